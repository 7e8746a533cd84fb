"""The reference arm's timing of full steps of the reference's own C++
(``bench.py --impl reference --ref-cpp``) where its library is built: one
response + createJacobian on the 2.5-D line (configuration 1)."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_cpp_arm():
    sys.path.insert(0, ROOT)
    from oracle import ref_driver
    if not ref_driver.available():
        pytest.skip("the reference's library is not built here (make -C oracle needs its sources)")
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--ref-cpp", "--workload", "line_2d",
                          "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])
    assert d["impl"] == "reference" and d["cpu_baseline"]["kind"] == "reference"
    assert d["value"] > 0 and d["steps"] == 1 and "createJacobian" in d["cpu_baseline"]["sample"]
