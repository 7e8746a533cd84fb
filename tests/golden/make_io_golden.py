"""Generate the file-format fixtures of tests/golden/io/ with the reference's
own C++ code (oracle/_ref/libgimli_ref.so, built by oracle/Makefile, driven
through oracle/ref_driver.py).

Run from the repository root after ``make -C oracle``:

    python tests/golden/make_io_golden.py

Unified data format: every hand-written input file in tests/golden/io/
(``*.dat``, ``*.ohm``) is loaded with ``DataContainerERT::load`` and the
parsed sensors and fields are stored in ``expected/<case>.npz``; the same
container is written back with ``DataContainer::save`` into
``expected/<case>_<format>.txt``.

Meshes: small meshes are built by the reference from the generators' arrays
(createNeighborInfos, optionally createP2), get a cell and a node data
array, and are written with ``Mesh::saveBinaryV2`` (``expected/<mesh>.bms``)
and ``Mesh::exportVTK`` (``expected/<mesh>.vtk``, cells; for linear meshes also
``expected/<mesh>_bnd.vtk``, boundaries, and the first binary format of
``Mesh::saveBinary`` in ``expected/<mesh>_v1.bms``).
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_driver as R  # noqa: E402
from pygimli_gb300.mesh import create_box_mesh_3d, create_para_mesh_2d  # noqa: E402

IO = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io")
EXP = os.path.join(IO, "expected")

# cases.json: case name, input file, sensor indices from one, remove invalid
# data, and the formats ({name: {format, no_filter}}) written back
with open(os.path.join(IO, "cases.json")) as f:
    DATA_CASES = json.load(f)


def data_cases():
    L = R.lib()
    for c in DATA_CASES:
        case, fname, from_one, remove = c["case"], c["file"], c["from_one"], c["remove_invalid"]
        src = os.path.join(IO, fname)
        h = L.ref_data_load(os.fsencode(src), int(from_one), int(remove))
        if not h:
            raise RuntimeError(L.ref_last_error().decode())
        try:
            sensors, tokens, fields = R.data_load(src, from_one, remove)
            np.savez(os.path.join(EXP, f"{case}.npz"), sensors=sensors, tokens=np.array(tokens),
                     **{f"f_{t}": v for t, v in fields.items()})
            for fmt_name, spec in c["formats"].items():
                fmt, no_filter = spec["format"], spec["no_filter"]
                out = os.path.join(EXP, f"{case}_{fmt_name}.txt")
                R._check(L.ref_data_save(h, os.fsencode(out), fmt.encode(), b"x y z", int(no_filter)))
        finally:
            L.ref_data_free(h)
        print(case, len(sensors), "sensors,", len(fields["valid"]), "data")


def _meshes():
    m2 = create_para_mesh_2d(np.arange(4.0), para_dx=0.5, para_depth=1.5, para_boundary=1.0)
    e = np.array([(0.0, 0.0), (2.0, 0.0)])
    m3 = create_box_mesh_3d(e, h=1.0, para_margin=(1, 1), para_depth=1.0, outer=6.0, growth=4.0, depth_growth=4.0)
    return [("mesh2d", m2, False), ("mesh2d_p2", m2, True), ("mesh3d", m3, False), ("mesh3d_p2", m3, True)]


def mesh_cases():
    for name, mesh, p2 in _meshes():
        rm = R.RefMesh(mesh, p2=p2)
        a = rm.arrays()
        C, n = len(a["cells"]), len(a["nodes"])
        rm.add_data("res", 10.0 + np.arange(C) * 0.5)
        rm.add_data("pot u", np.linspace(-1.0, 1.0, n) ** 3)
        rm.save_bms(os.path.join(EXP, name + ".bms"))
        rm.export_vtk(os.path.join(EXP, name + ".vtk"), True)
        if not p2:
            rm.export_vtk(os.path.join(EXP, name + "_bnd.vtk"), False)
            rm.save_bms_v1(os.path.join(EXP, name + "_v1.bms"))
            v1 = R.RefMesh(path=os.path.join(EXP, name + "_v1.bms"))  # the reference's fallback reader
            b = v1.arrays()
            assert all(np.array_equal(a[k], b[k]) for k in a), "v1 round trip"
            v1.close()
        print(name, n, "nodes,", C, "cells,", len(a["boundaries"]), "boundaries")
        rm.close()


def main():
    os.makedirs(EXP, exist_ok=True)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)  # the reference's validity check writes 'invalid.data' into the working directory
        try:
            data_cases()
            mesh_cases()
        finally:
            os.chdir(cwd)


if __name__ == "__main__":
    main()
