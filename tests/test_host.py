"""Host-side logic (no GPU): scheme generators, synthetic meshes, the C ABI
library build, its exported symbols and its error path without a device."""
import ctypes
import os
import re

import numpy as np
import pytest

from pygimli_gb300.data import createData, grid_line_scheme, grid_scheme_3d
from pygimli_gb300.mesh import create_box_mesh_3d, create_para_mesh_2d

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dipole_dipole_count():
    # 41 electrodes, default dipole-dipole: 741 configurations
    d = createData(np.arange(41.0), "dd")
    assert d.size() == 741
    ab = d.abmn()
    assert np.all(ab[:, 1] == ab[:, 0] + 1) and np.all(ab[:, 3] == ab[:, 2] + 1)
    assert np.all(ab[:, 2] > ab[:, 1])


def test_pole_dipole_and_wenner():
    pd = createData(np.arange(11.0), "pd").abmn()
    assert np.all(pd[:, 1] == -1) and np.all(pd[:, 3] == pd[:, 2] + 1)
    wa = createData(np.arange(11.0), "wa").abmn()
    s = wa[:, 2] - wa[:, 0]
    assert np.all(wa[:, 3] - wa[:, 2] == s) and np.all(wa[:, 1] - wa[:, 3] == s)


def test_grid_scheme_indices():
    ab = grid_line_scheme((12, 8), "dd")
    assert ab.min() >= 0 and ab.max() < 96 and len(ab) == 540
    ab = grid_scheme_3d(12, 8)
    assert len(ab) == 5336 and ab.max() < 96 and len(np.unique(ab, axis=0)) == len(ab)
    assert np.all((ab[:, 1] == -1) | (ab[:, 1] != ab[:, 0]))


def test_para_mesh_2d_config():
    m = create_para_mesh_2d(np.arange(41.0), para_dx=0.25, para_depth=10.0)
    assert 3000 <= m.nodeCount() <= 4500 and 5500 <= m.cellCount() <= 8000
    assert np.sum(m.node_markers == -99) == 41
    assert set(np.unique(m.boundary_markers)) == {-1, -2}
    assert np.all(m.boundary_cells >= 0)
    assert np.all(m.cellSizes() > 0)


def test_box_mesh_3d_config():
    e = np.array([(x, y) for x in np.arange(12) * 4.0 for y in np.arange(8) * 4.0])
    m = create_box_mesh_3d(e)
    assert 80000 <= m.nodeCount() <= 100000 and 450000 <= m.cellCount() <= 560000
    assert np.sum(m.node_markers == -99) == 96
    assert np.all(m.boundary_cells >= 0)
    lo, hi = m.nodes.min(0), m.nodes.max(0)
    assert np.allclose(lo, [-500, -500, -500]) and np.allclose(hi, [500, 500, 0])


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "ertgb.h")).read()
    return sorted(set(re.findall(r"\b(ertgb_[a-z_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def built_lib():
    from pygimli_gb300 import build
    return build.build()


def test_library_exports_every_header_symbol(built_lib):
    L = ctypes.CDLL(built_lib)
    syms = _header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), s
    from pygimli_gb300 import _native
    assert set(_native.SIGNATURES) == set(syms)


def test_library_fails_loudly_without_device(built_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from pygimli_gb300 import _native
    L = _native.load()
    ctx = ctypes.c_void_p()
    rc = L.ertgb_create(ctypes.byref(ctx), 0)
    assert rc == _native.CUDA_ERROR
    assert b"cuda" in L.ertgb_last_error(None).lower()


def test_estimate_error_forms():
    """estimateError (pygimli/physics/ert/ert.py:482-540) on hand values."""
    import numpy as np
    from pygimli_gb300.data import DataContainerERT, estimateError
    d = DataContainerERT(np.array([[0.0, 0, 0], [1, 0, 0], [2, 0, 0], [3, 0, 0]]), np.array([[0, 1, 2, 3]] * 2))
    d.set("rhoa", np.array([100.0, 50.0]))
    d.set("k", np.array([10.0, 20.0]))
    assert np.allclose(estimateError(d, 0.03, absoluteError=1.0), [0.04, 0.05])
    assert np.allclose(estimateError(d, 3.0), [0.03, 0.03])                    # percent
    u = np.array([100.0 / 10.0, 50.0 / 20.0]) * 0.1
    assert np.allclose(estimateError(d, 0.02, absoluteUError=1e-3), 1e-3 / u + 0.02)
    d.set("u", np.array([2.0, 4.0]))
    assert np.allclose(estimateError(d, 0.02, absoluteUError=1e-2), [0.025, 0.0225])


def test_data_container_editing():
    """remove / resize / add / translate / scale of DataContainerERT
    (core/src/datacontainer.cpp:139-168, 742-767, 930-940)."""
    import numpy as np
    from pygimli_gb300.data import createData
    d = createData(np.arange(6.0), "dd")
    n = d.size()
    d.set("rhoa", np.arange(n, dtype=float) + 1.0)
    d.remove(d["rhoa"] > n - 2)
    assert d.size() == n - 2 and d["rhoa"].max() == n - 2
    e = createData(np.arange(2.0, 8.0), "dd")         # shares sensors x = 2..5
    e.set("rhoa", np.full(e.size(), 7.0))
    m = d.size()
    d.add(e)
    assert d.sensorCount() == 8 and d.size() == m + e.size()
    assert np.allclose(d.sensorPositions()[d.abmn()[m:, 0], 0], e.sensorPositions()[e.abmn()[:, 0], 0])
    assert np.all(d["rhoa"][m:] == 7.0)
    d.resize(d.size() + 2)
    assert np.all(d.abmn()[-2:] == -1) and np.all(d["rhoa"][-2:] == 0.0)
    d.translate([1.0, 0.0])
    d.scale([2.0, 1.0, 1.0])
    assert np.isclose(d.sensorPosition(0)[0], 2.0)


def test_flip_imag():
    """The complex flip convention's vector helper (pg.utils.squeezeComplex
    with conj): [Re..., Im...] out, the imaginary part negated on request."""
    from pygimli_gb300.ert import flip_imag
    v = np.array([1.0, 2.0, 3.0, -4.0])
    assert np.array_equal(flip_imag(v, True), [1.0, 2.0, -3.0, 4.0])
    assert np.array_equal(flip_imag(v, False), v)
    assert np.array_equal(flip_imag(np.array([1 - 2j, 3 + 4j]), True), [1.0, 3.0, 2.0, -4.0])
    with pytest.raises(ValueError):
        flip_imag(np.ones(3), True)


def test_geometric_factors_hand_formula():
    """Half-space geometric factors against the closed form with mirror
    sources that the reference checks them with (pygimli/testing/
    test_geometricFactors.py): surface and buried electrodes."""
    from pygimli_gb300.data import DataContainerERT, geometricFactors

    def hand(p):
        d1, d2 = np.zeros(4), np.zeros(4)
        for i, (c, q) in enumerate(((0, 2), (0, 3), (1, 2), (1, 3))):
            d1[i] = np.sqrt(np.sum((p[c] - p[q]) ** 2))
            d2[i] = np.sqrt(np.sum((p[c, :2] - p[q, :2]) ** 2) + (-p[c, 2] - p[q, 2]) ** 2)
        dI = 1.0 / d1 + 1.0 / d2
        return 4.0 * np.pi / (dI[0] - dI[1] - dI[2] + dI[3])

    rng = np.random.default_rng(1)
    for z in ((0.0, 0.0, 0.0, 0.0), (-1.0, -2.0, -0.5, -3.0), (0.0, -1.0, 0.0, -2.0)):
        p = np.column_stack([np.arange(4.0), rng.normal(size=4), np.array(z)])
        d = DataContainerERT(p, np.array([[0, 1, 2, 3]], np.int32))
        np.testing.assert_allclose(geometricFactors(d, 3), [hand(p)], rtol=1e-13)
