"""H2 / P2 refinement on the GPU (``ertgb_refine``) against the host
restatements ``create_h2`` / ``create_p2``, which tests/test_oracle.py pins
to the reference's own Mesh::createH2 / createP2 (core/src/mesh.cpp:
1278-1600): node coordinates, node markers, cells, cell markers,
boundaries, boundary markers and the boundaries' adjacent cells equal."""
from __future__ import annotations

import os
import time

import numpy as np
import pytest

from pygimli_gb300.mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d

IO = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io", "expected")


@pytest.fixture(scope="module")
def refine():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import build
    build.build()
    from pygimli_gb300 import refine as r
    return r


def assert_same(dev, host, outer_only=False):
    assert np.array_equal(dev.nodes, host.nodes)
    assert np.array_equal(dev.node_markers, host.node_markers)
    assert np.array_equal(dev.cells, host.cells)
    assert np.array_equal(dev.cell_markers, host.cell_markers)
    assert np.array_equal(dev.boundaries, host.boundaries)
    assert np.array_equal(dev.boundary_markers, host.boundary_markers)
    sel = host.boundary_markers != 0 if outer_only else slice(None)
    assert np.array_equal(dev.boundary_cells[sel], host.boundary_cells[sel])


def _meshes():
    m2 = create_para_mesh_2d(np.arange(8.0), para_dx=0.5, para_depth=3.0)
    m3 = create_box_mesh_3d(np.array([(x, y) for x in (0.0, 2.0, 4.0) for y in (0.0, 2.0)]), h=1.0,
                            para_margin=(2, 2), para_depth=3.0, outer=30.0, growth=2.0, depth_growth=2.0)
    return {"2d": m2, "3d": m3}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["2d", "3d"])
@pytest.mark.parametrize("mode", ["H2", "P2", "H2P2"])
def test_device_refinement_equals_host(refine, name, mode):
    m = _meshes()[name]
    if mode == "H2":
        dev, host = refine.createH2(m), m.createH2()
    elif mode == "P2":
        dev, host = refine.createP2(m), m.createP2()
    else:  # the forward mesh with _refineP2: H2, then P2
        dev, host = refine.createP2(refine.createH2(m)), m.createH2().createP2()
    assert_same(dev, host)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mesh2d", "mesh3d"])
def test_device_refinement_of_reference_file(refine, name):
    """A mesh written by the reference (every facet a boundary, some outer
    facets with only a right cell): equal to the host refinement; every
    boundary's adjacent cell holds the boundary."""
    m = Mesh.load(os.path.join(IO, name + ".bms"))
    for dev, host in ((refine.createH2(m), m.createH2()), (refine.createP2(m), m.createP2())):
        assert_same(dev, host, outer_only=True)
        nv = dev.dim() + 1
        for b, c in zip(dev.boundaries[:, :dev.dim()], dev.boundary_cells):
            assert c >= 0 and set(b.tolist()) <= set(dev.cells[c, :nv].tolist())


@pytest.mark.gpu
def test_device_refinement_at_scale(refine):
    """box_3d's parameter mesh (485,640 tetrahedra): H2 gives 3,885,120
    tetrahedra, identical to the host restatement; the device is faster."""
    from pygimli_gb300.synthetic import box_3d
    r = box_3d()
    m = r[0] if isinstance(r, tuple) else r
    refine.createH2(m)  # first call: CUDA context, module load
    t0 = time.perf_counter()
    dev = refine.createH2(m)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    host = m.createH2()
    t_host = time.perf_counter() - t0
    print(f"H2 of {m.cellCount()} cells: device {t_dev:.3f} s, host {t_host:.3f} s")
    assert dev.cellCount() == 8 * m.cellCount()
    assert_same(dev, host)
    assert t_dev < t_host


@pytest.mark.gpu
def test_refine_rejects_bad_input(refine):
    from pygimli_gb300._native import ErtgbError
    m = _meshes()["2d"]
    bad = Mesh(2, m.nodes, m.cells, m.cell_markers, m.node_markers, m.boundaries, m.boundary_markers,
               m.boundary_cells)
    bad.cells = bad.cells.copy()
    bad.cells[3, 1] = m.nodeCount() + 5
    with pytest.raises(ErtgbError, match="out of range"):
        refine.createH2(bad)
