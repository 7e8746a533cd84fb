"""File formats against fixtures written by the reference's own C++ code
(tests/golden/make_io_golden.py): the unified data format
(DataContainer::load / save, core/src/datacontainer.cpp:209-615), the binary
mesh format (Mesh::saveBinaryV2 / loadBinaryV2, core/src/mesh_io.cpp:391-662)
and the VTK export (Mesh::exportVTK, core/src/mesh_io.cpp:674-992)."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from pygimli_gb300 import DataContainerERT, createData, geometricFactors
from pygimli_gb300.fileio import read_bms, read_unified, token_list
from pygimli_gb300.mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d

IO = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io")
EXP = os.path.join(IO, "expected")
with open(os.path.join(IO, "cases.json")) as _f:
    CASES = json.load(_f)
MESHES = ("mesh2d", "mesh2d_p2", "mesh3d", "mesh3d_p2")


@pytest.mark.parametrize("c", CASES, ids=[c["case"] for c in CASES])
def test_unified_load_matches_reference(c):
    """Sensors, token list and every field (sensor indices from zero) equal
    the reference loader's, bit for bit: aliases and unit scaling, comment
    and blank rows, duplicated sensors merged and unused ones dropped,
    invalid data marked or removed, r = u / i when only u and i are given."""
    z = np.load(os.path.join(EXP, c["case"] + ".npz"))
    u = read_unified(os.path.join(IO, c["file"]), c["from_one"], c["remove_invalid"])
    assert np.array_equal(u.sensors, z["sensors"])
    assert token_list(u.fields).split() == list(z["tokens"])
    for t in z["tokens"]:
        assert np.array_equal(u.fields[t], z["f_" + t], equal_nan=True), t


@pytest.mark.parametrize("c", CASES, ids=[c["case"] for c in CASES])
def test_unified_save_matches_reference(c, tmp_path):
    """DataContainerERT.load + save write the reference's text exactly."""
    d = DataContainerERT(os.path.join(IO, c["file"]), c["from_one"], c["remove_invalid"])
    for name, spec in c["formats"].items():
        out = tmp_path / f"{name}.txt"
        d.save(str(out), spec["format"], "x y z", spec["no_filter"])
        with open(os.path.join(EXP, f"{c['case']}_{name}.txt")) as f:
            assert out.read_text() == f.read(), name


def test_unified_container_fields():
    d = DataContainerERT(os.path.join(IO, "aliases.ohm"))
    assert d.sensorCount() == 5 and d.size() == 6
    assert d.abmn()[2].tolist() == [0, -1, 1, 2]           # b = 0 on file: pole at infinity
    assert np.allclose(d["u"][:2], [0.0125, 0.00825])       # u/mV scaled to V
    assert np.allclose(d["err"][:2], [0.03, 0.025])         # err/% scaled to a fraction
    assert np.allclose(d.sensorPosition(3), [3.0, 0.5, 0.0])  # x/mm, y/mm scaled to m
    assert d.exists("foo") and d.haveData("rhoa") and not d.haveData("k")
    d2 = DataContainerERT(os.path.join(IO, "line_basic.dat"))
    assert np.allclose(d2.additionalPoints(), [[0, 0, 0], [7, 0, 0]])


def test_unified_round_trip(tmp_path):
    """A generated scheme with geometric factors and apparent resistivities
    survives save + load (14 significant digits)."""
    d = createData(np.arange(12.0), "dd")
    d.set("k", geometricFactors(d, 2))
    rng = np.random.default_rng(3)
    d.set("rhoa", np.exp(rng.normal(4.0, 0.5, d.size())))
    d.set("err", np.full(d.size(), 0.03))
    p = tmp_path / "dd.dat"
    d.save(str(p), "a b m n rhoa err k")
    e = DataContainerERT(str(p))
    assert np.array_equal(e.abmn(), d.abmn())
    assert np.allclose(e.sensorPositions(), d.sensorPositions(), rtol=0, atol=1e-12)
    for t in ("rhoa", "err", "k"):
        assert np.allclose(e[t], d[t], rtol=1e-13, atol=0), t


def test_unified_bad_files(tmp_path):
    p = tmp_path / "bad.dat"
    p.write_text("3 4\n")
    with pytest.raises(ValueError):
        DataContainerERT(str(p))
    p.write_text("3\n0 0 0\n1 0 0\n")
    with pytest.raises(ValueError):
        DataContainerERT(str(p))
    p.write_text("2\n0 0 0\n1 0 0\n3\n# a b m n\n1 2 0 0\n")
    with pytest.raises(ValueError):
        DataContainerERT(str(p))


@pytest.mark.parametrize("name", MESHES)
def test_bms_round_trip_matches_reference(name, tmp_path):
    """Mesh.load of the reference's binary mesh and Mesh.save write the same
    bytes (all boundaries with left and right cells, the data map)."""
    src = os.path.join(EXP, name + ".bms")
    m = Mesh.load(src)
    out = m.save(str(tmp_path / name))
    assert out.endswith(".bms")
    with open(out, "rb") as a, open(src, "rb") as b:
        assert a.read() == b.read()
    assert sorted(m.dataMap()) == ["pot u", "res"]
    assert m.order == (2 if name.endswith("p2") else 1)


@pytest.mark.parametrize("name", MESHES)
def test_vtk_export_matches_reference(name, tmp_path):
    """exportVTK text equals the reference's except the creator line."""
    m = Mesh.load(os.path.join(EXP, name + ".bms"))
    modes = ((True, ""),) if name.endswith("p2") else ((True, ""), (False, "_bnd"))
    for cells, suffix in modes:
        out = m.exportVTK(str(tmp_path / (name + suffix)), cells)
        a = open(out).read().split("\n")
        with open(os.path.join(EXP, name + suffix + ".vtk")) as f:
            b = f.read().split("\n")
        assert a[1].startswith(f"d-{m.dim()}__ ")
        assert a[:1] + a[2:] == b[:1] + b[2:], suffix


@pytest.mark.parametrize("dim", (2, 3))
def test_bms_mesh_equals_generator(dim):
    """The reference built its mesh from the generators' arrays: the loaded
    file has the same nodes, cells and markers, and its marked boundaries
    are the generator's boundaries with their adjacent cells."""
    if dim == 2:
        g = create_para_mesh_2d(np.arange(4.0), para_dx=0.5, para_depth=1.5, para_boundary=1.0)
    else:
        g = create_box_mesh_3d(np.array([(0.0, 0.0), (2.0, 0.0)]), h=1.0, para_margin=(1, 1), para_depth=1.0,
                               outer=6.0, growth=4.0, depth_growth=4.0)
    m = Mesh.load(os.path.join(EXP, f"mesh{dim}d.bms"))
    assert np.array_equal(m.nodes, g.nodes)
    assert np.array_equal(m.cells, g.cells)
    assert np.array_equal(m.cell_markers, g.cell_markers)
    assert np.array_equal(m.node_markers, g.node_markers)
    mk = m.boundary_markers != 0
    key = lambda b: tuple(sorted(b))  # noqa: E731
    gb = {key(b): (int(k), int(c)) for b, k, c in zip(g.boundaries, g.boundary_markers, g.boundary_cells)}
    mb = {key(b): (int(k), int(c)) for b, k, c in zip(m.boundaries[mk], m.boundary_markers[mk],
                                                      m.boundary_cells[mk])}
    assert mb == gb


def test_bms_generated_round_trip(tmp_path):
    g = create_para_mesh_2d(np.arange(6.0), para_dx=0.5, para_depth=2.0).createP2()
    g["rho"] = np.arange(g.cellCount(), dtype=np.float64)
    out = g.save(str(tmp_path / "p2.bms"))
    r = read_bms(out)
    assert r["dim"] == 2 and r["cells"].shape == g.cells.shape
    m = Mesh.load(out)
    for a in ("nodes", "cells", "cell_markers", "node_markers", "boundaries", "boundary_markers",
              "boundary_cells"):
        assert np.array_equal(getattr(m, a), getattr(g, a)), a
    assert np.array_equal(m["rho"], g["rho"])


def test_loaded_mesh_forward_equals_generator():
    """The reference's file of a mesh (every facet a boundary, half the outer
    ones with only a right cell) gives the oracle the same apparent
    resistivities as the generator's mesh."""
    from oracle import ert_oracle as O
    g = create_para_mesh_2d(np.arange(4.0), para_dx=0.5, para_depth=1.5, para_boundary=1.0)
    m = Mesh.load(os.path.join(EXP, "mesh2d.bms"))
    d = createData(np.arange(4.0), "dd")
    d.set("k", geometricFactors(d, 2))
    rho = 50.0 + np.arange(g.cellCount()) % 7 * 10.0
    k, w = np.array([0.05, 0.5, 2.0]), np.array([1.0, 0.7, 0.3])
    r_g, _ = O.Problem(g, d.sensorPositions(), d.abmn(), d["k"], k, w).response(rho)
    r_m, _ = O.Problem(m, d.sensorPositions(), d.abmn(), d["k"], k, w).response(rho)
    assert np.allclose(r_m, r_g, rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", ("mesh2d", "mesh3d"))
def test_bms_first_format(name, tmp_path):
    """The first binary format (Mesh::saveBinary, read by Mesh::load when the
    v2/v3 header does not match): same mesh as the v3 file, and saveBinary
    writes the reference's bytes."""
    v3 = Mesh.load(os.path.join(EXP, name + ".bms"))
    src = os.path.join(EXP, name + "_v1.bms")
    v1 = Mesh.load(src)
    for a in ("nodes", "cells", "cell_markers", "node_markers", "boundaries", "boundary_markers",
              "boundary_cells", "boundary_left_cells", "boundary_right_cells"):
        assert np.array_equal(getattr(v1, a), getattr(v3, a)), a
    out = v1.saveBinary(str(tmp_path / name))
    with open(out, "rb") as a, open(src, "rb") as b:
        assert a.read() == b.read()


@pytest.mark.parametrize("name", MESHES)
def test_vtk_import(name):
    """Mesh::importVTK of the reference's VTK files: the nodes, cells (a
    Tetrahedron10 in the file's node order, as the reference reads it back),
    cell markers and data arrays of the mesh it exported; no boundaries."""
    m = Mesh.load(os.path.join(EXP, name + ".bms"))
    v = Mesh.load(os.path.join(EXP, name + ".vtk"))
    assert v.dim() == m.dim() and v.boundaryCount() == 0
    assert np.allclose(v.nodes, m.nodes, rtol=1e-13, atol=1e-13)  # the file holds 14 significant digits
    cells = m.cells[:, [0, 1, 2, 3, 4, 7, 5, 6, 9, 8]] if m.cells.shape[1] == 10 else m.cells
    assert np.array_equal(v.cells, cells)
    assert np.array_equal(v.cell_markers, m.cell_markers)
    assert np.allclose(v["res"], m["res"], rtol=1e-13, atol=0)
    assert np.allclose(v["pot_u"], m["pot u"], rtol=1e-13, atol=1e-300)
