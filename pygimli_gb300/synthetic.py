"""Seeded synthetic ERT workloads with the shapes of the benchmark
configurations (no field data is used anywhere):

``line_2d``  2.5-D, 41 surface electrodes at 1 m, dipole-dipole (741 data),
             para mesh paraDX 0.25 / paraDepth 10 m (~3.6k nodes, ~6.8k
             triangles), resistivity log-uniform in [50, 200] Ohm m with a
             10 and a 1000 Ohm m rectangle.
``box_3d_large`` 3-D, 256 electrodes on a 16 x 16 grid at 4 m, dipole-dipole +
             pole-dipole + Wenner lines (~8k data), ~807k tetrahedra / ~145k nodes
             (P1; ``p2=True`` refines the whole mesh with create_p2), resistivity
             as ``box_3d``.
``box_3d``   3-D, 96 electrodes on a 12 x 8 grid at 4 m, 5336 dipole-dipole /
             pole-dipole / cross-line data, tetrahedral mesh of the para box
             padded to +-500 m (~88k nodes, ~486k tetrahedra), resistivity
             log-normal (mu = ln 100, sigma = 1) with three ellipsoids.
             ``scheme="inline"`` keeps only the 540 inline dipole-dipole
             data (same mesh and sources; a 2 GB instead of a 21 GB
             Jacobian, used for profiler captures).
"""
from __future__ import annotations

import numpy as np

from .data import DataContainerERT, createData, geometricFactors, grid_line_scheme, grid_scheme_3d
from .mesh import create_box_mesh_3d, create_para_mesh_2d


def box_3d_large(seed=8, p2=False):
    nx = ny = 16
    mesh, data, rho = box_3d(seed=seed, nx=nx, ny=ny, scheme="inline")
    ab = np.vstack([grid_line_scheme((nx, ny), kind) for kind in ("dd", "pd", "wa")])
    data = DataContainerERT(data.sensorPositions(), ab)
    data.set("k", geometricFactors(data, 3))
    if p2:
        mesh = mesh.createP2()
    return mesh, data, rho


def line_2d(seed=1):
    xs = np.arange(41.0)
    mesh = create_para_mesh_2d(xs, para_dx=0.25, para_depth=10.0)
    data = createData(xs, "dd")
    data.set("k", geometricFactors(data, 2))
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.uniform(np.log(50.0), np.log(200.0), mesh.cellCount()))
    c = mesh.cellCenters()
    x1, x2 = rng.uniform(5.0, 17.0), rng.uniform(23.0, 35.0)
    rho[(np.abs(c[:, 0] - x1) < 3.0) & (c[:, 1] > -4.0) & (c[:, 1] < -1.0)] = 10.0
    rho[(np.abs(c[:, 0] - x2) < 3.0) & (c[:, 1] > -6.0) & (c[:, 1] < -2.0)] = 1000.0
    return mesh, data, rho


def box_3d(seed=7, nx=12, ny=8, spacing=4.0, scheme="full", **mesh_kw):
    e = np.array([(x, y) for x in np.arange(nx) * spacing for y in np.arange(ny) * spacing])
    mesh = create_box_mesh_3d(e, **mesh_kw)
    ab = grid_scheme_3d(nx, ny) if scheme == "full" else grid_line_scheme((nx, ny), "dd")
    data = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), ab)
    data.set("k", geometricFactors(data, 3))
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.normal(np.log(100.0), 1.0, mesh.cellCount()))
    c = mesh.cellCenters()
    span = np.array([(nx - 1) * spacing, (ny - 1) * spacing])
    for val in (10.0, 1000.0, 30.0):
        ctr = np.array([rng.uniform(0.1, 0.9) * span[0], rng.uniform(0.1, 0.9) * span[1],
                        -rng.uniform(3.0, 12.0)])
        ax = rng.uniform([3.0, 3.0, 1.5], [8.0, 6.0, 4.0])
        inside = np.sum(((c - ctr) / ax) ** 2, axis=1) <= 1.0
        rho[inside] = val
    return mesh, data, rho


def random_models(mesh, count, seed=0, n_blocks=(1, 4), contrast=(1e2, 1e5)):
    """Training / evaluation models on ``mesh``: log-normal background
    (mu = ln 100, sigma = 1) plus 1-4 blocky inclusions (ellipsoids in 3-D,
    rectangles in 2-D) whose resistivity sits a factor drawn log-uniformly in
    ``contrast`` above or below the background median."""
    rng = np.random.default_rng(seed)
    c = mesh.cellCenters()
    d = mesh.dim()
    lo = np.percentile(c[:, :d], 5, axis=0)
    hi = np.percentile(c[:, :d], 95, axis=0)
    # the inclusions live in the upper part of the model (the para region)
    depth_axis = d - 1
    span = hi - lo
    lo_in = lo.copy()
    lo_in[depth_axis] = hi[depth_axis] - 0.3 * span[depth_axis]
    out = []
    for _ in range(count):
        rho = np.exp(rng.normal(np.log(100.0), 1.0, mesh.cellCount()))
        for _ in range(int(rng.integers(n_blocks[0], n_blocks[1] + 1))):
            ctr = rng.uniform(lo_in, hi)
            ax = rng.uniform(0.03, 0.15, d) * span
            f = 10 ** rng.uniform(np.log10(contrast[0]), np.log10(contrast[1])) ** 0.5
            val = 100.0 * (f if rng.random() < 0.5 else 1.0 / f)
            if d == 3:
                inside = np.sum(((c - ctr) / ax) ** 2, axis=1) <= 1.0
            else:
                inside = np.all(np.abs(c[:, :2] - ctr) <= ax, axis=1)
            rho[inside] = val
        out.append(rho)
    return out


def batch_2d(n_problems=64, seed=3, nodes=(2000, 60000), electrodes=(24, 72)):
    """Independent 2.5-D problems for the batched solver: node counts drawn
    log-uniformly in ``nodes``, 24-72 electrodes at 1 m, dipole-dipole plus
    Wenner data, log-normal resistivity (mu = ln 100, sigma = 1) with a 10 and
    a 1000 Ohm m rectangle.  Returns a list of (mesh, data, rho)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_problems):
        target = float(np.exp(rng.uniform(np.log(nodes[0]), np.log(nodes[1]))))
        ne = int(rng.integers(electrodes[0], electrodes[1] + 1))
        xs = np.arange(float(ne))
        depth = ne / 4.0
        n2 = create_para_mesh_2d(xs, para_dx=0.5, para_depth=depth).nodeCount()
        n4 = create_para_mesh_2d(xs, para_dx=0.25, para_depth=depth).nodeCount()
        slope = (n4 - n2) / 2.0  # nodes grow affinely in 1 / para_dx
        k = max(1, int(round(2 + (target - n2) / slope)))
        mesh = create_para_mesh_2d(xs, para_dx=1.0 / k, para_depth=depth)
        while k > 1 and mesh.nodeCount() > 1.1 * nodes[1]:
            k -= 1
            mesh = create_para_mesh_2d(xs, para_dx=1.0 / k, para_depth=depth)
        dd = createData(xs, "dd")
        wa = createData(xs, "wa")
        data = DataContainerERT(dd.sensorPositions(), np.vstack([dd.abmn(), wa.abmn()]))
        data.set("k", geometricFactors(data, 2))
        rho = np.exp(rng.normal(np.log(100.0), 1.0, mesh.cellCount()))
        c = mesh.cellCenters()
        for val in (10.0, 1000.0):
            x0 = rng.uniform(0.15, 0.85) * (ne - 1)
            z0 = -rng.uniform(0.1, 0.6) * depth
            rho[(np.abs(c[:, 0] - x0) < 0.08 * ne) & (np.abs(c[:, 1] - z0) < 0.1 * depth)] = val
        out.append((mesh, data, rho))
    return out
