"""Uniform mesh refinement on the GPU (``ertgb_refine``): the quadratic mesh
of ``Mesh::createP2`` and the H2 mesh of ``Mesh::createH2`` with the
reference's numbering (core/src/mesh.cpp:1278-1600).  pyGIMLi refines every
parameter mesh given to the forward operator this way
(pygimli/frameworks/modelling.py:682-699); ``ERTModelling.setMesh`` calls
these.  ``Mesh.createH2`` / ``Mesh.createP2`` are the host restatements the
results are tested against.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .mesh import Mesh

P2, H2 = 1, 2


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def refine(mesh, mode, device=0):
    """Refined copy of the linear ``mesh`` (mode ``P2`` or ``H2``) computed on
    CUDA device ``device``."""
    if mesh.order != 1:
        raise ValueError("refinement needs a linear mesh")
    lib = _native.load()
    nodes = np.ascontiguousarray(mesh.nodes, np.float64)
    nm = np.ascontiguousarray(mesh.node_markers, np.int32)
    cells = np.ascontiguousarray(mesh.cells, np.int32)
    cm = np.ascontiguousarray(mesh.cell_markers, np.int32)
    bnd = np.ascontiguousarray(mesh.boundaries, np.int32)
    bm = np.ascontiguousarray(mesh.boundary_markers, np.int32)
    bc = np.ascontiguousarray(mesh.boundary_cells, np.int32)
    h = ctypes.c_void_p()
    _native.check(None, lib.ertgb_refine(int(device), mesh.dim(), int(mode), len(nodes), _ptr(nodes), _ptr(nm),
                                         len(cells), _ptr(cells), _ptr(cm), len(bnd), _ptr(bnd), _ptr(bm), _ptr(bc),
                                         ctypes.byref(h)))
    try:
        sz = [ctypes.c_int64() for _ in range(5)]
        _native.check(None, lib.ertgb_refined_sizes(h, *[ctypes.byref(x) for x in sz]))
        n, C, nv, B, nvb = [x.value for x in sz]
        out = dict(xyz=np.empty((n, 3)), nm=np.empty(n, np.int32), cells=np.empty((C, nv), np.int32),
                   cm=np.empty(C, np.int32), bnd=np.empty((B, nvb), np.int32), bm=np.empty(B, np.int32),
                   bc=np.empty(B, np.int32))
        _native.check(None, lib.ertgb_refined_get(h, *[_ptr(out[k]) for k in ("xyz", "nm", "cells", "cm", "bnd", "bm",
                                                                                "bc")]))
    finally:
        lib.ertgb_refined_free(h)
    return Mesh(mesh.dim(), out["xyz"], out["cells"], out["cm"], out["nm"], out["bnd"], out["bm"], out["bc"],
                check=False)


def createP2(mesh, device=0):
    return refine(mesh, P2, device)


def createH2(mesh, device=0):
    return refine(mesh, H2, device)
