"""Test infrastructure only: ctypes driver of the reference's own C++ ERT
modelling code (oracle/_ref/libgimli_ref.so, built by oracle/Makefile from
the reference sources with the project's entry shim oracle/ref_shim.cpp).

The reference normally factors each system matrix with CHOLMOD
(core/src/bert/dcfemmodelling.cpp:2199-2210), which is not available here.
``RefModelling`` injects an FP64 sparse LU (scipy SuperLU, partial pivoting
off-diagonal threshold 0 so the symmetric matrix is factored like a
Cholesky) through the reference's own solver hook
(core/src/bert/dcfemmodelling.h:266 setSolver).  Each captured system matrix
is kept so tests can compare the assembled CSR with the product's.

Only tests and the fixture generator use this module.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libgimli_ref.so")

_FACTOR = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_void_p)
_SOLVE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p)

_CFACTOR = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                            ctypes.c_void_p, ctypes.c_void_p)
_CSOLVE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p)

_lib = None


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.ref_create.restype = vp
        L.ref_create.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int, vp, vp,
                                 ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp, ctypes.c_int, vp,
                                 vp, ctypes.c_int, ctypes.c_int]
        L.ref_create_ex.restype = vp
        L.ref_create_ex.argtypes = L.ref_create.argtypes + [ctypes.c_int, ctypes.c_int, vp]
        L.ref_mesh_sizes.argtypes = [vp, vp, vp, vp, vp, vp]
        L.ref_mesh_arrays.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.ref_destroy.argtypes = [vp]
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_set_solver.argtypes = [vp, _FACTOR, _SOLVE]
        L.ref_set_threads.argtypes = [vp, ctypes.c_int]
        L.ref_set_complex_solver.argtypes = [vp, _CFACTOR, _CSOLVE]
        L.ref_response_complex.argtypes = [vp, vp, ctypes.c_int, vp]
        L.ref_jacobian_complex.argtypes = [vp, vp, ctypes.c_int, vp, vp, vp, vp]
        L.ref_set_kw.argtypes = [vp, ctypes.c_int, vp, vp]
        L.ref_set_primary.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
        L.ref_kw_count.argtypes = [vp]
        L.ref_get_kw.argtypes = [vp, vp, vp]
        L.ref_electrode_nodes.argtypes = [vp, vp]
        L.ref_geometric_factors.argtypes = [vp, vp]
        L.ref_response.argtypes = [vp, vp, ctypes.c_int, vp]
        L.ref_calculate_dipole.argtypes = [vp, vp, ctypes.c_int, vp, vp]
        L.ref_subpot_shape.argtypes = [vp, vp, vp]
        L.ref_subpotentials.argtypes = [vp, vp]
        L.ref_jacobian.argtypes = [vp, vp, ctypes.c_int, vp, vp, vp]
        L.ref_assemble.argtypes = [vp, vp, ctypes.c_double, vp, vp, vp, vp, vp, vp]
        L.ref_primary.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, vp]
        L.ref_besselK0.restype = ctypes.c_double
        L.ref_besselK0.argtypes = [ctypes.c_double]
        L.ref_besselK1.restype = ctypes.c_double
        L.ref_besselK1.argtypes = [ctypes.c_double]
        L.ref_gauss_legendre.argtypes = [ctypes.c_int, vp, vp]
        L.ref_gauss_laguerre.argtypes = [ctypes.c_int, vp, vp]
        cs = ctypes.c_char_p
        L.ref_mesh_create.restype = vp
        L.ref_mesh_create.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int, vp, vp,
                                      ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int]
        L.ref_mesh_load.restype = vp
        L.ref_mesh_load.argtypes = [cs]
        L.ref_mesh_dim.argtypes = [vp]
        L.ref_mesh_save_bms.argtypes = [vp, cs]
        L.ref_mesh_save_bms_v1.argtypes = [vp, cs]
        L.ref_mesh_boundary_cells.argtypes = [vp, vp, vp]
        L.ref_mesh_add_data.argtypes = [vp, cs, ctypes.c_int, vp]
        L.ref_mesh_export_vtk.argtypes = [vp, cs, ctypes.c_int]
        L.ref_regions.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, ctypes.c_int, vp, vp, vp, vp, vp]
        L.ref_region_constraints.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, ctypes.c_int, vp,
                                             vp, ctypes.c_int, vp, vp, vp, vp, vp, vp]
        L.ref_data_load.restype = vp
        L.ref_data_load.argtypes = [cs, ctypes.c_int, ctypes.c_int]
        L.ref_data_free.argtypes = [vp]
        L.ref_data_sizes.argtypes = [vp, vp, vp]
        L.ref_data_sensors.argtypes = [vp, vp]
        L.ref_data_tokens.argtypes = [vp, cs, ctypes.c_int]
        L.ref_data_get.argtypes = [vp, cs, vp]
        L.ref_data_save.argtypes = [vp, cs, cs, cs, ctypes.c_int]
        L.ref_cgls.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                               ctypes.c_double, vp, ctypes.c_int, ctypes.c_double]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(rc):
    if rc != 0:
        raise RuntimeError("reference call failed: " + lib().ref_last_error().decode())


class RefModelling:
    """The reference's DCSRMultiElectrodeModelling (sr=True) or
    DCMultiElectrodeModelling (sr=False: total potential, complete electrode
    model, bypass electrodes) on a given mesh/scheme."""

    def __init__(self, mesh, sensors, abmn, kfac=None, threads=1, keep_matrices=False, p2=False, h2=False,
                 sr=True, contact_impedance=None):
        L = lib()
        self.mesh = mesh
        self._keep = [np.ascontiguousarray(mesh.nodes, np.float64),
                      np.ascontiguousarray(mesh.node_markers, np.int32),
                      np.ascontiguousarray(mesh.cells, np.int32),
                      np.ascontiguousarray(mesh.cell_markers, np.int32),
                      np.ascontiguousarray(mesh.boundaries, np.int32),
                      np.ascontiguousarray(mesh.boundary_markers, np.int32),
                      np.ascontiguousarray(sensors, np.float64).reshape(-1, 3),
                      np.ascontiguousarray(abmn, np.int32).reshape(-1, 4)]
        kf = None if kfac is None else np.ascontiguousarray(kfac, np.float64)
        self._keep.append(kf)
        nodes, nm, cells, cm, bnd, bm, sens, ab = self._keep[:8]
        self.nData = len(ab)
        self.nE = len(sens)
        z = None if contact_impedance is None else np.ascontiguousarray(contact_impedance, np.float64)
        self._keep.append(z)
        h = L.ref_create_ex(mesh.dim(), len(nodes), _p(nodes), _p(nm), len(cells), cells.shape[1], _p(cells),
                            _p(cm), len(bnd), bnd.shape[1], _p(bnd), _p(bm), len(sens), _p(sens), len(ab),
                            _p(ab), None if kf is None else _p(kf), 0, 2 if h2 else int(bool(p2)), int(bool(sr)),
                            0 if z is None else len(z), None if z is None else _p(z))
        if not h:
            raise RuntimeError("ref_create failed: " + L.ref_last_error().decode())
        self.h = h
        self.keep_matrices = keep_matrices
        self.matrices = []
        self._lu = None

        def factor(n, nnz, rowptr, colidx, vals):
            try:
                rp = np.ctypeslib.as_array(ctypes.cast(rowptr, ctypes.POINTER(ctypes.c_int)), (n + 1,)).copy()
                ci = np.ctypeslib.as_array(ctypes.cast(colidx, ctypes.POINTER(ctypes.c_int)), (nnz,)).copy()
                va = np.ctypeslib.as_array(ctypes.cast(vals, ctypes.POINTER(ctypes.c_double)), (nnz,)).copy()
                A = sp.csr_matrix((va, ci, rp), shape=(n, n))
                if self.keep_matrices:
                    self.matrices.append((rp, ci, va))
                self._lu = spla.splu(A.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0)
                return 0
            except Exception:  # pragma: no cover - reported through the C layer
                return 1

        def solve(n, rhs, x):
            try:
                b = np.ctypeslib.as_array(ctypes.cast(rhs, ctypes.POINTER(ctypes.c_double)), (n,))
                out = np.ctypeslib.as_array(ctypes.cast(x, ctypes.POINTER(ctypes.c_double)), (n,))
                out[:] = self._lu.solve(np.array(b))
                return 0
            except Exception:  # pragma: no cover
                return 1

        self._clu = None

        def cfactor(n, nnz, rowptr, colidx, vals):
            try:
                rp = np.ctypeslib.as_array(ctypes.cast(rowptr, ctypes.POINTER(ctypes.c_int)), (n + 1,)).copy()
                ci = np.ctypeslib.as_array(ctypes.cast(colidx, ctypes.POINTER(ctypes.c_int)), (nnz,)).copy()
                va = np.ctypeslib.as_array(ctypes.cast(vals, ctypes.POINTER(ctypes.c_double)), (2 * nnz,))
                A = sp.csr_matrix((va[0::2] + 1j * va[1::2], ci, rp), shape=(n, n))
                if self.keep_matrices:
                    self.matrices.append((rp, ci, va[0::2] + 1j * va[1::2]))
                self._clu = spla.splu(A.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0)
                return 0
            except Exception:  # pragma: no cover - reported through the C layer
                return 1

        def csolve(n, rhs, x):
            try:
                b = np.ctypeslib.as_array(ctypes.cast(rhs, ctypes.POINTER(ctypes.c_double)), (2 * n,))
                out = np.ctypeslib.as_array(ctypes.cast(x, ctypes.POINTER(ctypes.c_double)), (2 * n,))
                sol = self._clu.solve(b[0::2] + 1j * b[1::2])
                out[0::2] = sol.real
                out[1::2] = sol.imag
                return 0
            except Exception:  # pragma: no cover
                return 1

        self._cb = (_FACTOR(factor), _SOLVE(solve), _CFACTOR(cfactor), _CSOLVE(csolve))
        _check(L.ref_set_solver(h, self._cb[0], self._cb[1]))
        _check(L.ref_set_complex_solver(h, self._cb[2], self._cb[3]))
        _check(L.ref_set_threads(h, int(threads)))

    def mesh_arrays(self):
        """Mesh the reference operator runs on (nodes, node markers, cells,
        cell markers, boundaries, boundary markers)."""
        v = [ctypes.c_int() for _ in range(5)]
        lib().ref_mesh_sizes(self.h, *[ctypes.byref(x) for x in v])
        n, C, nv, B, nvb = [x.value for x in v]
        xyz = np.zeros((n, 3))
        nm = np.zeros(n, np.int32)
        cells = np.zeros((C, nv), np.int32)
        cm = np.zeros(C, np.int32)
        bnd = np.zeros((B, nvb), np.int32)
        bm = np.zeros(B, np.int32)
        _check(lib().ref_mesh_arrays(self.h, _p(xyz), _p(nm), _p(cells), _p(cm), _p(bnd), _p(bm)))
        return xyz, nm, cells, cm, bnd, bm

    def close(self):
        if self.h:
            lib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_kw(self, k, w):
        k = np.ascontiguousarray(k, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        _check(lib().ref_set_kw(self.h, len(k), _p(k), _p(w)))

    def kw(self):
        n = lib().ref_kw_count(self.h)
        k = np.zeros(n)
        w = np.zeros(n)
        _check(lib().ref_get_kw(self.h, _p(k), _p(w)))
        return k, w

    def electrode_nodes(self):
        out = np.zeros(self.nE, np.int32)
        _check(lib().ref_electrode_nodes(self.h, _p(out)))
        return out

    def geometric_factors(self):
        out = np.zeros(self.nData)
        _check(lib().ref_geometric_factors(self.h, _p(out)))
        return out

    def response(self, model):
        m = np.ascontiguousarray(model, np.float64)
        out = np.zeros(self.nData)
        self.matrices = []
        _check(lib().ref_response(self.h, _p(m), len(m), _p(out)))
        return out

    def calculate_dipole(self, model):
        """Voltages (unit current) of the data with the dipole current
        pattern (calculate(DataContainerERT &) with setDipoleCurrentPattern);
        returns (u, number of (a, b) patterns solved)."""
        m = np.ascontiguousarray(model, np.float64)
        out = np.zeros(self.nData)
        npat = ctypes.c_int()
        _check(lib().ref_calculate_dipole(self.h, _p(m), len(m), _p(out), ctypes.byref(npat)))
        return out, npat.value

    def set_primary(self, prim):
        """Primary potentials (rows = source + k * nE, cols = nodes) for the
        singularity-removal operator (setPrimaryPotential)."""
        P = np.ascontiguousarray(prim, np.float64)
        self._prim = P
        _check(lib().ref_set_primary(self.h, P.shape[0], P.shape[1], _p(P)))

    def subpotentials(self):
        r = ctypes.c_int()
        c = ctypes.c_int()
        lib().ref_subpot_shape(self.h, ctypes.byref(r), ctypes.byref(c))
        out = np.zeros((r.value, c.value))
        _check(lib().ref_subpotentials(self.h, _p(out)))
        return out

    def response_complex(self, model_re, model_im):
        """Complex resistivity: [Re, Im] of the apparent resistivities for the
        model (Re, Im) (setComplex(true) + response)."""
        m = np.ascontiguousarray(np.concatenate([model_re, model_im]), np.float64)
        out = np.zeros(2 * self.nData)
        _check(lib().ref_response_complex(self.h, _p(m), len(m), _p(out)))
        return out[:self.nData] + 1j * out[self.nData:]

    def jacobian_complex(self, model_re, model_im):
        m = np.ascontiguousarray(np.concatenate([model_re, model_im]), np.float64)
        r, c = ctypes.c_int(), ctypes.c_int()
        _check(lib().ref_jacobian_complex(self.h, _p(m), len(m), None, None, ctypes.byref(r), ctypes.byref(c)))
        Jr = np.zeros((r.value, c.value))
        Ji = np.zeros((r.value, c.value))
        _check(lib().ref_jacobian_complex(self.h, _p(m), len(m), _p(Jr), _p(Ji), ctypes.byref(r), ctypes.byref(c)))
        return Jr + 1j * Ji

    def create_jacobian(self, model):
        """createJacobian(model) alone (the Jacobian stays in the reference's
        RMatrix); returns its shape."""
        m = np.ascontiguousarray(model, np.float64)
        r = ctypes.c_int()
        c = ctypes.c_int()
        _check(lib().ref_jacobian(self.h, _p(m), len(m), None, ctypes.byref(r), ctypes.byref(c)))
        return r.value, c.value

    def jacobian(self, model):
        m = np.ascontiguousarray(model, np.float64)
        r = ctypes.c_int()
        c = ctypes.c_int()
        _check(lib().ref_jacobian(self.h, _p(m), len(m), None, ctypes.byref(r), ctypes.byref(c)))
        J = np.zeros((r.value, c.value))
        _check(lib().ref_jacobian(self.h, _p(m), len(m), _p(J), ctypes.byref(r), ctypes.byref(c)))
        return J

    def assemble(self, rho_cell, k, src_center):
        """System matrix as the SR calculateK builds it (CSR tuple)."""
        rho = np.ascontiguousarray(rho_cell, np.float64)
        sc = np.ascontiguousarray(src_center, np.float64)
        n = ctypes.c_int()
        nnz = ctypes.c_int()
        _check(lib().ref_assemble(self.h, _p(rho), float(k), _p(sc), ctypes.byref(n), ctypes.byref(nnz),
                                  None, None, None))
        rp = np.zeros(n.value + 1, np.int32)
        ci = np.zeros(nnz.value, np.int32)
        va = np.zeros(nnz.value)
        _check(lib().ref_assemble(self.h, _p(rho), float(k), _p(sc), ctypes.byref(n), ctypes.byref(nnz),
                                  _p(rp), _p(ci), _p(va)))
        return rp, ci, va

    def node_count(self):
        """Nodes of the mesh the reference operator runs on (after createP2)."""
        v = [ctypes.c_int() for _ in range(5)]
        lib().ref_mesh_sizes(self.h, *[ctypes.byref(x) for x in v])
        return v[0].value

    def primary(self, e, k, surface_z=0.0):
        out = np.zeros(self.node_count())
        _check(lib().ref_primary(self.h, int(e), float(k), float(surface_z), _p(out)))
        return out


def besselK0(x):
    return lib().ref_besselK0(float(x))


def besselK1(x):
    return lib().ref_besselK1(float(x))


def _mesh_arrays(h):
    v = [ctypes.c_int() for _ in range(5)]
    lib().ref_mesh_sizes(h, *[ctypes.byref(x) for x in v])
    n, C, nv, B, nvb = [x.value for x in v]
    xyz = np.zeros((n, 3))
    nm = np.zeros(n, np.int32)
    cells = np.zeros((C, nv), np.int32)
    cm = np.zeros(C, np.int32)
    bnd = np.zeros((B, nvb), np.int32)
    bm = np.zeros(B, np.int32)
    _check(lib().ref_mesh_arrays(h, _p(xyz), _p(nm), _p(cells), _p(cm), _p(bnd), _p(bm)))
    left = np.zeros(B, np.int32)
    right = np.zeros(B, np.int32)
    _check(lib().ref_mesh_boundary_cells(h, _p(left), _p(right)))
    return {"dim": lib().ref_mesh_dim(h), "nodes": xyz, "node_markers": nm, "cells": cells, "cell_markers": cm,
            "boundaries": bnd, "boundary_markers": bm, "left": left, "right": right}


class RefMesh:
    """A reference ``GIMLI::Mesh`` alone: built from arrays (with
    createNeighborInfos, optionally createP2 / createH2) or loaded from a
    binary mesh file; saved with saveBinaryV2 or exported with exportVTK."""

    def __init__(self, mesh=None, p2=False, h2=False, path=None):
        L = lib()
        if path is not None:
            self.h = L.ref_mesh_load(os.fsencode(path))
        else:
            a = [np.ascontiguousarray(mesh.nodes, np.float64), np.ascontiguousarray(mesh.node_markers, np.int32),
                 np.ascontiguousarray(mesh.cells, np.int32), np.ascontiguousarray(mesh.cell_markers, np.int32),
                 np.ascontiguousarray(mesh.boundaries, np.int32),
                 np.ascontiguousarray(mesh.boundary_markers, np.int32)]
            self._keep = a
            nodes, nm, cells, cm, bnd, bm = a
            self.h = L.ref_mesh_create(mesh.dim(), len(nodes), _p(nodes), _p(nm), len(cells), cells.shape[1],
                                       _p(cells), _p(cm), len(bnd), bnd.shape[1], _p(bnd), _p(bm),
                                       2 if h2 else int(bool(p2)))
        if not self.h:
            raise RuntimeError("reference mesh failed: " + L.ref_last_error().decode())

    def arrays(self):
        return _mesh_arrays(self.h)

    def regions(self, default_background=True, background=(), single=(), fix=None):
        """The reference's RegionManager on this mesh: (renumbered cell
        markers, parameter count, para-domain cell count)."""
        fix = fix or {}
        bg = np.ascontiguousarray(list(background) or [0], np.int32)
        sg = np.ascontiguousarray(list(single) or [0], np.int32)
        fm = np.ascontiguousarray(list(fix) or [0], np.int32)
        fv = np.ascontiguousarray(list(fix.values()) or [0.0], np.float64)
        C = len(self.arrays()["cells"])
        out = np.zeros(C, np.int32)
        npar, ncell = ctypes.c_int(), ctypes.c_int()
        _check(lib().ref_regions(self.h, int(default_background), len(background), _p(bg), len(single), _p(sg),
                                 len(fix), _p(fm), _p(fv), _p(out), ctypes.byref(npar), ctypes.byref(ncell)))
        return out, npar.value, ncell.value

    def constraints(self, default_background=True, background=(), single=(), fix=None):
        """The reference's RegionManager::fillConstraints for these region
        settings: (rows, cols, vals, n_rows, n_cols), entries row-major."""
        fix = fix or {}
        bg = np.ascontiguousarray(list(background) or [0], np.int32)
        sg = np.ascontiguousarray(list(single) or [0], np.int32)
        fm = np.ascontiguousarray(list(fix) or [0], np.int32)
        fv = np.ascontiguousarray(list(fix.values()) or [0.0], np.float64)
        nr, nc, ne = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        args = (self.h, int(default_background), len(background), _p(bg), len(single), _p(sg), len(fix), _p(fm),
                _p(fv))
        _check(lib().ref_region_constraints(*args, 0, ctypes.byref(nr), ctypes.byref(nc), ctypes.byref(ne),
                                            None, None, None))
        r = np.zeros(max(ne.value, 1), np.int32)
        c = np.zeros(max(ne.value, 1), np.int32)
        v = np.zeros(max(ne.value, 1))
        _check(lib().ref_region_constraints(*args, ne.value, ctypes.byref(nr), ctypes.byref(nc), ctypes.byref(ne),
                                            _p(r), _p(c), _p(v)))
        return r[:ne.value], c[:ne.value], v[:ne.value], nr.value, nc.value

    def add_data(self, name, values):
        v = np.ascontiguousarray(values, np.float64)
        _check(lib().ref_mesh_add_data(self.h, name.encode(), len(v), _p(v)))

    def save_bms(self, path):
        _check(lib().ref_mesh_save_bms(self.h, os.fsencode(path)))

    def save_bms_v1(self, path):
        _check(lib().ref_mesh_save_bms_v1(self.h, os.fsencode(path)))

    def export_vtk(self, path, cells=True):
        _check(lib().ref_mesh_export_vtk(self.h, os.fsencode(path), int(bool(cells))))

    def close(self):
        if self.h:
            lib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover
            pass


def data_load(path, from_one=True, remove_invalid=True):
    """The reference's ``DataContainerERT::load``: returns (sensors (S, 3),
    token list, {token: values})."""
    L = lib()
    h = L.ref_data_load(os.fsencode(path), int(bool(from_one)), int(bool(remove_invalid)))
    if not h:
        raise RuntimeError("reference data load failed: " + L.ref_last_error().decode())
    try:
        nS, nD = ctypes.c_int(), ctypes.c_int()
        L.ref_data_sizes(h, ctypes.byref(nS), ctypes.byref(nD))
        xyz = np.zeros((nS.value, 3))
        _check(L.ref_data_sensors(h, _p(xyz)))
        buf = ctypes.create_string_buffer(4096)
        assert L.ref_data_tokens(h, buf, 4096) == 0
        tokens = buf.value.decode().split()
        fields = {}
        for t in tokens:
            v = np.zeros(nD.value)
            _check(L.ref_data_get(h, t.encode(), _p(v)))
            fields[t] = v
        return xyz, tokens, fields
    finally:
        L.ref_data_free(h)


def data_resave(path_in, path_out, fmt_data="all", fmt_sensor="x y z", no_filter=False, from_one=True):
    """Load ``path_in`` with the reference and write it back with its
    ``DataContainer::save``."""
    L = lib()
    h = L.ref_data_load(os.fsencode(path_in), int(bool(from_one)), 1)
    if not h:
        raise RuntimeError("reference data load failed: " + L.ref_last_error().decode())
    try:
        _check(L.ref_data_save(h, os.fsencode(path_out), fmt_data.encode(), fmt_sensor.encode(),
                               int(bool(no_filter))))
    finally:
        L.ref_data_free(h)


def cgls(J, C, dW, b, x0, wc, wm, tm, td, lam, rough, max_iter=200, tol=-1.0):
    """The reference's solveCGLSCDWWhtrans (core/src/solver.cpp:27-212): J
    dense (nData x nModel), C = (rowptr, colidx, values, nModel) in CSR."""
    rp, ci, cv, P = C
    f = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
    Jc = f(J)
    rp = np.ascontiguousarray(rp, np.int32)
    ci = np.ascontiguousarray(ci, np.int32)
    arrs = [f(cv), f(dW), f(b), f(wc), f(wm), f(tm), f(td), f(rough)]
    x = f(x0).copy()
    cvv, dWv, bv, wcv, wmv, tmv, tdv, rv = arrs
    _check(lib().ref_cgls(Jc.shape[0], Jc.shape[1], _p(Jc), len(rp) - 1, _p(rp), _p(ci), _p(cvv), _p(dWv), _p(bv),
                          _p(x), _p(wcv), _p(wmv), _p(tmv), _p(tdv), float(lam), _p(rv), int(max_iter), float(tol)))
    return x
