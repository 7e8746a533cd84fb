"""Drop-in ERT forward operator on one GB300: ``ERTModelling``.

Mirrors the method surface of pyGIMLi's ``pg.physics.ert.ERTModelling``
(pygimli/physics/ert/ertModelling.py:73-246) over the singularity-removal
operator ``DCSRMultiElectrodeModelling`` (core/src/bert/dcfemmodelling.h:344)
or, with ``sr=False``, the total-potential operator
``DCMultiElectrodeModelling`` (dcfemmodelling.h:105) with complete-electrode-
model and bypass electrodes:
``setMesh``, ``setData``, ``response(model)``, ``createJacobian(model)``,
``jacobian()``, ``mesh()``, ``parameterCount``, ``solution()``,
``calcGeometricFactor``, ``mapERTModel``, ``setkValues/setWeights``.
Every numerical step runs in libertgb.so (hand-written sm_103a CUDA behind
the C ABI of include/ertgb.h); this module only does setup bookkeeping
(electrode search, wavenumbers, model mapping) and moves buffers.

Scope (raises otherwise): node electrodes (marker -99) and electrodes inside
cells, with sr=False also CEM and bypass electrodes; mixed far-field,
homogeneous Neumann and homogeneous Dirichlet (-3) boundaries, closed
(Neumann-only) domains with calibration nodes (-1000) and a reference
electrode (node marker -999 or the last electrode); pole current patterns
or patterns against the reference electrode, and the dipole current pattern
(forward voltages, ``setDipoleCurrentPattern`` + ``calculate``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .cem import electrode_setup, has_cem_markers
from .data import DataContainerERT, geometricFactors
from .kwave import init_kwave_list
from .mesh import (MARKER_BOUND_HOMOGEN_DIRICHLET, MARKER_BOUND_HOMOGEN_NEUMANN, MARKER_BOUND_MIXED,
                   MARKER_NODE_ELECTRODE, Mesh)
from .modelmap import map_model

TOLERANCE = 1e-12
MARKER_BOUND_DIRICHLET = -4
MARKER_NODE_REFERENCEELECTRODE = -999
MARKER_NODE_CALIBRATION = -1000


def _torch():
    import torch
    return torch


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def sensor_positions(mesh, sensors):
    """Sensor positions in mesh coordinates: 2-D sensors given as (x, 0, z)
    are swapped to (x, z) (dcfemmodelling.cpp:859-867)."""
    ePos = np.asarray(sensors, dtype=np.float64).reshape(-1, 3).copy()
    if mesh.dim() == 2:
        zvar = np.ptp(ePos[:, 2]) > 0 or np.max(np.abs(ePos[:, 2])) > 0
        yvar = np.ptp(ePos[:, 1]) > 0
        if zvar and not yvar and np.max(np.abs(ePos[:, 1])) < 1e-8:
            ePos[:, [1, 2]] = ePos[:, [2, 1]]
    return ePos


def find_cell(mesh, p, tol=1e-12):
    """The cell that holds point p (linear cells; the lowest cell index whose
    barycentric coordinates are all >= -tol, as Mesh::findCell returns the
    one holding cell), or -1."""
    d = mesh.dim()
    if mesh.cells.shape[1] != d + 1:
        raise NotImplementedError("electrodes inside cells need linear cells")
    x = mesh.nodes[mesh.cells][:, :, :d]
    near = np.nonzero(np.all((x.min(axis=1) <= p[:d] + 1e-9) & (x.max(axis=1) >= p[:d] - 1e-9), axis=1))[0]
    if len(near) == 0:
        return -1
    xs = x[near]
    A = np.transpose(xs[:, 1:, :] - xs[:, :1, :], (0, 2, 1))
    lam = np.linalg.solve(A, (p[:d][None, :] - xs[:, 0, :])[:, :, None])[:, :, 0]
    bary = np.column_stack([1.0 - lam.sum(axis=1), lam])
    ok = np.nonzero(np.all(bary >= -tol, axis=1))[0]
    return int(near[ok[0]]) if len(ok) else -1


class ElectrodeSearch:
    """Electrodes of the singularity-removal operator in data order: a node
    (nodes[i] >= 0) or, with no electrode node within 1 cm, the cell that
    holds the sensor (cells[i] >= 0, ElectrodeShapeEntity); pos: the sensor
    positions in mesh coordinates."""

    def __init__(self, nodes, cells, pos):
        self.nodes, self.cells, self.pos = nodes, cells, pos

    @property
    def entity(self):
        return bool(np.any(self.cells >= 0))


def search_electrodes(mesh, sensors):
    """Electrodes as DCMultiElectrodeModelling::searchElectrodes_ finds them
    for node and free electrodes (core/src/bert/dcfemmodelling.cpp:790-1030):
    sensor i takes the first still-unused node with marker -99 within 1 cm,
    else the cell that holds it (:924-937)."""
    ePos = sensor_positions(mesh, sensors)
    cand = np.nonzero(mesh.node_markers == MARKER_NODE_ELECTRODE)[0]
    used = np.zeros(len(cand), bool)
    nodes = np.full(len(ePos), -1, np.int32)
    cells = np.full(len(ePos), -1, np.int32)
    cpos = mesh.nodes[cand]
    for i, p in enumerate(ePos):
        d = np.linalg.norm(cpos - p, axis=1)
        ok = np.nonzero((d < 0.01) & ~used)[0]
        if len(ok):
            used[ok[0]] = True
            nodes[i] = cand[ok[0]]
            continue
        cells[i] = find_cell(mesh, p)
        if cells[i] < 0:
            raise ValueError(f"There is a requested electrode that does not match the given mesh: {p}")
    return ElectrodeSearch(nodes, cells, ePos)


def surface_info(mesh):
    """surfaceZ and topography flag of updateMeshDependency_
    (core/src/bert/dcfemmodelling.cpp:711-773); a domain without mixed and
    Dirichlet boundaries counts as topography (:750-755)."""
    bm = mesh.boundary_markers
    neu = np.nonzero(bm == MARKER_BOUND_HOMOGEN_NEUMANN)[0]
    closed = not np.any((bm == MARKER_BOUND_MIXED) | (bm == MARKER_BOUND_HOMOGEN_DIRICHLET))
    if len(neu) == 0:
        return -np.finfo(np.float64).max, closed
    c = mesh.nodes[mesh.boundaries[neu]].mean(axis=1)[:, mesh.dim() - 1]
    return float(c[0]), bool(np.any(c != c[0])) or closed


class BoundarySetup:
    """Boundary conditions and current reference of a mesh with n_elec
    electrodes, as updateMeshDependency_ and searchElectrodes_ choose them
    (core/src/bert/dcfemmodelling.cpp:711-773, 799-802, 1011-1073):
    ``neumann`` (no mixed, no Dirichlet boundary), ``topography``,
    ``dirichlet`` (nodes of -3 boundaries), ``calib`` (a closed 3-D domain:
    the nodes with marker -1000, else node 0), ``ref_node`` (the first node
    with marker -999, in any domain; -1: none) and ``ref_elec`` (a closed
    3-D domain without reference node: the last electrode; else -1)."""

    def __init__(self, neumann, topography, dirichlet, calib, ref_node, ref_elec):
        self.neumann, self.topography = neumann, topography
        self.dirichlet, self.calib = dirichlet, calib
        self.ref_node, self.ref_elec = ref_node, ref_elec


def boundary_setup(mesh, n_elec, dipole=False):
    bm = np.asarray(mesh.boundary_markers)
    if np.any(bm == MARKER_BOUND_DIRICHLET):
        raise NotImplementedError("inhomogeneous Dirichlet boundaries (marker -4) are not implemented")
    _, topo = surface_info(mesh)
    neumann = not np.any((bm == MARKER_BOUND_MIXED) | (bm == MARKER_BOUND_HOMOGEN_DIRICHLET))
    d = mesh.boundaries[bm == MARKER_BOUND_HOMOGEN_DIRICHLET]
    dirichlet = np.unique(d) if d.size else np.zeros(0, np.int64)
    nm = np.asarray(mesh.node_markers)
    refs = np.flatnonzero(nm == MARKER_NODE_REFERENCEELECTRODE)
    ref_node = int(refs[0]) if len(refs) else -1
    calib, ref_elec = np.zeros(0, np.int64), -1
    if neumann and mesh.dim() == 3:  # 2.5-D is never a Neumann domain (:758-766)
        calib = np.flatnonzero(nm == MARKER_NODE_CALIBRATION)
        if len(calib) == 0:
            calib = np.zeros(1, np.int64)
        if ref_node < 0 and n_elec > 0 and not dipole:
            ref_elec = n_elec - 1
    if dipole:  # the dipole current pattern pairs the data's own electrodes (no reference)
        ref_node = -1
    return BoundarySetup(neumann, topo, dirichlet, calib, ref_node, ref_elec)


class ERTModelling:
    """ERT forward operator on one GB300.

    sr=True (default): singularity removal (pyGIMLi's
    DCSRMultiElectrodeModelling).  sr=False: total potentials
    (DCMultiElectrodeModelling, pygimli/physics/ert/ertModelling.py:102-106),
    the formulation that also takes complete-electrode-model (CEM) and bypass
    electrodes from the mesh markers (see ``pygimli_gb300.cem``)."""

    def __init__(self, sr=True, verbose=False, device=0, rtol=1e-10, maxIter=20000, precision="fp64",
                 precond="jacobi", weights=None):
        self.verbose = verbose
        self._lib = _native.load()
        self._ctx = ctypes.c_void_p()
        _native.check(None, self._lib.ertgb_create(ctypes.byref(self._ctx), int(device)))
        self.device = int(device)
        self._sr = bool(sr)
        self._check(self._lib.ertgb_set_formulation(self._ctx, 0 if self._sr else 1))
        self._contact_z = None    # setContactImpedances
        self._bypass_r = None     # setBypassResistances
        self._electrodes = None   # electrode setup of the total-potential operator
        self._mesh = None
        self._data = None
        self._k = None
        self._w = None
        self._kw_user = False
        self._topo = False        # forward mesh surface is not flat (set by setMesh)
        self._J = None
        self._elec_nodes = None
        self._last_model = None
        self._precond = 0
        # forward-mesh refinement applied by setMesh(mesh) without
        # ignoreRegionManager (MeshModelling, pygimli/frameworks/modelling.py:584-586)
        self._refineH2 = True
        self._refineP2 = False
        self._complex = False     # complex resistivity (setComplex)
        self._conjImag = False    # complex start model flipped to a positive imaginary part
        self._dipole = False      # dipole current pattern (setDipoleCurrentPattern)
        self._mapped = None       # cell resistivities of the last mapERTModel / response
        self._rm = None           # region manager of the parameter mesh (setMesh without ignoreRegionManager)
        self._fwd_parent = None   # forward-mesh cell -> parameter-mesh cell
        self.setSolverTolerance(rtol, maxIter)
        self.setPrecision(precision)
        self.setPreconditioner(precond, weights)

    def setPrecision(self, precision):
        """Solver arithmetic: ``"fp64"`` or ``"mixed"`` (FP32 recurrence with
        FP64 reliable updates; same converged accuracy)."""
        modes = {"fp64": 0, "mixed": 1}
        if precision not in modes:
            raise ValueError(f"precision must be one of {sorted(modes)}")
        self._check(self._lib.ertgb_set_precision(self._ctx, modes[precision]))
        self.precision = precision

    def __del__(self):
        try:
            if getattr(self, "_ctx", None) and self._ctx.value:
                self._lib.ertgb_destroy(self._ctx)
                self._ctx = ctypes.c_void_p()
        except Exception:
            pass

    def _check(self, rc):
        return _native.check(self._ctx, rc)

    # -------------------------------------------------------------- setup
    def setVerbose(self, v):
        self.verbose = bool(v)

    def setThreadCount(self, n):
        """No-op: the work runs on the GPU."""

    def setSolver(self, solver):
        raise NotImplementedError("the linear solver is the built-in GPU block PCG")

    def setSolverTolerance(self, rtol=1e-10, maxIter=20000):
        self._rtol, self._maxIter = float(rtol), int(maxIter)
        self._check(self._lib.ertgb_set_solver(self._ctx, self._rtol, self._maxIter, self._precond))

    def setPreconditioner(self, precond, weights=None):
        """``"jacobi"``, ``"fsai"`` (factorized sparse approximate inverse) or
        ``"learned"`` (network-emitted factor; ``weights``: a
        LearnedPreconditioner, a weight array or an .npz path).  FSAI and
        learned need mixed precision; stalled columns finish with FP64 Jacobi."""
        codes = {"jacobi": 0, "fsai": 1, "learned": 2, "ic0": 3, "band": 4}
        if precond not in codes:
            raise ValueError(f"precond must be one of {sorted(codes)}")
        if weights is not None:
            from .learned import LearnedPreconditioner
            if isinstance(weights, str):
                weights = LearnedPreconditioner.load(weights)
            w = weights.weights if isinstance(weights, LearnedPreconditioner) else np.asarray(weights)
            w = np.ascontiguousarray(w, np.float32)
            self._check(self._lib.ertgb_set_precond_weights(self._ctx, _ptr(w), w.size))
            self._have_weights = True
        if precond == "learned" and not getattr(self, "_have_weights", False):
            raise ValueError("the learned preconditioner needs weights")
        self._precond = codes[precond]
        self._check(self._lib.ertgb_set_solver(self._ctx, self._rtol, self._maxIter, self._precond))

    def createRefinedFwdMesh(self, mesh):
        """Forward mesh of a parameter mesh: H2 refinement, then P2, as
        enabled by ``_refineH2`` / ``_refineP2``
        (pygimli/frameworks/modelling.py:682-699), computed on this
        operator's GPU (``refine.py``).  Refined cells keep their parent's
        marker, so the model stays one value per parameter."""
        from . import refine
        m = mesh
        if self._refineH2:
            m = refine.createH2(m, self.device)
        if self._refineP2:
            m = refine.createP2(m, self.device)
        return m

    def setMesh(self, mesh, ignoreRegionManager=False):
        """Set the mesh (MeshModelling.setMesh, pygimli/frameworks/
        modelling.py:730-757).  ``ignoreRegionManager=True`` solves on
        ``mesh`` itself with its cell markers as parameter indices.
        Otherwise the region manager takes the cell markers as regions (the
        lowest of several becomes background, regions.py), renumbers them
        into parameter indices, and the forward mesh is
        ``createRefinedFwdMesh`` of the renumbered mesh."""
        if not isinstance(mesh, Mesh):
            raise TypeError("mesh must be a pygimli_gb300.mesh.Mesh")
        if ignoreRegionManager:
            self._rm = None
            self._fwd_parent = None
            self._set_fwd_mesh(mesh)
            return
        from .regions import RegionManager
        rm = RegionManager()
        rm.setMesh(mesh)
        rm.setDefaultBackground()
        self._rm = rm
        para = Mesh(mesh.dim(), mesh.nodes, mesh.cells, rm.paraMarkers(), mesh.node_markers, mesh.boundaries,
                    mesh.boundary_markers, mesh.boundary_cells, check=False)
        fwd = self.createRefinedFwdMesh(para)
        ratio = fwd.cellCount() // para.cellCount()
        self._fwd_parent = np.arange(fwd.cellCount(), dtype=np.int64) // ratio
        self._set_fwd_mesh(fwd)

    def regionManager(self):
        return self._rm

    def setDefaultBackground(self):
        """With several regions, the one with the lowest marker becomes
        background (MeshModelling.setDefaultBackground, pygimli/frameworks/
        modelling.py:759-767; ERTModelling.setDefaultBackground,
        ertModelling.py:131-144).  ``setMesh`` applies it already."""
        if self._rm is None:
            raise RuntimeError("no region manager: setMesh(mesh) without ignoreRegionManager first")
        ids = self._rm.regionIdxs()
        if len(ids) > 1:
            self.setRegionProperties(ids[0], background=True)

    def setDataPost(self, data):
        """The framework's hook after setData (ertModelling.py:240-242)."""
        self.setData(data)

    def setMeshPost(self, mesh):
        """The framework's hook after setMesh: the mesh as the forward mesh
        (ertModelling.py:244-246)."""
        self.setMesh(mesh, ignoreRegionManager=True)

    def setRegionProperties(self, regionNr, background=None, single=None, fix=None, **kwargs):
        """Background / single / fixed-value flags of a region ("*": all),
        as MeshModelling.setRegionProperties (pygimli/frameworks/
        modelling.py:330-390); the parameters are renumbered.  Start
        models, bounds and constraint settings belong to the inversion and
        are not kept."""
        if self._rm is None:
            raise RuntimeError("no region manager: setMesh(mesh) without ignoreRegionManager first")
        self._rm.setRegionProperties(regionNr, background=background, single=single, fix=fix)
        fwd = self._mesh
        fwd.setCellMarkers(self._rm.paraMarkers()[self._fwd_parent])
        self._set_fwd_mesh(fwd)

    @property
    def paraDomain(self):
        """Mesh of the parameter cells (the region manager's para domain);
        without a region manager the forward mesh."""
        return self._rm.paraDomain() if self._rm is not None else self._mesh

    def _set_fwd_mesh(self, mesh):
        surf, topo = surface_info(mesh)
        if topo and self._sr and mesh.order != 1:
            raise NotImplementedError("singularity removal on a topographic surface computes its primary "
                                      "potentials on createP2 of the mesh: the mesh must be linear")
        boundary_setup(mesh, 0)  # refuses -4 boundaries
        b = np.ascontiguousarray(mesh.boundaries, np.int32)
        self._check(self._lib.ertgb_set_mesh(
            self._ctx, mesh.dim(), mesh.order, mesh.nodeCount(), _ptr(mesh.nodes), mesh.cellCount(),
            _ptr(mesh.cells), _ptr(mesh.cell_markers), len(b), _ptr(b),
            _ptr(mesh.boundary_markers), _ptr(mesh.boundary_cells)))
        self._mesh = mesh
        self._surface_z = surf
        self._topo = bool(topo)
        self._J = None
        if self._data is not None:
            self._update_data()

    def mesh(self):
        return self._mesh

    def setData(self, data):
        if not isinstance(data, DataContainerERT):
            raise TypeError("data must be a pygimli_gb300.data.DataContainerERT")
        self._data = data
        self._J = None
        if self._mesh is not None:
            self._update_data()

    @property
    def data(self):
        return self._data

    def setContactImpedances(self, zi):
        """Contact impedances (Ohm m^2) of the CEM electrodes, one per
        electrode then per passive body (DCMultiElectrodeModelling::
        setContactImpedances, dcfemmodelling.cpp:786-788; default 1).  Point
        electrodes always couple with 1 (dcfemmodelling.cpp:344-350)."""
        self._contact_z = None if zi is None else np.asarray(zi, np.float64).copy()
        self._J = None
        if self._mesh is not None and self._data is not None:
            self._update_data()

    def setBypassResistances(self, resistances):
        """Bypass resistances {node marker: Ohm} (the reference reads them
        from electrodeBypassResistances.map, dcfemmodelling.cpp:672-686;
        default 1e-6 Ohm)."""
        self._bypass_r = None if resistances is None else dict(resistances)
        self._J = None
        if self._mesh is not None and self._data is not None:
            self._update_data()

    def _update_data(self):
        mesh, data = self._mesh, self._data
        if self._sr:
            if has_cem_markers(mesh):
                raise ValueError("complete-electrode-model and bypass electrodes need the total-potential "
                                 "operator: ERTModelling(sr=False)")
            es = search_electrodes(mesh, data.sensorPositions())
            self._elec_nodes = es.nodes
            self._electrodes = None
        else:
            setup = electrode_setup(mesh, data.sensorPositions(), self._contact_z, self._bypass_r)
            self._electrodes = setup
            self._elec_nodes = setup.enode
            es = setup.search
        self._check(self._lib.ertgb_set_electrodes(self._ctx, len(self._elec_nodes),
                                                   _ptr(self._elec_nodes), float(self._surface_z)))
        self._esearch = es
        self._entity = es is not None and es.entity
        if self._entity:
            cells = np.ascontiguousarray(es.cells, np.int32)
            pos = np.ascontiguousarray(es.pos, np.float64)
            self._check(self._lib.ertgb_set_electrode_shapes(self._ctx, len(cells), _ptr(cells), _ptr(pos)))
        if self._electrodes is not None and (self._electrodes.cem or len(self._electrodes.rows)):
            e = self._electrodes
            self._check(self._lib.ertgb_set_extension(
                self._ctx, int(e.n_ext), len(e.rows), _ptr(e.rows), _ptr(e.cols), _ptr(e.vals), _ptr(e.src_row),
                _ptr(e.src_center), 1 if e.cem else 0))
        bc = boundary_setup(mesh, len(self._elec_nodes), self._dipole)
        if bc.ref_node >= 0 or bc.ref_elec >= 0:
            if self._electrodes is not None and (self._electrodes.cem or len(self._electrodes.rows)):
                raise NotImplementedError("a reference electrode with complete-electrode-model or bypass "
                                          "electrodes is not supported")
        calib = np.ascontiguousarray(bc.calib, np.int32)
        self._check(self._lib.ertgb_set_reference(self._ctx, int(bc.ref_elec), int(bc.ref_node), len(calib),
                                                  _ptr(calib) if len(calib) else None))
        self._bc = bc
        if not self._kw_user:
            self._k, self._w = init_kwave_list(mesh.dim(), data.sensorPositions())
        self._push_kw()
        if self._sr and self._topo:
            self._push_numerical_primary()
        self._push_scheme()

    def _push_numerical_primary(self):
        """Primary potentials of singularity removal on a topographic surface
        (DCSRMultiElectrodeModelling::checkPrimpotentials_, core/src/bert/
        dcfemmodelling.cpp:2008-2068): the total potential at 1 Ohm m on
        createP2 of the forward mesh (GPU refinement, total-potential operator
        in FP64 to rtol 1e-12, this operator's wavenumbers), taken at the
        forward mesh's nodes, which createP2 keeps first (the reference's
        interpolation to a vertex is its nodal value)."""
        from . import refine
        mesh = self._mesh
        m2 = refine.createP2(mesh, self.device)
        fop = ERTModelling(sr=False, device=self.device, rtol=1e-12, maxIter=max(self._maxIter, 100000),
                           precision="fp64")
        fop.setkValues(self._k)
        fop.setWeights(self._w)
        fop._dipole = self._dipole  # the same current patterns (pure poles for the dipole pattern)
        unit = self._data.copy()
        unit.set("k", np.ones(unit.size()))
        fop.setData(unit)
        fop.setMesh(m2, ignoreRegionManager=True)
        fop._forward(np.ones(m2.cellCount()))
        up = np.ascontiguousarray(fop.subPotentials()[:, :, :mesh.nodeCount()])
        del fop
        self._check(self._lib.ertgb_set_primary(self._ctx, up.shape[0], up.shape[1], up.shape[2], _ptr(up)))

    def _push_kw(self):
        k = np.ascontiguousarray(self._k, np.float64)
        w = np.ascontiguousarray(self._w, np.float64)
        self._check(self._lib.ertgb_set_kw(self._ctx, len(k), _ptr(k), _ptr(w)))

    def _push_scheme(self):
        data = self._data
        kf = data["k"]
        if data.size() == 0:
            raise ValueError("data container is empty")
        if np.min(np.abs(kf)) < TOLERANCE:
            # the reference computes missing factors analytically only for a flat
            # surface without CEM electrodes (DCMultiElectrodeModelling::response,
            # core/src/bert/dcfemmodelling.cpp:1088-1097)
            if self._topo or (self._electrodes is not None and self._electrodes.cem):
                raise ValueError("data contains no K-factors (topography or complete electrode model: "
                                 "give them, e.g. from calcGeometricFactor)")
            kf = self.calcGeometricFactor(data)
            data.set("k", kf)
        ab = np.ascontiguousarray(data.abmn(), np.int32)
        kf = np.ascontiguousarray(kf, np.float64)
        self._check(self._lib.ertgb_set_scheme(self._ctx, len(ab), _ptr(ab), _ptr(kf)))

    def setkValues(self, k):
        self._k = np.asarray(k, np.float64).copy()
        self._kw_user = True
        if self._w is not None and len(self._w) == len(self._k) and self._elec_nodes is not None:
            self._push_kw()

    def setWeights(self, w):
        self._w = np.asarray(w, np.float64).copy()
        self._kw_user = True
        if self._k is not None and len(self._w) == len(self._k) and self._elec_nodes is not None:
            self._push_kw()

    def kValues(self):
        return None if self._k is None else self._k.copy()

    def weights(self):
        return None if self._w is None else self._w.copy()

    @property
    def parameterCount(self):
        """Model parameters (twice the real count with complex resistivity,
        real parts first, as pygimli/physics/ert/ertModelling.py:146-149)."""
        return self._real_parameter_count() * (2 if self._complex else 1)

    def _real_parameter_count(self):
        if self._rm is not None:
            return self._rm.parameterCount()
        return int(self._mesh.cell_markers.max()) + 1

    # ------------------------------------------------- complex resistivity
    def setComplex(self, c=True):
        """Complex resistivity (induced polarisation): models and responses
        are [Re..., Im...] vectors and createJacobian returns the complex
        Jacobian (DCMultiElectrodeModelling::setComplex,
        core/src/bert/dcfemmodelling.cpp:573-583).  The reference then solves
        the total-potential problem (no singularity removal); so does this
        operator (ertgb_response_complex)."""
        self._complex = bool(c)
        self._J = None

    def complex(self):
        return self._complex

    def createStartModel(self, dataVals):
        """Start model: the median of the data values for every parameter
        (Modelling.createStartModel, pygimli/frameworks/modelling.py:231-244);
        complex: medians of the real and imaginary parts, a negative
        imaginary part flipped to positive, after which ``response`` and
        ``createJacobian`` work on the flipped convention: the model's
        imaginary part flipped before, the response's after, the Jacobian
        conjugated (ertModelling.py:168-238)."""
        v = np.asarray(dataVals)
        if not self._complex:
            return np.full(self.parameterCount, float(np.median(v)))
        z = v if np.iscomplexobj(v) else v[:len(v) // 2] + 1j * v[len(v) // 2:]
        P = self._real_parameter_count()
        re, im = np.median(z.real), np.median(z.imag)
        if im < 0:
            self._conjImag = True
            im = -im
        return np.concatenate([np.full(P, re), np.full(P, im)])

    def flipImagPart(self, v):
        """[Re..., Im...] of ``v`` ([Re..., Im...] or complex) with the
        imaginary part negated when the start model flipped it
        (ERTModelling.flipImagPart, ertModelling.py:188-202)."""
        return flip_imag(v, self._conjImag)

    def _complex_cells(self, model):
        """Per-cell (Re, Im) of a complex model [Re..., Im...]: one value per
        cell as given, else mapped like the reference's mapERTModel(CVector)
        (dcfemmodelling.cpp:1199-1210): the real part with prolongation of
        empty cells, the imaginary part as its own mapped model."""
        m = np.asarray(model)
        if np.iscomplexobj(m):
            re, im = m.real.astype(np.float64), m.imag.astype(np.float64)
        else:
            m = m.astype(np.float64)
            if len(m) % 2:
                raise ValueError("a complex model needs [Re..., Im...] (even length)")
            re, im = m[:len(m) // 2], m[len(m) // 2:]
        if len(re) == self._mesh.cellCount():
            return np.ascontiguousarray(re), np.ascontiguousarray(im)
        return (np.ascontiguousarray(self.mapERTModel(re)), np.ascontiguousarray(self.mapERTModel(im)))

    def _response_complex(self, model):
        torch = _torch()
        dev = torch.device("cuda", self.device)
        re, im = self._complex_cells(model)
        if np.min(np.hypot(re, im)) < TOLERANCE:
            raise ValueError("complex response for abs model with negative or zero resistivity is not defined")
        re_d = torch.from_numpy(re).to(dev)
        im_d = torch.from_numpy(im).to(dev)
        D = self._data.size()
        out = torch.empty((2, D), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        self._check(self._lib.ertgb_response_complex(self._ctx, ctypes.c_void_p(re_d.data_ptr()),
                                                     ctypes.c_void_p(im_d.data_ptr()),
                                                     ctypes.c_void_p(out[0].data_ptr()),
                                                     ctypes.c_void_p(out[1].data_ptr()), ctypes.c_void_p(stream)))
        self._last_model = np.asarray(model)
        return out.reshape(-1).cpu().numpy()

    def _jacobian_complex(self, model):
        torch = _torch()
        dev = torch.device("cuda", self.device)
        P = self._real_parameter_count()
        m = np.asarray(model)
        if np.iscomplexobj(m):
            mr, mi = m.real.astype(np.float64), m.imag.astype(np.float64)
        else:
            m = m.astype(np.float64)
            mr, mi = m[:len(m) // 2], m[len(m) // 2:]
        mr_d = torch.from_numpy(np.ascontiguousarray(mr)).to(dev)
        mi_d = torch.from_numpy(np.ascontiguousarray(mi)).to(dev)
        J = torch.empty((self._data.size(), P), dtype=torch.complex128, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        self._check(self._lib.ertgb_jacobian_complex(self._ctx, ctypes.c_void_p(mr_d.data_ptr()),
                                                     ctypes.c_void_p(mi_d.data_ptr()), int(len(mr)),
                                                     ctypes.c_void_p(J.data_ptr()), ctypes.c_void_p(stream)))
        self._J = J
        return J

    def calcGeometricFactor(self, data=None):
        """Geometric factors (DCMultiElectrodeModelling::calcGeometricFactor,
        core/src/bert/dcfemmodelling.cpp:1527-1557): analytic half-space
        factors for a flat surface without CEM electrodes, otherwise
        numerical ones, 1 / (u + 1e-12) with u the voltages of this operator
        (its formulation, forward mesh, electrodes and contact impedances) for
        a unit resistivity."""
        data = self._data if data is None else data
        cem = self._electrodes is not None and self._electrodes.cem
        if not (getattr(self, "_topo", False) or cem):
            return geometricFactors(data, self._mesh.dim())
        fop = ERTModelling(sr=self._sr, device=self.device, rtol=self._rtol, maxIter=self._maxIter,
                           precision=self.precision)
        if self._contact_z is not None:
            fop.setContactImpedances(self._contact_z)
        if self._bypass_r is not None:
            fop.setBypassResistances(self._bypass_r)
        if self._kw_user:
            fop.setkValues(self._k)
            fop.setWeights(self._w)
        unit = data.copy()
        unit.set("k", np.ones(unit.size()))
        fop.setData(unit)
        fop.setMesh(self._mesh, ignoreRegionManager=True)
        fop.response(np.ones(self._mesh.cellCount()))
        u = datamap_voltages(fop.electrodePotentials(), data.abmn())
        return 1.0 / (u + TOLERANCE)

    def mapERTModel(self, model, background=-9e99):
        """Cell resistivities of ``model`` (per cell or per parameter, the
        region manager's fixed values and ``background`` for unmapped cells),
        kept for ``calculate`` as the reference keeps them as cell attributes
        (DCMultiElectrodeModelling::mapERTModel, dcfemmodelling.cpp:1211-1218)."""
        fixed = self._rm.fixedValues() if self._rm is not None else None
        rho = map_model(self._mesh, model, background, fixed)
        self._mapped = rho
        return rho

    # ---------------------------------------------------------- forward
    def _ready(self):
        if self._mesh is None or self._data is None:
            raise RuntimeError("mesh and data must be set")
        if self._data.exists("k") and np.min(np.abs(self._data["k"])) >= TOLERANCE:
            return
        self._push_scheme()

    def response(self, model):
        """Apparent resistivities for ``model`` (numpy in -> numpy out, or a
        CUDA tensor of per-cell resistivities -> CUDA tensor).  With
        setComplex(True): [Re..., Im...] of the complex apparent
        resistivities for a model [Re..., Im...] (or a complex array)."""
        if self._dipole:
            # DCMultiElectrodeModelling::response_ throws there (dcfemmodelling.cpp:1231-1233)
            raise NotImplementedError("response with the dipole current pattern is not implemented (neither in "
                                      "the reference); calculate(data) gives its voltages")
        return self._forward(model)

    def _forward(self, model):
        self._ready()
        if self._complex:
            if not self._conjImag:
                return self._response_complex(model)
            return self.flipImagPart(self._response_complex(self.flipImagPart(model)))
        torch = _torch()
        if isinstance(model, torch.Tensor) and model.is_cuda:
            rho = model.to(torch.float64).contiguous()
            if rho.numel() != self._mesh.cellCount():
                raise ValueError("device models must be per-cell resistivities")
            out = torch.empty(self._data.size(), dtype=torch.float64, device=rho.device)
            self._response_dev(rho, out)
            self._last_model = rho
            self._mapped = rho
            return out
        m = np.asarray(model, np.float64)
        if np.min(m) < TOLERANCE:
            raise ValueError(f"response for model with negative or zero resistivity is not defined: "
                             f"min={m.min()}")
        rho = np.ascontiguousarray(self.mapERTModel(m), np.float64)
        dev = torch.device("cuda", self.device)
        rho_d = torch.from_numpy(rho).pin_memory().to(dev, non_blocking=True)
        out = torch.empty(self._data.size(), dtype=torch.float64, device=dev)
        self._response_dev(rho_d, out)
        self._last_model = m
        self._mapped = rho
        return out.cpu().numpy()

    def _response_dev(self, rho, out):
        torch = _torch()
        stream = torch.cuda.current_stream(rho.device).cuda_stream
        self._check(self._lib.ertgb_response(self._ctx, ctypes.c_void_p(rho.data_ptr()),
                                             ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream)))

    # ------------------------------------------- learned preconditioner
    def assemble(self, model):
        """Assemble the system matrices of every wavenumber for ``model``
        without solving (training data of the learned preconditioner)."""
        self._ready()
        torch = _torch()
        dev = torch.device("cuda", self.device)
        if isinstance(model, torch.Tensor) and model.is_cuda:
            rho = model.to(torch.float64).contiguous()
        else:
            rho = torch.from_numpy(np.ascontiguousarray(self.mapERTModel(np.asarray(model, np.float64)))).to(dev)
        if rho.numel() != self._mesh.cellCount():
            raise ValueError("model does not match the mesh")
        stream = torch.cuda.current_stream(dev).cuda_stream
        self._check(self._lib.ertgb_assemble(self._ctx, ctypes.c_void_p(rho.data_ptr()), ctypes.c_void_p(stream)))
        self._assembled = rho  # keep the buffer alive until the stream has used it

    def lpForward(self, theta):
        """Network factor G of the assembled matrices for device weights
        ``theta``: (n_k, n_lower) float32 tensor, A's lower triangle row-major."""
        torch = _torch()
        n, nnz, _, _ = self.sizes()
        nL = (nnz + n) // 2
        G = torch.empty((len(self._k), nL), dtype=torch.float32, device=theta.device)
        stream = torch.cuda.current_stream(theta.device).cuda_stream
        self._check(self._lib.ertgb_lp_forward(self._ctx, ctypes.c_void_p(theta.data_ptr()),
                                               ctypes.c_void_p(G.data_ptr()), ctypes.c_void_p(stream)))
        return G

    def lpLossGrad(self, theta, grad=None):
        """Kaporin loss of the assembled matrices (float) and, into ``grad``
        (device tensor of the weights' size), its gradient."""
        torch = _torch()
        loss = ctypes.c_double()
        stream = torch.cuda.current_stream(theta.device).cuda_stream
        self._check(self._lib.ertgb_lp_loss_grad(
            self._ctx, ctypes.c_void_p(theta.data_ptr()), None if grad is None else ctypes.c_void_p(grad.data_ptr()),
            ctypes.byref(loss), ctypes.c_void_p(stream)))
        return loss.value

    def lpFeatures(self):
        """Network inputs of the assembled matrices: node (n_k, n, 4) and edge
        (n_k, nnz, 4) features (device tensors)."""
        torch = _torch()
        n, nnz, _, _ = self.sizes()
        dev = torch.device("cuda", self.device)
        x = torch.empty((len(self._k), n, 4), dtype=torch.float32, device=dev)
        f = torch.empty((len(self._k), nnz, 4), dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        self._check(self._lib.ertgb_lp_features(self._ctx, ctypes.c_void_p(x.data_ptr()),
                                                ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(stream)))
        return x, f

    def createJacobian(self, model, dtype="float64"):
        """Jacobian d rhoa / d model from the potentials of the last response
        (like the reference, which reuses its stored sub-potentials).  Stored
        on the device; ``jacobian()`` returns it."""
        torch = _torch()
        if self._mesh is None:
            raise RuntimeError("no mesh")
        if self._dipole:
            # the reference has no working dipole-pattern Jacobian: prepareJacobianT_
            # takes one potential row per (a, b) pattern from calculate(DataContainerERT &)
            # (dcfemmodelling.cpp:1290-1292), and the Jacobian's pattern branch
            # (core/src/bert/bertJacobian.cpp:172-181) looks the pattern up from its
            # zero-initialised a, b, m, n before it reads any datum's electrodes
            raise NotImplementedError("createJacobian with the dipole current pattern is not implemented "
                                      "(neither in the reference)")
        if self._complex:
            if not self._conjImag:
                return self._jacobian_complex(model)
            J = self._jacobian_complex(self.flipImagPart(model))
            J.imag.neg_()  # conjugate in place (the complex Jacobian can be tens of GB)
            return J
        P = self.parameterCount
        D = self._data.size()
        tdt = torch.float64 if dtype in ("float64", torch.float64) else torch.float32
        dev = torch.device("cuda", self.device)
        if isinstance(model, torch.Tensor):
            md = model.to(device=dev, dtype=torch.float64).contiguous()
        else:
            md = torch.from_numpy(np.ascontiguousarray(model, np.float64)).to(dev)
        J = torch.empty((D, P), dtype=tdt, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream

        def run():
            return self._lib.ertgb_jacobian(self._ctx, ctypes.c_void_p(md.data_ptr()), int(md.numel()),
                                            ctypes.c_void_p(J.data_ptr()), 0 if tdt == torch.float64 else 1,
                                            ctypes.c_void_p(stream))

        rc = run()
        if rc == _native.STATE:
            self._potentials_for_jacobian(md.cpu().numpy() if isinstance(model, torch.Tensor) else model)
            rc = run()
        self._check(rc)
        self._J = J
        return J

    def _potentials_for_jacobian(self, model):
        """Sub-potentials for a Jacobian requested before any response
        (prepareJacobianT_, core/src/bert/dcfemmodelling.cpp:1262-1301): for a
        homogeneous model (standard deviation <= 1e-7) on a flat surface
        without CEM electrodes the analytic half-space potentials scaled by
        model[0]; otherwise the potentials of a response to the model."""
        m = np.asarray(model, np.float64).ravel()
        sd = float(np.std(m, ddof=1)) if m.size > 1 else 0.0
        cem = self._electrodes is not None and (self._electrodes.cem or len(self._electrodes.rows) > 0)
        if sd <= TOLERANCE * 1e5 and not self._topo and not cem:
            self._check(self._lib.ertgb_analytic_potentials(self._ctx, float(m[0])))
        else:
            self.response(model)

    def jacobian(self):
        return self._J

    # ---------------------------------------------------- inspection
    def sizes(self):
        n = ctypes.c_int64()
        nnz = ctypes.c_int64()
        p = ctypes.c_int64()
        r = ctypes.c_int64()
        self._check(self._lib.ertgb_sizes(self._ctx, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(p),
                                          ctypes.byref(r)))
        return n.value, nnz.value, p.value, r.value

    def pattern(self):
        n, nnz, _, _ = self.sizes()
        rp = np.zeros(n + 1, np.int32)
        ci = np.zeros(nnz, np.int32)
        self._check(self._lib.ertgb_get_pattern(self._ctx, _ptr(rp), _ptr(ci)))
        return rp, ci

    def matrix(self, k_index=0, which=0):
        _, nnz, _, _ = self.sizes()
        v = np.zeros(nnz)
        self._check(self._lib.ertgb_get_matrix(self._ctx, int(k_index), int(which), _ptr(v)))
        return v

    def subPotentials(self):
        """[k][electrode][node] total potentials of the last response."""
        n, _, _, _ = self.sizes()
        out = np.zeros((len(self._k), len(self._elec_nodes), n))
        self._check(self._lib.ertgb_get_potentials(self._ctx, _ptr(out)))
        return out

    def primaryPotentials(self):
        n, _, _, _ = self.sizes()
        out = np.zeros((len(self._k), len(self._elec_nodes), n))
        self._check(self._lib.ertgb_get_primary(self._ctx, _ptr(out)))
        return out

    def solution(self):
        """k-summed potentials per electrode source (nE x rows), the
        reference's solutions_ (dcfemmodelling.cpp:1707-1729): the first
        wavenumber's term, then the others added in order."""
        u = self.subPotentials()
        sol = u[0] * self._w[0]
        for ki in range(1, len(self._w)):
            sol += u[ki] * self._w[ki]
        return sol

    def electrodePotentials(self):
        """U[e, f]: potential at electrode f for the unit current of pattern
        e after the last response -- the reference's DataMap
        (DataMap::collect, core/src/bert/datamap.cpp:57-98): the k-summed
        solution at the electrodes (a node, or the shape functions of the
        cell that holds the electrode); with CEM the extension rows of the
        last wavenumber, unweighted (dcfemmodelling.cpp:1642-1644).
        Collected on the device (ertgb_get_electrode_potentials)."""
        nE = len(self._elec_nodes)
        U = np.zeros((nE, nE))
        self._check(self._lib.ertgb_get_electrode_potentials(self._ctx, _ptr(U)))
        return U

    # ------------------------------------------------ dipole current pattern
    def setDipoleCurrentPattern(self, dipole=True):
        """One current pattern per distinct (a, b) pair of the data instead
        of one per electrode (DCMultiElectrodeModelling::
        setDipoleCurrentPattern, core/src/bert/dcfemmodelling.h:211;
        createCurrentPattern, dcfemmodelling.cpp:1488-1513).  Forward only,
        as in the reference: ``calculate(data)`` gives the voltages,
        ``response`` and ``createJacobian`` refuse the mode.

        The (a, b) pattern is solved as the difference of the pure poles a and
        b: +1 at one electrode and no reference electrode (in a closed domain
        the current drains at the calibration nodes).  The difference is the
        dipole solution itself, not an approximation of it: each wavenumber
        has one system matrix S for every source (its mixed boundaries use one
        source centre, 2181-2182), the total-potential right-hand side is
        linear in the source, and the singularity-removal potential u = u_p +
        u_s solves S u = S1 (p_a - p_b) at the free nodes whatever the source
        resistivity rho_s (u_p = rho_s (p_a - p_b), rhs = S1 u_p / rho_s -
        S u_p, 2228-2254).  Only at the fixed-potential nodes of singularity
        removal (calibration, homogeneous Dirichlet) does the reference keep
        u = u_p with the pattern's own rho_s; ``calculate`` refuses a
        measuring electrode there.  Solving the poles costs one solve per
        electrode and wavenumber instead of one per (a, b) pattern."""
        dipole = bool(dipole)
        if dipole != self._dipole:
            self._dipole = dipole
            self._J = None
            if self._mesh is not None and self._data is not None:
                self._update_data()

    def dipoleCurrentPattern(self):
        return self._dipole

    def calculate(self, data=None, reciprocity=False):
        """Voltages for a unit current of ``data`` (default: the operator's
        own) at the cell resistivities of the last ``mapERTModel`` or
        ``response``, written to data 'u' and returned
        (DCMultiElectrodeModelling::calculate(DataContainerERT &, bool),
        core/src/bert/dcfemmodelling.cpp:1558-1618): u = (U[a,m] - U[a,n]) -
        (U[b,m] - U[b,n]) of ``electrodePotentials``, signed, without the
        rounding and the reciprocal mean of ``response``.  ``reciprocity``
        changes nothing, as in the reference (1566, 1628-1639).  With the
        dipole current pattern every datum's (a, b) pair must be one of the
        operator's own data (the reference finds no pattern index otherwise,
        1581-1586).  The operator's data need geometric factors where
        ``response`` needs them (topography, CEM); their values do not enter."""
        if self._complex:
            raise NotImplementedError("calculate with complex resistivity is not implemented (the reference "
                                      "refuses it, dcfemmodelling.cpp:1562)")
        if self._mapped is None:
            raise RuntimeError("no model: call mapERTModel(model) or response(model) first")
        self._ready()
        data = self._data if data is None else data
        ab = np.asarray(data.abmn(), np.int64).reshape(-1, 4)
        nE = len(self._elec_nodes)
        if ab.size and (ab.max() >= nE or ab.min() < -1):
            raise ValueError("electrode index out of range of the operator's electrodes")
        if self._dipole:
            own = {tuple(p) for p in np.asarray(self._data.abmn(), np.int64)[:, :2].tolist()}
            for p in ab[:, :2].tolist():
                if tuple(p) not in own:
                    raise ValueError(f"current pattern (a, b) = {tuple(p)} is not among the operator's data")
            if self._sr:
                self._refuse_fixed_measuring(ab)
        torch = _torch()
        dev = torch.device("cuda", self.device)
        rho = self._mapped
        if isinstance(rho, torch.Tensor):
            rho_d = rho.to(device=dev, dtype=torch.float64).contiguous()
        else:
            rho_d = torch.from_numpy(np.ascontiguousarray(rho, np.float64)).to(dev)
        if rho_d.numel() != self._mesh.cellCount():
            raise ValueError("the mapped model must give one resistivity per cell")
        out = torch.empty(self._data.size(), dtype=torch.float64, device=dev)
        self._response_dev(rho_d, out)
        u = datamap_voltages(self.electrodePotentials(), ab)
        data.set("u", u)
        return u

    def _refuse_fixed_measuring(self, ab):
        """Singularity removal with the dipole pattern: no measuring
        electrode on a calibration or homogeneous Dirichlet node."""
        bc = self._bc
        fixed = np.union1d(np.asarray(bc.calib, np.int64), np.asarray(bc.dirichlet, np.int64))
        if not len(fixed):
            return
        es = self._esearch
        for e in np.unique(ab[:, 2:][ab[:, 2:] >= 0]):
            support = [es.nodes[e]] if es.nodes[e] >= 0 else self._mesh.cells[es.cells[e]]
            if np.isin(support, fixed).any():
                raise NotImplementedError(f"the dipole current pattern with singularity removal and measuring "
                                          f"electrode {int(e)} on a fixed-potential (calibration or Dirichlet) "
                                          f"node is not implemented")

    def stats(self):
        s = _native.Stats()
        self._check(self._lib.ertgb_get_stats(self._ctx, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def electrodeNodes(self):
        return None if self._elec_nodes is None else self._elec_nodes.copy()


def _cell_values(mesh, res):
    """The forms of ``res`` simulate accepts: a number (real or complex), one
    value per cell, a map [[marker, value], ...] (pyGIMLi's parseArgToArray)
    or N x cellCount rows.  Returns (array, is_rows)."""
    C = mesh.cellCount()
    if np.isscalar(res):
        return np.full(C, res, dtype=complex if np.iscomplexobj(res) else float), False
    first = res[0]
    if hasattr(first, "__iter__") and len(first) == 2 and len(res) != C:
        markers = mesh.cell_markers
        table = {int(m): v for m, v in res}
        missing = sorted(set(np.unique(markers).tolist()) - set(table))
        if missing:
            raise ValueError(f"Mesh contains markers without assigned resistivities {missing}. Please fix given rhomap.")
        vals = np.array([table[int(m)] for m in markers])
        return vals, False
    arr = np.asarray(res)
    if arr.ndim == 2:
        return arr, True
    if len(arr) != C:
        raise IndexError("Simulate called with wrong resistivity array.")
    return arr, False


def flip_imag(v, conj):
    """[Re..., Im...] of ``v`` ([Re..., Im...] or a complex array), the
    imaginary part negated when ``conj`` (pg.utils.squeezeComplex(toComplex(v),
    conj=...))."""
    a = np.asarray(v)
    if np.iscomplexobj(a):
        re, im = a.real, a.imag
    else:
        a = a.astype(np.float64)
        if len(a) % 2:
            raise ValueError("a complex vector needs [Re..., Im...] (even length)")
        re, im = a[:len(a) // 2], a[len(a) // 2:]
    return np.concatenate([re, -im if conj else im]).astype(np.float64)


def datamap_voltages(U, abmn):
    """Voltages of the scheme from the electrode potential matrix, without
    rounding or reciprocity (DataMap::data, core/src/bert/datamap.cpp:
    159-231): (U[a,m] - U[a,n]) - (U[b,m] - U[b,n]), index -1 = infinity."""
    U = np.asarray(U, np.float64)
    ab = np.asarray(abmn, np.int64).reshape(-1, 4)

    def g(i, j):
        ok = (i != -1) & (j != -1)
        return np.where(ok, U[np.where(ok, i, 0), np.where(ok, j, 0)], 0.0)

    a, b, m, n = ab[:, 0], ab[:, 1], ab[:, 2], ab[:, 3]
    return (g(a, m) - g(a, n)) - (g(b, m) - g(b, n))


def createGeometricFactors(scheme, numerical=None, mesh=None, dim=3, h2=True, p2=True, verbose=False, **kwargs):
    """Geometric factors (pg.physics.ert.createGeometricFactors,
    pygimli/physics/ert/ert.py:323-397): analytic half-space factors, or
    with ``numerical`` the inverse voltages of a unit-resistivity
    total-potential simulation on ``mesh`` refined by H2 then P2 (``h2``,
    ``p2``), which holds topography.  A mesh must be given: the reference's
    default inversion mesh needs a mesh generator.  Keywords of
    ERTModelling (device, precision, ...) are passed on."""
    if not numerical and mesh is None:
        return geometricFactors(scheme, dim)
    if mesh is None:
        raise NotImplementedError("numerical geometric factors need a mesh (no mesh generator here)")
    m = mesh
    if h2:
        m = m.createH2()
    if p2:
        m = m.createP2()
    d = simulate(m, scheme, 1.0, sr=False, calcOnly=True, **kwargs)
    return 1.0 / d["u"]


def simulate(mesh, scheme, res, **kwargs):
    """Simulate an ERT measurement (pg.physics.ert.simulate,
    pygimli/physics/ert/ert.py:12-285): apparent resistivities of ``res`` for
    ``scheme`` on ``mesh``, with apparent phases ('phia') for complex
    resistivity; ``noiseLevel`` > 0 adds Gaussian noise with the errors of
    ``estimateError`` (``noiseAbs`` V at 1 A; ``seed`` fixes it, numpy's
    generator: the draws differ from pyGIMLi's); ``returnArray`` returns
    rhoa (and phia) instead of the container.  ``calcOnly``: the voltages
    only ('r' per unit current, 'i' = ``current``, 'u'), no geometric
    factors (ert.py:186-201); ``returnFields``: the k-summed potentials per
    source; ``contactImpedances`` (a value or one per electrode): CEM contact
    impedances of the total-potential operator (``sr=False``) -- the
    reference passes fixed values there instead (ert.py:123-128).  Keywords
    of ERTModelling (sr, device, precision, precond, ...) are passed on."""
    from .data import estimateError
    calc_only = bool(kwargs.pop("calcOnly", False))
    return_fields = bool(kwargs.pop("returnFields", False))
    contact = kwargs.pop("contactImpedances", None)
    kwargs.pop("verbose", None)
    return_array = kwargs.pop("returnArray", False)
    noise_level = float(kwargs.pop("noiseLevel", 0.0))
    noise_abs = kwargs.pop("noiseAbs", 1e-4)
    seed = kwargs.pop("seed", None)
    phi_err = kwargs.pop("phiErr", None)
    current = kwargs.pop("current", 1.0)
    return_fop = kwargs.pop("returnFOP", False)
    fop = ERTModelling(**kwargs)
    if contact is not None:
        z = np.asarray(contact, np.float64)
        fop.setContactImpedances(np.full(scheme.sensorCount(), float(z)) if z.ndim == 0 else z)
    data = scheme.copy()
    vals, rows = _cell_values(mesh, res)
    cplx = np.iscomplexobj(vals)
    fop.setComplex(cplx)
    k_given = data.allNonZero("k")
    if calc_only:
        if cplx:
            raise NotImplementedError("simulate(calcOnly=True) with complex resistivity (the reference has none)")
        if rows:
            raise ValueError("simulate(calcOnly=True) takes one resistivity per cell")
        # the scheme's factors only scale apparent resistivities, which calcOnly does not return
        k_saved = data["k"].copy() if data.exists("k") else None
        data.set("k", np.ones(data.size()))
    elif not k_given:
        data.set("k", geometricFactors(data, mesh.dim()))
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    D = data.size()
    if calc_only:
        fop.response(vals)
        if return_fields:
            return fop.solution()
        r = datamap_voltages(fop.electrodePotentials(), data.abmn())
        if k_saved is not None:
            data.set("k", k_saved)
        else:
            data.set("k", np.zeros(D))
        data.set("r", r)
        data.set("i", np.full(D, float(current)))
        data.set("u", r * float(current))
        return data
    for t in ("u", "i", "r"):
        data.set(t, np.zeros(D))

    def one(v):
        out = fop.response(v)
        if cplx:
            z = out[:D] + 1j * out[D:]
            return np.abs(z), np.angle(z)
        return np.asarray(out), None

    if rows:
        both = [one(v) for v in vals]
        rhoa = np.array([b[0] for b in both])
        phia = np.array([b[1] for b in both]) if cplx else None
        data.set("rhoa", rhoa[0])
        if cplx:
            data.set("phia", phia[0])
    else:
        rhoa, phia = one(vals)
        data.set("rhoa", rhoa)
        if cplx:
            data.set("phia", phia)
    if return_fields:
        return fop.solution()
    if noise_level > 0 and not rows:
        rng = np.random.default_rng(seed)
        if not data.allNonZero("err"):
            data.set("err", estimateError(data, relativeError=noise_level, absoluteUError=noise_abs,
                                          absoluteCurrent=1))
        rhoa = rhoa * (1.0 + rng.standard_normal(D) * data["err"])
        data.set("rhoa", rhoa)
        if phia is not None:
            if data.allNonZero("iperr"):
                ip_err = data["iperr"]
            else:
                level = noise_level / 100.0 if noise_level > 0.5 else noise_level
                ip_err = np.full(D, phi_err / 1000.0) if phi_err is not None else np.abs(phia) * level
            phia = phia + rng.standard_normal(D) * ip_err
            data.set("iperr", ip_err)
            data.set("phia", phia)
    if data.allNonZero("k"):
        data.set("r", data["rhoa"] / data["k"])
        data.set("i", np.full(D, float(current)))
        data.set("u", data["r"] * data["i"])
    if return_array:
        return (rhoa, phia) if phia is not None else rhoa
    data.set("valid", np.ones(D))
    return (data, fop) if return_fop else data
