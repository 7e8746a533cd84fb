// Test infrastructure only: a C entry layer over the reference's own C++
// ERT modelling code, compiled from the reference sources into
// oracle/_ref/libgimli_ref.so by oracle/Makefile.  Nothing in the product
// links or loads this file; tests and fixture generation call it through
// ctypes (oracle/ref_driver.py) to obtain reference outputs.
//
// What it drives (reference file:line):
//   mesh construction      core/src/mesh.h:183-217 (createNode/createTriangle/
//                          createTetrahedron/createEdge/createTriangleFace),
//                          mesh.h:457 createNeighborInfos
//   data container         core/src/bert/bertDataContainer.h:62 addFourPointData
//   forward operator       core/src/bert/dcfemmodelling.h:344 DCSRMultiElectrodeModelling,
//                          dcfemmodelling.h:105 DCMultiElectrodeModelling (total potential,
//                          complete electrode model, bypass electrodes)
//   response / Jacobian    core/src/bert/dcfemmodelling.cpp:1085-1197, 1446-1476
//   mesh / data I/O        core/src/mesh_io.cpp:391-662 (binary mesh v3),
//                          mesh_io.cpp:674-992 exportVTK,
//                          core/src/datacontainer.cpp:209-470 load, 518-615 save
//   regularised CGLS       core/src/solver.cpp:27-212 solveCGLSCDWWhtrans
//   solver injection       core/src/bert/dcfemmodelling.h:266 setSolver,
//                          core/src/solverWrapper.h:26-56 SolverWrapper
// The reference's default direct solver (CHOLMOD/UMFPACK) is not available,
// so the solve is delegated to a host callback (an FP64 sparse direct solver
// supplied by the caller).  Every other step is the reference's own code.

#include <gimli.h>
#include <mesh.h>
#include <node.h>
#include <meshentities.h>
#include <sparsematrix.h>
#include <regionManager.h>
#include <solverWrapper.h>
#include <bert/dcfemmodelling.h>
#include <bert/bertDataContainer.h>
#include <bert/bertMisc.h>
#include <bert/bertJacobian.h>
#include <solver.h>

#include <cstring>
#include <exception>
#include <string>
#include <vector>

namespace GIMLI {
// Defined (not declared in a header) in core/src/bert/dcfemmodelling.cpp:300-304.
void dcfemBoundaryAssembleStiffnessMatrix(RSparseMatrix &S, const Mesh &mesh,
                                          const RVector3 &source, double k);
}

using namespace GIMLI;

extern "C" {
// factor(n, nnz, rowptr, colidx, vals): called once per system matrix.
typedef int (*ref_factor_fn)(int n, int nnz, const int *rowptr,
                             const int *colidx, const double *vals);
// solve(n, rhs, x): x = A^{-1} rhs for the last factored matrix.
typedef int (*ref_solve_fn)(int n, const double *rhs, double *x);
// complex variants (values, right-hand side and solution interleaved re, im)
typedef int (*ref_cfactor_fn)(int n, int nnz, const int *rowptr, const int *colidx, const double *vals);
typedef int (*ref_csolve_fn)(int n, const double *rhs, double *x);
}

namespace {

std::string g_last_error;

class CallbackSolver : public SolverWrapper {
public:
    CallbackSolver(ref_factor_fn f, ref_solve_fn s) : SolverWrapper(false), f_(f), s_(s) {}
    void setMatrix(const RSparseMatrix &S) override {
        const std::vector<int> &cp = S.vecColPtr();
        const std::vector<int> &ri = S.vecRowIdx();
        const RVector &v = S.vecVals();
        n_ = (int)S.rows();
        int rc = f_(n_, (int)ri.size(), cp.data(), ri.data(), &v[0]);
        if (rc != 0) throwError("oracle factor callback failed");
    }
    void solve(const RVector &rhs, RVector &sol) override {
        if ((int)sol.size() != n_) sol.resize(n_);
        int rc = s_(n_, &rhs[0], &sol[0]);
        if (rc != 0) throwError("oracle solve callback failed");
    }
    void setComplex(ref_cfactor_fn f, ref_csolve_fn s) { cf_ = f; cs_ = s; }
    void setMatrix(const CSparseMatrix &S) override {
        if (!cf_) throwError("no complex solver callback");
        const std::vector<int> &cp = S.vecColPtr();
        const std::vector<int> &ri = S.vecRowIdx();
        const CVector &v = S.vecVals();
        n_ = (int)S.rows();
        int rc = cf_(n_, (int)ri.size(), cp.data(), ri.data(), reinterpret_cast<const double *>(&v[0]));
        if (rc != 0) throwError("oracle complex factor callback failed");
    }
    void solve(const CVector &rhs, CVector &sol) override {
        if ((int)sol.size() != n_) sol.resize(n_);
        int rc = cs_(n_, reinterpret_cast<const double *>(&rhs[0]), reinterpret_cast<double *>(&sol[0]));
        if (rc != 0) throwError("oracle complex solve callback failed");
    }
private:
    ref_factor_fn f_;
    ref_solve_fn s_;
    ref_cfactor_fn cf_ = nullptr;
    ref_csolve_fn cs_ = nullptr;
    int n_ = 0;
};

// The reference operator (singularity removal: DCSRMultiElectrodeModelling;
// total potential: DCMultiElectrodeModelling) plus one helper: drop the
// caller-owned real sub-potential matrix so that the complex path allocates
// its own.
template <class Base> struct ShimFop : Base {
    explicit ShimFop(bool verbose) : Base(verbose) {}
    void detachSubpotentials() {
        if (!this->subpotOwner_) {
            this->subSolutions_ = nullptr;
            this->subpotOwner_ = true;
        }
    }
    static void detach(DCMultiElectrodeModelling *f) { static_cast<ShimFop *>(f)->detachSubpotentials(); }
};

struct RefHandle {
    Mesh mesh;
    DataContainerERT data;
    DCMultiElectrodeModelling *fop = nullptr;
    void (*detach)(DCMultiElectrodeModelling *) = nullptr;
    CallbackSolver *solver = nullptr;
    RMatrix subpots;          // collected sub-potentials (nE*nK x nNodes)
    RMatrix prim;             // primary potentials given to the singularity-removal operator
    RefHandle(int dim) : mesh(dim) {}
    ~RefHandle() { delete fop; delete solver; }
};

template <class F> int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch (std::exception &e) {
        g_last_error = e.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

}  // namespace

extern "C" {

const char *ref_last_error() { return g_last_error.c_str(); }

// Build mesh + data container + forward operator: sr = 1 the singularity-
// removal operator (DCSRMultiElectrodeModelling), sr = 0 the total-potential
// operator (DCMultiElectrodeModelling, which alone builds the complete
// electrode model and bypass resistors, dcfemmodelling.cpp:1786-1833).
// cellNodes: nCells*nv (nv=3 triangle, 4 tetrahedron), bndNodes: nBnd*nvb.
// abmn: nData*4 with -1 for an electrode at infinity.  kfac may be NULL.
// contactZ (nZ values, may be NULL): setContactImpedances (dcfemmodelling.cpp:786-788).
void *ref_create_ex(int dim, int nNodes, const double *xyz, const int *nodeMarker,
                    int nCells, int nv, const int *cellNodes, const int *cellMarker,
                    int nBnd, int nvb, const int *bndNodes, const int *bndMarker,
                    int nSensors, const double *sensorXyz, int nData, const int *abmn,
                    const double *kfac, int verbose, int p2, int sr, int nZ, const double *contactZ) {
    RefHandle *h = nullptr;
    int rc = guarded([&] {
        h = new RefHandle(dim);
        Mesh &m = h->mesh;
        for (int i = 0; i < nNodes; i++)
            m.createNode(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], nodeMarker[i]);
        for (int c = 0; c < nCells; c++) {
            const int *cn = cellNodes + (size_t)c * nv;
            if (nv == 3) m.createTriangle(m.node(cn[0]), m.node(cn[1]), m.node(cn[2]), cellMarker[c]);
            else if (nv == 4) m.createTetrahedron(m.node(cn[0]), m.node(cn[1]), m.node(cn[2]), m.node(cn[3]), cellMarker[c]);
            else throwError("unsupported cell node count");
        }
        for (int b = 0; b < nBnd; b++) {
            const int *bn = bndNodes + (size_t)b * nvb;
            if (nvb == 2) m.createEdge(m.node(bn[0]), m.node(bn[1]), bndMarker[b]);
            else if (nvb == 3) m.createTriangleFace(m.node(bn[0]), m.node(bn[1]), m.node(bn[2]), bndMarker[b]);
            else throwError("unsupported boundary node count");
        }
        m.createNeighborInfos();
        if (p2) {  // 1: quadratic elements, 2: uniform H2 refinement (the reference's own)
            Mesh m2 = p2 == 2 ? m.createH2() : m.createP2();
            h->mesh = m2;
            h->mesh.createNeighborInfos();
        }
        for (int s = 0; s < nSensors; s++)
            h->data.createSensor(RVector3(sensorXyz[3 * s], sensorXyz[3 * s + 1], sensorXyz[3 * s + 2]), 1e-9);
        for (int d = 0; d < nData; d++)
            h->data.addFourPointData(abmn[4 * d], abmn[4 * d + 1], abmn[4 * d + 2], abmn[4 * d + 3]);
        if (kfac) {
            RVector k(nData);
            for (int d = 0; d < nData; d++) k[d] = kfac[d];
            h->data.set("k", k);
        }
        if (sr) {
            h->fop = new ShimFop<DCSRMultiElectrodeModelling>(verbose != 0);
            h->detach = &ShimFop<DCSRMultiElectrodeModelling>::detach;
        } else {
            h->fop = new ShimFop<DCMultiElectrodeModelling>(verbose != 0);
            h->detach = &ShimFop<DCMultiElectrodeModelling>::detach;
        }
        if (contactZ && nZ > 0) {
            RVector z(nZ);
            for (int i = 0; i < nZ; i++) z[i] = contactZ[i];
            h->fop->setContactImpedances(z);
        }
        h->fop->setData(h->data);
        h->fop->setMesh(h->mesh, true);
        h->fop->collectSubPotentials(h->subpots);
        h->fop->initJacobian();
    });
    if (rc) { delete h; return nullptr; }
    return h;
}

// The singularity-removal operator (the original entry point).
void *ref_create(int dim, int nNodes, const double *xyz, const int *nodeMarker,
                 int nCells, int nv, const int *cellNodes, const int *cellMarker,
                 int nBnd, int nvb, const int *bndNodes, const int *bndMarker,
                 int nSensors, const double *sensorXyz, int nData, const int *abmn,
                 const double *kfac, int verbose, int p2) {
    return ref_create_ex(dim, nNodes, xyz, nodeMarker, nCells, nv, cellNodes, cellMarker, nBnd, nvb, bndNodes,
                         bndMarker, nSensors, sensorXyz, nData, abmn, kfac, verbose, p2, 1, 0, nullptr);
}

void ref_destroy(void *hp) { delete (RefHandle *)hp; }

// Sizes and arrays of the mesh the operator runs on (after createP2).
int ref_mesh_sizes(void *hp, int *n, int *C, int *nv, int *B, int *nvb) {
    RefHandle *h = (RefHandle *)hp;
    Mesh &m = h->mesh;
    *n = (int)m.nodeCount();
    *C = (int)m.cellCount();
    *nv = m.cellCount() ? (int)m.cell(0).nodeCount() : 0;
    *B = (int)m.boundaryCount();
    *nvb = m.boundaryCount() ? (int)m.boundary(0).nodeCount() : 0;
    return 0;
}

int ref_mesh_arrays(void *hp, double *xyz, int *nodeMarker, int *cells, int *cellMarker, int *bnd, int *bndMarker) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        Mesh &m = h->mesh;
        for (Index i = 0; i < m.nodeCount(); i++) {
            xyz[3 * i] = m.node(i).pos()[0];
            xyz[3 * i + 1] = m.node(i).pos()[1];
            xyz[3 * i + 2] = m.node(i).pos()[2];
            nodeMarker[i] = m.node(i).marker();
        }
        for (Index c = 0; c < m.cellCount(); c++) {
            const Cell &cl = m.cell(c);
            for (Index j = 0; j < cl.nodeCount(); j++) cells[c * cl.nodeCount() + j] = (int)cl.node(j).id();
            cellMarker[c] = cl.marker();
        }
        for (Index b = 0; b < m.boundaryCount(); b++) {
            const Boundary &bd = m.boundary(b);
            for (Index j = 0; j < bd.nodeCount(); j++) bnd[b * bd.nodeCount() + j] = (int)bd.node(j).id();
            bndMarker[b] = bd.marker();
        }
    });
}

// Primary potentials of the singularity-removal operator given by the caller
// (rows = current source + wavenumber * sources, cols = nodes): the
// reference's setPrimaryPotential (core/src/bert/dcfemmodelling.h:374);
// checkPrimpotentials_ (dcfemmodelling.cpp:1986-2141) then takes them as they are.
int ref_set_primary(void *hp, int rows, int cols, const double *P) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        auto *sr = dynamic_cast<DCSRMultiElectrodeModelling *>(h->fop);
        if (!sr) throwError("primary potentials need the singularity-removal operator");
        h->prim.resize(rows, cols);
        for (int i = 0; i < rows; i++)
            for (int j = 0; j < cols; j++) h->prim[i][j] = P[(size_t)i * cols + j];
        sr->setPrimaryPotential(h->prim);
    });
}

int ref_set_solver(void *hp, ref_factor_fn f, ref_solve_fn s) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        delete h->solver;
        h->solver = new CallbackSolver(f, s);
        h->fop->setSolver(h->solver);
    });
}

// Complex solve callbacks (the complex-resistivity path factors complex
// symmetric matrices, core/src/bert/dcfemmodelling.cpp:1756-1929).
int ref_set_complex_solver(void *hp, ref_cfactor_fn f, ref_csolve_fn s) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        if (!h->solver) throwError("set the real solver first");
        h->solver->setComplex(f, s);
    });
}

// Complex resistivity: setComplex(true) and response([re, im]) -> [re, im]
// of the apparent resistivities (dcfemmodelling.cpp:1103-1119).
int ref_response_complex(void *hp, const double *model, int nModel2, double *out) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        h->detach(h->fop);
        h->fop->setComplex(true);
        RVector m(nModel2);
        for (int i = 0; i < nModel2; i++) m[i] = model[i];
        RVector r(h->fop->response(m));
        for (Index i = 0; i < r.size(); i++) out[i] = r[i];
    });
}

// createJacobian([re, im]) in complex mode, J (rows x cols complex) as
// separate real and imaginary parts.
int ref_jacobian_complex(void *hp, const double *model, int nModel2, double *J_re, double *J_im, int *rows,
                         int *cols) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        h->detach(h->fop);
        h->fop->setComplex(true);
        RVector m(nModel2);
        for (int i = 0; i < nModel2; i++) m[i] = model[i];
        h->fop->createJacobian(m);
        CMatrix *Jm = dynamic_cast<CMatrix *>(h->fop->jacobian());
        if (!Jm) throwError("no complex Jacobian");
        *rows = (int)Jm->rows();
        *cols = (int)Jm->cols();
        if (J_re) {
            for (Index i = 0; i < Jm->rows(); i++)
                for (Index j = 0; j < Jm->cols(); j++) {
                    J_re[i * Jm->cols() + j] = (*Jm)[i][j].real();
                    J_im[i * Jm->cols() + j] = (*Jm)[i][j].imag();
                }
        }
    });
}

int ref_set_threads(void *hp, int n) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] { h->fop->setThreadCount(n); });
}

int ref_set_kw(void *hp, int nK, const double *k, const double *w) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        RVector kv(nK), wv(nK);
        for (int i = 0; i < nK; i++) { kv[i] = k[i]; wv[i] = w[i]; }
        h->fop->setkValues(kv);
        h->fop->setWeights(wv);
    });
}

// Number of wavenumbers chosen by the reference (initKWaveList) or set.
int ref_kw_count(void *hp) { return (int)((RefHandle *)hp)->fop->kValues().size(); }

int ref_get_kw(void *hp, double *k, double *w) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        const RVector &kv = h->fop->kValues();
        const RVector &wv = h->fop->weights();
        for (Index i = 0; i < kv.size(); i++) { k[i] = kv[i]; w[i] = wv[i]; }
    });
}

// Electrode node ids as matched by searchElectrodes_ (-1 if not a node electrode),
// plus sourceCenterPos_-equivalent and surfaceZ are not exposed by the reference.
int ref_electrode_nodes(void *hp, int *nodeIds) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        const std::vector<ElectrodeShape *> &el = h->fop->electrodes();
        for (size_t i = 0; i < el.size(); i++) nodeIds[i] = el[i]->mID();
    });
}

int ref_geometric_factors(void *hp, double *kout) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        RVector k(geometricFactors(h->data, h->mesh.dim(), false));
        for (Index i = 0; i < k.size(); i++) kout[i] = k[i];
    });
}

int ref_response(void *hp, const double *model, int nModel, double *rhoa) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        RVector m(nModel);
        for (int i = 0; i < nModel; i++) m[i] = model[i];
        RVector r(h->fop->response(m));
        for (Index i = 0; i < r.size(); i++) rhoa[i] = r[i];
    });
}

// The dipole current pattern: setDipoleCurrentPattern(true), the model
// mapped to the cells (mapERTModel), calculate(DataContainerERT &)
// (dcfemmodelling.cpp:1558-1618: one solve per distinct (a, b) pair of the
// data, createCurrentPattern 1488-1513), then the data's "u" (unit current)
// and the number of patterns solved.  The operator is back in pole mode
// afterwards.
int ref_calculate_dipole(void *hp, const double *model, int nModel, double *u, int *n_patterns) {
    RefHandle *h = (RefHandle *)hp;
    int rc = guarded([&] {
        RVector m(nModel);
        for (int i = 0; i < nModel; i++) m[i] = model[i];
        h->fop->setDipoleCurrentPattern(true);
        h->fop->mapERTModel(m, -9e99);
        h->fop->calculate(h->data, false);
        const RVector &uu = h->data("u");
        for (Index i = 0; i < uu.size(); i++) u[i] = uu[i];
        *n_patterns = (int)h->data.currentPattern(false).size();
    });
    h->fop->setDipoleCurrentPattern(false);
    return rc;
}

// Sub-potentials of the last response: rows (i + kIdx*nE), cols nodes.
int ref_subpot_shape(void *hp, int *rows, int *cols) {
    RefHandle *h = (RefHandle *)hp;
    *rows = (int)h->subpots.rows();
    *cols = h->subpots.rows() ? (int)h->subpots[0].size() : 0;
    return 0;
}

int ref_subpotentials(void *hp, double *out) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        Index r = h->subpots.rows();
        for (Index i = 0; i < r; i++) {
            const RVector &row = h->subpots[i];
            std::memcpy(out + i * row.size(), &row[0], row.size() * sizeof(double));
        }
    });
}

// createJacobian(model) then copy J (rows x cols, row-major).
int ref_jacobian(void *hp, const double *model, int nModel, double *J, int *rows, int *cols) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        RVector m(nModel);
        for (int i = 0; i < nModel; i++) m[i] = model[i];
        h->fop->createJacobian(m);
        RMatrix *Jm = dynamic_cast<RMatrix *>(h->fop->jacobian());
        if (!Jm) throwError("no real Jacobian");
        *rows = (int)Jm->rows();
        *cols = (int)Jm->cols();
        if (J) {
            for (Index i = 0; i < Jm->rows(); i++)
                std::memcpy(J + i * Jm->cols(), &(*Jm)[i][0], Jm->cols() * sizeof(double));
        }
    });
}

// The system matrix exactly as the SR calculateK builds it
// (dcfemmodelling.cpp:2174-2182): pattern, domain assembly with the given
// per-cell resistivity, mixed boundary terms at the mean electrode position,
// calibration Dirichlet rows.  srcCenter is the mean electrode position.
// Call once with vals == NULL to get nnz, then with buffers of that size.
int ref_assemble(void *hp, const double *rho, double k, const double *srcCenter,
                 int *n, int *nnz, int *rowptr, int *colidx, double *vals) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        Mesh &m = h->mesh;
        RVector att(m.cellCount());
        for (Index c = 0; c < m.cellCount(); c++) att[c] = rho[c];
        Mesh mm(m);
        mm.setCellAttributes(att);
        RSparseMatrix S;
        S.buildSparsityPattern(mm);
        dcfemDomainAssembleStiffnessMatrix(S, mm, k);
        dcfemBoundaryAssembleStiffnessMatrix(S, mm, RVector3(srcCenter[0], srcCenter[1], srcCenter[2]), k);
        *n = (int)S.rows();
        *nnz = (int)S.nVals();
        if (vals) {
            const std::vector<int> &cp = S.vecColPtr();
            const std::vector<int> &ri = S.vecRowIdx();
            for (size_t i = 0; i < cp.size(); i++) rowptr[i] = cp[i];
            for (size_t i = 0; i < ri.size(); i++) colidx[i] = ri[i];
            for (Index i = 0; i < S.nVals(); i++) vals[i] = S.vecVals()[i];
        }
    });
}

// Analytic primary potential of the reference (bertMisc.cpp:186-271) at all
// nodes for electrode index e (singular value set as in the SR path).
int ref_primary(void *hp, int e, double k, double surfaceZ, double *out) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        const std::vector<ElectrodeShape *> &el = h->fop->electrodes();
        RVector u(exactDCSolution(h->mesh, el[e], k, surfaceZ, true));
        for (Index i = 0; i < u.size(); i++) out[i] = u[i];
    });
}

double ref_besselK0(double x) { return besselK0(x); }
double ref_besselK1(double x) { return besselK1(x); }

int ref_gauss_legendre(int n, double *x, double *w) {
    return guarded([&] {
        RVector xv, wv;
        GaussLegendre(0.0, 1.0, n, xv, wv);
        for (int i = 0; i < n; i++) { x[i] = xv[i]; w[i] = wv[i]; }
    });
}

int ref_gauss_laguerre(int n, double *x, double *w) {
    return guarded([&] {
        RVector xv, wv;
        GaussLaguerre(n, xv, wv);
        for (int i = 0; i < n; i++) { x[i] = xv[i]; w[i] = wv[i]; }
    });
}

// ---- mesh and data I/O (core/src/mesh_io.cpp, core/src/datacontainer.cpp) ----

// A handle holding only a mesh, built like ref_create's (no data, no operator).
void *ref_mesh_create(int dim, int nNodes, const double *xyz, const int *nodeMarker,
                      int nCells, int nv, const int *cellNodes, const int *cellMarker,
                      int nBnd, int nvb, const int *bndNodes, const int *bndMarker, int p2) {
    RefHandle *h = nullptr;
    int rc = guarded([&] {
        h = new RefHandle(dim);
        Mesh &m = h->mesh;
        for (int i = 0; i < nNodes; i++)
            m.createNode(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], nodeMarker[i]);
        for (int c = 0; c < nCells; c++) {
            const int *cn = cellNodes + (size_t)c * nv;
            if (nv == 3) m.createTriangle(m.node(cn[0]), m.node(cn[1]), m.node(cn[2]), cellMarker[c]);
            else if (nv == 4) m.createTetrahedron(m.node(cn[0]), m.node(cn[1]), m.node(cn[2]), m.node(cn[3]), cellMarker[c]);
            else throwError("unsupported cell node count");
        }
        for (int b = 0; b < nBnd; b++) {
            const int *bn = bndNodes + (size_t)b * nvb;
            if (nvb == 2) m.createEdge(m.node(bn[0]), m.node(bn[1]), bndMarker[b]);
            else if (nvb == 3) m.createTriangleFace(m.node(bn[0]), m.node(bn[1]), m.node(bn[2]), bndMarker[b]);
            else throwError("unsupported boundary node count");
        }
        m.createNeighborInfos();
        if (p2) {
            Mesh m2 = p2 == 2 ? m.createH2() : m.createP2();
            h->mesh = m2;
            h->mesh.createNeighborInfos();
        }
    });
    if (rc) { delete h; return nullptr; }
    return h;
}

// Mesh::load (binary format v2/v3 for a .bms name), without createNeighborInfos.
void *ref_mesh_load(const char *path) {
    RefHandle *h = nullptr;
    int rc = guarded([&] {
        h = new RefHandle(3);
        h->mesh.load(path, false);
    });
    if (rc) { delete h; return nullptr; }
    return h;
}

int ref_mesh_dim(void *hp) { return (int)((RefHandle *)hp)->mesh.dim(); }

int ref_mesh_save_bms(void *hp, const char *path) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] { h->mesh.saveBinaryV2(path); });
}

// The first binary format (Mesh::saveBinary, read by Mesh::load as fallback).
int ref_mesh_save_bms_v1(void *hp, const char *path) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] { h->mesh.saveBinary(path); });
}

int ref_mesh_boundary_cells(void *hp, int *left, int *right) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        Mesh &m = h->mesh;
        for (Index b = 0; b < m.boundaryCount(); b++) {
            Boundary &bd = m.boundary(b);
            left[b] = bd.leftCell() ? (int)bd.leftCell()->id() : -1;
            right[b] = bd.rightCell() ? (int)bd.rightCell()->id() : -1;
        }
    });
}

int ref_mesh_add_data(void *hp, const char *name, int n, const double *vals) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        RVector v(n);
        for (int i = 0; i < n; i++) v[i] = vals[i];
        h->mesh.addData(name, v);
    });
}

int ref_mesh_export_vtk(void *hp, const char *path, int writeCells) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] { h->mesh.exportVTK(path, writeCells != 0); });
}

// RegionManager (core/src/regionManager.cpp) on the handle's mesh: regions
// from the cell markers; with default_background the lowest of several
// regions becomes background (pyGIMLi's setDefaultBackground); then the
// given regions are set background, single or fixed, in that order.  Out:
// the renumbered cell markers of the manager's mesh copy, the parameter count
// and the cell count of its para domain.
int ref_regions(void *hp, int default_background, int n_bg, const int *bg, int n_single, const int *single,
                int n_fix, const int *fix_marker, const double *fix_value, int *cell_markers, int *n_param,
                int *n_para_cells) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        RegionManager rm(false);
        rm.setMesh(h->mesh);
        IVector ids(rm.regionIdxs());
        if (default_background && ids.size() > 1) rm.region(min(ids))->setBackground(true);
        for (int i = 0; i < n_bg; i++) rm.region(bg[i])->setBackground(true);
        for (int i = 0; i < n_single; i++) rm.region(single[i])->setSingle(true);
        for (int i = 0; i < n_fix; i++) rm.region(fix_marker[i])->setFixValue(fix_value[i]);
        const Mesh &m = rm.mesh();
        for (Index c = 0; c < m.cellCount(); c++) cell_markers[c] = m.cell(c).marker();
        *n_param = (int)rm.parameterCount();
        *n_para_cells = (int)rm.paraDomain().cellCount();
    });
}

// The region manager's constraint matrix (RegionManager::fillConstraints,
// core/src/regionManager.cpp:920-990, default first-order rows per region,
// Region::fillConstraints 305-404) for the same region settings as
// ref_regions: n_rows x n_param with its entries as (row, col, value)
// triplets in row-major order.  Call with cap = 0 for the sizes first.
int ref_region_constraints(void *hp, int default_background, int n_bg, const int *bg, int n_single,
                           const int *single, int n_fix, const int *fix_marker, const double *fix_value, int cap,
                           int *n_rows, int *n_cols, int *n_entries, int *rows, int *cols, double *vals) {
    RefHandle *h = (RefHandle *)hp;
    return guarded([&] {
        RegionManager rm(false);
        rm.setMesh(h->mesh);
        IVector ids(rm.regionIdxs());
        if (default_background && ids.size() > 1) rm.region(min(ids))->setBackground(true);
        for (int i = 0; i < n_bg; i++) rm.region(bg[i])->setBackground(true);
        for (int i = 0; i < n_single; i++) rm.region(single[i])->setSingle(true);
        for (int i = 0; i < n_fix; i++) rm.region(fix_marker[i])->setFixValue(fix_value[i]);
        rm.parameterCount();
        RSparseMapMatrix C;
        rm.fillConstraints(C);
        *n_rows = (int)C.rows();
        *n_cols = (int)C.cols();
        *n_entries = (int)C.size();
        if (cap >= (int)C.size()) {
            int q = 0;
            for (auto it = C.begin(); it != C.end(); it++, q++) {
                rows[q] = (int)it->first.first;
                cols[q] = (int)it->first.second;
                vals[q] = it->second;
            }
        }
    });
}

// DataContainerERT::load (unified data format).
void *ref_data_load(const char *path, int fromOne, int removeInvalid) {
    DataContainerERT *d = nullptr;
    int rc = guarded([&] {
        d = new DataContainerERT();
        d->load(path, fromOne != 0, removeInvalid != 0);
    });
    if (rc) { delete d; return nullptr; }
    return d;
}

void ref_data_free(void *dp) { delete (DataContainerERT *)dp; }

int ref_data_sizes(void *dp, int *nSensors, int *nData) {
    DataContainerERT *d = (DataContainerERT *)dp;
    *nSensors = (int)d->sensorCount();
    *nData = (int)d->size();
    return 0;
}

int ref_data_sensors(void *dp, double *xyz) {
    DataContainerERT *d = (DataContainerERT *)dp;
    return guarded([&] {
        for (Index i = 0; i < d->sensorCount(); i++)
            for (int j = 0; j < 3; j++) xyz[3 * i + j] = d->sensorPosition(i)[j];
    });
}

// Space-separated token list (DataContainer::tokenList(false)).
int ref_data_tokens(void *dp, char *buf, int len) {
    DataContainerERT *d = (DataContainerERT *)dp;
    std::string t = d->tokenList(false);
    if ((int)t.size() + 1 > len) return (int)t.size() + 1;
    std::memcpy(buf, t.c_str(), t.size() + 1);
    return 0;
}

int ref_data_get(void *dp, const char *token, double *out) {
    DataContainerERT *d = (DataContainerERT *)dp;
    return guarded([&] {
        const RVector &v = d->get(token);
        for (Index i = 0; i < v.size(); i++) out[i] = v[i];
    });
}

int ref_data_save(void *dp, const char *path, const char *fmtData, const char *fmtSensor, int noFilter) {
    DataContainerERT *d = (DataContainerERT *)dp;
    return guarded([&] { d->save(path, fmtData, fmtSensor, noFilter != 0, false); });
}

// The reference's regularised CGLS (solveCGLSCDWWhtrans, core/src/solver.cpp:
// 27-212) on a dense J (nData x nModel, row-major) and a constraint matrix
// given as CSR (nConst rows, built into the reference's RSparseMapMatrix);
// x is the start vector on input and the solution on output.
int ref_cgls(int nData, int nModel, const double *J, int nConst, const int *crp, const int *cci, const double *cv,
             const double *dW, const double *b, double *x, const double *wc, const double *wm, const double *tm,
             const double *td, double lambda, const double *rough, int maxIter, double tol) {
    return guarded([&] {
        RMatrix S(nData, nModel);
        for (int i = 0; i < nData; i++)
            for (int j = 0; j < nModel; j++) S[i][j] = J[(size_t)i * nModel + j];
        RSparseMapMatrix C(nConst, nModel);
        for (int i = 0; i < nConst; i++)
            for (int q = crp[i]; q < crp[i + 1]; q++) C.setVal(i, cci[q], cv[q]);
        auto vec = [](const double *v, int n) {
            RVector r(n);
            for (int i = 0; i < n; i++) r[i] = v[i];
            return r;
        };
        RVector xv(vec(x, nModel));
        solveCGLSCDWWhtrans(S, C, vec(dW, nData), vec(b, nData), xv, vec(wc, nConst), vec(wm, nModel),
                            vec(tm, nModel), vec(td, nData), lambda, vec(rough, nConst), maxIter, tol, false);
        for (int i = 0; i < nModel; i++) x[i] = xv[i];
    });
}

}  // extern "C"
