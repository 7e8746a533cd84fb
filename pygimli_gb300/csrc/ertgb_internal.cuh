// Internal definitions of libertgb: the context, device buffers and the
// kernel launchers shared between translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ertgb.h"

namespace ertgb {

// Error carried across the C ABI as a status code plus message.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define ERTGB_CUDA(call)                                                                   \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            if (e_ == cudaErrorMemoryAllocation)                                           \
                throw ::ertgb::Error(ERTGB_OOM, std::string(#call) + ": " + cudaGetErrorString(e_)); \
            throw ::ertgb::Error(ERTGB_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                                  \
    } while (0)

#define ERTGB_REQUIRE(cond, msg)                                                           \
    do {                                                                                   \
        if (!(cond)) throw ::ertgb::Error(ERTGB_BAD_INPUT, msg);                           \
    } while (0)

// Owning device buffer (raw cudaMalloc; the library's own workspaces).
template <class T> struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count == n && p) return;
        release();
        if (count == 0) return;
        ERTGB_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    void upload(const T *h, size_t count, cudaStream_t s) {
        alloc(count);
        if (count) ERTGB_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T> &h, cudaStream_t s) { upload(h.data(), h.size(), s); }
    void zero(cudaStream_t s) {
        if (n) ERTGB_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

// Level schedule of the IC(0) factorization and triangular solves: rows of
// the lower (forward) and upper (backward) pattern ordered by level.
struct Ic0Plan {
    bool ready = false;
    std::vector<int32_t> frow, flev, brow, blev;
    DBuf<int32_t> d_frow, d_brow;
};

// Band ordering of the direct solve: the mesh's own order or reverse
// Cuthill-McKee, whichever has the smaller bandwidth b (usable if b <= kMaxBand).
constexpr int kMaxBand = 256;
struct BandPlan {
    bool built = false, ok = false;
    int b = 0;
    std::vector<int32_t> perm, pos;  // band index -> row, row -> band index
    DBuf<int32_t> d_perm, d_pos;
};

// Mesh-dependent structures.
struct MeshData {
    int dim = 0, order = 1, nv = 0, nvb = 0;  // nv / nvb: nodes per cell / boundary
    int64_t n = 0, C = 0, B = 0;  // matrix rows (nodes + extension rows), cells, mixed boundaries
    int64_t nn = 0;               // mesh nodes (the first nn rows)
    int64_t nnz = 0;
    int64_t P = 0;                // parameters = max(cell marker) + 1
    std::vector<double> xyz;      // host copy (n x 3)
    std::vector<int32_t> cells;   // C x nv
    std::vector<int32_t> marker;  // C
    std::vector<int32_t> rowptr, colidx;
    std::vector<int32_t> bnd_nodes, bnd_cell;  // mixed boundaries only
    std::vector<int32_t> dir_nodes;            // nodes of homogeneous Dirichlet boundaries (sorted)
    // FSAI factor pattern: lower triangle of A and its transpose
    std::vector<int32_t> Lrowptr, Lcolidx, LtoA, Urowptr, Ucolidx, UtoL;
    DBuf<int32_t> d_Lrowptr, d_Lcolidx, d_LtoA, d_Urowptr, d_Ucolidx, d_UtoL;
    Ic0Plan ic0;  // built on first use of the IC(0) preconditioner
    BandPlan band;  // built on first use of the banded direct solve
    // device
    DBuf<double> d_xyz;
    DBuf<int32_t> d_cells, d_rowptr, d_colidx, d_diag;
    DBuf<int32_t> d_cptr, d_centry;  // per-slot contribution lists
    DBuf<double> d_K, d_M;           // per-cell element matrices (C x nv*nv)
    DBuf<int32_t> d_bnd_nodes, d_bnd_cell;
    DBuf<double> d_bnd_mass, d_bnd_center, d_bnd_normal;  // B x nvb^2, B x 3, B x 3
    // constant matrix extension (complete electrode model, bypass resistors):
    // n_ext rows after the nodes; entries added after assembly, per slot in
    // the order given (ext_ptr: nnz + 1 offsets into ext_val)
    int64_t n_ext = 0;
    std::vector<int32_t> ext_rows, ext_cols;
    std::vector<double> ext_vals;
    DBuf<int32_t> d_ext_ptr;
    DBuf<double> d_ext_val;
    // parameter -> cells (sorted by parameter), for the Jacobian
    std::vector<int32_t> pcell_ptr, pcell;
    DBuf<int32_t> d_pcell_ptr, d_pcell;
};

// A contiguous range of data [d0, d1) with its own distinct current and
// potential dipoles (indices local to the chunk), for schemes whose dipole
// tables of one cell exceed shared memory.
struct JacChunk {
    int64_t d0 = 0, d1 = 0;
    int nA = 0, nM = 0;
    DBuf<int32_t> dip_a, dip_m, data_dip;
};

// Jacobian tiles for one table precision: parameter boundaries of each tile
// and the cells one tile may stage.
struct JacTiles {
    std::vector<int32_t> tile_p;
    DBuf<int32_t> d_tile_p;
    int max_cells = 0;    // tile width TW (cells, = parameters when one cell each)
    int stage_cells = 0;  // cells whose potentials are staged at a time
    std::vector<std::unique_ptr<JacChunk>> chunks;  // empty: the whole scheme in one pass
};

// Plan of the stiffness-only Jacobian kernel (one wavenumber k = 0, at most
// one cell per parameter) for one J precision: tiles of 32 parameters with
// their distinct nodes (node list per tile; local node index per slot and
// cell node, 0xff for an empty slot), data chunks (descriptors of 12 ints)
// with their dipoles as potential-row columns (nE = the electrode at
// infinity), and the records of each chunk sorted by current dipole (datum,
// ia | im << 16, geometric factor).
struct JacStiff {
    bool ok = false;
    int nchunks = 0, RS = 0;  // chunks, staged row length (columns)
    int64_t ntiles = 0;
    size_t tab_bytes = 0, stage_bytes = 0, smem = 0;
    DBuf<int32_t> d_pc, d_nptr, d_tnodes, d_dipa, d_dipm, d_chunks, d_meta;
    DBuf<uint8_t> d_lidx;
};

// Learned preconditioner (learned.cu): graph of the system matrix, network
// weights, activations of every layer and the training buffers.  bf16
// tensors are stored as uint16_t.
struct LPState {
    bool graph_ready = false;
    int64_t n = 0, E = 0, nL = 0;
    int T1 = 0;                           // row-aligned edge tiles per matrix
    int nKb = 0;                          // matrices the activation buffers hold
    bool train_alloc = false;
    DBuf<int32_t> d_erow, d_T, d_tile_row, d_LtoU;
    DBuf<float> d_theta;                  // inference weights (ERTGB_LP_NPARAM)
    bool have_weights = false;
    DBuf<float> x, f, dsq, delta;
    DBuf<uint16_t> h, e, z, a, y;         // (layers + 1) x rows x 64 / layers x rows x 64
    DBuf<double> gA, kpart, kq;
    DBuf<float> dh0, dh1, de, dXj, dhrow, da, ddelta, wpart, gnorm;
    DBuf<uint16_t> dz;
    DBuf<int32_t> err;
};

// Complex resistivity (complex.cu): complex system matrices and the block
// COCG state, all n x Rpad arrays of (re, im) pairs.
struct ComplexState {
    DBuf<double2> sigma;            // C: 1 / rho*
    DBuf<double2> S, dinv;          // nK x nnz, nK x n
    DBuf<double2> x, r, z, p, q;    // n x Rpad
    DBuf<double> part;              // partial sums (5 x NB x Rpad)
    DBuf<double> col;               // per-column scalars
    DBuf<int32_t> active;           // Rpad flags, Rpad iterations, counter
    DBuf<double2> U;                // nE x nE electrode potentials
    // mixed precision: FP32 matrices, Jacobi diagonal and recurrence vectors
    DBuf<float2> S32, dinv32, r32, z32, p32, q32, y32;
    DBuf<int32_t> stalled;          // Rpad flags + counter
    bool have_pot = false;
    int32_t iterations = 0;
    int32_t stalled_columns = 0;
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8];
    std::string last_error;
    MeshData mesh;
    bool have_mesh = false;
    // electrodes
    int nE = 0;
    std::vector<int32_t> enode;
    double surface_z = 0.0;
    double src_center[3] = {0, 0, 0};
    std::vector<double> emin_r;              // singular radius per electrode
    std::vector<double> epos_h;              // electrode positions (nE x 3)
    std::vector<int32_t> ent_cell;           // cell holding an electrode that is no node (-1: none)
    std::vector<double> ent_w;               // nE x nv: shape functions of that cell at the electrode
    DBuf<int32_t> d_ew_ptr, d_ew_row;        // source / collect rows and weights per electrode
    DBuf<double> d_ew_w;
    std::vector<int32_t> ecell_ptr, ecell;   // incident cells per electrode
    DBuf<int32_t> d_enode, d_ecell_ptr, d_ecell;
    // current reference: the pattern of electrode e carries +1 at e and -1 at
    // the reference electrode (an electrode, ref_elec, or a node, ref_node;
    // neither: the current leaves at infinity)
    int ref_elec = -1, ref_node = -1;
    double ref_pos[3] = {0, 0, 0};
    double ref_minr = 0.0;                   // singular radius of the reference node
    std::vector<int32_t> ref_cells;          // cells around the reference node
    DBuf<int32_t> d_ref_cells;
    DBuf<int32_t> d_sink_row;                // rows and weights of the reference's -1
    DBuf<double> d_sink_w;
    int n_sink = 0;
    // rows held at zero potential: calibration nodes (zero singularity-removal
    // right-hand side) and Dirichlet nodes; fixed[row] = 1 cleans row and column
    std::vector<int32_t> calib;
    DBuf<int32_t> d_calib;
    DBuf<uint8_t> d_fixed;
    bool have_fixed = false;
    // formulation (ertgb_formulation); total potential: the row of each
    // electrode's current and potential, and the CEM collect of the last
    // wavenumber only
    int formulation = ERTGB_FORMULATION_SINGULARITY_REMOVAL;
    std::vector<int32_t> src_row;
    DBuf<int32_t> d_src_row;
    bool collect_last_k = false;
    DBuf<double> d_emin_r, d_epos;
    bool have_elec = false;
    // wavenumbers
    int nK = 0;
    std::vector<double> k, w;
    DBuf<double> d_k, d_w;
    bool have_kw = false;
    // scheme
    int64_t D = 0;
    std::vector<int32_t> abmn_h;  // host copy of the scheme (D x 4)
    DBuf<int32_t> d_abmn;
    DBuf<double> d_kfac;
    std::vector<double> kfac_h;   // host copy of the geometric factors
    bool have_scheme = false;
    // distinct current (a, b) and potential (m, n) dipoles of the scheme
    int nA = 0, nM = 0;
    DBuf<int32_t> d_dip_a, d_dip_m, d_data_dip;  // nA x 2, nM x 2, D x 2 (ia, im)
    JacTiles jtiles[2];                          // FP64 and FP32 tables
    JacStiff jstiff[2];                          // stiffness-only plans (FP64, FP32 J)
    DBuf<float2> d_xhl;                          // FP32 J: potentials split into (hi, lo)
    bool jac_ready = false;
    DBuf<char> d_jscale;                         // per-datum / per-parameter scales
    // solver
    double rtol = 1e-10;
    int max_iter = 20000;
    int precond = ERTGB_PRECOND_JACOBI;
    int precision = ERTGB_PRECISION_FP64;
    int rhs_align = 32;           // Rpad granularity (batches use 128)
    // derived per (mesh, electrodes, kw)
    int64_t R = 0, Rpad = 0;     // right-hand sides nK*nE, padded to 32
    bool prim_ready = false;
    DBuf<double> d_alpha;         // nK x B mixed-boundary coefficients
    DBuf<double> d_up;            // unit primary potential  n x Rpad
    std::vector<double> up_user;  // given unit primary potentials (nK x nE x n), empty: analytic
    DBuf<double> d_S1;            // nK x nnz (unit resistivity)
    bool s1_ready = false;
    // per response
    DBuf<double> d_S;             // nK x nnz
    DBuf<double> d_dinv;          // nK x n  (1 / diag)
    DBuf<double> d_pnorm2;        // Rpad: ||S1 u_p / rho_s||^2 per right-hand side (convergence reference floor)
    DBuf<double> d_rhos;          // nE source resistivity
    DBuf<double> d_x, d_r, d_p, d_q;  // n x Rpad (d_r holds the right-hand sides)
    // mixed precision: FP32 matrix, Jacobi diagonal and recurrence vectors
    DBuf<float> d_S32, d_dinv32, d_r32, d_p32, d_q32, d_y32;
    // FSAI preconditioner M^-1 = G^T G: G (lower) and G^T values per wavenumber
    DBuf<double> d_G;
    DBuf<float> d_G32, d_GT32, d_t32, d_z32;
    int32_t fsai_fallback_rows = 0;
    // IC(0) preconditioner: factor values per wavenumber (lower pattern),
    // its pivot-breakdown counter, and the preconditioned residual
    DBuf<double> d_ic, d_z;
    DBuf<double> d_band;  // banded Cholesky factors, nK x n x (b + 1)
    DBuf<int32_t> d_ic_bad;
    int32_t ic0_breakdowns = 0;
    // mixed precision: wavenumbers whose columns stalled in FP32 in the last
    // response start in FP64 next time (cleared with the mesh / k / w)
    std::vector<uint8_t> fp64_k;
    DBuf<int32_t> d_pre;
    DBuf<double> d_part;          // reduction partials
    DBuf<double> d_col;           // per-column scalars (see pcg.cu)
    DBuf<int32_t> d_active;
    DBuf<double> d_U;             // nE x nE collected electrode potentials
    DBuf<double> d_inv_rho;       // 1/rho per cell of the last assembly
    DBuf<double> d_rhoa;
    bool have_pot = false;
    bool have_S = false;          // d_S holds the matrices of the current setup
    const double *d_rho_last = nullptr;  // resistivity of the last response (caller's buffer)
    DBuf<double> d_rho_tmp, d_model_tmp;
    DBuf<char> d_J_tmp;
    LPState lp;
    ComplexState cx;
    ertgb_stats stats{};
};

// --- launchers (defined in the .cu files) -----------------------------------
// assemble.cu
void build_mesh_device(Context &c);
void compute_boundary_alpha(Context &c);
void compute_primary(Context &c);
// given primary potentials (c.up_user, nK x nE x n) into d_up (n x Rpad)
void upload_primary(Context &c);
// analytic half-space potentials of every source (the unit primaries, with
// the source node's singular value) times rho into out (n x Rpad)
void analytic_potentials(Context &c, double rho, double *out);
void assemble_all(Context &c, const double *rho_cell, double *vals_out, cudaStream_t s);
void assemble_unit(Context &c, cudaStream_t s);
void compute_source_rho(Context &c, const double *rho_cell, cudaStream_t s);
void build_rhs(Context &c, cudaStream_t s);
// ||S1 u_p / rho_s||^2 per column into d_pnorm2 (after build_rhs)
void compute_rhs_scale(Context &c, cudaStream_t s);
// Floor of the convergence reference: ||b||^2 is raised to kRhsFloor2 ||S1 u_p / rho_s||^2
// where the singularity-removal right-hand side cancels (homogeneous ground around a source).
constexpr double kRhsFloor2 = 1e-6;
void finish_potentials(Context &c, cudaStream_t s);
void collect_potentials(Context &c, cudaStream_t s);  // d_U = k-summed potentials at the electrodes
void collect_response(Context &c, double *rhoa, cudaStream_t s);
// total potential: unit currents at the electrodes' source rows into d_r
void build_rhs_total(Context &c, cudaStream_t s);
// rows and weights of every electrode's source and potential (its node / source
// row with weight 1, or the shape functions of the cell holding it), the
// reference electrode's sink and the fixed-row flags
void build_electrode_weights(Context &c);
// homogeneous Dirichlet rows and columns (diagonal 1) of the fixed rows in
// nK matrices of the pattern
void clean_fixed_rows(Context &c, double *vals, cudaStream_t s);
void check_rho(Context &c, const double *rho_cell, cudaStream_t s);
// pcg.cu
// mask: warm start (x kept) on the columns with mask[t] != 0; nullptr = cold start, all columns
int pcg_solve(Context &c, cudaStream_t s, const int32_t *mask = nullptr);
// allocate pcg_solve's workspaces ahead (no allocation inside a later solve)
void pcg_prepare(Context &c);
void pcg_finish_init(dim3 g, dim3 b, cudaStream_t s, int64_t Rpad, int64_t R, int NB, const double *pa,
                     const double *pb, double *col, int32_t *active, int32_t *iters, int32_t *nactive,
                     const double *pnorm2);
// pcg_mixed.cu
int pcg_solve_mixed(Context &c, cudaStream_t s);
void profile_spmm32(Context &c, int reps, double *ms, double *bytes, double *flops);
void profile_spmm(Context &c, int reps, double *ms, double *bytes, double *flops);
// Y = A X with column dots (the PCG operator kernel) on raw CSR arrays; the
// NB x ld block partials live in ``partials``.
int spmm_partial_rows(int64_t n, int cap);
void spmm_dot_launch(int64_t n, int64_t nnz, const int32_t *rowptr, const int32_t *colidx, const double *vals, int nK,
                     int n_per_k, int64_t ld, const double *X, double *Y, double *dots, double *partials, int NB,
                     cudaStream_t s);
// Message returned by ertgb_last_error(NULL) for the context-free entry points.
void set_free_error(const std::string &msg);

// complex resistivity (complex.cu): response [Re, Im] per datum and the
// complex Jacobian (interleaved re, im; D x n_model)
int complex_response(Context &c, const double *rho_re, const double *rho_im, double *out_re, double *out_im,
                     cudaStream_t s);
void complex_jacobian(Context &c, const double *m_re, const double *m_im, int n_model, double *J, cudaStream_t s);

// device mesh refinement (refine.cu)
struct Refined;
Refined *refine_mesh(int device, int dim, int mode, int64_t n0, const double *xyz, const int32_t *nmark, int64_t C,
                     const int32_t *cells, const int32_t *cmark, int64_t B, const int32_t *bnd, const int32_t *bmark,
                     const int32_t *bcell);
void refined_sizes(const Refined *r, int64_t *n, int64_t *C, int64_t *nv, int64_t *B, int64_t *nvb);
void refined_get(const Refined *r, double *xyz, int32_t *nmark, int32_t *cells, int32_t *cmark, int32_t *bnd,
                 int32_t *bmark, int32_t *bcell);
void refined_free(Refined *r);
// Checks shared by the context-free operator entry points; throws Error.
void check_spmm_args(int64_t n, int64_t nnz, const void *rowptr, const void *colidx, const void *vals, int n_k,
                     int n_per_k, int64_t ld, const void *X, const void *Y, const void *dots);
void profile_assemble(Context &c, int reps, double *ms, double *bytes, double *flops);
void profile_jacobian(Context &c, int reps, void *J, int dtype, double *ms, double *bytes, double *flops);
// jacobian.cu
void jacobian(Context &c, const double *model, int n_model, void *J, int dtype, cudaStream_t s);
// setup.cpp
void build_pattern(MeshData &m);
void build_assembly_map(MeshData &m, std::vector<int32_t> &cptr, std::vector<int32_t> &centry,
                        std::vector<int32_t> &diag);
void build_jacobian_tiles(Context &c);
void build_lower_pattern(MeshData &m);
void build_extension_map(const MeshData &m, std::vector<int32_t> &ptr, std::vector<double> &val);
// fsai.cu
void fsai_setup(Context &c, cudaStream_t s);
// ic0.cu: factor every wavenumber's matrix (d_S) into d_ic; z = (L L^T)^-1 r
// on all columns; kernel launches of one application
void ic0_setup(Context &c, cudaStream_t s);
void ic0_apply(Context &c, const double *r, double *z, cudaStream_t s);
int ic0_launches(const Context &c);
// band.cu: x = A^-1 b for every column (FP64 banded Cholesky per wavenumber)
int band_solve(Context &c, cudaStream_t s);
// batch.cu: batched mixed-precision PCG over the contexts' assembled systems
int batch_solve(std::vector<Context *> &cs, cudaStream_t s, ertgb_batch_info *info, int *stalled);
// cgls.cu: regularised Gauss-Newton update (all pointers device, vectors FP64)
int cgls_solve(const void *J, int dtype, int64_t D, int64_t P, int64_t NC, const int32_t *c_rp, const int32_t *c_ci,
               const double *c_v, const int32_t *ct_rp, const int32_t *ct_ci, const double *ct_v, const double *dW,
               const double *b, double *x, const double *wc, const double *wm, const double *tm, const double *td,
               double lambda, const double *rough, int max_iter, double tol, int *iters, cudaStream_t s);
// learned.cu
void lp_setup(Context &c, cudaStream_t s);  // network G into d_G32 / d_GT32 (the solver's factor)
void lp_forward(Context &c, const float *theta, cudaStream_t s);
double lp_loss_grad(Context &c, const float *theta, float *grad, cudaStream_t s);
void lp_features(Context &c, float *x, float *f, cudaStream_t s);
void lp_adam(float *theta, const float *grad, float *m, float *v, int64_t n, double lr, double beta1,
             double beta2, double eps, int step, double clip, float *gnorm_scratch, cudaStream_t s);

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace ertgb
