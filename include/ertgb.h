/* ertgb — GB300-native ERT (DC resistivity) forward operator and Jacobian.
 *
 * C ABI of libertgb.so.  Plain pointers and sizes only; every function
 * returns an ertgb_status and never throws.  Arrays named *_host live in host
 * memory, arrays named *_dev in device memory of the context's GPU.  A
 * ``stream`` argument is a cudaStream_t passed as void* (NULL = the
 * context's own stream): the call's work is ordered after the work already
 * queued on that stream, and later work on it is ordered after the call.
 * Compute calls also return only after their work is done, because the
 * solver decides on the host when to stop.
 *
 * The operator is the singularity-removal (SR) DC forward operator of
 * pyGIMLi: pg.physics.ert.ERTModelling(sr=True) -> C++
 * GIMLI::DCSRMultiElectrodeModelling.  Each entry point below names the
 * reference interface it replaces (paths inside the pyGIMLi tree).
 */
#ifndef ERTGB_H
#define ERTGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ertgb_ctx ertgb_ctx;

typedef enum {
    ERTGB_OK = 0,
    ERTGB_BAD_INPUT = 1,     /* sizes, indices, non-positive resistivity ... */
    ERTGB_NOT_CONVERGED = 2, /* PCG hit max_iter before the tolerance      */
    ERTGB_OOM = 3,           /* device allocation failed                     */
    ERTGB_CUDA_ERROR = 4,    /* a CUDA runtime call failed                   */
    ERTGB_STATE = 5          /* call order (e.g. jacobian before response)   */
} ertgb_status;

/* Preconditioners of the block PCG.  JACOBI: diagonal.  FSAI: factorized
 * sparse approximate inverse M^-1 = G^T G, G lower triangular on A's pattern
 * (mixed precision only; columns that stall finish with FP64 Jacobi).
 * LEARNED: M^-1 = G^T G with G emitted by a message-passing network on the
 * graph of A (weights: ertgb_set_precond_weights), same pattern, same
 * application and the same FP64 Jacobi fallback as FSAI. */
/* IC0: incomplete Cholesky on A's lower pattern (no fill), factored on the
 * device per response and wavenumber, level-scheduled triangular solves;
 * FP64 precision only (the incomplete counterpart of the reference's CHOLMOD
 * factorization, core/src/cholmodWrapper.cpp:309-420).
 * BAND: no iteration: the exact Cholesky factor of every wavenumber's matrix
 * in band storage (the mesh's order or reverse Cuthill-McKee, bandwidth at
 * most 256: the 2-D meshes of the 2.5-D path) and a forward and backward
 * substitution per source, as the reference's direct solve
 * (dcfemmodelling.cpp:2199-2210); FP64 precision only. */
typedef enum {
    ERTGB_PRECOND_JACOBI = 0,
    ERTGB_PRECOND_FSAI = 1,
    ERTGB_PRECOND_LEARNED = 2,
    ERTGB_PRECOND_IC0 = 3,
    ERTGB_PRECOND_BAND = 4
} ertgb_precond;

/* Length of the learned preconditioner's FP32 parameter vector: encoders
 * (2 x (64x4 + 64)), 4 layers of (W1 64x192, b1 64, W2 64x128, b2 64) and the
 * decoder (wo 64, bo, wd 64, bd), in that order. */
#define ERTGB_LP_NPARAM 83202

/* Arithmetic of the block PCG.  FP64: everything in FP64.  MIXED: FP32
 * recurrence (operator, preconditioner, vectors) with FP64 reliable updates
 * every 64 iterations (the FP64 solution accumulates the FP32 increments and
 * the residual restarts from the FP64 true residual); convergence is tested
 * on the FP64 true residual, so the tolerance means the same in both.
 * Columns whose true residual stops falling (systems too ill-conditioned
 * for FP32) are finished by the FP64 solver from where they stalled. */
typedef enum { ERTGB_PRECISION_FP64 = 0, ERTGB_PRECISION_MIXED = 1 } ertgb_precision;

/* Solver statistics of the last response. */
typedef struct {
    int32_t iterations;       /* PCG iterations until every column converged */
    int32_t n_rhs;            /* right-hand sides = electrodes x wavenumbers */
    double max_rel_residual;  /* max_j ||b_j - A x_j|| / ||b_j|| (recursive)  */
    double ms_assemble;       /* device time of the last response's phases   */
    double ms_rhs;
    double ms_solve;
    double ms_collect;
    double ms_jacobian;       /* device time of the last jacobian            */
    int64_t launches_response; /* kernels launched by the last response       */
    int64_t launches_jacobian; /* kernels launched by the last jacobian       */
    int32_t stalled_columns;   /* mixed precision: columns finished in FP64   */
} ertgb_stats;

/* Kernels that ertgb_profile_kernel can time. */
typedef enum {
    ERTGB_KERNEL_SPMM = 0,     /* PCG operator q = A p with column dots       */
    ERTGB_KERNEL_JACOBIAN = 1, /* Jacobian of the last response (FP64 J)      */
    ERTGB_KERNEL_ASSEMBLE = 2, /* system matrices of the last response        */
    ERTGB_KERNEL_SPMM32 = 3,   /* FP32 operator of the mixed-precision PCG    */
    ERTGB_KERNEL_JACOBIAN32 = 4 /* Jacobian of the last response (FP32 J)     */
} ertgb_kernel;

/* Create a context on CUDA device ``device``.  Replaces the construction of
 * DCSRMultiElectrodeModelling (core/src/bert/dcfemmodelling.h:346-359,
 * pygimli/physics/ert/ertModelling.py:87-122). */
int ertgb_create(ertgb_ctx **ctx, int device);
int ertgb_destroy(ertgb_ctx *ctx);
/* Message of the last failing call on this context ("" if none). */
const char *ertgb_last_error(const ertgb_ctx *ctx);

/* Mesh: replaces ModellingBase::setMesh (core/src/modellingbase.cpp:179-206)
 * with DCMultiElectrodeModelling::updateMeshDependency_
 * (core/src/bert/dcfemmodelling.cpp:711-773).  dim 2 (triangles, y = depth,
 * 2.5-D) or 3 (tetrahedra); order 1 (linear) or 2 (quadratic: Triangle6 /
 * Tetrahedron10 in the node order of Mesh::createP2, core/src/mesh.cpp:
 * 1284-1600).  xyz: n_nodes x 3.  cell_nodes: n_cells x (dim+1) for order 1,
 * x 6 / 10 for order 2.  bnd_nodes: n_bnd x dim (order 1) or x 3 / 6
 * (order 2), bnd_marker -1 Neumann / -2 mixed / -3 homogeneous Dirichlet
 * (the boundary's nodes get Dirichlet rows and columns, diagonal 1:
 * dcfemBoundaryAssembleStiffnessMatrix, core/src/bert/dcfemmodelling.cpp:
 * 279-298; -4 is refused as by the reference, :293),
 * bnd_cell: adjacent cell of each boundary.  Builds the CSR pattern
 * (core/src/sparsematrix.h:966-1024), the per-slot assembly map and the
 * element matrices (core/src/elementmatrix.cpp:683-1122). */
int ertgb_set_mesh(ertgb_ctx *ctx, int dim, int order, int n_nodes, const double *xyz_host,
                   int n_cells, const int32_t *cell_nodes_host, const int32_t *cell_marker_host,
                   int n_bnd, const int32_t *bnd_nodes_host, const int32_t *bnd_marker_host,
                   const int32_t *bnd_cell_host);

/* Node electrodes as matched by DCMultiElectrodeModelling::searchElectrodes_
 * (core/src/bert/dcfemmodelling.cpp:790-1030): node id of each electrode,
 * the surface coordinate on axis dim-1 of the Neumann boundary
 * (updateMeshDependency_, :727-745).  Replaces that search's results; the
 * mean electrode position (sourceCenterPos_, :1026-1030), the singular
 * radii (core/src/bert/electrode.cpp:154-197) and the incident cells
 * (electrode.cpp:102-127) are derived here.  Node -1: an electrode given by
 * a matrix extension row (ertgb_set_extension) or by the cell that holds it
 * (ertgb_set_electrode_shapes). */
int ertgb_set_electrodes(ertgb_ctx *ctx, int n_elec, const int32_t *elec_node_host,
                         double surface_z);

/* Electrodes that are not mesh nodes (after ertgb_set_electrodes, which gives
 * them node -1): cell_host[e] >= 0 is the cell holding electrode e (linear
 * cells), pos_host[3e..3e+2] its position in mesh coordinates; -1 keeps the
 * node electrode.  The source enters with the cell's shape functions at the
 * position, the electrode potential is the interpolation there, the source
 * resistivity of singularity removal is the cell's.  Replaces
 * ElectrodeShapeEntity (core/src/bert/electrode.cpp:252-290) as chosen by
 * DCMultiElectrodeModelling::searchElectrodes_
 * (core/src/bert/dcfemmodelling.cpp:924-937). */
int ertgb_set_electrode_shapes(ertgb_ctx *ctx, int n_elec, const int32_t *cell_host, const double *pos_host);

/* Current reference and calibration (after ertgb_set_electrodes; setting the
 * mesh or the electrodes clears them).  The pattern of electrode e then
 * carries +1 at e and -1 at the reference electrode: electrode ref_electrode
 * (its own pattern is empty) or mesh node ref_node; both -1: the current
 * leaves at infinity.  Replaces DCMultiElectrodeModelling::searchElectrodes_
 * (core/src/bert/dcfemmodelling.cpp:1011-1073: node marker -999, or the
 * last electrode in a 3-D domain without mixed and Dirichlet boundaries) and
 * createCurrentPattern (:1515-1523).  Singularity removal subtracts the
 * reference's primary potential (:2085-2090) and averages the two source
 * resistivities (:2236-2266).  calib_host: n_calib calibration nodes (node
 * marker -1000, else node 0, in such a closed 3-D domain): Dirichlet rows
 * and columns in every system matrix (:1835, 2182-2192) and a zero
 * singularity-removal right-hand side there (:2281-2283).  A closed 3-D
 * domain needs at least one. */
int ertgb_set_reference(ertgb_ctx *ctx, int ref_electrode, int ref_node, int n_calib, const int32_t *calib_host);

/* Formulation of the forward operator.  SINGULARITY_REMOVAL (default):
 * DCSRMultiElectrodeModelling, pyGIMLi ERTModelling(sr=True)
 * (core/src/bert/dcfemmodelling.cpp:2152-2296).  TOTAL_POTENTIAL:
 * DCMultiElectrodeModelling, ERTModelling(sr=False) (ertModelling.py:102-106):
 * total potentials of unit point currents (calculateK_,
 * dcfemmodelling.cpp:1756-1929), no primary field; the only formulation that
 * takes a matrix extension (complete electrode model, bypass resistors).
 * With TOTAL_POTENTIAL an electrode node may be -1 (an electrode given by
 * its extension row only).  Setting the formulation drops an extension. */
typedef enum {
    ERTGB_FORMULATION_SINGULARITY_REMOVAL = 0,
    ERTGB_FORMULATION_TOTAL_POTENTIAL = 1
} ertgb_formulation;
int ertgb_set_formulation(ertgb_ctx *ctx, int formulation);

/* Constant extension of the total-potential system matrix: the complete
 * electrode model (assembleCompleteElectrodeModel_, dcfemmodelling.cpp:
 * 315-414, called at :1786-1831) and bypass resistors
 * (assembleStiffnessMatrixDCFEMByPass_, :601-709).  n_ext rows / columns
 * follow the mesh nodes (one per electrode, then per passive body).  The
 * n_entries (row, col, value) entries are added, in the order given, to the
 * assembled matrix of every wavenumber after the domain and boundary terms
 * (rows / columns < n_nodes + n_ext).  src_row[e] (n_elec values): the row
 * of electrode e's unit current and of its potential (its node without CEM,
 * n_nodes + e with CEM: electrode.cpp:133-150, 341-355).  src_center: the
 * mean electrode position of the mixed boundary condition (sourceCenterPos_,
 * :1026-1030; may be NULL).  collect_last_k != 0: the electrode potentials
 * are those of the last wavenumber, unweighted, as the reference's
 * potentialsCEM_ (overwritten per wavenumber, :1829, 1912; collected at
 * :1642-1644).  Call after ertgb_set_electrodes; needs TOTAL_POTENTIAL. */
int ertgb_set_extension(ertgb_ctx *ctx, int n_ext, int64_t n_entries, const int32_t *rows_host,
                        const int32_t *cols_host, const double *vals_host, const int32_t *src_row_host,
                        const double *src_center_host, int collect_last_k);

/* Wavenumbers and weights: DCMultiElectrodeModelling::setkValues/setWeights
 * (core/src/bert/dcfemmodelling.h:239-243). */
int ertgb_set_kw(ertgb_ctx *ctx, int n_k, const double *k_host, const double *w_host);

/* Unit primary potentials for singularity removal (host, n_k x n_elec x
 * n_nodes, node fastest), used instead of the analytic half-space
 * potentials until the mesh, electrodes or wavenumbers change: the numerical
 * primaries of a topographic surface.  Replaces setPrimaryPotential
 * (core/src/bert/dcfemmodelling.h:374) and the topography branch of
 * DCSRMultiElectrodeModelling::checkPrimpotentials_
 * (core/src/bert/dcfemmodelling.cpp:2008-2068), whose total-potential solve
 * on createP2 the caller runs (ERTModelling does it on the GPU). */
int ertgb_set_primary(ertgb_ctx *ctx, int n_k, int n_elec, int64_t n_nodes, const double *up_host);

/* Potentials of a homogeneous model of resistivity rho without a solve: the
 * analytic half-space potentials of every source (with the source node's
 * singular value) times rho, as the sub-potentials of the next Jacobian.
 * Replaces the analytic branch of prepareJacobianT_
 * (core/src/bert/dcfemmodelling.cpp:1262-1301: createJacobian before any
 * response on a model with standard deviation <= 1e-7, calculateKAnalyt
 * 1737-1753, scaled by model[0]).  Node electrodes, flat surface. */
int ertgb_analytic_potentials(ertgb_ctx *ctx, double rho);

/* Measurement scheme: the a b m n columns (-1 = at infinity) and geometric
 * factors k of DataContainerERT (core/src/bert/bertDataContainer.h:62),
 * as read by DataMap::data (core/src/bert/datamap.cpp:159-231). */
int ertgb_set_scheme(ertgb_ctx *ctx, int n_data, const int32_t *abmn_host, const double *kfac_host);

/* Solver controls: relative residual tolerance, iteration cap, preconditioner. */
int ertgb_set_solver(ertgb_ctx *ctx, double rtol, int max_iter, int precond);
/* Solver arithmetic (ertgb_precision).  No counterpart in the reference,
 * whose direct solver is FP64. */
int ertgb_set_precision(ertgb_ctx *ctx, int precision);

/* Forward response: DCMultiElectrodeModelling::response
 * (core/src/bert/dcfemmodelling.cpp:1085-1197) for a per-cell resistivity
 * (the result of mapERTModel, :1199-1218).  Writes n_data apparent
 * resistivities sqrt(|rhoa * rhoa_reciprocal|).  Keeps the sub-potentials
 * on the device for ertgb_jacobian (the reference keeps subSolutions_). */
int ertgb_response(ertgb_ctx *ctx, const double *rho_cell_dev, double *rhoa_dev, void *stream);
/* Same with host buffers (copies included). */
int ertgb_response_host(ertgb_ctx *ctx, const double *rho_cell_host, double *rhoa_host);

/* Jacobian: DCMultiElectrodeModelling::createJacobian
 * (core/src/bert/dcfemmodelling.cpp:1446-1476, createSensitivityCol
 * core/src/bert/bertJacobian.cpp:267-421, calc2 :70-119) from the
 * sub-potentials of the last response.  J is n_data x n_param row-major,
 * n_param = max(cell marker) + 1, FP64 (dtype 0) or FP32 (dtype 1).  When
 * n_model == n_param the rows are scaled by k_i / model_j^2
 * (dcfemmodelling.cpp:1377-1384). */
int ertgb_jacobian(ertgb_ctx *ctx, const double *model_dev, int n_model, void *J_dev, int dtype,
                   void *stream);
/* Same with host buffers (model and J on the host). */
int ertgb_jacobian_host(ertgb_ctx *ctx, const double *model_host, int n_model, void *J_host,
                        int dtype);

/* Sizes after set_mesh/set_electrodes/set_kw/set_scheme.  n_nodes: rows of
 * the system matrix (mesh nodes plus the rows of ertgb_set_extension); the
 * potentials of ertgb_get_potentials have that many entries per column. */
int ertgb_sizes(const ertgb_ctx *ctx, int64_t *n_nodes, int64_t *nnz, int64_t *n_param,
                int64_t *n_rhs);

/* Parity accessors (host outputs). */
int ertgb_get_pattern(ertgb_ctx *ctx, int32_t *rowptr_host, int32_t *colidx_host);
/* System matrix values of wavenumber k_index from the last response:
 * which 0 = S (model), 1 = S1 (unit resistivity). */
int ertgb_get_matrix(ertgb_ctx *ctx, int k_index, int which, double *vals_host);
/* Sub-potentials of the last response, laid out [k][electrode][node]
 * like the reference's subSolutions_ rows (i + k*nElecs). */
int ertgb_get_potentials(ertgb_ctx *ctx, double *pot_host);
/* Electrode potential matrix of the last real-valued response (ertgb_response,
 * ertgb_response_host, or the analytic potentials), n_elec x n_elec row-major:
 * U[e][f] = potential at electrode f for the unit current of pattern e,
 * summed over the wavenumbers with their weights (the complete electrode
 * model: its extension row, last wavenumber) -- the reference's DataMap
 * (DataMap::collect, core/src/bert/datamap.cpp:57-98), from which
 * DCMultiElectrodeModelling::calculate(DataContainerERT &)
 * (core/src/bert/dcfemmodelling.cpp:1558-1618) takes its voltages. */
int ertgb_get_electrode_potentials(ertgb_ctx *ctx, double *U_host);
/* Unit-current primary potentials [k][electrode][node]. */
int ertgb_get_primary(ertgb_ctx *ctx, double *prim_host);
int ertgb_get_stats(const ertgb_ctx *ctx, ertgb_stats *stats);

/* Multi-right-hand-side CSR product with column dot products, the block
 * PCG's operator kernel, for callers that run their own Krylov iterations
 * on device arrays:  Y[:, t] = A_{k(t)} X[:, t] and dots[t] = X[:, t] . Y[:, t],
 * k(t) = min(t / n_per_k, n_k - 1).  CSR int32 (rowptr n+1, colidx nnz),
 * vals n_k x nnz, X and Y n x ld row-major (ld a multiple of 32), dots ld.
 * Replaces the reference's SparseMatrix::mult (core/src/sparsematrix.h:
 * 825-876) applied column by column.  Context free; scratch for the block
 * partials is taken from the stream-ordered allocator.  Errors are reported
 * through ertgb_last_error(NULL). */
int ertgb_csr_spmm_dot(int64_t n, int64_t nnz, const int32_t *rowptr_dev, const int32_t *colidx_dev,
                       const double *vals_dev, int n_k, int n_per_k, int64_t ld, const double *X_dev,
                       double *Y_dev, double *dots_dev, void *stream);

/* Allocation-free variant of ertgb_csr_spmm_dot, for callers that cannot
 * allocate device memory at call time (a host framework that owns the device
 * memory through its own pool, or a loop that must not allocate after
 * start-up).  No counterpart in the reference.  Same arguments and results;
 * the block partials live in a fixed 2 MiB device array of the library
 * (every GPU that loads the library holds it until exit), so ld is limited
 * to 1024 columns (larger ld: ERTGB_BAD_INPUT).  Calls no allocator.  The
 * first call on a device looks up the array's address and should come
 * before any stream capture; the address is kept for the life of the
 * process, so no device may be reset (cudaDeviceReset) nor its primary
 * context torn down while the library is loaded.  All calls share the array:
 * calls that overlap on the GPU race and must be ordered by the caller. */
int ertgb_csr_spmm_dot_noalloc(int64_t n, int64_t nnz, const int32_t *rowptr_dev, const int32_t *colidx_dev,
                               const double *vals_dev, int n_k, int n_per_k, int64_t ld, const double *X_dev,
                               double *Y_dev, double *dots_dev, void *stream);

/* Measurement helper with no counterpart in the reference: launches one
 * kernel ``reps`` times on the context stream (on the state of the last
 * response) and returns the mean launch time from CUDA events, with the
 * algorithmic DRAM bytes and FLOPs of one launch.  J_scratch_dev must hold
 * n_data x n_param doubles for ERTGB_KERNEL_JACOBIAN (else unused). */
int ertgb_profile_kernel(ertgb_ctx *ctx, int kernel, int reps, void *J_scratch_dev, double *ms_per_launch,
                         double *bytes_per_launch, double *flops_per_launch);

/* ---- learned preconditioner (no counterpart in the reference, which
 * factors every system with CHOLMOD: core/src/bert/dcfemmodelling.cpp:2199-2210).
 * The network runs on the system matrices of the context. */

/* Network weights used by ERTGB_PRECOND_LEARNED (host, ERTGB_LP_NPARAM floats). */
int ertgb_set_precond_weights(ertgb_ctx *ctx, const float *theta_host, int64_t n);

/* Assemble the system matrices of every wavenumber for a per-cell
 * resistivity (device) without solving: the training data of the network. */
int ertgb_assemble(ertgb_ctx *ctx, const double *rho_cell_dev, void *stream);

/* Network factor of the current matrices (device weights): G values in the
 * row-major order of A's lower triangle, n_k x n_lower floats (G_dev may be
 * NULL). */
int ertgb_lp_forward(ertgb_ctx *ctx, const float *theta_dev, float *G_dev, void *stream);

/* Training loss (Kaporin's condition number of G A G^T, mean over the
 * wavenumbers; host scalar) and, if grad_dev is not NULL, its gradient in the
 * weights (device, ERTGB_LP_NPARAM floats, overwritten). */
int ertgb_lp_loss_grad(ertgb_ctx *ctx, const float *theta_dev, float *grad_dev, double *loss_host, void *stream);

/* One Adam step on device vectors (gradient clipped to norm clip if clip > 0;
 * step counts from 1). */
int ertgb_lp_adam(float *theta_dev, const float *grad_dev, float *m_dev, float *v_dev, int64_t n, double lr,
                  double beta1, double beta2, double eps, int step, double clip, void *stream);

/* Network input features of the current matrices: node features n_k x n x 4,
 * edge features n_k x nnz x 4 (device; either may be NULL). */
int ertgb_lp_features(ertgb_ctx *ctx, float *x_dev, float *f_dev, void *stream);

/* ---- batches of independent problems (one context each) -------------- */

/* Tile shape chosen by the batch autotuner, its candidates, and the work of
 * the last batched response. */
typedef struct {
    int32_t rows_per_tile;    /* matrix rows per tile                         */
    int32_t rhs_width;        /* right-hand-side columns per operator tile    */
    int32_t n_candidates;     /* shapes timed (0 when the shape was cached)   */
    int32_t cached;           /* 1: shape reused from an earlier identical batch */
    int32_t cand_rows[16], cand_width[16];
    double cand_ms[16];       /* operator time of every candidate             */
    int64_t spmm_tiles, vector_tiles, columns;
    int32_t iterations;       /* batched PCG iterations (all problems)        */
    int32_t stalled_columns;  /* columns finished by their problem's FP64 PCG */
    int64_t launches;         /* kernel launches of the batched iterations    */
    double ms_assemble, ms_solve, ms_collect;
} ertgb_batch_info;

/* Apparent resistivities of n independent problems in one batched solve.
 * Every context needs mesh, electrodes, wavenumbers and scheme set; rho_dev[i]
 * is problem i's per-cell resistivity and rhoa_dev[i] its output (device).
 * Assembly, right-hand sides and collection run per problem; the linear
 * systems of all problems (all sources x wavenumbers) are solved together by
 * the mixed-precision block PCG (Jacobi, FP64 reliable updates, FP64 true
 * residual to each context's rtol; stalled columns finish in FP64), whose
 * kernels each cover every problem in one launch.  The potentials stay in
 * each context (ertgb_jacobian works afterwards).  info may be NULL. */
int ertgb_batch_response(ertgb_ctx *const *ctxs, int n, const double *const *rho_dev, double *const *rhoa_dev,
                         ertgb_batch_info *info, void *stream);

/* ---- Gauss-Newton model update ------------------------------------------ */

/* The regularised CGLS of pyGIMLi's inversion step (solveCGLSCDWWhtrans,
 * core/src/solver.cpp:27-212, called by RInversion::oneStep,
 * core/src/inversion.cpp:249-372): solves for the transformed model update x
 *   (Jt^T Wd^2 Jt + lambda (Wc C Wm)^T (Wc C Wm)) x = Jt^T Wd^2 b - lambda (Wc C Wm)^T rough
 * with Jt = diag(td) J diag(1/tm), starting from x.  J: device D x P row-major,
 * dtype 0 FP64 / 1 FP32 (as written by ertgb_jacobian).  C: n_constr x P CSR
 * (FP64 values) and its transpose (P x n_constr CSR).  Every vector is a
 * device FP64 array: dweight, b, td (D); x, wm, tm (P); wc, rough (n_constr).
 * tol < 0: stop when ||r||^2 <= max(1e-12, 1e-8 ||r_0||^2) as the reference.
 * iterations_out receives the CGLS iterations. */
int ertgb_cgls(const void *J_dev, int dtype, int64_t n_data, int64_t n_model, int64_t n_constr,
               const int32_t *c_rowptr, const int32_t *c_colidx, const double *c_vals, const int32_t *ct_rowptr,
               const int32_t *ct_colidx, const double *ct_vals, const double *dweight, const double *b, double *x,
               const double *wc, const double *wm, const double *tm, const double *td, double lambda,
               const double *rough, int max_iter, double tol, int32_t *iterations_out, void *stream);

/* Complex resistivity (induced polarisation): the response of
 * DCMultiElectrodeModelling with setComplex(true) (core/src/bert/
 * dcfemmodelling.cpp:573-583, 1103-1119), which with complex resistivities
 * uses the total-potential formulation (calculateK_, :1756-1929: complex
 * symmetric matrices, unit point sources, no singularity removal) — solved
 * here by a block COCG with Jacobi preconditioning in FP64 to the context's
 * tolerance.  rho_re / rho_im: per-cell complex resistivity (device, n_cells
 * each); rhoa_re / rhoa_im: complex apparent resistivities k * u (device,
 * n_data each; the reference returns them as [re, im]). */
int ertgb_response_complex(ertgb_ctx *ctx, const double *rho_re_dev, const double *rho_im_dev, double *rhoa_re_dev,
                           double *rhoa_im_dev, void *stream);
/* Complex Jacobian of the last complex response (createJacobian in complex
 * mode, dcfemmodelling.cpp:1410-1431, 1446-1458): J_dev receives n_data x
 * n_param complex values, interleaved (re, im), row-major; with a model of
 * one complex value per parameter (n_model = n_param) J is divided by
 * model^2 / k as the reference does (no conjugation); other n_model: the
 * unscaled sensitivities. */
int ertgb_jacobian_complex(ertgb_ctx *ctx, const double *model_re_dev, const double *model_im_dev, int n_model,
                           double *J_dev, void *stream);

/* Uniform refinement of a linear simplex mesh on device ``device``.  mode 1:
 * the quadratic mesh of Mesh::createP2 (Triangle6 / Tetrahedron10, one
 * midpoint node per edge); mode 2: Mesh::createH2 (every triangle into 4,
 * every tetrahedron into 8, boundaries into 2 / 4).  Node, cell and boundary
 * numbering and markers are the reference's createRefined_
 * (core/src/mesh.cpp:1278-1600), which pyGIMLi applies to every parameter
 * mesh handed to the forward operator (pygimli/frameworks/modelling.py:
 * 682-699, MeshModelling.createRefinedFwdMesh).  Inputs in host memory as
 * for ertgb_set_mesh with order 1; bnd_cell (the adjacent cell of each
 * boundary) may be NULL.  H2 boundaries get the child of their parent's
 * adjacent cell that holds them (-1 without one).  The refined mesh stays on
 * the device until ertgb_refined_get copies it out; errors:
 * ertgb_last_error(NULL). */
typedef struct ertgb_refined ertgb_refined;
int ertgb_refine(int device, int dim, int mode, int64_t n_nodes, const double *xyz_host,
                 const int32_t *node_marker_host, int64_t n_cells, const int32_t *cell_nodes_host,
                 const int32_t *cell_marker_host, int64_t n_bnd, const int32_t *bnd_nodes_host,
                 const int32_t *bnd_marker_host, const int32_t *bnd_cell_host, ertgb_refined **out);
/* Nodes, cells, nodes per cell, boundaries and nodes per boundary of a refined mesh. */
int ertgb_refined_sizes(const ertgb_refined *r, int64_t *n_nodes, int64_t *n_cells, int64_t *nv, int64_t *n_bnd,
                        int64_t *nvb);
/* Copy a refined mesh into host arrays sized by ertgb_refined_sizes (xyz:
 * n_nodes x 3); a NULL array is skipped. */
int ertgb_refined_get(const ertgb_refined *r, double *xyz_host, int32_t *node_marker_host, int32_t *cell_nodes_host,
                      int32_t *cell_marker_host, int32_t *bnd_nodes_host, int32_t *bnd_marker_host,
                      int32_t *bnd_cell_host);
int ertgb_refined_free(ertgb_refined *r);

#ifdef __cplusplus
}
#endif

#endif /* ERTGB_H */
