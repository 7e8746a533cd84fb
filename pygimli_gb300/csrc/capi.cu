// C ABI of libertgb (declared in include/ertgb.h).  Every entry point
// catches all exceptions and returns a status; messages are kept per context.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <set>

#include "ertgb_internal.cuh"

using namespace ertgb;

namespace {

std::string g_create_error;
thread_local std::string g_free_error;  // last error of the context-free entry points

template <class F> int guard_free(F &&f) {
    try {
        f();
        g_free_error.clear();
        return ERTGB_OK;
    } catch (Error &e) {
        g_free_error = e.what();
        return e.code;
    } catch (std::exception &e) {
        g_free_error = e.what();
        return ERTGB_BAD_INPUT;
    }
}

template <class F> int guard(Context *c, F &&f) {
    if (!c) return ERTGB_BAD_INPUT;
    try {
        f();
        c->last_error.clear();
        return ERTGB_OK;
    } catch (Error &e) {
        c->last_error = e.what();
        return e.code;
    } catch (std::exception &e) {
        c->last_error = e.what();
        return ERTGB_BAD_INPUT;
    } catch (...) {
        c->last_error = "unknown error";
        return ERTGB_BAD_INPUT;
    }
}

void clear_reference(Context &c) {
    c.ref_elec = -1;
    c.ref_node = -1;
    c.ref_minr = 0.0;
    c.ref_cells.clear();
    c.calib.clear();
}

void invalidate_derived(Context &c) {
    c.fp64_k.clear();
    c.up_user.clear();  // given primaries belong to the mesh, electrodes and wavenumbers they were set for
    c.prim_ready = false;
    c.s1_ready = false;
    c.have_pot = false;
    c.have_S = false;
}

// Join the caller's stream into the context stream and back.  A null stream
// is the caller's legacy default stream: the context stream is created
// non-blocking, so it is ordered against the legacy stream explicitly
// (work the caller queued there, such as the copy of the model, comes first).
struct StreamJoin {
    Context &c;
    cudaStream_t user;
    StreamJoin(Context &ctx, void *stream)
        : c(ctx), user(stream ? (cudaStream_t)stream : cudaStreamLegacy) {
        if (user != c.stream) {
            ERTGB_CUDA(cudaEventRecord(c.ev[6], user));
            ERTGB_CUDA(cudaStreamWaitEvent(c.stream, c.ev[6], 0));
        }
    }
    void done() {
        if (user != c.stream) {
            ERTGB_CUDA(cudaEventRecord(c.ev[7], c.stream));
            ERTGB_CUDA(cudaStreamWaitEvent(user, c.ev[7], 0));
        }
    }
};

}  // namespace

void ertgb::set_free_error(const std::string &msg) { g_free_error = msg; }

void ertgb::check_spmm_args(int64_t n, int64_t nnz, const void *rowptr, const void *colidx, const void *vals, int n_k,
                            int n_per_k, int64_t ld, const void *X, const void *Y, const void *dots) {
    ERTGB_REQUIRE(n > 0 && nnz > 0 && n_k > 0 && n_per_k > 0, "empty operator");
    ERTGB_REQUIRE(ld > 0 && ld % 32 == 0, "ld must be a positive multiple of 32");
    ERTGB_REQUIRE(rowptr && colidx && vals && X && Y && dots, "null device pointer");
    ERTGB_REQUIRE(n <= INT32_MAX && nnz <= INT32_MAX, "int32 CSR indices");
}

namespace {

// Device -> host copy of a large result.  Into page-locked (or device)
// memory the copy engines run at full speed; into ordinary pageable memory
// the driver's staged copy varied from call to call on the GB300 machine
// (24-193 GB/s for the same array), while the GPU's own stores through the
// host page tables (devices that report pageable memory access, as Grace
// systems do) held 170 GB/s, so such destinations are written by a
// grid-stride copy kernel.
__global__ void k_copy_out16(uint4 *__restrict__ dst, const uint4 *__restrict__ src, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}
__global__ void k_copy_out4(uint32_t *__restrict__ dst, const uint32_t *__restrict__ src, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

void copy_to_host(Context &c, void *dst, const void *src, size_t bytes) {
    cudaPointerAttributes a{};
    const bool known = cudaPointerGetAttributes(&a, dst) == cudaSuccess;
    cudaGetLastError();  // an unregistered host pointer may leave an error on older drivers
    int pageable = 0, sms = 1;
    ERTGB_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c.device));
    ERTGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
    const bool unregistered = known && a.type == cudaMemoryTypeUnregistered;
    if (!unregistered || !pageable || bytes % 4) {
        ERTGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c.stream));
        return;
    }
    if (((uintptr_t)dst % 16 == 0) && ((uintptr_t)src % 16 == 0) && bytes % 16 == 0)
        k_copy_out16<<<(unsigned)(4 * sms), 512, 0, c.stream>>>((uint4 *)dst, (const uint4 *)src, bytes / 16);
    else
        k_copy_out4<<<(unsigned)(4 * sms), 512, 0, c.stream>>>((uint32_t *)dst, (const uint32_t *)src, bytes / 4);
    ERTGB_CUDA(cudaGetLastError());
}

void ensure_derived(Context &c) {
    if (!c.have_mesh) throw Error(ERTGB_STATE, "no mesh set");
    if (!c.have_elec) throw Error(ERTGB_STATE, "no electrodes set");
    if (!c.have_kw) throw Error(ERTGB_STATE, "no wavenumbers set");
    if (!c.have_scheme) throw Error(ERTGB_STATE, "no measurement scheme set");
    ERTGB_CUDA(cudaSetDevice(c.device));
    const bool total = c.formulation == ERTGB_FORMULATION_TOTAL_POTENTIAL;
    if (total) {
        if ((int)c.src_row.size() != c.nE) throw Error(ERTGB_STATE, "electrode source rows do not match the electrodes");
        for (int e = 0; e < c.nE; e++)
            if ((c.src_row[e] < 0 || c.src_row[e] >= c.mesh.n) && c.ent_cell[e] < 0)
                throw Error(ERTGB_STATE, "an electrode has no source row (set the matrix extension after the electrodes)");
    } else {
        for (int e = 0; e < c.nE; e++)
            if (c.enode[e] < 0 && c.ent_cell[e] < 0)
                throw Error(ERTGB_STATE, "singularity removal needs a node or a cell for every electrode");
    }
    const MeshData &m = c.mesh;
    if (m.dim == 3 && m.B == 0 && m.dir_nodes.empty() && c.calib.empty())
        throw Error(ERTGB_STATE, "a closed (Neumann-only) 3-D domain needs a calibration node (ertgb_set_reference)");
    if (!m.ext_rows.empty() || m.n_ext > 0) {
        if (c.ref_elec >= 0 || c.ref_node >= 0)
            throw Error(ERTGB_STATE, "a reference electrode with complete-electrode-model or bypass electrodes "
                                     "is not supported");
        if (!m.dir_nodes.empty()) {
            std::vector<uint8_t> fixed((size_t)m.nn, 0);
            for (int32_t v : m.dir_nodes) fixed[v] = 1;
            for (size_t i = 0; i < m.ext_rows.size(); i++)
                if ((m.ext_rows[i] < m.nn && fixed[m.ext_rows[i]]) || (m.ext_cols[i] < m.nn && fixed[m.ext_cols[i]]))
                    throw Error(ERTGB_STATE, "a complete-electrode-model or bypass entry on a Dirichlet boundary node");
        }
    }
    if (!c.prim_ready) {
        build_electrode_weights(c);
        c.R = (int64_t)c.nE * c.nK;
        c.Rpad = ceil_div(c.R, c.rhs_align) * c.rhs_align;
        compute_boundary_alpha(c);
        if (total) c.d_up.release();  // no primary field
        else if (!c.up_user.empty()) upload_primary(c);
        else compute_primary(c);
        c.prim_ready = true;
        c.s1_ready = false;
        c.jac_ready = false;
    }
    if (!c.jac_ready) {
        build_jacobian_tiles(c);
        c.jac_ready = true;
    }
    if (!c.s1_ready) {
        if (total) c.d_S1.release();  // the unit-resistivity matrix only serves singularity removal
        else assemble_unit(c, c.stream);
        c.s1_ready = true;
    }
}

float elapsed(Context &c, int a, int b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c.ev[a], c.ev[b]);
    return ms;
}

int do_response(Context &c, const double *rho, double *rhoa, void *stream) {
    int status = ERTGB_OK;
    StreamJoin j(c, stream);
    ensure_derived(c);
    cudaStream_t s = c.stream;
    c.have_pot = false;
    c.stats.launches_response = 0;
    c.stats.stalled_columns = 0;
    check_rho(c, rho, s);
    c.d_rho_last = rho;
    MeshData &m = c.mesh;
    ERTGB_CUDA(cudaEventRecord(c.ev[0], s));
    const bool total = c.formulation == ERTGB_FORMULATION_TOTAL_POTENTIAL;
    const bool fp64_only = c.precond == ERTGB_PRECOND_IC0 || c.precond == ERTGB_PRECOND_BAND;
    if (c.precision != ERTGB_PRECISION_MIXED && c.precond != ERTGB_PRECOND_JACOBI && !fp64_only)
        throw Error(ERTGB_BAD_INPUT, "the FSAI and learned preconditioners need mixed precision");
    if (c.precision == ERTGB_PRECISION_MIXED && fp64_only)
        throw Error(ERTGB_BAD_INPUT, "the IC(0) preconditioner and the banded direct solve need FP64 precision");
    if (c.precond == ERTGB_PRECOND_LEARNED && !m.ext_rows.empty())
        throw Error(ERTGB_BAD_INPUT, "the learned preconditioner does not cover a matrix extension (CEM, bypass)");
    c.d_S.alloc((size_t)c.nK * m.nnz);
    assemble_all(c, rho, c.d_S.p, s);
    if (!total) compute_source_rho(c, rho, s);
    ERTGB_CUDA(cudaEventRecord(c.ev[1], s));
    c.d_r.alloc((size_t)m.n * c.Rpad);
    if (total) {
        build_rhs_total(c, s);
    } else {
        build_rhs(c, s);
        compute_rhs_scale(c, s);
    }
    ERTGB_CUDA(cudaEventRecord(c.ev[2], s));
    c.have_S = true;
    status = (c.precision == ERTGB_PRECISION_MIXED) ? pcg_solve_mixed(c, s) : pcg_solve(c, s);
    ERTGB_CUDA(cudaEventRecord(c.ev[3], s));
    if (!total) finish_potentials(c, s);
    collect_response(c, rhoa, s);
    ERTGB_CUDA(cudaEventRecord(c.ev[4], s));
    ERTGB_CUDA(cudaEventSynchronize(c.ev[4]));
    c.stats.ms_assemble = elapsed(c, 0, 1);
    c.stats.ms_rhs = elapsed(c, 1, 2);
    c.stats.ms_solve = elapsed(c, 2, 3);
    c.stats.ms_collect = elapsed(c, 3, 4);
    // check_rho, inv_rho, assemble, dinv, source_rho, rhs, finish_pot, collect, response
    // (total potential: check_rho, inv_rho, assemble, dinv, rhs, collect, response)
    c.stats.launches_response += total ? 7 : 9;
    c.have_pot = true;
    j.done();
    return status;
}

// Replace the matrix extension (rows / cols / vals after the nodes) and
// rebuild the pattern and the device structures that derive from it.
void set_mesh_extension(Context &c, int64_t n_ext, std::vector<int32_t> rows, std::vector<int32_t> cols,
                        std::vector<double> vals) {
    MeshData &m = c.mesh;
    m.n_ext = n_ext;
    m.n = m.nn + n_ext;
    m.ext_rows.swap(rows);
    m.ext_cols.swap(cols);
    m.ext_vals.swap(vals);
    build_pattern(m);
    build_mesh_device(c);
    c.lp.graph_ready = false;
}
void do_jacobian(Context &c, const double *model, int n_model, void *J, int dtype, void *stream) {
    if (!c.have_pot) throw Error(ERTGB_STATE, "createJacobian needs the potentials of a response first");
    if (dtype != 0 && dtype != 1) throw Error(ERTGB_BAD_INPUT, "dtype must be 0 (FP64) or 1 (FP32)");
    StreamJoin j(c, stream);
    cudaStream_t s = c.stream;
    ERTGB_CUDA(cudaEventRecord(c.ev[4], s));
    jacobian(c, model, n_model, J, dtype, s);
    ERTGB_CUDA(cudaEventRecord(c.ev[5], s));
    ERTGB_CUDA(cudaEventSynchronize(c.ev[5]));
    c.stats.ms_jacobian = elapsed(c, 4, 5);
    c.stats.launches_jacobian = 1;
    j.done();
}

}  // namespace

extern "C" {

int ertgb_create(ertgb_ctx **out, int device) {
    if (!out) return ERTGB_BAD_INPUT;
    *out = nullptr;
    Context *c = new Context();
    int rc = guard(c, [&] {
        c->device = device;
        ERTGB_CUDA(cudaSetDevice(device));
        ERTGB_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        for (auto &e : c->ev) ERTGB_CUDA(cudaEventCreate(&e));
    });
    if (rc != ERTGB_OK) {
        g_create_error = c->last_error;
        delete c;
        return rc;
    }
    *out = reinterpret_cast<ertgb_ctx *>(c);
    return ERTGB_OK;
}

int ertgb_destroy(ertgb_ctx *ctx) {
    Context *c = reinterpret_cast<Context *>(ctx);
    if (!c) return ERTGB_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    cudaStream_t s = c->stream;
    delete c;
    if (s) cudaStreamDestroy(s);
    return ERTGB_OK;
}

const char *ertgb_last_error(const ertgb_ctx *ctx) {
    const Context *c = reinterpret_cast<const Context *>(ctx);
    if (!c) return g_free_error.empty() ? g_create_error.c_str() : g_free_error.c_str();
    return c->last_error.c_str();
}

int ertgb_set_mesh(ertgb_ctx *ctx, int dim, int order, int n_nodes, const double *xyz, int n_cells,
                   const int32_t *cell_nodes, const int32_t *cell_marker, int n_bnd, const int32_t *bnd_nodes,
                   const int32_t *bnd_marker, const int32_t *bnd_cell) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
        ERTGB_REQUIRE(order == 1 || order == 2, "order must be 1 (linear) or 2 (quadratic)");
        ERTGB_REQUIRE(n_nodes > 0 && n_cells > 0 && n_bnd >= 0, "empty mesh");
        ERTGB_REQUIRE(xyz && cell_nodes && cell_marker, "null mesh array");
        ERTGB_CUDA(cudaSetDevice(c->device));
        c->mesh.~MeshData();  // release the previous mesh's device buffers
        new (&c->mesh) MeshData();
        c->lp.graph_ready = false;
        MeshData &m = c->mesh;
        m.dim = dim;
        m.order = order;
        m.nv = order == 1 ? dim + 1 : (dim == 2 ? 6 : 10);
        m.nvb = order == 1 ? dim : (dim == 2 ? 3 : 6);
        m.n = n_nodes;
        m.nn = n_nodes;
        m.C = n_cells;
        m.xyz.assign(xyz, xyz + (size_t)n_nodes * 3);
        m.cells.assign(cell_nodes, cell_nodes + (size_t)n_cells * m.nv);
        m.marker.assign(cell_marker, cell_marker + n_cells);
        for (int32_t v : m.cells) ERTGB_REQUIRE(v >= 0 && v < n_nodes, "cell node index out of range");
        int32_t pmax = -1;
        for (int32_t v : m.marker) pmax = std::max(pmax, v);
        m.P = (int64_t)pmax + 1;
        std::set<int32_t> dir;
        for (int b = 0; b < n_bnd; b++) {
            const int mk = bnd_marker[b];
            if (mk == -4)  // the reference throws here as well (dcfemmodelling.cpp:293)
                throw Error(ERTGB_BAD_INPUT, "inhomogeneous Dirichlet boundaries (marker -4) are not implemented");
            if (mk == -3) {  // homogeneous Dirichlet: the boundary's nodes are fixed rows
                for (int i = 0; i < m.nvb; i++) {
                    const int32_t v = bnd_nodes[(size_t)b * m.nvb + i];
                    ERTGB_REQUIRE(v >= 0 && v < n_nodes, "boundary node index out of range");
                    dir.insert(v);
                }
                continue;
            }
            if (mk != -2) continue;
            for (int i = 0; i < m.nvb; i++) {
                const int32_t v = bnd_nodes[(size_t)b * m.nvb + i];
                ERTGB_REQUIRE(v >= 0 && v < n_nodes, "boundary node index out of range");
                m.bnd_nodes.push_back(v);
            }
            ERTGB_REQUIRE(bnd_cell && bnd_cell[b] >= 0 && bnd_cell[b] < n_cells,
                          "mixed boundary without an adjacent cell");
            m.bnd_cell.push_back(bnd_cell[b]);
        }
        m.dir_nodes.assign(dir.begin(), dir.end());
        m.B = (int64_t)m.bnd_cell.size();
        build_pattern(m);
        build_mesh_device(*c);
        c->have_mesh = true;
        c->have_elec = false;
        clear_reference(*c);
        c->src_row.clear();
        c->collect_last_k = false;
        invalidate_derived(*c);
    });
}

int ertgb_set_electrodes(ertgb_ctx *ctx, int n_elec, const int32_t *elec_node, double surface_z) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (!c->have_mesh) throw Error(ERTGB_STATE, "set the mesh before the electrodes");
        ERTGB_REQUIRE(n_elec > 0 && elec_node, "no electrodes");
        MeshData &m = c->mesh;
        c->nE = n_elec;
        c->enode.assign(elec_node, elec_node + n_elec);
        std::set<int32_t> uniq;
        for (int32_t v : c->enode) {
            // -1: an electrode given by its extension row (total potential) or by
            // the cell that holds it (ertgb_set_electrode_shapes)
            if (v == -1) continue;
            ERTGB_REQUIRE(v >= 0 && v < m.nn, "electrode node index out of range");
            ERTGB_REQUIRE(uniq.insert(v).second, "two electrodes on the same node");
        }
        c->surface_z = surface_z;
        // source centre = mean electrode position (an extension may replace it)
        double sc[3] = {0, 0, 0};
        std::vector<double> epos((size_t)n_elec * 3, 0.0);
        for (int e = 0; e < n_elec; e++)
            for (int d = 0; d < 3; d++) {
                if (c->enode[e] >= 0) epos[3 * e + d] = m.xyz[3 * (size_t)c->enode[e] + d];
                sc[d] += epos[3 * e + d];
            }
        for (int d = 0; d < 3; d++) c->src_center[d] = sc[d] / (double)n_elec;
        c->epos_h = epos;
        c->ent_cell.assign(n_elec, -1);
        c->ent_w.assign((size_t)n_elec * m.nv, 0.0);
        // incident cells and smallest neighbour distance per electrode node
        std::vector<std::vector<int32_t>> inc(n_elec);
        std::vector<int> slot(m.nn, -1);
        for (int e = 0; e < n_elec; e++)
            if (c->enode[e] >= 0) slot[c->enode[e]] = e;
        for (int64_t cc = 0; cc < m.C; cc++)
            for (int i = 0; i < m.nv; i++) {
                const int e = slot[m.cells[cc * m.nv + i]];
                if (e >= 0) inc[e].push_back((int32_t)cc);
            }
        c->ecell_ptr.assign(n_elec + 1, 0);
        c->ecell.clear();
        c->emin_r.assign(n_elec, DBL_MAX);
        for (int e = 0; e < n_elec; e++) {
            if (c->enode[e] < 0) {
                c->emin_r[e] = 0.0;
                c->ecell_ptr[e + 1] = (int32_t)c->ecell.size();
                continue;
            }
            ERTGB_REQUIRE(!inc[e].empty(), "electrode node belongs to no cell");
            const int32_t nd = c->enode[e];
            for (int32_t cc : inc[e]) {
                c->ecell.push_back(cc);
                for (int i = 0; i < m.nv; i++) {
                    const int32_t o = m.cells[(size_t)cc * m.nv + i];
                    if (o == nd) continue;
                    double d2 = 0;
                    for (int d = 0; d < 3; d++) {
                        const double dd = m.xyz[3 * (size_t)nd + d] - m.xyz[3 * (size_t)o + d];
                        d2 += dd * dd;
                    }
                    c->emin_r[e] = std::min(c->emin_r[e], std::sqrt(d2));
                }
            }
            c->ecell_ptr[e + 1] = (int32_t)c->ecell.size();
        }
        cudaStream_t s = c->stream;
        c->d_enode.upload(c->enode, s);
        c->d_epos.upload(epos, s);
        c->d_emin_r.upload(c->emin_r, s);
        c->d_ecell_ptr.upload(c->ecell_ptr, s);
        c->d_ecell.upload(c->ecell, s);
        // total potential: the current enters on the electrode node unless an
        // extension gives other rows
        c->src_row = c->enode;
        c->collect_last_k = false;
        c->d_src_row.upload(c->src_row, s);
        ERTGB_CUDA(cudaStreamSynchronize(s));
        c->have_elec = true;
        clear_reference(*c);
        invalidate_derived(*c);
    });
}

int ertgb_set_reference(ertgb_ctx *ctx, int ref_electrode, int ref_node, int n_calib, const int32_t *calib) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (!c->have_mesh || !c->have_elec) throw Error(ERTGB_STATE, "set the mesh and the electrodes first");
        MeshData &m = c->mesh;
        ERTGB_REQUIRE(ref_electrode >= -1 && ref_electrode < c->nE, "reference electrode out of range");
        ERTGB_REQUIRE(ref_node >= -1 && ref_node < m.nn, "reference node out of range");
        ERTGB_REQUIRE(ref_electrode < 0 || ref_node < 0, "give either a reference electrode or a reference node");
        ERTGB_REQUIRE(n_calib >= 0 && (n_calib == 0 || calib), "null calibration nodes");
        std::set<int32_t> cal;
        for (int i = 0; i < n_calib; i++) {
            ERTGB_REQUIRE(calib[i] >= 0 && calib[i] < m.nn, "calibration node out of range");
            cal.insert(calib[i]);
        }
        clear_reference(*c);
        c->ref_elec = ref_electrode;
        c->ref_node = ref_node;
        if (ref_node >= 0) {
            for (int d = 0; d < 3; d++) c->ref_pos[d] = m.xyz[3 * (size_t)ref_node + d];
            double mr = DBL_MAX;
            for (int64_t cc = 0; cc < m.C; cc++) {
                const int32_t *cn = &m.cells[(size_t)cc * m.nv];
                bool has = false;
                for (int i = 0; i < m.nv; i++) has |= cn[i] == ref_node;
                if (!has) continue;
                c->ref_cells.push_back((int32_t)cc);
                for (int i = 0; i < m.nv; i++) {
                    if (cn[i] == ref_node) continue;
                    double d2 = 0;
                    for (int d = 0; d < 3; d++) {
                        const double dd = m.xyz[3 * (size_t)ref_node + d] - m.xyz[3 * (size_t)cn[i] + d];
                        d2 += dd * dd;
                    }
                    mr = std::min(mr, std::sqrt(d2));
                }
            }
            ERTGB_REQUIRE(!c->ref_cells.empty(), "reference node belongs to no cell");
            c->ref_minr = mr;
        }
        c->calib.assign(cal.begin(), cal.end());
        invalidate_derived(*c);
    });
}

int ertgb_set_electrode_shapes(ertgb_ctx *ctx, int n_elec, const int32_t *cell, const double *pos) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (!c->have_elec) throw Error(ERTGB_STATE, "set the electrodes first");
        ERTGB_REQUIRE(n_elec == c->nE && cell && pos, "one cell and position per electrode");
        MeshData &m = c->mesh;
        const int d = m.dim;
        for (int e = 0; e < n_elec; e++) {
            if (cell[e] < 0) continue;
            ERTGB_REQUIRE(c->enode[e] < 0, "an electrode inside a cell must have no node");
            ERTGB_REQUIRE(cell[e] < m.C, "electrode cell out of range");
            ERTGB_REQUIRE(m.order == 1 && m.nv == d + 1, "electrodes inside cells need linear cells");
            // barycentric coordinates = the linear shape functions at the electrode
            const int32_t *cn = &m.cells[(size_t)cell[e] * m.nv];
            double A[3][3] = {{0}}, r[3] = {0}, lam[3] = {0};
            for (int i = 0; i < d; i++) {
                for (int j = 0; j < d; j++) A[i][j] = m.xyz[3 * (size_t)cn[j + 1] + i] - m.xyz[3 * (size_t)cn[0] + i];
                r[i] = pos[3 * e + i] - m.xyz[3 * (size_t)cn[0] + i];
            }
            // Gaussian elimination with partial pivoting (d <= 3)
            int piv[3] = {0, 1, 2};
            for (int k = 0; k < d; k++) {
                int b = k;
                for (int i = k + 1; i < d; i++)
                    if (std::fabs(A[piv[i]][k]) > std::fabs(A[piv[b]][k])) b = i;
                std::swap(piv[k], piv[b]);
                ERTGB_REQUIRE(std::fabs(A[piv[k]][k]) > 0.0, "degenerate electrode cell");
                for (int i = k + 1; i < d; i++) {
                    const double f = A[piv[i]][k] / A[piv[k]][k];
                    for (int j = k; j < d; j++) A[piv[i]][j] -= f * A[piv[k]][j];
                    r[piv[i]] -= f * r[piv[k]];
                }
            }
            for (int k = d - 1; k >= 0; k--) {
                double s2 = r[piv[k]];
                for (int j = k + 1; j < d; j++) s2 -= A[piv[k]][j] * lam[j];
                lam[k] = s2 / A[piv[k]][k];
            }
            double l0 = 1.0;
            for (int i = 0; i < d; i++) l0 -= lam[i];
            ERTGB_REQUIRE(l0 >= -1e-9 && lam[0] >= -1e-9 && lam[1] >= -1e-9 && (d < 3 || lam[2] >= -1e-9),
                          "electrode position outside its cell");
            c->ent_cell[e] = cell[e];
            c->ent_w[(size_t)e * m.nv] = l0;
            for (int i = 0; i < d; i++) c->ent_w[(size_t)e * m.nv + i + 1] = lam[i];
            for (int i = 0; i < 3; i++) c->epos_h[3 * e + i] = pos[3 * e + i];
            c->emin_r[e] = 0.0;
        }
        // source resistivity of an electrode inside a cell: that cell's
        std::vector<int32_t> ptr(1, 0), lst;
        for (int e = 0; e < c->nE; e++) {
            if (c->ent_cell[e] >= 0) lst.push_back(c->ent_cell[e]);
            else lst.insert(lst.end(), c->ecell.begin() + c->ecell_ptr[e], c->ecell.begin() + c->ecell_ptr[e + 1]);
            ptr.push_back((int32_t)lst.size());
        }
        c->ecell_ptr.swap(ptr);
        c->ecell.swap(lst);
        double sc[3] = {0, 0, 0};
        for (int e = 0; e < c->nE; e++)
            for (int i = 0; i < 3; i++) sc[i] += c->epos_h[3 * e + i];
        for (int i = 0; i < 3; i++) c->src_center[i] = sc[i] / (double)c->nE;
        cudaStream_t s = c->stream;
        c->d_epos.upload(c->epos_h, s);
        c->d_emin_r.upload(c->emin_r, s);
        c->d_ecell_ptr.upload(c->ecell_ptr, s);
        c->d_ecell.upload(c->ecell, s);
        ERTGB_CUDA(cudaStreamSynchronize(s));
        invalidate_derived(*c);
    });
}

int ertgb_set_formulation(ertgb_ctx *ctx, int formulation) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(formulation == ERTGB_FORMULATION_SINGULARITY_REMOVAL ||
                          formulation == ERTGB_FORMULATION_TOTAL_POTENTIAL,
                      "formulation must be 0 (singularity removal) or 1 (total potential)");
        ERTGB_CUDA(cudaSetDevice(c->device));
        if (c->have_mesh && (c->mesh.n_ext > 0 || !c->mesh.ext_rows.empty()))
            set_mesh_extension(*c, 0, {}, {}, {});
        c->formulation = formulation;
        c->src_row = c->enode;
        c->collect_last_k = false;
        if (c->have_elec) c->d_src_row.upload(c->src_row, c->stream);
        invalidate_derived(*c);
    });
}

int ertgb_set_extension(ertgb_ctx *ctx, int n_ext, int64_t n_entries, const int32_t *rows, const int32_t *cols,
                        const double *vals, const int32_t *src_row, const double *src_center, int collect_last_k) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (!c->have_mesh || !c->have_elec) throw Error(ERTGB_STATE, "set the mesh and the electrodes before the extension");
        if (c->formulation != ERTGB_FORMULATION_TOTAL_POTENTIAL)
            throw Error(ERTGB_STATE, "a matrix extension needs the total-potential formulation");
        ERTGB_REQUIRE(n_ext >= 0 && n_entries >= 0, "negative extension size");
        ERTGB_REQUIRE(n_entries == 0 || (rows && cols && vals), "null extension entries");
        ERTGB_REQUIRE(src_row, "null source rows");
        const int64_t N = c->mesh.nn + n_ext;
        ERTGB_REQUIRE(N <= INT32_MAX && n_entries <= INT32_MAX, "extension too large for int32 indices");
        std::vector<int32_t> r(rows, rows + n_entries), q(cols, cols + n_entries);
        std::vector<double> v(vals, vals + n_entries);
        for (int64_t i = 0; i < n_entries; i++) {
            ERTGB_REQUIRE(r[i] >= 0 && r[i] < N && q[i] >= 0 && q[i] < N, "extension entry out of range");
            ERTGB_REQUIRE(std::isfinite(v[i]), "extension value not finite");
        }
        std::vector<int32_t> sr(src_row, src_row + c->nE);
        for (int e = 0; e < c->nE; e++)  // an electrode inside a cell has no source row
            ERTGB_REQUIRE((sr[e] >= 0 && sr[e] < N) || (e < (int)c->ent_cell.size() && c->ent_cell[e] >= 0),
                          "electrode source row out of range");
        ERTGB_CUDA(cudaSetDevice(c->device));
        set_mesh_extension(*c, n_ext, std::move(r), std::move(q), std::move(v));
        c->src_row = sr;
        c->d_src_row.upload(c->src_row, c->stream);
        if (src_center)
            for (int d = 0; d < 3; d++) c->src_center[d] = src_center[d];
        c->collect_last_k = collect_last_k != 0;
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        invalidate_derived(*c);
    });
}

int ertgb_analytic_potentials(ertgb_ctx *ctx, double rho) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(std::isfinite(rho) && rho > 0.0, "resistivity must be positive");
        ensure_derived(*c);
        if (c->mesh.n_ext > 0 || !c->mesh.ext_rows.empty())
            throw Error(ERTGB_STATE, "no analytic potentials with complete-electrode-model or bypass electrodes");
        if (!c->up_user.empty())
            throw Error(ERTGB_STATE, "no analytic potentials on a topographic surface");
        for (int32_t v : c->enode)
            if (v < 0) throw Error(ERTGB_STATE, "analytic potentials need node electrodes");
        c->d_x.alloc((size_t)c->mesh.n * c->Rpad);
        analytic_potentials(*c, rho, c->d_x.p);
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        c->have_pot = true;
    });
}

int ertgb_set_primary(ertgb_ctx *ctx, int n_k, int n_elec, int64_t n_nodes, const double *up) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (c->formulation != ERTGB_FORMULATION_SINGULARITY_REMOVAL)
            throw Error(ERTGB_STATE, "primary potentials belong to the singularity-removal formulation");
        if (!c->have_mesh || !c->have_elec || !c->have_kw)
            throw Error(ERTGB_STATE, "set mesh, electrodes and wavenumbers before the primary potentials");
        ERTGB_REQUIRE(up, "null buffer");
        ERTGB_REQUIRE(n_k == c->nK && n_elec == c->nE && n_nodes == c->mesh.n,
                      "primary potentials must be n_k x n_elec x n_nodes of the context");
        const size_t total = (size_t)n_k * n_elec * n_nodes;
        for (size_t i = 0; i < total; i++) ERTGB_REQUIRE(std::isfinite(up[i]), "non-finite primary potential");
        c->up_user.assign(up, up + total);
        c->prim_ready = false;
        c->have_pot = false;
        c->have_S = false;
    });
}

int ertgb_set_kw(ertgb_ctx *ctx, int n_k, const double *k, const double *w) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(n_k > 0 && k && w, "no wavenumbers");
        for (int i = 0; i < n_k; i++) ERTGB_REQUIRE(k[i] >= 0.0 && std::isfinite(k[i]) && std::isfinite(w[i]),
                                                    "wavenumbers must be finite and non-negative");
        c->nK = n_k;
        c->k.assign(k, k + n_k);
        c->w.assign(w, w + n_k);
        c->d_k.upload(c->k, c->stream);
        c->d_w.upload(c->w, c->stream);
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        c->have_kw = true;
        invalidate_derived(*c);
    });
}

int ertgb_set_scheme(ertgb_ctx *ctx, int n_data, const int32_t *abmn, const double *kfac) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(n_data > 0 && abmn && kfac, "empty scheme");
        if (!c->have_elec) throw Error(ERTGB_STATE, "set the electrodes before the scheme");
        for (int64_t i = 0; i < 4 * (int64_t)n_data; i++)
            ERTGB_REQUIRE(abmn[i] >= -1 && abmn[i] < c->nE, "electrode index out of range in scheme");
        c->D = n_data;
        c->abmn_h.assign(abmn, abmn + (size_t)4 * n_data);
        c->d_abmn.upload(abmn, (size_t)4 * n_data, c->stream);
        c->d_kfac.upload(kfac, (size_t)n_data, c->stream);
        c->kfac_h.assign(kfac, kfac + n_data);
        // distinct current and potential dipoles, in order of first use
        std::map<std::pair<int32_t, int32_t>, int32_t> amap, mmap;
        std::vector<int32_t> dip_a, dip_m, data_dip((size_t)2 * n_data);
        for (int64_t d = 0; d < n_data; d++) {
            const auto ka = std::make_pair(abmn[4 * d], abmn[4 * d + 1]);
            const auto km = std::make_pair(abmn[4 * d + 2], abmn[4 * d + 3]);
            auto ia = amap.emplace(ka, (int32_t)amap.size());
            if (ia.second) { dip_a.push_back(ka.first); dip_a.push_back(ka.second); }
            auto im = mmap.emplace(km, (int32_t)mmap.size());
            if (im.second) { dip_m.push_back(km.first); dip_m.push_back(km.second); }
            data_dip[2 * d] = ia.first->second;
            data_dip[2 * d + 1] = im.first->second;
        }
        c->nA = (int)amap.size();
        c->nM = (int)mmap.size();
        c->d_dip_a.upload(dip_a, c->stream);
        c->d_dip_m.upload(dip_m, c->stream);
        c->d_data_dip.upload(data_dip, c->stream);
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        c->have_scheme = true;
        c->have_pot = false;
        c->jac_ready = false;
    });
}

int ertgb_set_solver(ertgb_ctx *ctx, double rtol, int max_iter, int precond) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(rtol > 0.0 && rtol < 1.0, "rtol must be in (0, 1)");
        ERTGB_REQUIRE(max_iter > 0, "max_iter must be positive");
        ERTGB_REQUIRE(precond == ERTGB_PRECOND_JACOBI || precond == ERTGB_PRECOND_FSAI ||
                          precond == ERTGB_PRECOND_LEARNED || precond == ERTGB_PRECOND_IC0 ||
                          precond == ERTGB_PRECOND_BAND,
                      "unknown preconditioner");
        c->rtol = rtol;
        c->max_iter = max_iter;
        c->precond = precond;
    });
}

int ertgb_set_precision(ertgb_ctx *ctx, int precision) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(precision == ERTGB_PRECISION_FP64 || precision == ERTGB_PRECISION_MIXED, "unknown precision");
        c->precision = precision;
    });
}

int ertgb_response(ertgb_ctx *ctx, const double *rho_cell_dev, double *rhoa_dev, void *stream) {
    Context *c = reinterpret_cast<Context *>(ctx);
    int status = ERTGB_OK;
    int rc = guard(c, [&] {
        ERTGB_REQUIRE(rho_cell_dev && rhoa_dev, "null buffer");
        status = do_response(*c, rho_cell_dev, rhoa_dev, stream);
        if (status == ERTGB_NOT_CONVERGED) throw Error(ERTGB_NOT_CONVERGED, "PCG did not converge");
    });
    return rc;
}

int ertgb_response_host(ertgb_ctx *ctx, const double *rho_cell, double *rhoa) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(rho_cell && rhoa, "null buffer");
        if (!c->have_mesh || !c->have_scheme) throw Error(ERTGB_STATE, "mesh and scheme needed");
        ERTGB_CUDA(cudaSetDevice(c->device));
        c->d_rho_tmp.upload(rho_cell, (size_t)c->mesh.C, c->stream);
        c->d_rhoa.alloc((size_t)c->D);
        int st = do_response(*c, c->d_rho_tmp.p, c->d_rhoa.p, nullptr);
        ERTGB_CUDA(cudaMemcpyAsync(rhoa, c->d_rhoa.p, sizeof(double) * c->D, cudaMemcpyDeviceToHost, c->stream));
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        if (st == ERTGB_NOT_CONVERGED) throw Error(ERTGB_NOT_CONVERGED, "PCG did not converge");
    });
}

int ertgb_jacobian(ertgb_ctx *ctx, const double *model_dev, int n_model, void *J_dev, int dtype, void *stream) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(J_dev, "null buffer");
        ERTGB_REQUIRE(n_model == 0 || model_dev, "null model");
        do_jacobian(*c, model_dev, n_model, J_dev, dtype, stream);
    });
}

int ertgb_jacobian_host(ertgb_ctx *ctx, const double *model, int n_model, void *J, int dtype) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(J, "null buffer");
        ERTGB_CUDA(cudaSetDevice(c->device));
        const double *md = nullptr;
        if (n_model > 0) {
            ERTGB_REQUIRE(model, "null model");
            c->d_model_tmp.upload(model, (size_t)n_model, c->stream);
            md = c->d_model_tmp.p;
        }
        const size_t bytes = (size_t)c->D * c->mesh.P * (dtype == 0 ? 8 : 4);
        c->d_J_tmp.alloc(bytes);
        do_jacobian(*c, md, n_model, c->d_J_tmp.p, dtype, nullptr);
        copy_to_host(*c, J, c->d_J_tmp.p, bytes);
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int ertgb_sizes(const ertgb_ctx *ctx, int64_t *n_nodes, int64_t *nnz, int64_t *n_param, int64_t *n_rhs) {
    const Context *c = reinterpret_cast<const Context *>(ctx);
    if (!c) return ERTGB_BAD_INPUT;
    if (n_nodes) *n_nodes = c->mesh.n;
    if (nnz) *nnz = c->mesh.nnz;
    if (n_param) *n_param = c->mesh.P;
    if (n_rhs) *n_rhs = (int64_t)c->nE * c->nK;
    return ERTGB_OK;
}

int ertgb_get_pattern(ertgb_ctx *ctx, int32_t *rowptr, int32_t *colidx) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (!c->have_mesh) throw Error(ERTGB_STATE, "no mesh");
        if (rowptr) std::memcpy(rowptr, c->mesh.rowptr.data(), sizeof(int32_t) * c->mesh.rowptr.size());
        if (colidx) std::memcpy(colidx, c->mesh.colidx.data(), sizeof(int32_t) * c->mesh.colidx.size());
    });
}

int ertgb_get_matrix(ertgb_ctx *ctx, int k_index, int which, double *vals) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(k_index >= 0 && k_index < c->nK && vals, "bad k index");
        const DBuf<double> &src = which == 0 ? c->d_S : c->d_S1;
        if (src.n < (size_t)c->nK * c->mesh.nnz) throw Error(ERTGB_STATE, "matrix not assembled yet");
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        ERTGB_CUDA(cudaMemcpy(vals, src.p + (size_t)k_index * c->mesh.nnz, sizeof(double) * c->mesh.nnz,
                              cudaMemcpyDeviceToHost));
    });
}

static void copy_blocked(Context &c, const double *dev, double *host) {
    const int64_t n = c.mesh.n;
    std::vector<double> tmp((size_t)n * c.Rpad);
    ERTGB_CUDA(cudaMemcpy(tmp.data(), dev, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost));
    for (int ki = 0; ki < c.nK; ki++)
        for (int e = 0; e < c.nE; e++) {
            double *o = host + ((size_t)ki * c.nE + e) * n;
            const int64_t t = (int64_t)ki * c.nE + e;
            for (int64_t i = 0; i < n; i++) o[i] = tmp[(size_t)i * c.Rpad + t];
        }
}

int ertgb_get_potentials(ertgb_ctx *ctx, double *pot) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (!c->have_pot) throw Error(ERTGB_STATE, "no potentials yet");
        ERTGB_REQUIRE(pot, "null buffer");
        copy_blocked(*c, c->d_x.p, pot);
    });
}

int ertgb_get_electrode_potentials(ertgb_ctx *ctx, double *U) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (!c->have_pot) throw Error(ERTGB_STATE, "no potentials yet");
        ERTGB_REQUIRE(U, "null buffer");
        collect_potentials(*c, c->stream);
        ERTGB_CUDA(cudaMemcpyAsync(U, c->d_U.p, sizeof(double) * (size_t)c->nE * c->nE, cudaMemcpyDeviceToHost,
                                   c->stream));
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int ertgb_get_primary(ertgb_ctx *ctx, double *prim) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(prim, "null buffer");
        if (c->formulation == ERTGB_FORMULATION_TOTAL_POTENTIAL)
            throw Error(ERTGB_STATE, "the total-potential formulation has no primary potentials");
        ensure_derived(*c);
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        copy_blocked(*c, c->d_up.p, prim);
    });
}

int ertgb_get_stats(const ertgb_ctx *ctx, ertgb_stats *stats) {
    const Context *c = reinterpret_cast<const Context *>(ctx);
    if (!c || !stats) return ERTGB_BAD_INPUT;
    *stats = c->stats;
    return ERTGB_OK;
}

int ertgb_csr_spmm_dot(int64_t n, int64_t nnz, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                       int n_k, int n_per_k, int64_t ld, const double *X, double *Y, double *dots, void *stream) {
    return guard_free([&] {
        check_spmm_args(n, nnz, rowptr, colidx, vals, n_k, n_per_k, ld, X, Y, dots);
        cudaStream_t s = (cudaStream_t)stream;
        const int NB = spmm_partial_rows(n, 608);
        double *part = nullptr;
        ERTGB_CUDA(cudaMallocAsync((void **)&part, sizeof(double) * (size_t)NB * ld, s));
        try {
            spmm_dot_launch(n, nnz, rowptr, colidx, vals, n_k, n_per_k, ld, X, Y, dots, part, NB, s);
        } catch (...) {
            cudaFreeAsync(part, s);
            throw;
        }
        ERTGB_CUDA(cudaFreeAsync(part, s));
    });
}

int ertgb_profile_kernel(ertgb_ctx *ctx, int kernel, int reps, void *J_scratch, double *ms, double *bytes,
                         double *flops) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(reps > 0 && ms && bytes && flops, "bad profile arguments");
        if (!c->have_pot) throw Error(ERTGB_STATE, "profile needs a completed response");
        ERTGB_CUDA(cudaSetDevice(c->device));
        switch (kernel) {
            case ERTGB_KERNEL_SPMM: profile_spmm(*c, reps, ms, bytes, flops); break;
            case ERTGB_KERNEL_JACOBIAN:
            case ERTGB_KERNEL_JACOBIAN32:
                ERTGB_REQUIRE(J_scratch, "Jacobian profile needs a scratch J");
                profile_jacobian(*c, reps, J_scratch, kernel == ERTGB_KERNEL_JACOBIAN ? 0 : 1, ms, bytes, flops);
                break;
            case ERTGB_KERNEL_ASSEMBLE: profile_assemble(*c, reps, ms, bytes, flops); break;
            case ERTGB_KERNEL_SPMM32: profile_spmm32(*c, reps, ms, bytes, flops); break;
            default: throw Error(ERTGB_BAD_INPUT, "unknown kernel id");
        }
    });
}

int ertgb_set_precond_weights(ertgb_ctx *ctx, const float *theta, int64_t n) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(theta && n == ERTGB_LP_NPARAM, "weights must be ERTGB_LP_NPARAM floats");
        for (int64_t i = 0; i < n; ++i) ERTGB_REQUIRE(std::isfinite(theta[i]), "non-finite weight");
        ERTGB_CUDA(cudaSetDevice(c->device));
        c->lp.d_theta.upload(theta, (size_t)n, c->stream);
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        c->lp.have_weights = true;
    });
}

int ertgb_assemble(ertgb_ctx *ctx, const double *rho, void *stream) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(rho, "null resistivity");
        StreamJoin j(*c, stream);
        ensure_derived(*c);
        c->have_pot = false;
        check_rho(*c, rho, c->stream);
        c->d_S.alloc((size_t)c->nK * c->mesh.nnz);
        assemble_all(*c, rho, c->d_S.p, c->stream);
        c->have_S = true;
        j.done();
    });
}

int ertgb_lp_forward(ertgb_ctx *ctx, const float *theta, float *G, void *stream) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(theta, "null weights");
        if (!c->have_S) throw Error(ERTGB_STATE, "no assembled matrices (ertgb_assemble or a response first)");
        StreamJoin j(*c, stream);
        lp_forward(*c, theta, c->stream);
        if (G)
            ERTGB_CUDA(cudaMemcpyAsync(G, c->d_G32.p, (size_t)c->lp.nL * c->nK * sizeof(float),
                                       cudaMemcpyDeviceToDevice, c->stream));
        j.done();
    });
}

int ertgb_lp_loss_grad(ertgb_ctx *ctx, const float *theta, float *grad, double *loss, void *stream) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(theta && loss, "null weights or loss");
        if (!c->have_S) throw Error(ERTGB_STATE, "no assembled matrices (ertgb_assemble or a response first)");
        StreamJoin j(*c, stream);
        *loss = lp_loss_grad(*c, theta, grad, c->stream);
        j.done();
    });
}

int ertgb_lp_adam(float *theta, const float *grad, float *m, float *v, int64_t n, double lr, double beta1,
                  double beta2, double eps, int step, double clip, void *stream) {
    try {
        ERTGB_REQUIRE(theta && grad && m && v && n > 0, "null Adam vector");
        ERTGB_REQUIRE(step >= 1 && lr > 0.0 && beta1 >= 0.0 && beta1 < 1.0 && beta2 >= 0.0 && beta2 < 1.0,
                      "bad Adam hyper-parameters");
        static thread_local DBuf<float> scratch;
        scratch.alloc(1);
        lp_adam(theta, grad, m, v, n, lr, beta1, beta2, eps, step, clip, scratch.p, (cudaStream_t)stream);
        return ERTGB_OK;
    } catch (Error &e) {
        set_free_error(e.what());
        return e.code;
    }
}

int ertgb_lp_features(ertgb_ctx *ctx, float *x, float *f, void *stream) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        if (!c->have_S) throw Error(ERTGB_STATE, "no assembled matrices (ertgb_assemble or a response first)");
        StreamJoin j(*c, stream);
        lp_features(*c, x, f, c->stream);
        ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        j.done();
    });
}

int ertgb_batch_response(ertgb_ctx *const *ctxs, int n, const double *const *rho, double *const *rhoa,
                         ertgb_batch_info *info, void *stream) {
    try {
        ERTGB_REQUIRE(ctxs && rho && rhoa && n > 0, "empty batch");
        std::vector<Context *> cs((size_t)n);
        for (int i = 0; i < n; i++) {
            cs[i] = reinterpret_cast<Context *>(ctxs[i]);
            ERTGB_REQUIRE(cs[i] && rho[i] && rhoa[i], "null context or buffer in the batch");
            ERTGB_REQUIRE(cs[i]->device == cs[0]->device, "all problems of a batch must be on one device");
            ERTGB_REQUIRE(cs[i]->formulation == ERTGB_FORMULATION_SINGULARITY_REMOVAL,
                          "batched responses use the singularity-removal formulation");
            for (int j = 0; j < i; j++) ERTGB_REQUIRE(cs[j] != cs[i], "a context appears twice in the batch");
        }
        Context &c0 = *cs[0];
        ERTGB_CUDA(cudaSetDevice(c0.device));
        for (Context *c : cs) {
            if (c->rhs_align != 128) {
                c->rhs_align = 128;
                invalidate_derived(*c);
            }
            ensure_derived(*c);
        }
        // derived data (primary potentials, boundary terms, unit matrices) is
        // built on each context's stream; the batch runs on the first one
        for (Context *c : cs) ERTGB_CUDA(cudaStreamSynchronize(c->stream));
        StreamJoin j(c0, stream);
        cudaStream_t s = c0.stream;
        ertgb_batch_info local{};
        ertgb_batch_info *inf = info ? info : &local;
        std::memset(inf, 0, sizeof(*inf));
        ERTGB_CUDA(cudaEventRecord(c0.ev[0], s));
        for (int i = 0; i < n; i++) {
            Context &c = *cs[i];
            c.have_pot = false;
            c.stats = ertgb_stats{};
            check_rho(c, rho[i], s);
            c.d_rho_last = rho[i];
            c.d_S.alloc((size_t)c.nK * c.mesh.nnz);
            assemble_all(c, rho[i], c.d_S.p, s);
            compute_source_rho(c, rho[i], s);
            c.d_r.alloc((size_t)c.mesh.n * c.Rpad);
            build_rhs(c, s);
            compute_rhs_scale(c, s);
            c.have_S = true;
        }
        ERTGB_CUDA(cudaEventRecord(c0.ev[1], s));
        int stalled = 0;
        const int status = batch_solve(cs, s, inf, &stalled);
        inf->stalled_columns = stalled;
        ERTGB_CUDA(cudaEventRecord(c0.ev[2], s));
        for (int i = 0; i < n; i++) {
            finish_potentials(*cs[i], s);
            collect_response(*cs[i], rhoa[i], s);
        }
        ERTGB_CUDA(cudaEventRecord(c0.ev[3], s));
        ERTGB_CUDA(cudaEventSynchronize(c0.ev[3]));
        inf->ms_assemble = elapsed(c0, 0, 1);
        inf->ms_solve = elapsed(c0, 1, 2);
        inf->ms_collect = elapsed(c0, 2, 3);
        for (Context *c : cs) c->have_pot = status == ERTGB_OK;
        j.done();
        if (status != ERTGB_OK) {
            set_free_error("batched solve did not converge within max_iter");
            return status;
        }
        return ERTGB_OK;
    } catch (Error &e) {
        set_free_error(e.what());
        return e.code;
    } catch (std::exception &e) {
        set_free_error(e.what());
        return ERTGB_BAD_INPUT;
    }
}

int ertgb_cgls(const void *J, int dtype, int64_t D, int64_t P, int64_t NC, const int32_t *c_rp, const int32_t *c_ci,
               const double *c_v, const int32_t *ct_rp, const int32_t *ct_ci, const double *ct_v, const double *dW,
               const double *b, double *x, const double *wc, const double *wm, const double *tm, const double *td,
               double lambda, const double *rough, int max_iter, double tol, int32_t *iters, void *stream) {
    try {
        ERTGB_REQUIRE(J && D > 0 && P > 0 && NC >= 0 && (dtype == 0 || dtype == 1), "bad CGLS sizes or dtype");
        ERTGB_REQUIRE(dW && b && x && wm && tm && td && max_iter >= 0, "null CGLS vector");
        ERTGB_REQUIRE(NC == 0 || (c_rp && c_ci && c_v && ct_rp && ct_ci && ct_v && wc && rough),
                      "null constraint array");
        int it = 0;
        const int rc = cgls_solve(J, dtype, D, P, NC, c_rp, c_ci, c_v, ct_rp, ct_ci, ct_v, dW, b, x, wc, wm, tm, td,
                                  lambda, rough, max_iter, tol, &it, (cudaStream_t)stream);
        if (iters) *iters = it;
        if (rc != ERTGB_OK) set_free_error("CGLS produced a non-finite residual");
        return rc;
    } catch (Error &e) {
        set_free_error(e.what());
        return e.code;
    }
}

int ertgb_response_complex(ertgb_ctx *ctx, const double *rho_re, const double *rho_im, double *out_re,
                           double *out_im, void *stream) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(rho_re && rho_im && out_re && out_im, "null buffer");
        StreamJoin j(*c, stream);
        ensure_derived(*c);
        const int st = complex_response(*c, rho_re, rho_im, out_re, out_im, c->stream);
        j.done();
        if (st == ERTGB_NOT_CONVERGED) throw Error(ERTGB_NOT_CONVERGED, "complex COCG did not converge");
    });
}

int ertgb_jacobian_complex(ertgb_ctx *ctx, const double *m_re, const double *m_im, int n_model, double *J,
                           void *stream) {
    Context *c = reinterpret_cast<Context *>(ctx);
    return guard(c, [&] {
        ERTGB_REQUIRE(J, "null buffer");
        StreamJoin j(*c, stream);
        ensure_derived(*c);
        complex_jacobian(*c, m_re, m_im, n_model, J, c->stream);
        j.done();
    });
}

int ertgb_refine(int device, int dim, int mode, int64_t n_nodes, const double *xyz, const int32_t *nmark,
                 int64_t n_cells, const int32_t *cells, const int32_t *cmark, int64_t n_bnd, const int32_t *bnd,
                 const int32_t *bmark, const int32_t *bcell, ertgb_refined **out) {
    return guard_free([&] {
        ERTGB_REQUIRE(out, "null output handle");
        *out = nullptr;
        *out = reinterpret_cast<ertgb_refined *>(
            refine_mesh(device, dim, mode, n_nodes, xyz, nmark, n_cells, cells, cmark, n_bnd, bnd, bmark, bcell));
    });
}

int ertgb_refined_sizes(const ertgb_refined *r, int64_t *n_nodes, int64_t *n_cells, int64_t *nv, int64_t *n_bnd,
                        int64_t *nvb) {
    return guard_free([&] {
        ERTGB_REQUIRE(r && n_nodes && n_cells && nv && n_bnd && nvb, "null argument");
        refined_sizes(reinterpret_cast<const Refined *>(r), n_nodes, n_cells, nv, n_bnd, nvb);
    });
}

int ertgb_refined_get(const ertgb_refined *r, double *xyz, int32_t *nmark, int32_t *cells, int32_t *cmark,
                      int32_t *bnd, int32_t *bmark, int32_t *bcell) {
    return guard_free([&] {
        ERTGB_REQUIRE(r, "null refined mesh");
        refined_get(reinterpret_cast<const Refined *>(r), xyz, nmark, cells, cmark, bnd, bmark, bcell);
    });
}

int ertgb_refined_free(ertgb_refined *r) {
    refined_free(reinterpret_cast<Refined *>(r));
    return ERTGB_OK;
}

}  // extern "C"
