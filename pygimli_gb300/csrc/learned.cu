// Learned preconditioner: a message-passing network on the graph of the
// system matrix A emits the lower-triangular factor G of M^-1 = G^T G,
//
//     G_ii = exp(tanh(delta_ii)) / sqrt(A_ii),   G_ij = delta_ij / sqrt(A_jj)  (j < i),
//
// a correction of the Jacobi factor that keeps G^T G SPD for any output.  The
// solver applies G and G^T with the FSAI kernels (same lower pattern).
//
// Network (hidden 64, 4 layers): encoders h = relu(Wn x + bn), e = relu(We f
// + be); per layer z_q = W1 [h_i; h_j; e_q] + b1, m = relu(z), e += m,
// a_i = mean_{q in row i} m_q, y = W2 [h; a] + b2, h += relu(y); decoder
// delta_q = wo . e_q + bo (lower off-diagonal), delta_ii = wd . h_i + bd.
// Node (x) and edge (f) features use only the Jacobi-scaled matrix, so the
// network is blind to a common scale of A.
//
// The two GEMMs of every layer, their input-gradient GEMMs and their
// weight-gradient GEMMs run on the tensor cores (tcgen05.mma, BF16 operands
// staged in shared memory, FP32 accumulators in TMEM; umma.cuh).  Edge tiles
// hold whole matrix rows (at most 128 stored entries), so the per-row mean of
// the messages and the per-row sums of the backward pass are finished inside
// the tile without atomics.  Weight gradients are accumulated in TMEM per CTA
// and summed over CTAs in a fixed order: every result is deterministic.
//
// Training minimises Kaporin's condition number of G A G^T (exact, per
// matrix):  K = log(sum_i q_i / n) - (2/n) sum_i log G_ii,  q_i = (G A G^T)_ii.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "ertgb_internal.cuh"
#include "umma.cuh"

namespace ertgb {

namespace {

using bf16 = __nv_bfloat16;
constexpr int H = 64;
constexpr int NLAYER = 4;
constexpr float kClamp = 1.0f;
constexpr int kTile = 128;
constexpr uint32_t kWaitLimit = 1u << 22;  // mbarrier polls before a tile gives up

// flat FP32 parameter vector
constexpr int P_ENC_N_W = 0, P_ENC_N_B = 256, P_ENC_E_W = 320, P_ENC_E_B = 576, P_LAYER0 = 640;
constexpr int P_LAYER = H * 3 * H + H + H * 2 * H + H;
__host__ __device__ constexpr int p_W1(int l) { return P_LAYER0 + l * P_LAYER; }
__host__ __device__ constexpr int p_b1(int l) { return p_W1(l) + H * 3 * H; }
__host__ __device__ constexpr int p_W2(int l) { return p_b1(l) + H; }
__host__ __device__ constexpr int p_b2(int l) { return p_W2(l) + H * 2 * H; }
constexpr int P_WO = P_LAYER0 + NLAYER * P_LAYER;
constexpr int P_BO = P_WO + H, P_WD = P_BO + 1, P_BD = P_WD + H;
constexpr int NPARAM = P_BD + 1;
static_assert(NPARAM == ERTGB_LP_NPARAM, "parameter layout");
static_assert(P_ENC_E_W == P_ENC_N_B + H && P_ENC_E_B == P_ENC_E_W + 4 * H && P_LAYER0 == P_ENC_E_B + H, "layout");

// partial-gradient widths of the kernels that produce them
constexpr int W_DEC = 2 * H + 2;          // wo, bo, wd, bd
constexpr int W_NODE = H * 2 * H + H;     // W2, b2
constexpr int W_EDGE = H * 3 * H + H;     // W1, b1
constexpr int W_ENC = 2 * (4 * H + H);    // Wn, bn, We, be

// dynamic shared memory of the tcgen05 kernels (bytes)
constexpr int SM_EDGE_FWD = 128 * 192 * 2 + 64 * 192 * 2 + 128 * 65 * 4;
constexpr int SM_NODE_FWD = 128 * 128 * 2 + 64 * 128 * 2;
constexpr int SM_NODE_BWD = 128 * 64 * 2 + 128 * 64 * 2 + 128 * 128 * 2 + 64 * 128 * 2;
// sized so that at most two CTAs (2 x 256 TMEM columns) share an SM
constexpr int SM_EDGE_DX = 80 * 1024;
constexpr int SM_EDGE_DW = 128 * 128 * 2 * 2 + 64 * 128 * 2;

__device__ __forceinline__ int64_t dceil(int64_t a, int64_t b) { return (a + b - 1) / b; }
__device__ __forceinline__ int64_t dmin(int64_t a, int64_t b) { return a < b ? a : b; }

__device__ __forceinline__ uint4 pack8(const float *v) {
    uint4 r;
    __nv_bfloat162 *p = reinterpret_cast<__nv_bfloat162 *>(&r);
#pragma unroll
    for (int u = 0; u < 4; ++u) p[u] = __floats2bfloat162_rn(v[2 * u], v[2 * u + 1]);
    return r;
}
__device__ __forceinline__ void unpack8(const uint4 &r, float *v) {
    const __nv_bfloat162 *p = reinterpret_cast<const __nv_bfloat162 *>(&r);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const float2 f = __bfloat1622float2(p[u]);
        v[2 * u] = f.x;
        v[2 * u + 1] = f.y;
    }
}
__device__ __forceinline__ uint16_t bf16_bits(float v) {
    return __bfloat16_as_ushort(__float2bfloat16(v));
}
__device__ __forceinline__ float bits_float(uint16_t b) {
    return __bfloat162float(__ushort_as_bfloat16(b));
}

struct Graph {
    int64_t n, E;
    int T1;
    const int32_t *rowptr, *cols, *erow, *tile_row;
};

// ---------------------------------------------------------------- features
__global__ void k_features(int64_t n, int64_t E, int nK, const int32_t *__restrict__ rowptr,
                           const int32_t *__restrict__ cols, const int32_t *__restrict__ diag,
                           const double *__restrict__ A, float *__restrict__ x, float *__restrict__ f,
                           float *__restrict__ dsq) {
    const int64_t total = n * nK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / n;
        const int32_t i = (int32_t)(t - k * n);
        const double *Ak = A + k * E;
        const double di = Ak[diag[i]];
        const int32_t q0 = rowptr[i], q1 = rowptr[i + 1];
        double sabs = 0.0, ssum = 0.0, a2ii = 0.0;
        for (int32_t q = q0; q < q1; ++q) {
            const int32_t j = cols[q];
            const double dj = Ak[diag[j]];
            const double sij = sqrt(di * dj);
            const double ah = Ak[q] / sij;
            // (Ahat^2)_ij = sum_k A_ik A_kj / (A_kk sqrt(A_ii A_jj)): merge of rows i and j
            double s = 0.0;
            int32_t a = q0, b = rowptr[j];
            const int32_t b1 = rowptr[j + 1];
            while (a < q1 && b < b1) {
                const int32_t ca = cols[a], cb = cols[b];
                if (ca == cb) {
                    s += Ak[a] * Ak[b] / Ak[diag[ca]];
                    ++a;
                    ++b;
                } else if (ca < cb) {
                    ++a;
                } else {
                    ++b;
                }
            }
            const double a2 = s / sij;
            reinterpret_cast<float4 *>(f)[k * E + q] =
                make_float4((float)ah, (float)a2, (float)log(di / dj), j == i ? 1.f : 0.f);
            if (j == i) {
                a2ii = a2;
            } else {
                sabs += fabs(ah);
                ssum += ah;
            }
        }
        reinterpret_cast<float4 *>(x)[t] = make_float4((float)sabs, (float)(q1 - q0) / 16.f, (float)a2ii, (float)ssum);
        dsq[t] = (float)(1.0 / sqrt(di));
    }
}

// ---------------------------------------------------------------- encoders
__global__ void k_encode(int64_t nb, int64_t Eb, const float *__restrict__ x, const float *__restrict__ f,
                         const float *__restrict__ theta, uint16_t *__restrict__ h0, uint16_t *__restrict__ e0) {
    __shared__ float W[W_ENC];
    for (int i = threadIdx.x; i < W_ENC; i += blockDim.x) W[i] = theta[P_ENC_N_W + i];
    __syncthreads();
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nb + Eb; t += (int64_t)gridDim.x * blockDim.x) {
        const bool edge = t >= nb;
        const int64_t row = edge ? t - nb : t;
        const float4 in = reinterpret_cast<const float4 *>(edge ? f : x)[row];
        const float *w = W + (edge ? 5 * H : 0);
        uint16_t *out = (edge ? e0 : h0) + row * H;
        for (int c = 0; c < 8; ++c) {
            float v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int o = c * 8 + u;
                const float p = w[4 * H + o] + w[4 * o] * in.x + w[4 * o + 1] * in.y + w[4 * o + 2] * in.z +
                                w[4 * o + 3] * in.w;
                v[u] = fmaxf(p, 0.f);
            }
            reinterpret_cast<uint4 *>(out)[c] = pack8(v);
        }
    }
}

// stage rows [0, R) x K of a row-major FP32 weight matrix W (ld = K) as a
// bf16 B operand (N = R rows, K-major)
__device__ void stage_weight(unsigned char *sB, const float *__restrict__ W, int R, int K) {
    for (int idx = threadIdx.x; idx < R * (K / 8); idx += blockDim.x) {
        const int r = idx / (K / 8), c = idx % (K / 8);
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = W[(int64_t)r * K + c * 8 + u];
        *reinterpret_cast<uint4 *>(sB + umma::kmajor_chunk(r, c, K)) = pack8(v);
    }
}
// stage the transpose of a row-major FP32 matrix W (Rw x Kw): B operand with
// N = Kw rows and K = Rw, element (n, k) = W[k][n]
__device__ void stage_weight_t(unsigned char *sB, const float *__restrict__ W, int Rw, int Kw) {
    for (int idx = threadIdx.x; idx < Kw * (Rw / 8); idx += blockDim.x) {
        const int nrow = idx % Kw, c = idx / Kw;
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = W[(int64_t)(c * 8 + u) * Kw + nrow];
        *reinterpret_cast<uint4 *>(sB + umma::kmajor_chunk(nrow, c, Rw)) = pack8(v);
    }
}

// Common prologue / epilogue of the persistent tcgen05 kernels.
struct TC {
    uint64_t *mbar;
    uint32_t *tbase;
    uint32_t phase;
    __device__ void start(uint32_t ncols) {
        if (threadIdx.x == 0) umma::mbar_init(mbar, 1);
        if (threadIdx.x < 32) umma::tmem_alloc(tbase, ncols);
        umma::fence_before();
        __syncthreads();
        umma::fence_after();
        phase = 0;
    }
    // wait for the commit of the MMAs issued by thread 0; block-uniform result
    __device__ bool wait(int *err) {
        const bool ok = umma::mbar_wait(mbar, phase, kWaitLimit);
        phase ^= 1u;
        umma::fence_after();
        const int all = __syncthreads_and(ok ? 1 : 0);
        if (!all && threadIdx.x == 0) atomicExch(err, 1);
        return all != 0;
    }
    __device__ void finish(uint32_t ncols, bool failed) {
        if (failed) umma::mbar_wait(mbar, phase ^ 1u, kWaitLimit);  // let an MMA in flight land
        umma::fence_before();
        __syncthreads();
        umma::fence_after();
        if (threadIdx.x < 32) umma::tmem_dealloc(*tbase, ncols);
    }
};

__device__ __forceinline__ void issue_barrier() {
    umma::fence_async_smem();
    umma::fence_before();
    __syncthreads();
}

// ------------------------------------------------------ edge layer (forward)
__global__ void __launch_bounds__(128) k_edge_fwd(Graph g, int nK, const float *__restrict__ theta, int layer,
                                                  const uint16_t *__restrict__ h, const uint16_t *__restrict__ e,
                                                  uint16_t *__restrict__ z_out, uint16_t *__restrict__ e_out,
                                                  uint16_t *__restrict__ a_out, int *err) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *sA = smem;
    unsigned char *sB = smem + 128 * 192 * 2;
    float *sM = reinterpret_cast<float *>(smem + 128 * 192 * 2 + 64 * 192 * 2);
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    __shared__ float sb[H];
    TC tc{&mbar, &tbase, 0};
    const int tid = threadIdx.x, warp = tid >> 5;
    stage_weight(sB, theta + p_W1(layer), H, 3 * H);
    if (tid < H) sb[tid] = theta[p_b1(layer) + tid];
    tc.start(64);
    const uint32_t tmem = tbase;
    bool failed = false;
    const int64_t ntiles = (int64_t)g.T1 * nK;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t k = t / g.T1;
        const int lt = (int)(t - k * g.T1);
        const int32_t r0 = g.tile_row[lt], r1 = g.tile_row[lt + 1];
        const int32_t q0 = g.rowptr[r0], ne = g.rowptr[r1] - q0;
        const uint16_t *hk = h + k * g.n * H;
        const uint16_t *ek = e + k * g.E * H;
        for (int idx = tid; idx < kTile * 24; idx += 128) {
            const int r = idx / 24, c = idx % 24;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (r < ne) {
                const int32_t q = q0 + r;
                const uint16_t *src = c < 8    ? hk + (int64_t)g.erow[q] * H + c * 8
                                      : c < 16 ? hk + (int64_t)g.cols[q] * H + (c - 8) * 8
                                               : ek + (int64_t)q * H + (c - 16) * 8;
                v = *reinterpret_cast<const uint4 *>(src);
            }
            *reinterpret_cast<uint4 *>(sA + umma::kmajor_chunk(r, c, 192)) = v;
        }
        issue_barrier();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, umma::smem_u32(sA), umma::smem_u32(sB), 64, 192, false);
            umma::mma_commit(&mbar);
        }
        if (!tc.wait(err)) {
            failed = true;
            break;
        }
        float v[64];
        umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), v);
        umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + 32, v + 32);
        const int r = tid;
        if (r < ne) {
            const int64_t q = k * g.E + q0 + r;
            for (int c = 0; c < 8; ++c) {
                float eo[8], zz[8], en[8];
                unpack8(*reinterpret_cast<const uint4 *>(sA + umma::kmajor_chunk(r, 16 + c, 192)), eo);
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int o = c * 8 + u;
                    zz[u] = v[o] + sb[o];
                    const float m = fmaxf(zz[u], 0.f);
                    en[u] = eo[u] + m;
                    sM[r * 65 + o] = m;
                }
                reinterpret_cast<uint4 *>(z_out + q * H)[c] = pack8(zz);
                reinterpret_cast<uint4 *>(e_out + q * H)[c] = pack8(en);
            }
        }
        __syncthreads();
        const int nr = r1 - r0;
        for (int idx = tid; idx < nr * H; idx += 128) {
            const int rr = idx >> 6, o = idx & 63;
            const int32_t a0 = g.rowptr[r0 + rr] - q0, a1 = g.rowptr[r0 + rr + 1] - q0;
            float s = 0.f;
            for (int qq = a0; qq < a1; ++qq) s += sM[qq * 65 + o];
            a_out[(k * g.n + r0 + rr) * H + o] = bf16_bits(s / (float)(a1 - a0));
        }
        umma::fence_before();
        __syncthreads();
    }
    tc.finish(64, failed);
}

// ------------------------------------------------------ node layer (forward)
__global__ void __launch_bounds__(128) k_node_fwd(int64_t nb, const float *__restrict__ theta, int layer,
                                                  const uint16_t *__restrict__ h, const uint16_t *__restrict__ a,
                                                  uint16_t *__restrict__ y_out, uint16_t *__restrict__ h_out,
                                                  int *err) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *sA = smem;
    unsigned char *sB = smem + 128 * 128 * 2;
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    __shared__ float sb[H];
    TC tc{&mbar, &tbase, 0};
    const int tid = threadIdx.x, warp = tid >> 5;
    stage_weight(sB, theta + p_W2(layer), H, 2 * H);
    if (tid < H) sb[tid] = theta[p_b2(layer) + tid];
    tc.start(64);
    const uint32_t tmem = tbase;
    bool failed = false;
    const int64_t ntiles = dceil(nb, kTile);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t base = t * kTile;
        for (int idx = tid; idx < kTile * 16; idx += 128) {
            const int r = idx / 16, c = idx % 16;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (base + r < nb)
                v = *reinterpret_cast<const uint4 *>((c < 8 ? h : a) + (base + r) * H + (c & 7) * 8);
            *reinterpret_cast<uint4 *>(sA + umma::kmajor_chunk(r, c, 128)) = v;
        }
        issue_barrier();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, umma::smem_u32(sA), umma::smem_u32(sB), 64, 128, false);
            umma::mma_commit(&mbar);
        }
        if (!tc.wait(err)) {
            failed = true;
            break;
        }
        float v[64];
        umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), v);
        umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + 32, v + 32);
        const int64_t node = base + tid;
        if (node < nb) {
            for (int c = 0; c < 8; ++c) {
                float ho[8], yy[8], hn[8];
                unpack8(*reinterpret_cast<const uint4 *>(sA + umma::kmajor_chunk(tid, c, 128)), ho);
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int o = c * 8 + u;
                    yy[u] = v[o] + sb[o];
                    hn[u] = ho[u] + fmaxf(yy[u], 0.f);
                }
                reinterpret_cast<uint4 *>(y_out + node * H)[c] = pack8(yy);
                reinterpret_cast<uint4 *>(h_out + node * H)[c] = pack8(hn);
            }
        }
        umma::fence_before();
        __syncthreads();
    }
    tc.finish(64, failed);
}

// ---------------------------------------------------------------- decoder
__global__ void k_decode(int64_t n, int nK, int64_t E, int64_t nL, const int32_t *__restrict__ rowptr,
                         const int32_t *__restrict__ Lrowptr, const int32_t *__restrict__ cols,
                         const int32_t *__restrict__ LtoU, const float *__restrict__ theta,
                         const uint16_t *__restrict__ hL, const uint16_t *__restrict__ eL,
                         const float *__restrict__ dsq, float *__restrict__ delta, float *__restrict__ G32,
                         float *__restrict__ GT32) {
    __shared__ float W[W_DEC];
    for (int i = threadIdx.x; i < W_DEC; i += blockDim.x) W[i] = theta[P_WO + i];
    __syncthreads();
    const int64_t total = n * nK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / n;
        const int32_t i = (int32_t)(t - k * n);
        const int32_t p0 = Lrowptr[i], p1 = Lrowptr[i + 1], qb = rowptr[i];
        for (int32_t p = p0; p < p1; ++p) {
            const int32_t q = qb + (p - p0);
            const int32_t j = cols[q];
            const bool dg = j == i;
            const uint4 *src = reinterpret_cast<const uint4 *>(dg ? hL + t * H : eL + (k * E + q) * H);
            const float *w = dg ? W + H + 1 : W;
            float d = dg ? W[2 * H + 1] : W[H];
            for (int c = 0; c < 8; ++c) {
                float v[8];
                unpack8(src[c], v);
#pragma unroll
                for (int u = 0; u < 8; ++u) d += w[c * 8 + u] * v[u];
            }
            const float G = dg ? expf(kClamp * tanhf(d)) * dsq[t] : d * dsq[k * n + j];
            delta[k * nL + p] = d;
            if (G32) G32[k * nL + p] = G;
            if (GT32) GT32[k * nL + LtoU[p]] = G;
        }
    }
}

// ------------------------------------------------------------ Kaporin loss
// q_i = sum_{a,b in S_i} G_ia A_ab G_ib with S_i the lower pattern of row i;
// gA[p] = (A g_i)_a for every entry p = (i, a).  One block row per matrix.
__global__ void k_kap_row(int64_t n, int64_t E, int64_t nL, const int32_t *__restrict__ rowptr,
                          const int32_t *__restrict__ cols, const int32_t *__restrict__ Lrowptr,
                          const int32_t *__restrict__ Lcol, const double *__restrict__ A,
                          const float *__restrict__ G, double *__restrict__ gA, double *__restrict__ part) {
    __shared__ double red[2][256];
    const int64_t k = blockIdx.y;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double qi = 0.0, lg = 0.0;
    if (i < n) {
        const double *Ak = A + k * E;
        const float *Gk = G + k * nL;
        const int32_t p0 = Lrowptr[i], p1 = Lrowptr[i + 1];
        for (int32_t pa = p0; pa < p1; ++pa) {
            const int32_t arow = Lcol[pa];
            double s = 0.0;
            int32_t qa = rowptr[arow], pb = p0;
            const int32_t qa1 = rowptr[arow + 1];
            while (qa < qa1 && pb < p1) {
                const int32_t ca = cols[qa], cb = Lcol[pb];
                if (ca == cb) {
                    s += Ak[qa] * (double)Gk[pb];
                    ++qa;
                    ++pb;
                } else if (ca < cb) {
                    ++qa;
                } else {
                    ++pb;
                }
            }
            gA[k * nL + pa] = s;
            qi += (double)Gk[pa] * s;
        }
        lg = log((double)Gk[p1 - 1]);
    }
    red[0][threadIdx.x] = qi;
    red[1][threadIdx.x] = lg;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            red[0][threadIdx.x] += red[0][threadIdx.x + w];
            red[1][threadIdx.x] += red[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[(k * gridDim.x + blockIdx.x) * 2] = red[0][0];
        part[(k * gridDim.x + blockIdx.x) * 2 + 1] = red[1][0];
    }
}

// Q_k = sum_i q_i per matrix and the mean loss over the matrices
__global__ void k_kap_finish(int64_t n, int nK, int nblk, const double *__restrict__ part, double *__restrict__ Q,
                             double *__restrict__ loss) {
    __shared__ double sl[64];
    double acc = 0.0;
    for (int k = threadIdx.x; k < nK; k += blockDim.x) {
        double q = 0.0, lg = 0.0;
        for (int b = 0; b < nblk; ++b) {
            q += part[((int64_t)k * nblk + b) * 2];
            lg += part[((int64_t)k * nblk + b) * 2 + 1];
        }
        Q[k] = q;
        acc += log(q / (double)n) - 2.0 * lg / (double)n;
    }
    sl[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < (int)blockDim.x; ++i) s += sl[i];
        *loss = s / (double)nK;
    }
}

// dK/dG -> d delta, the decoder's input gradients (de_L, dh_L)
__global__ void k_kap_grad(int64_t n, int nK, int64_t E, int64_t nL, const int32_t *__restrict__ rowptr,
                           const int32_t *__restrict__ Lrowptr, const int32_t *__restrict__ cols,
                           const float *__restrict__ theta, const float *__restrict__ G, const float *__restrict__ delta,
                           const double *__restrict__ gA, const double *__restrict__ Q, const float *__restrict__ dsq,
                           float *__restrict__ ddelta, float *__restrict__ deL, float *__restrict__ dhL) {
    __shared__ float wo[H], wd[H];
    if (threadIdx.x < H) {
        wo[threadIdx.x] = theta[P_WO + threadIdx.x];
        wd[threadIdx.x] = theta[P_WD + threadIdx.x];
    }
    __syncthreads();
    const int64_t total = n * nK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / n;
        const int32_t i = (int32_t)(t - k * n);
        const int32_t p0 = Lrowptr[i], p1 = Lrowptr[i + 1], q0 = rowptr[i], q1 = rowptr[i + 1];
        const double inv_nk = 1.0 / (double)nK;
        const float Gii = G[k * nL + p1 - 1];
        for (int32_t q = q0; q < q1; ++q) {
            const int32_t p = p0 + (q - q0);
            float *dst = deL + (k * E + q) * H;
            if (p < p1 - 1) {
                const int32_t j = cols[q];
                const double dG = (2.0 * gA[k * nL + p] / Q[k]) * inv_nk;
                const float dd = (float)dG * dsq[k * n + j];
                ddelta[k * nL + p] = dd;
                for (int o = 0; o < H; o += 4)
                    *reinterpret_cast<float4 *>(dst + o) =
                        make_float4(dd * wo[o], dd * wo[o + 1], dd * wo[o + 2], dd * wo[o + 3]);
            } else {
                if (p == p1 - 1) {
                    const double dG =
                        (2.0 * gA[k * nL + p] / Q[k] - 2.0 / ((double)n * (double)Gii)) * inv_nk;
                    const float th = tanhf(delta[k * nL + p]);
                    const float dd = (float)dG * Gii * kClamp * (1.f - th * th);
                    ddelta[k * nL + p] = dd;
                    float *dh = dhL + t * H;
                    for (int o = 0; o < H; o += 4)
                        *reinterpret_cast<float4 *>(dh + o) =
                            make_float4(dd * wd[o], dd * wd[o + 1], dd * wd[o + 2], dd * wd[o + 3]);
                }
                for (int o = 0; o < H; o += 4) *reinterpret_cast<float4 *>(dst + o) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    }
}

// decoder weight gradients: 64 threads (one per feature) over a chunk of rows
__global__ void k_dec_wgrad(int64_t n, int nK, int64_t E, int64_t nL, const int32_t *__restrict__ rowptr,
                            const int32_t *__restrict__ Lrowptr, const uint16_t *__restrict__ hL,
                            const uint16_t *__restrict__ eL, const float *__restrict__ ddelta,
                            float *__restrict__ part) {
    const int o = threadIdx.x;
    const int64_t total = n * nK;
    const int64_t chunk = dceil(total, gridDim.x);
    const int64_t t0 = blockIdx.x * chunk, t1 = dmin(total, t0 + chunk);
    float gwo = 0.f, gbo = 0.f, gwd = 0.f, gbd = 0.f;
    for (int64_t t = t0; t < t1; ++t) {
        const int64_t k = t / n;
        const int32_t i = (int32_t)(t - k * n);
        const int32_t p0 = Lrowptr[i], p1 = Lrowptr[i + 1], qb = rowptr[i];
        for (int32_t p = p0; p < p1 - 1; ++p) {
            const float dd = ddelta[k * nL + p];
            gwo += dd * bits_float(eL[(k * E + qb + (p - p0)) * H + o]);
            gbo += dd;
        }
        const float dd = ddelta[k * nL + p1 - 1];
        gwd += dd * bits_float(hL[t * H + o]);
        gbd += dd;
    }
    float *dst = part + (int64_t)blockIdx.x * W_DEC;
    dst[o] = gwo;
    dst[H + 1 + o] = gwd;
    if (o == 0) {
        dst[H] = gbo;
        dst[2 * H + 1] = gbd;
    }
}

// ------------------------------------------------------ node layer (backward)
// dy = dh o [y > 0];  [dh_h; da] = dy W2;  dW2^T += [h; a]^T dy;  db2 += sum dy
__global__ void __launch_bounds__(128) k_node_bwd(int64_t nb, const float *__restrict__ theta, int layer,
                                                  const float *__restrict__ dh_in, const uint16_t *__restrict__ y,
                                                  const uint16_t *__restrict__ h, const uint16_t *__restrict__ a,
                                                  float *__restrict__ dh_mid, float *__restrict__ da,
                                                  float *__restrict__ part, int *err) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *sDy = smem;                       // 128 nodes x 64 (A of dX)
    unsigned char *sW2T = sDy + 128 * 64 * 2;        // 128 x 64      (B of dX)
    unsigned char *sYT = sW2T + 128 * 64 * 2;        // 128 feat x 128 nodes (A of dW)
    unsigned char *sDyT = sYT + 128 * 128 * 2;       // 64 x 128 nodes (B of dW)
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    TC tc{&mbar, &tbase, 0};
    const int tid = threadIdx.x, warp = tid >> 5;
    stage_weight_t(sW2T, theta + p_W2(layer), H, 2 * H);
    tc.start(256);
    const uint32_t tmem = tbase;
    bool failed = false, first = true;
    float db = 0.f;
    const int64_t ntiles = dceil(nb, kTile);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t node = t * kTile + tid;
        const bool valid = node < nb;
        for (int c = 0; c < 8; ++c) {
            float dy[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (valid) {
                float yy[8];
                unpack8(reinterpret_cast<const uint4 *>(y + node * H)[c], yy);
                const float4 g0 = reinterpret_cast<const float4 *>(dh_in + node * H)[2 * c];
                const float4 g1 = reinterpret_cast<const float4 *>(dh_in + node * H)[2 * c + 1];
                const float gg[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
#pragma unroll
                for (int u = 0; u < 8; ++u) dy[u] = yy[u] > 0.f ? gg[u] : 0.f;
            }
            const uint4 pk = pack8(dy);
            *reinterpret_cast<uint4 *>(sDy + umma::kmajor_chunk(tid, c, 64)) = pk;
            const uint16_t *bits = reinterpret_cast<const uint16_t *>(&pk);
#pragma unroll
            for (int u = 0; u < 8; ++u)
                *reinterpret_cast<uint16_t *>(sDyT + umma::kmajor_offset(c * 8 + u, tid, 128)) = bits[u];
        }
        for (int c = 0; c < 16; ++c) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (valid) v = reinterpret_cast<const uint4 *>((c < 8 ? h : a) + node * H)[c & 7];
            const uint16_t *bits = reinterpret_cast<const uint16_t *>(&v);
#pragma unroll
            for (int u = 0; u < 8; ++u)
                *reinterpret_cast<uint16_t *>(sYT + umma::kmajor_offset(c * 8 + u, tid, 128)) = bits[u];
        }
        issue_barrier();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, umma::smem_u32(sDy), umma::smem_u32(sW2T), 128, 64, false);
            umma::mma_tile(tmem + 128, umma::smem_u32(sYT), umma::smem_u32(sDyT), 64, 128, !first);
            umma::mma_commit(&mbar);
        }
        first = false;
        if (!tc.wait(err)) {
            failed = true;
            break;
        }
        if (tid < H)
            for (int r = 0; r < kTile; ++r)
                db += bits_float(*reinterpret_cast<const uint16_t *>(sDyT + umma::kmajor_offset(tid, r, 128)));
        for (int c = 0; c < 4; ++c) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c * 32, v);
            if (valid) {
                if (c < 2) {
                    const float4 *src = reinterpret_cast<const float4 *>(dh_in + node * H + c * 32);
                    float4 *dst = reinterpret_cast<float4 *>(dh_mid + node * H + c * 32);
                    for (int u = 0; u < 8; ++u) {
                        const float4 s4 = src[u];
                        dst[u] = make_float4(s4.x + v[4 * u], s4.y + v[4 * u + 1], s4.z + v[4 * u + 2],
                                             s4.w + v[4 * u + 3]);
                    }
                } else {
                    float4 *dst = reinterpret_cast<float4 *>(da + node * H + (c - 2) * 32);
                    for (int u = 0; u < 8; ++u)
                        dst[u] = make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
                }
            }
        }
        umma::fence_before();
        __syncthreads();
    }
    // dW2^T partial: lane f (feature of [h; a]), columns o
    float *dst = part + (int64_t)blockIdx.x * W_NODE;
    if (!failed) {
        for (int c = 0; c < 2; ++c) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + 128 + c * 32, v);
            for (int u = 0; u < 32; ++u) dst[(c * 32 + u) * 2 * H + tid] = first ? 0.f : v[u];
        }
        if (tid < H) dst[H * 2 * H + tid] = db;
    }
    tc.finish(256, failed);
}

// ------------------------------------------------------ edge layer (backward)
// dz = (de + da_i / deg_i) o [z > 0];  dX = dz W1 -> row sums (dh_i), per-edge
// dh_j parts (gathered through the transpose later), de += dX_e
__global__ void __launch_bounds__(128) k_edge_bwd_dx(Graph g, int nK, const float *__restrict__ theta, int layer,
                                                     float *__restrict__ de, const float *__restrict__ da,
                                                     const uint16_t *__restrict__ z, uint16_t *__restrict__ dz_out,
                                                     float *__restrict__ dXj, float *__restrict__ dhrow, int *err) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *sDz = smem;                       // 128 x 64
    unsigned char *sW1T = sDz + 128 * 64 * 2;        // 192 x 64
    float *sM = reinterpret_cast<float *>(sW1T + 192 * 64 * 2);  // 128 x 65
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    TC tc{&mbar, &tbase, 0};
    const int tid = threadIdx.x, warp = tid >> 5;
    stage_weight_t(sW1T, theta + p_W1(layer), H, 3 * H);
    tc.start(256);
    const uint32_t tmem = tbase;
    bool failed = false;
    const int64_t ntiles = (int64_t)g.T1 * nK;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t k = t / g.T1;
        const int lt = (int)(t - k * g.T1);
        const int32_t r0 = g.tile_row[lt], r1 = g.tile_row[lt + 1];
        const int32_t q0 = g.rowptr[r0], ne = g.rowptr[r1] - q0;
        for (int idx = tid; idx < kTile * 8; idx += 128) {
            const int r = idx / 8, c = idx % 8;
            float dz[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (r < ne) {
                const int32_t ql = q0 + r;
                const int64_t q = k * g.E + ql;
                const int32_t i = g.erow[ql];
                const float inv = 1.f / (float)(g.rowptr[i + 1] - g.rowptr[i]);
                float zz[8];
                unpack8(reinterpret_cast<const uint4 *>(z + q * H)[c], zz);
                const float4 *dep = reinterpret_cast<const float4 *>(de + q * H + c * 8);
                const float4 *dap = reinterpret_cast<const float4 *>(da + (k * g.n + i) * H + c * 8);
                const float4 e0 = dep[0], e1 = dep[1], a0 = dap[0], a1 = dap[1];
                const float dm[8] = {e0.x + a0.x * inv, e0.y + a0.y * inv, e0.z + a0.z * inv, e0.w + a0.w * inv,
                                     e1.x + a1.x * inv, e1.y + a1.y * inv, e1.z + a1.z * inv, e1.w + a1.w * inv};
#pragma unroll
                for (int u = 0; u < 8; ++u) dz[u] = zz[u] > 0.f ? dm[u] : 0.f;
            }
            const uint4 pk = pack8(dz);
            *reinterpret_cast<uint4 *>(sDz + umma::kmajor_chunk(r, c, 64)) = pk;
            if (r < ne) reinterpret_cast<uint4 *>(dz_out + (k * g.E + q0 + r) * H)[c] = pk;
        }
        issue_barrier();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, umma::smem_u32(sDz), umma::smem_u32(sW1T), 192, 64, false);
            umma::mma_commit(&mbar);
        }
        if (!tc.wait(err)) {
            failed = true;
            break;
        }
        const int r = tid;
        const int64_t q = k * g.E + q0 + r;
        for (int c = 0; c < 6; ++c) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c * 32, v);
            if (r < ne) {
                if (c < 2) {
                    for (int u = 0; u < 32; ++u) sM[r * 65 + c * 32 + u] = v[u];
                } else if (c < 4) {
                    float4 *dst = reinterpret_cast<float4 *>(dXj + q * H + (c - 2) * 32);
                    for (int u = 0; u < 8; ++u)
                        dst[u] = make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
                } else {
                    float4 *dst = reinterpret_cast<float4 *>(de + q * H + (c - 4) * 32);
                    for (int u = 0; u < 8; ++u) {
                        const float4 s4 = dst[u];
                        dst[u] = make_float4(s4.x + v[4 * u], s4.y + v[4 * u + 1], s4.z + v[4 * u + 2],
                                             s4.w + v[4 * u + 3]);
                    }
                }
            }
        }
        __syncthreads();
        const int nr = r1 - r0;
        for (int idx = tid; idx < nr * H; idx += 128) {
            const int rr = idx >> 6, o = idx & 63;
            const int32_t a0 = g.rowptr[r0 + rr] - q0, a1 = g.rowptr[r0 + rr + 1] - q0;
            float s = 0.f;
            for (int qq = a0; qq < a1; ++qq) s += sM[qq * 65 + o];
            dhrow[(k * g.n + r0 + rr) * H + o] = s;
        }
        umma::fence_before();
        __syncthreads();
    }
    tc.finish(256, failed);
}

// dW1^T += X^T dz over the edge tiles of this CTA (features 0..127 and 128..191)
__global__ void __launch_bounds__(128) k_edge_bwd_dw(Graph g, int nK, const uint16_t *__restrict__ h,
                                                     const uint16_t *__restrict__ e, const uint16_t *__restrict__ dz,
                                                     float *__restrict__ part, int *err) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *sXlo = smem;                      // 128 feat x 128 edges
    unsigned char *sXhi = sXlo + 128 * 128 * 2;      // rows 0..63: features 128..191, rows 64..127 zero
    unsigned char *sDzT = sXhi + 128 * 128 * 2;      // 64 x 128 edges
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    TC tc{&mbar, &tbase, 0};
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int idx = tid; idx < 64 * 16; idx += 128) {
        const int r = 64 + idx / 16, c = idx % 16;
        *reinterpret_cast<uint4 *>(sXhi + umma::kmajor_chunk(r, c, 128)) = make_uint4(0, 0, 0, 0);
    }
    tc.start(128);
    const uint32_t tmem = tbase;
    bool failed = false, first = true;
    float db = 0.f;
    const int64_t ntiles = (int64_t)g.T1 * nK;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t k = t / g.T1;
        const int lt = (int)(t - k * g.T1);
        const int32_t r0 = g.tile_row[lt], r1 = g.tile_row[lt + 1];
        const int32_t q0 = g.rowptr[r0], ne = g.rowptr[r1] - q0;
        const uint16_t *hk = h + k * g.n * H;
        const uint16_t *ek = e + k * g.E * H;
        for (int idx = tid; idx < kTile * 32; idx += 128) {
            const int r = idx % kTile, c = idx / kTile;  // consecutive threads: consecutive edges
            uint4 v = make_uint4(0, 0, 0, 0);
            if (r < ne) {
                const int32_t ql = q0 + r;
                const uint16_t *src = c < 8    ? hk + (int64_t)g.erow[ql] * H + c * 8
                                      : c < 16 ? hk + (int64_t)g.cols[ql] * H + (c - 8) * 8
                                      : c < 24 ? ek + (int64_t)ql * H + (c - 16) * 8
                                               : dz + (k * g.E + ql) * H + (c - 24) * 8;
                v = *reinterpret_cast<const uint4 *>(src);
            }
            const uint16_t *bits = reinterpret_cast<const uint16_t *>(&v);
            unsigned char *dstm = c < 16 ? sXlo : (c < 24 ? sXhi : sDzT);
            const int fb = c < 16 ? c * 8 : (c < 24 ? (c - 16) * 8 : (c - 24) * 8);
#pragma unroll
            for (int u = 0; u < 8; ++u)
                *reinterpret_cast<uint16_t *>(dstm + umma::kmajor_offset(fb + u, r, 128)) = bits[u];
        }
        issue_barrier();
        if (tid == 0) {
            umma::fence_after();
            umma::mma_tile(tmem, umma::smem_u32(sXlo), umma::smem_u32(sDzT), 64, 128, !first);
            umma::mma_tile(tmem + 64, umma::smem_u32(sXhi), umma::smem_u32(sDzT), 64, 128, !first);
            umma::mma_commit(&mbar);
        }
        first = false;
        if (!tc.wait(err)) {
            failed = true;
            break;
        }
        if (tid < H)
            for (int r = 0; r < kTile; ++r)
                db += bits_float(*reinterpret_cast<const uint16_t *>(sDzT + umma::kmajor_offset(tid, r, 128)));
        umma::fence_before();
        __syncthreads();
    }
    float *dst = part + (int64_t)blockIdx.x * W_EDGE;
    if (!failed) {
        for (int c = 0; c < 4; ++c) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c * 32, v);
            const int f = c < 2 ? tid : 128 + tid;
            if (c < 2 || tid < 64)
                for (int u = 0; u < 32; ++u) dst[((c & 1) * 32 + u) * 3 * H + f] = first ? 0.f : v[u];
        }
        if (tid < H) dst[H * 3 * H + tid] = db;
    }
    tc.finish(128, failed);
}

// dh_prev_i = dh_mid_i + dhrow_i + sum_{q in row i} dXj[T(q)]
__global__ void k_gather_dh(int64_t n, int nK, int64_t E, const int32_t *__restrict__ rowptr,
                            const int32_t *__restrict__ T, const float *__restrict__ dh_mid,
                            const float *__restrict__ dhrow, const float *__restrict__ dXj, float *__restrict__ dh_out) {
    const int64_t total = n * nK * H;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / H;
        const int o = (int)(t - row * H);
        const int64_t k = row / n;
        const int32_t i = (int32_t)(row - k * n);
        float s = dh_mid[t] + dhrow[t];
        for (int32_t q = rowptr[i]; q < rowptr[i + 1]; ++q) s += dXj[(k * E + T[q]) * H + o];
        dh_out[t] = s;
    }
}

// encoder weight gradients: threads 0..63 node features, 64..127 edge features
__global__ void k_encode_bwd(int64_t nb, int64_t Eb, const float *__restrict__ x, const float *__restrict__ f,
                             const float *__restrict__ theta, const float *__restrict__ dh0,
                             const float *__restrict__ de0, float *__restrict__ part) {
    const int o = threadIdx.x & 63;
    const bool edge = threadIdx.x >= 64;
    const float *W = theta + (edge ? P_ENC_E_W : P_ENC_N_W);
    const float w0 = W[4 * o], w1 = W[4 * o + 1], w2 = W[4 * o + 2], w3 = W[4 * o + 3], bb = W[4 * H + o];
    const int64_t rows = edge ? Eb : nb;
    const float *in = edge ? f : x;
    const float *g = edge ? de0 : dh0;
    const int64_t chunk = dceil(rows, gridDim.x);
    const int64_t t0 = blockIdx.x * chunk, t1 = dmin(rows, t0 + chunk);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, ab = 0.f;
    for (int64_t r = t0; r < t1; ++r) {
        const float4 v = reinterpret_cast<const float4 *>(in)[r];
        const float pre = bb + w0 * v.x + w1 * v.y + w2 * v.z + w3 * v.w;
        if (pre > 0.f) {
            const float gg = g[r * H + o];
            a0 += gg * v.x;
            a1 += gg * v.y;
            a2 += gg * v.z;
            a3 += gg * v.w;
            ab += gg;
        }
    }
    float *dst = part + (int64_t)blockIdx.x * W_ENC + (edge ? 5 * H : 0);
    dst[4 * o] = a0;
    dst[4 * o + 1] = a1;
    dst[4 * o + 2] = a2;
    dst[4 * o + 3] = a3;
    dst[4 * H + o] = ab;
}

// out[j] = sum_b part[b][j] in block order
__global__ void k_reduce(const float *__restrict__ part, int nblk, int width, float *__restrict__ out) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < width; j += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * width + j];
        out[j] = s;
    }
}

__global__ void k_sumsq(const float *__restrict__ v, int64_t n, float *__restrict__ out) {
    __shared__ float red[1024];
    float s = 0.f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += v[i] * v[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}

__global__ void k_adam(float *__restrict__ theta, const float *__restrict__ grad, float *__restrict__ m,
                       float *__restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                       float clip, const float *__restrict__ sumsq) {
    const float gn = sqrtf(sumsq[0]);
    const float scale = (clip > 0.f && gn > clip) ? clip / gn : 1.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float g = grad[i] * scale;
        const float mi = b1 * m[i] + (1.f - b1) * g;
        const float vi = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        theta[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

int num_sms(int device) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    return v > 0 ? v : 1;
}

template <class K> void set_smem(K kernel, int bytes) {
    ERTGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

// graph of the current mesh: row of each entry, transpose map, edge tiles,
// position of each lower entry in the transposed (upper) order
void prepare_graph(Context &c) {
    LPState &L = c.lp;
    MeshData &m = c.mesh;
    if (L.graph_ready && L.n == m.n && L.E == m.nnz) return;
    const int64_t n = m.n, E = m.nnz;
    std::vector<int32_t> erow(E), T(E), tile{0};
    for (int64_t i = 0; i < n; ++i)
        for (int32_t q = m.rowptr[i]; q < m.rowptr[i + 1]; ++q) erow[q] = (int32_t)i;
    for (int64_t i = 0; i < n; ++i) {
        const int32_t deg = m.rowptr[i + 1] - m.rowptr[i];
        if (deg > kTile) throw Error(ERTGB_BAD_INPUT, "learned preconditioner: a matrix row has more than 128 entries");
        for (int32_t q = m.rowptr[i]; q < m.rowptr[i + 1]; ++q) {
            const int32_t j = m.colidx[q];
            const int32_t *b = m.colidx.data() + m.rowptr[j], *e = m.colidx.data() + m.rowptr[j + 1];
            const int32_t *pos = std::lower_bound(b, e, (int32_t)i);
            if (pos == e || *pos != i) throw Error(ERTGB_BAD_INPUT, "learned preconditioner: pattern is not symmetric");
            T[q] = (int32_t)(pos - m.colidx.data());
        }
    }
    int64_t r0 = 0;
    while (r0 < n) {
        int64_t r1 = r0, cnt = 0;
        while (r1 < n && cnt + (m.rowptr[r1 + 1] - m.rowptr[r1]) <= kTile) {
            cnt += m.rowptr[r1 + 1] - m.rowptr[r1];
            ++r1;
        }
        tile.push_back((int32_t)r1);
        r0 = r1;
    }
    const int64_t nL = (int64_t)m.Lcolidx.size();
    std::vector<int32_t> LtoU(nL);
    for (int64_t u = 0; u < nL; ++u) LtoU[m.UtoL[u]] = (int32_t)u;
    L.d_erow.upload(erow, c.stream);
    L.d_T.upload(T, c.stream);
    L.d_tile_row.upload(tile, c.stream);
    L.d_LtoU.upload(LtoU, c.stream);
    L.T1 = (int)tile.size() - 1;
    L.n = n;
    L.E = E;
    L.nL = nL;
    L.nKb = 0;
    L.train_alloc = false;
    L.graph_ready = true;
    ERTGB_CUDA(cudaStreamSynchronize(c.stream));
}

void alloc_buffers(Context &c, bool training) {
    LPState &L = c.lp;
    const int nK = c.nK;
    if (L.nKb != nK) {
        const size_t nb = (size_t)L.n * nK, Eb = (size_t)L.E * nK;
        L.x.alloc(nb * 4);
        L.f.alloc(Eb * 4);
        L.dsq.alloc(nb);
        L.delta.alloc((size_t)L.nL * nK);
        L.h.alloc((NLAYER + 1) * nb * H);
        L.e.alloc((NLAYER + 1) * Eb * H);
        L.z.alloc(NLAYER * Eb * H);
        L.a.alloc(NLAYER * nb * H);
        L.y.alloc(NLAYER * nb * H);
        L.err.alloc(1);
        L.nKb = nK;
        L.train_alloc = false;
    }
    if (training && !L.train_alloc) {
        const size_t nb = (size_t)L.n * nK, Eb = (size_t)L.E * nK;
        L.gA.alloc((size_t)L.nL * nK);
        L.kq.alloc(nK);
        L.dh0.alloc(nb * H);
        L.dh1.alloc(nb * H);
        L.da.alloc(nb * H);
        L.dhrow.alloc(nb * H);
        L.de.alloc(Eb * H);
        L.dXj.alloc(Eb * H);
        L.dz.alloc(Eb * H);
        L.ddelta.alloc((size_t)L.nL * nK);
        L.train_alloc = true;
    }
}

Graph graph_of(Context &c) {
    LPState &L = c.lp;
    return Graph{L.n, L.E, L.T1, c.mesh.d_rowptr.p, c.mesh.d_colidx.p, L.d_erow.p, L.d_tile_row.p};
}

void check_err(Context &c, cudaStream_t s) {
    int32_t e = 0;
    ERTGB_CUDA(cudaMemcpyAsync(&e, c.lp.err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    if (e) throw Error(ERTGB_CUDA_ERROR, "learned preconditioner: a tensor-core tile timed out");
}

// features, encoders, layers, decoder (G32 / GT32 may be null)
void forward_impl(Context &c, const float *theta, float *G32, float *GT32, cudaStream_t s) {
    MeshData &m = c.mesh;
    LPState &L = c.lp;
    const int nK = c.nK;
    const int64_t nb = L.n * nK, Eb = L.E * nK;
    const int sms = num_sms(c.device);
    set_smem(k_edge_fwd, SM_EDGE_FWD);
    set_smem(k_node_fwd, SM_NODE_FWD);
    L.err.zero(s);
    k_features<<<(unsigned)std::min<int64_t>(ceil_div(nb, 128), 8 * sms), 128, 0, s>>>(
        L.n, L.E, nK, m.d_rowptr.p, m.d_colidx.p, m.d_diag.p, c.d_S.p, L.x.p, L.f.p, L.dsq.p);
    ERTGB_CUDA(cudaGetLastError());
    k_encode<<<(unsigned)std::min<int64_t>(ceil_div(nb + Eb, 256), 8 * sms), 256, 0, s>>>(nb, Eb, L.x.p, L.f.p, theta,
                                                                                          L.h.p, L.e.p);
    ERTGB_CUDA(cudaGetLastError());
    const Graph g = graph_of(c);
    const int64_t etiles = (int64_t)L.T1 * nK, ntiles = ceil_div(nb, kTile);
    for (int l = 0; l < NLAYER; ++l) {
        k_edge_fwd<<<(unsigned)std::min<int64_t>(etiles, 2 * sms), 128, SM_EDGE_FWD, s>>>(
            g, nK, theta, l, L.h.p + l * nb * H, L.e.p + l * Eb * H, L.z.p + l * Eb * H, L.e.p + (l + 1) * Eb * H,
            L.a.p + l * nb * H, L.err.p);
        ERTGB_CUDA(cudaGetLastError());
        k_node_fwd<<<(unsigned)std::min<int64_t>(ntiles, 3 * sms), 128, SM_NODE_FWD, s>>>(
            nb, theta, l, L.h.p + l * nb * H, L.a.p + l * nb * H, L.y.p + l * nb * H, L.h.p + (l + 1) * nb * H,
            L.err.p);
        ERTGB_CUDA(cudaGetLastError());
    }
    k_decode<<<(unsigned)std::min<int64_t>(ceil_div(nb, 128), 8 * sms), 128, 0, s>>>(
        L.n, nK, L.E, L.nL, m.d_rowptr.p, m.d_Lrowptr.p, m.d_colidx.p, L.d_LtoU.p, theta, L.h.p + NLAYER * nb * H,
        L.e.p + NLAYER * Eb * H, L.dsq.p, L.delta.p, G32, GT32);
    ERTGB_CUDA(cudaGetLastError());
}

}  // namespace

void lp_forward(Context &c, const float *theta, cudaStream_t s) {
    prepare_graph(c);
    alloc_buffers(c, false);
    const size_t nLk = (size_t)c.lp.nL * c.nK;
    c.d_G32.alloc(nLk);
    c.d_GT32.alloc(nLk);
    forward_impl(c, theta, c.d_G32.p, c.d_GT32.p, s);
    check_err(c, s);
}

void lp_setup(Context &c, cudaStream_t s) {
    if (!c.lp.have_weights) throw Error(ERTGB_STATE, "the learned preconditioner needs weights (ertgb_set_precond_weights)");
    lp_forward(c, c.lp.d_theta.p, s);
    c.stats.launches_response += 3 + 2 * NLAYER;
}

void lp_features(Context &c, float *x, float *f, cudaStream_t s) {
    prepare_graph(c);
    alloc_buffers(c, false);
    MeshData &m = c.mesh;
    LPState &L = c.lp;
    const int64_t nb = L.n * c.nK;
    k_features<<<(unsigned)std::min<int64_t>(ceil_div(nb, 128), 8 * num_sms(c.device)), 128, 0, s>>>(
        L.n, L.E, c.nK, m.d_rowptr.p, m.d_colidx.p, m.d_diag.p, c.d_S.p, L.x.p, L.f.p, L.dsq.p);
    ERTGB_CUDA(cudaGetLastError());
    if (x) ERTGB_CUDA(cudaMemcpyAsync(x, L.x.p, nb * 4 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    if (f) ERTGB_CUDA(cudaMemcpyAsync(f, L.f.p, L.E * c.nK * 4 * sizeof(float), cudaMemcpyDeviceToDevice, s));
}

double lp_loss_grad(Context &c, const float *theta, float *grad, cudaStream_t s) {
    prepare_graph(c);
    alloc_buffers(c, true);
    MeshData &m = c.mesh;
    LPState &L = c.lp;
    const int nK = c.nK;
    const int64_t nb = L.n * nK, Eb = L.E * nK;
    const int sms = num_sms(c.device);
    const size_t nLk = (size_t)L.nL * nK;
    c.d_G32.alloc(nLk);
    c.d_GT32.alloc(nLk);
    forward_impl(c, theta, c.d_G32.p, c.d_GT32.p, s);
    // loss
    const int kb = (int)ceil_div(L.n, 256);
    L.kpart.alloc((size_t)nK * kb * 2);
    k_kap_row<<<dim3(kb, nK), 256, 0, s>>>(L.n, L.E, L.nL, m.d_rowptr.p, m.d_colidx.p, m.d_Lrowptr.p, m.d_Lcolidx.p,
                                             c.d_S.p, c.d_G32.p, L.gA.p, L.kpart.p);
    ERTGB_CUDA(cudaGetLastError());
    DBuf<double> dloss;
    dloss.alloc(1);
    k_kap_finish<<<1, 64, 0, s>>>(L.n, nK, kb, L.kpart.p, L.kq.p, dloss.p);
    ERTGB_CUDA(cudaGetLastError());
    double loss = 0.0;
    if (grad) {
        const int rows_grid = (int)std::min<int64_t>(ceil_div(nb, 128), 8 * sms);
        float *dh = L.dh0.p, *dh_alt = L.dh1.p;
        k_kap_grad<<<rows_grid, 128, 0, s>>>(L.n, nK, L.E, L.nL, m.d_rowptr.p, m.d_Lrowptr.p, m.d_colidx.p, theta,
                                             c.d_G32.p, L.delta.p, L.gA.p, L.kq.p, L.dsq.p, L.ddelta.p, L.de.p, dh);
        ERTGB_CUDA(cudaGetLastError());
        // partial buffers: the widest user
        const int g_dec = std::min<int>(2 * sms, (int)std::max<int64_t>(1, nb / 64));
        const int64_t etiles = (int64_t)L.T1 * nK, ntiles = ceil_div(nb, kTile);
        const int g_node = (int)std::min<int64_t>(ntiles, 2 * sms), g_edge = (int)std::min<int64_t>(etiles, 2 * sms);
        const int g_enc = std::min<int>(2 * sms, (int)std::max<int64_t>(1, nb / 64));
        const size_t need = std::max({(size_t)g_dec * W_DEC, (size_t)g_node * W_NODE, (size_t)g_edge * W_EDGE,
                                      (size_t)g_enc * W_ENC});
        L.wpart.alloc(std::max(need, L.wpart.n));
        k_dec_wgrad<<<g_dec, H, 0, s>>>(L.n, nK, L.E, L.nL, m.d_rowptr.p, m.d_Lrowptr.p, L.h.p + NLAYER * nb * H,
                                        L.e.p + NLAYER * Eb * H, L.ddelta.p, L.wpart.p);
        ERTGB_CUDA(cudaGetLastError());
        k_reduce<<<1, 256, 0, s>>>(L.wpart.p, g_dec, W_DEC, grad + P_WO);
        ERTGB_CUDA(cudaGetLastError());
        set_smem(k_node_bwd, SM_NODE_BWD);
        set_smem(k_edge_bwd_dx, SM_EDGE_DX);
        set_smem(k_edge_bwd_dw, SM_EDGE_DW);
        const Graph g = graph_of(c);
        for (int l = NLAYER - 1; l >= 0; --l) {
            k_node_bwd<<<g_node, 128, SM_NODE_BWD, s>>>(nb, theta, l, dh, L.y.p + l * nb * H, L.h.p + l * nb * H,
                                                        L.a.p + l * nb * H, dh_alt, L.da.p, L.wpart.p, L.err.p);
            ERTGB_CUDA(cudaGetLastError());
            k_reduce<<<(unsigned)ceil_div(W_NODE, 256), 256, 0, s>>>(L.wpart.p, g_node, W_NODE, grad + p_W2(l));
            ERTGB_CUDA(cudaGetLastError());
            k_edge_bwd_dx<<<g_edge, 128, SM_EDGE_DX, s>>>(g, nK, theta, l, L.de.p, L.da.p, L.z.p + l * Eb * H, L.dz.p,
                                                          L.dXj.p, L.dhrow.p, L.err.p);
            ERTGB_CUDA(cudaGetLastError());
            k_edge_bwd_dw<<<g_edge, 128, SM_EDGE_DW, s>>>(g, nK, L.h.p + l * nb * H, L.e.p + l * Eb * H, L.dz.p,
                                                          L.wpart.p, L.err.p);
            ERTGB_CUDA(cudaGetLastError());
            k_reduce<<<(unsigned)ceil_div(W_EDGE, 256), 256, 0, s>>>(L.wpart.p, g_edge, W_EDGE, grad + p_W1(l));
            ERTGB_CUDA(cudaGetLastError());
            k_gather_dh<<<(unsigned)std::min<int64_t>(ceil_div(nb * H, 256), 16 * sms), 256, 0, s>>>(
                L.n, nK, L.E, m.d_rowptr.p, L.d_T.p, dh_alt, L.dhrow.p, L.dXj.p, dh);
            ERTGB_CUDA(cudaGetLastError());
        }
        k_encode_bwd<<<g_enc, 128, 0, s>>>(nb, Eb, L.x.p, L.f.p, theta, dh, L.de.p, L.wpart.p);
        ERTGB_CUDA(cudaGetLastError());
        k_reduce<<<(unsigned)ceil_div(W_ENC, 256), 256, 0, s>>>(L.wpart.p, g_enc, W_ENC, grad + P_ENC_N_W);
        ERTGB_CUDA(cudaGetLastError());
    }
    ERTGB_CUDA(cudaMemcpyAsync(&loss, dloss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    check_err(c, s);
    return loss;
}

void lp_adam(float *theta, const float *grad, float *m, float *v, int64_t n, double lr, double beta1, double beta2,
             double eps, int step, double clip, float *gnorm_scratch, cudaStream_t s) {
    k_sumsq<<<1, 1024, 0, s>>>(grad, n, gnorm_scratch);
    ERTGB_CUDA(cudaGetLastError());
    const float c1 = (float)(1.0 - std::pow(beta1, step)), c2 = (float)(1.0 - std::pow(beta2, step));
    k_adam<<<(unsigned)std::min<int64_t>(ceil_div(n, 256), 1024), 256, 0, s>>>(
        theta, grad, m, v, n, (float)lr, (float)beta1, (float)beta2, (float)eps, c1, c2, (float)clip, gnorm_scratch);
    ERTGB_CUDA(cudaGetLastError());
}

}  // namespace ertgb
