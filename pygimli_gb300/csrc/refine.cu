// Uniform refinement of a linear simplex mesh on the device: the quadratic
// mesh of Mesh::createP2 and the H2 mesh of Mesh::createH2 (core/src/mesh.cpp:
// 1278-1288, createRefined_ 1315-1600), with the reference's numbering.
//
// Edge slots are the cells' edges (Triangle6 / Tetrahedron10 edge order,
// cells in order), then the boundaries' edges.  Every slot's edge key
// (lo * n + hi) goes into an open-addressing hash table that keeps, per
// edge, the smallest slot using it (atomicMin: the same result whatever the
// insertion order).  A slot that is its edge's first use creates the
// midpoint node; an exclusive prefix sum of these flags in slot order gives
// the midpoint ids n + rank — the order in which createRefinementNode_
// creates them when it walks the cells and then the boundaries.  H2 then
// splits every cell into 4 / 8 children and every boundary into 2 / 4.
//
// Memory per refinement: the hash table (2^ceil(log2(2 S)) x 16 bytes for S
// slots), the slot arrays (S x 20 bytes) and the output mesh.
#include "ertgb_internal.cuh"

#include <algorithm>

namespace ertgb {
namespace {

constexpr unsigned long long kEmptyKey = ~0ull;

// edge tables: Tetrahedron10 (Zienkiewicz) and Triangle6 edge order; the
// boundary triangles' and segments' edges
__constant__ int8_t c_tet_edges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {2, 3}, {3, 1}};
__constant__ int8_t c_tri_edges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
// H2 children in Tetrahedron10 / Triangle6 node numbers (mesh.cpp:1357-1406)
__constant__ int8_t c_tet_h2[8][4] = {{4, 6, 5, 0}, {4, 5, 6, 9}, {7, 9, 4, 1}, {7, 4, 9, 5},
                                      {8, 7, 5, 2}, {8, 5, 7, 9}, {6, 9, 8, 3}, {6, 8, 9, 5}};
__constant__ int8_t c_tri_h2[4][3] = {{0, 3, 5}, {1, 4, 3}, {2, 5, 4}, {3, 4, 5}};
__constant__ int8_t c_seg_h2[2][2] = {{0, 2}, {2, 1}};

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    // splitmix64 finaliser (Steele, Lea, Flood 2014)
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

struct Slots {
    int dim;
    int64_t n0, C, B, SC, S;  // nodes, cells, boundaries, cell slots, all slots
    int E, Eb, nv, nvb;       // edges per cell / boundary, nodes per cell / boundary
};

__device__ __forceinline__ void slot_edge(const Slots &q, const int32_t *cells, const int32_t *bnd, int64_t s,
                                          int32_t &a, int32_t &b) {
    if (s < q.SC) {
        const int64_t c = s / q.E;
        const int e = (int)(s - c * q.E);
        const int ia = q.dim == 3 ? c_tet_edges[e][0] : c_tri_edges[e][0];
        const int ib = q.dim == 3 ? c_tet_edges[e][1] : c_tri_edges[e][1];
        a = cells[c * q.nv + ia];
        b = cells[c * q.nv + ib];
    } else {
        const int64_t r = s - q.SC;
        const int64_t f = r / q.Eb;
        const int e = (int)(r - f * q.Eb);
        a = bnd[f * q.nvb + c_tri_edges[e][0]];
        b = bnd[f * q.nvb + (q.dim == 3 ? c_tri_edges[e][1] : 1)];
    }
}

__device__ __forceinline__ unsigned long long edge_key(int64_t n0, int32_t a, int32_t b) {
    const unsigned long long lo = (unsigned long long)min(a, b), hi = (unsigned long long)max(a, b);
    return lo * (unsigned long long)n0 + hi;
}

// table insert: first use per edge (the probe sequence is bounded by the
// table size; the table is at least twice the slot count, so it never fills)
__global__ void k_insert(Slots q, const int32_t *__restrict__ cells, const int32_t *__restrict__ bnd,
                         unsigned long long *__restrict__ tkey, long long *__restrict__ tfirst,
                         unsigned long long mask, int32_t *__restrict__ err) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < q.S; s += (int64_t)gridDim.x * blockDim.x) {
        int32_t a, b;
        slot_edge(q, cells, bnd, s, a, b);
        const unsigned long long k = edge_key(q.n0, a, b);
        unsigned long long h = mix64(k) & mask;
        bool done = false;
        for (unsigned long long probe = 0; probe <= mask; probe++) {
            const unsigned long long prev = atomicCAS(&tkey[h], kEmptyKey, k);
            if (prev == kEmptyKey || prev == k) {
                atomicMin(&tfirst[h], (long long)s);
                done = true;
                break;
            }
            h = (h + 1) & mask;
        }
        if (!done) atomicExch(err, 1);
    }
}

// first use of every slot's edge; flag = 1 on first uses
__global__ void k_lookup(Slots q, const int32_t *__restrict__ cells, const int32_t *__restrict__ bnd,
                         const unsigned long long *__restrict__ tkey, const long long *__restrict__ tfirst,
                         unsigned long long mask, int32_t *__restrict__ first, int32_t *__restrict__ flag,
                         int32_t *__restrict__ err) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < q.S; s += (int64_t)gridDim.x * blockDim.x) {
        int32_t a, b;
        slot_edge(q, cells, bnd, s, a, b);
        const unsigned long long k = edge_key(q.n0, a, b);
        unsigned long long h = mix64(k) & mask;
        long long f = -1;
        for (unsigned long long probe = 0; probe <= mask; probe++) {
            const unsigned long long tk = tkey[h];
            if (tk == k) {
                f = tfirst[h];
                break;
            }
            if (tk == kEmptyKey) break;
            h = (h + 1) & mask;
        }
        if (f < 0) {
            atomicExch(err, 2);
            f = s;
        }
        first[s] = (int32_t)f;
        flag[s] = (f == s) ? 1 : 0;
    }
}

// exclusive scan of int32 in blocks of kScanBlock: per-block scan + block totals
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanBlock = kScanThreads * kScanPer;

__global__ void k_scan_block(int64_t n, const int32_t *__restrict__ in, int32_t *__restrict__ out,
                             int32_t *__restrict__ totals) {
    __shared__ int32_t warp_sum[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
    int32_t v[kScanPer];
    int32_t local = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; j++) {
        v[j] = (base + j < n) ? in[base + j] : 0;
        local += v[j];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
        int32_t ws = warp_sum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += y;
        }
        warp_sum[lane] = ws;  // inclusive over warps
    }
    __syncthreads();
    int32_t run = incl - local + (w > 0 ? warp_sum[w - 1] : 0);
#pragma unroll
    for (int j = 0; j < kScanPer; j++) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (threadIdx.x == kScanThreads - 1) totals[blockIdx.x] = warp_sum[31];
}

__global__ void k_scan_add(int64_t n, int32_t *__restrict__ out, const int32_t *__restrict__ offsets) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += offsets[i / kScanBlock];
}

// exclusive scan of n values (recursive over the block totals); returns the total
int32_t exclusive_scan(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    DBuf<int32_t> totals, offsets;
    totals.alloc((size_t)nb + 1);
    k_scan_block<<<(unsigned)nb, kScanThreads, 0, s>>>(n, in, out, totals.p);
    ERTGB_CUDA(cudaGetLastError());
    int32_t total = 0;
    if (nb > 1) {
        offsets.alloc((size_t)nb);
        total = exclusive_scan(totals.p, offsets.p, nb, s);
        k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, out, offsets.p);
        ERTGB_CUDA(cudaGetLastError());
        ERTGB_CUDA(cudaStreamSynchronize(s));  // before this level's buffers are freed
    } else {
        ERTGB_CUDA(cudaMemcpyAsync(&total, totals.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        ERTGB_CUDA(cudaStreamSynchronize(s));
    }
    return total;
}

__device__ __forceinline__ int32_t marker_mid(int32_t m0, int32_t m1) {
    // core/src/mesh.cpp:1293-1299
    if (m0 == -99 && m1 == -99) return -1;
    if (m0 == -99) return m1;
    if (m1 == -99) return m0;
    return m0 == m1 ? m1 : 0;
}

// new nodes (first uses) and the midpoint id of every slot
__global__ void k_midpoints(Slots q, const int32_t *__restrict__ cells, const int32_t *__restrict__ bnd,
                            const double *__restrict__ xyz, const int32_t *__restrict__ nmark,
                            const int32_t *__restrict__ first, const int32_t *__restrict__ rank,
                            double *__restrict__ xyz2, int32_t *__restrict__ nmark2, int32_t *__restrict__ mid) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < q.S; s += (int64_t)gridDim.x * blockDim.x) {
        const int32_t f = first[s];
        mid[s] = (int32_t)(q.n0 + rank[f]);
        if (f == s) {
            int32_t a, b;
            slot_edge(q, cells, bnd, s, a, b);
            const int64_t id = q.n0 + rank[s];
#pragma unroll
            for (int d = 0; d < 3; d++) xyz2[id * 3 + d] = 0.5 * (xyz[(int64_t)a * 3 + d] + xyz[(int64_t)b * 3 + d]);
            nmark2[id] = marker_mid(nmark[a], nmark[b]);
        }
    }
}

__device__ __forceinline__ int32_t full_node(const Slots &q, const int32_t *cells, const int32_t *mid, int64_t c,
                                             int i) {
    return i < q.nv ? cells[c * q.nv + i] : mid[c * q.E + (i - q.nv)];
}

__global__ void k_cells_p2(Slots q, const int32_t *__restrict__ cells, const int32_t *__restrict__ mid,
                           int32_t *__restrict__ out) {
    const int nv2 = q.nv + q.E;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < q.C; c += (int64_t)gridDim.x * blockDim.x)
        for (int i = 0; i < nv2; i++) out[c * nv2 + i] = full_node(q, cells, mid, c, i);
}

__global__ void k_cells_h2(Slots q, const int32_t *__restrict__ cells, const int32_t *__restrict__ mid,
                           const int32_t *__restrict__ marker, int32_t *__restrict__ out,
                           int32_t *__restrict__ marker2) {
    const int nch = q.dim == 3 ? 8 : 4;
    const int64_t total = q.C * nch;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = i / nch;
        const int k = (int)(i - c * nch);
        for (int j = 0; j < q.nv; j++) {
            const int loc = q.dim == 3 ? c_tet_h2[k][j] : c_tri_h2[k][j];
            out[i * q.nv + j] = full_node(q, cells, mid, c, loc);
        }
        marker2[i] = marker[c];
    }
}

__global__ void k_bnd_p2(Slots q, const int32_t *__restrict__ bnd, const int32_t *__restrict__ mid,
                         int32_t *__restrict__ out) {
    const int nvb2 = q.nvb + q.Eb;
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < q.B; f += (int64_t)gridDim.x * blockDim.x) {
        for (int i = 0; i < q.nvb; i++) out[f * nvb2 + i] = bnd[f * q.nvb + i];
        for (int e = 0; e < q.Eb; e++) out[f * nvb2 + q.nvb + e] = mid[q.SC + f * q.Eb + e];
    }
}

// H2 boundaries: 4 triangles / 2 segments per parent with its marker; the
// adjacent cell is the child of the parent boundary's cell holding the facet
__global__ void k_bnd_h2(Slots q, const int32_t *__restrict__ bnd, const int32_t *__restrict__ bmark,
                         const int32_t *__restrict__ bcell, const int32_t *__restrict__ cells2,
                         const int32_t *__restrict__ mid, int32_t *__restrict__ out, int32_t *__restrict__ bmark2,
                         int32_t *__restrict__ bcell2) {
    const int nch = q.dim == 3 ? 4 : 2;   // children per boundary
    const int cch = q.dim == 3 ? 8 : 4;   // children per cell
    const int64_t total = q.B * nch;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = i / nch;
        const int k = (int)(i - f * nch);
        int32_t node[3];
        for (int j = 0; j < q.nvb; j++) {
            const int loc = q.dim == 3 ? c_tri_h2[k][j] : c_seg_h2[k][j];
            node[j] = loc < q.nvb ? bnd[f * q.nvb + loc] : mid[q.SC + f * q.Eb + (loc - q.nvb)];
            out[i * q.nvb + j] = node[j];
        }
        bmark2[i] = bmark[f];
        const int32_t pc = bcell ? bcell[f] : -1;
        int32_t found = -1;
        if (pc >= 0 && pc < q.C) {
            for (int ch = 0; ch < cch && found < 0; ch++) {
                const int32_t *cn = cells2 + ((int64_t)pc * cch + ch) * q.nv;
                bool all = true;
                for (int j = 0; j < q.nvb; j++) {
                    bool in = false;
                    for (int v = 0; v < q.nv; v++) in |= (cn[v] == node[j]);
                    all &= in;
                }
                if (all) found = (int32_t)((int64_t)pc * cch + ch);
            }
        }
        bcell2[i] = found;
    }
}

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

}  // namespace

struct Refined {
    int device = 0, dim = 0, nv = 0, nvb = 0;
    int64_t n = 0, C = 0, B = 0;
    DBuf<double> xyz;
    DBuf<int32_t> nmark, cells, cmark, bnd, bmark, bcell;
};

Refined *refine_mesh(int device, int dim, int mode, int64_t n0, const double *xyz_h, const int32_t *nmark_h,
                     int64_t C, const int32_t *cells_h, const int32_t *cmark_h, int64_t B, const int32_t *bnd_h,
                     const int32_t *bmark_h, const int32_t *bcell_h) {
    ERTGB_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
    ERTGB_REQUIRE(mode == 1 || mode == 2, "mode must be 1 (P2) or 2 (H2)");
    ERTGB_REQUIRE(n0 > 0 && C > 0 && B >= 0 && xyz_h && nmark_h && cells_h && cmark_h, "empty mesh or null array");
    ERTGB_REQUIRE(B == 0 || (bnd_h && bmark_h), "null boundary array");
    Slots q;
    q.dim = dim;
    q.n0 = n0;
    q.C = C;
    q.B = B;
    q.nv = dim + 1;
    q.nvb = dim;
    q.E = dim == 3 ? 6 : 3;
    q.Eb = dim == 3 ? 3 : 1;
    q.SC = C * q.E;
    q.S = q.SC + B * q.Eb;
    const int nch = dim == 3 ? 8 : 4, bch = dim == 3 ? 4 : 2;
    ERTGB_REQUIRE(n0 + q.S < INT32_MAX && (mode == 1 || C * nch < INT32_MAX), "refined mesh exceeds int32 ids");
    // the kernels index only what these checks admit
    for (int64_t i = 0; i < C * q.nv; i++)
        ERTGB_REQUIRE(cells_h[i] >= 0 && cells_h[i] < n0, "cell node index out of range");
    for (int64_t i = 0; i < B * q.nvb; i++)
        ERTGB_REQUIRE(bnd_h[i] >= 0 && bnd_h[i] < n0, "boundary node index out of range");

    int prev_dev = 0;
    ERTGB_CUDA(cudaGetDevice(&prev_dev));
    ERTGB_CUDA(cudaSetDevice(device));
    struct Restore {
        int d;
        ~Restore() { cudaSetDevice(d); }
    } restore{prev_dev};
    cudaStream_t s;
    ERTGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{s};

    DBuf<double> xyz;
    DBuf<int32_t> nmark, cells, cmark, bnd, bmark, bcell;
    xyz.upload(xyz_h, (size_t)n0 * 3, s);
    nmark.upload(nmark_h, (size_t)n0, s);
    cells.upload(cells_h, (size_t)(C * q.nv), s);
    cmark.upload(cmark_h, (size_t)C, s);
    if (B) {
        bnd.upload(bnd_h, (size_t)(B * q.nvb), s);
        bmark.upload(bmark_h, (size_t)B, s);
        if (bcell_h) bcell.upload(bcell_h, (size_t)B, s);
    }

    unsigned long long tsize = 1;
    while (tsize < (unsigned long long)(2 * q.S)) tsize <<= 1;
    DBuf<unsigned long long> tkey;
    DBuf<long long> tfirst;
    DBuf<int32_t> first, flag, rank, mid, err;
    tkey.alloc(tsize);
    tfirst.alloc(tsize);
    first.alloc((size_t)q.S);
    flag.alloc((size_t)q.S);
    rank.alloc((size_t)q.S);
    mid.alloc((size_t)q.S);
    err.alloc(1);
    ERTGB_CUDA(cudaMemsetAsync(tkey.p, 0xff, tsize * sizeof(unsigned long long), s));
    ERTGB_CUDA(cudaMemsetAsync(tfirst.p, 0x7f, tsize * sizeof(long long), s));
    err.zero(s);
    const unsigned g = grid_for(q.S);
    k_insert<<<g, 256, 0, s>>>(q, cells.p, bnd.p, tkey.p, tfirst.p, tsize - 1, err.p);
    ERTGB_CUDA(cudaGetLastError());
    k_lookup<<<g, 256, 0, s>>>(q, cells.p, bnd.p, tkey.p, tfirst.p, tsize - 1, first.p, flag.p, err.p);
    ERTGB_CUDA(cudaGetLastError());
    const int32_t n_new = exclusive_scan(flag.p, rank.p, q.S, s);
    int32_t h_err = 0;
    ERTGB_CUDA(cudaMemcpyAsync(&h_err, err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    if (h_err) throw Error(ERTGB_CUDA_ERROR, "edge table probe failed");
    tkey.release();
    tfirst.release();

    std::unique_ptr<Refined> r(new Refined);
    r->device = device;
    r->dim = dim;
    r->n = n0 + n_new;
    r->xyz.alloc((size_t)r->n * 3);
    r->nmark.alloc((size_t)r->n);
    ERTGB_CUDA(cudaMemcpyAsync(r->xyz.p, xyz.p, sizeof(double) * n0 * 3, cudaMemcpyDeviceToDevice, s));
    ERTGB_CUDA(cudaMemcpyAsync(r->nmark.p, nmark.p, sizeof(int32_t) * n0, cudaMemcpyDeviceToDevice, s));
    k_midpoints<<<g, 256, 0, s>>>(q, cells.p, bnd.p, xyz.p, nmark.p, first.p, rank.p, r->xyz.p, r->nmark.p, mid.p);
    ERTGB_CUDA(cudaGetLastError());
    if (mode == 1) {
        r->nv = q.nv + q.E;
        r->nvb = q.nvb + q.Eb;
        r->C = C;
        r->B = B;
        r->cells.alloc((size_t)(C * r->nv));
        k_cells_p2<<<grid_for(C), 256, 0, s>>>(q, cells.p, mid.p, r->cells.p);
        ERTGB_CUDA(cudaGetLastError());
        r->cmark.alloc((size_t)C);
        ERTGB_CUDA(cudaMemcpyAsync(r->cmark.p, cmark.p, sizeof(int32_t) * C, cudaMemcpyDeviceToDevice, s));
        if (B) {
            r->bnd.alloc((size_t)(B * r->nvb));
            k_bnd_p2<<<grid_for(B), 256, 0, s>>>(q, bnd.p, mid.p, r->bnd.p);
            ERTGB_CUDA(cudaGetLastError());
            r->bmark.alloc((size_t)B);
            r->bcell.alloc((size_t)B);
            ERTGB_CUDA(cudaMemcpyAsync(r->bmark.p, bmark.p, sizeof(int32_t) * B, cudaMemcpyDeviceToDevice, s));
            if (bcell_h)
                ERTGB_CUDA(cudaMemcpyAsync(r->bcell.p, bcell.p, sizeof(int32_t) * B, cudaMemcpyDeviceToDevice, s));
            else
                ERTGB_CUDA(cudaMemsetAsync(r->bcell.p, 0xff, sizeof(int32_t) * B, s));
        }
    } else {
        r->nv = q.nv;
        r->nvb = q.nvb;
        r->C = C * nch;
        r->B = B * bch;
        r->cells.alloc((size_t)(r->C * r->nv));
        r->cmark.alloc((size_t)r->C);
        k_cells_h2<<<grid_for(r->C), 256, 0, s>>>(q, cells.p, mid.p, cmark.p, r->cells.p, r->cmark.p);
        ERTGB_CUDA(cudaGetLastError());
        if (B) {
            r->bnd.alloc((size_t)(r->B * r->nvb));
            r->bmark.alloc((size_t)r->B);
            r->bcell.alloc((size_t)r->B);
            k_bnd_h2<<<grid_for(r->B), 256, 0, s>>>(q, bnd.p, bmark.p, bcell_h ? bcell.p : nullptr, r->cells.p, mid.p,
                                                    r->bnd.p, r->bmark.p, r->bcell.p);
            ERTGB_CUDA(cudaGetLastError());
        }
    }
    ERTGB_CUDA(cudaStreamSynchronize(s));
    return r.release();
}

void refined_get(const Refined *r, double *xyz, int32_t *nmark, int32_t *cells, int32_t *cmark, int32_t *bnd,
                 int32_t *bmark, int32_t *bcell) {
    int prev_dev = 0;
    ERTGB_CUDA(cudaGetDevice(&prev_dev));
    ERTGB_CUDA(cudaSetDevice(r->device));
    struct Restore {
        int d;
        ~Restore() { cudaSetDevice(d); }
    } restore{prev_dev};
    auto get = [](void *dst, const void *src, size_t bytes) {
        if (dst && bytes) ERTGB_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    };
    get(xyz, r->xyz.p, sizeof(double) * r->n * 3);
    get(nmark, r->nmark.p, sizeof(int32_t) * r->n);
    get(cells, r->cells.p, sizeof(int32_t) * r->C * r->nv);
    get(cmark, r->cmark.p, sizeof(int32_t) * r->C);
    get(bnd, r->bnd.p, sizeof(int32_t) * r->B * r->nvb);
    get(bmark, r->bmark.p, sizeof(int32_t) * r->B);
    get(bcell, r->bcell.p, sizeof(int32_t) * r->B);
}

void refined_sizes(const Refined *r, int64_t *n, int64_t *C, int64_t *nv, int64_t *B, int64_t *nvb) {
    *n = r->n;
    *C = r->C;
    *nv = r->nv;
    *B = r->B;
    *nvb = r->nvb;
}

void refined_free(Refined *r) {
    if (!r) return;
    int prev_dev = 0;
    cudaGetDevice(&prev_dev);
    cudaSetDevice(r->device);
    delete r;
    cudaSetDevice(prev_dev);
}

}  // namespace ertgb
