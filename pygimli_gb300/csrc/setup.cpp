// Host-side setup of libertgb: CSR sparsity pattern, the conflict-free
// per-slot assembly map and the Jacobian parameter tiles.
//
// Pattern: same content and order as SparseMatrix::buildSparsityPattern
// (core/src/sparsematrix.h:966-1024): for every node the set of nodes that
// share a cell with it, diagonal included, rows and columns ascending, int32;
// with a matrix extension (complete electrode model, bypass resistors) the
// positions of its entries are merged in and its rows follow the nodes, as
// the reference's map matrix grows (dcfemmodelling.cpp:315-414, 701-708).
//
// Assembly map: for every CSR slot the list of element-matrix entries that
// land on it, cell entries first in ascending cell order, then mixed-boundary
// entries in ascending boundary order.  A gather over this list sums in the
// same order as the reference's scatter (SparseMatrix::add over cells,
// core/src/sparsematrix.cpp:247-266, then over boundaries), with no atomics.
#include <algorithm>
#include <cstring>

#include "ertgb_internal.cuh"

namespace ertgb {

void build_pattern(MeshData &m) {
    const int64_t n = m.n, nn = m.nn, C = m.C;
    const int nv = m.nv;
    // node -> cells
    std::vector<int64_t> nc_ptr(nn + 1, 0);
    for (int64_t c = 0; c < C; c++)
        for (int i = 0; i < nv; i++) nc_ptr[m.cells[c * nv + i] + 1]++;
    for (int64_t i = 0; i < nn; i++) nc_ptr[i + 1] += nc_ptr[i];
    std::vector<int32_t> nc(nc_ptr[nn]);
    {
        std::vector<int64_t> pos(nc_ptr.begin(), nc_ptr.end() - 1);
        for (int64_t c = 0; c < C; c++)
            for (int i = 0; i < nv; i++) nc[pos[m.cells[c * nv + i]]++] = (int32_t)c;
    }
    // extension entries by row
    const size_t nx = m.ext_rows.size();
    std::vector<int64_t> x_ptr(n + 1, 0);
    for (size_t q = 0; q < nx; q++) x_ptr[m.ext_rows[q] + 1]++;
    for (int64_t i = 0; i < n; i++) x_ptr[i + 1] += x_ptr[i];
    std::vector<int32_t> x_col(nx);
    {
        std::vector<int64_t> pos(x_ptr.begin(), x_ptr.end() - 1);
        for (size_t q = 0; q < nx; q++) x_col[pos[m.ext_rows[q]]++] = m.ext_cols[q];
    }
    // rows
    m.rowptr.assign(n + 1, 0);
    std::vector<int32_t> mark(n, -1);
    std::vector<int32_t> row;
    std::vector<int32_t> cols;
    cols.reserve((size_t)C * nv * 4 + nx);
    for (int64_t r = 0; r < n; r++) {
        row.clear();
        if (r < nn) {
            for (int64_t q = nc_ptr[r]; q < nc_ptr[r + 1]; q++) {
                const int32_t *cn = &m.cells[(int64_t)nc[q] * nv];
                for (int i = 0; i < nv; i++) {
                    if (mark[cn[i]] != (int32_t)r) {
                        mark[cn[i]] = (int32_t)r;
                        row.push_back(cn[i]);
                    }
                }
            }
            if (row.empty()) throw Error(ERTGB_BAD_INPUT, "mesh has a node that belongs to no cell");
        }
        for (int64_t q = x_ptr[r]; q < x_ptr[r + 1]; q++) {
            if (mark[x_col[q]] != (int32_t)r) {
                mark[x_col[q]] = (int32_t)r;
                row.push_back(x_col[q]);
            }
        }
        if (row.empty()) throw Error(ERTGB_BAD_INPUT, "extension row without entries");
        std::sort(row.begin(), row.end());
        cols.insert(cols.end(), row.begin(), row.end());
        if (cols.size() > (size_t)INT32_MAX) throw Error(ERTGB_BAD_INPUT, "matrix too large for int32 indices");
        m.rowptr[r + 1] = (int32_t)cols.size();
    }
    m.colidx.swap(cols);
    m.nnz = (int64_t)m.colidx.size();
}

namespace {
inline int32_t find_slot(const MeshData &m, int32_t r, int32_t c) {
    const int32_t *b = m.colidx.data() + m.rowptr[r];
    const int32_t *e = m.colidx.data() + m.rowptr[r + 1];
    const int32_t *it = std::lower_bound(b, e, c);
    if (it == e || *it != c) throw Error(ERTGB_BAD_INPUT, "boundary facet not part of any cell");
    return (int32_t)(it - m.colidx.data());
}
}  // namespace

// Per-slot contribution lists (host) -> cptr (nnz+1), centry.
void build_assembly_map(MeshData &m, std::vector<int32_t> &cptr, std::vector<int32_t> &centry,
                        std::vector<int32_t> &diag) {
    const int nv = m.nv, nvb = m.nvb;
    const int64_t C = m.C, B = m.B;
    if ((double)C * nv * nv + (double)B * nvb * nvb > (double)INT32_MAX)
        throw Error(ERTGB_BAD_INPUT, "mesh too large for int32 assembly entries");
    std::vector<int32_t> cell_slot((size_t)C * nv * nv);
    for (int64_t c = 0; c < C; c++) {
        const int32_t *cn = &m.cells[c * nv];
        for (int i = 0; i < nv; i++)
            for (int j = 0; j < nv; j++) cell_slot[(c * nv + i) * nv + j] = find_slot(m, cn[i], cn[j]);
    }
    std::vector<int32_t> bnd_slot((size_t)B * nvb * nvb);
    for (int64_t b = 0; b < B; b++) {
        const int32_t *bn = &m.bnd_nodes[b * nvb];
        for (int i = 0; i < nvb; i++)
            for (int j = 0; j < nvb; j++) bnd_slot[(b * nvb + i) * nvb + j] = find_slot(m, bn[i], bn[j]);
    }
    cptr.assign(m.nnz + 1, 0);
    for (int32_t s : cell_slot) cptr[s + 1]++;
    for (int32_t s : bnd_slot) cptr[s + 1]++;
    for (int64_t i = 0; i < m.nnz; i++) cptr[i + 1] += cptr[i];
    centry.assign(cptr[m.nnz], 0);
    std::vector<int32_t> pos(cptr.begin(), cptr.end() - 1);
    const int32_t nv2 = nv * nv, nvb2 = nvb * nvb;
    for (int64_t e = 0; e < C * nv2; e++) centry[pos[cell_slot[e]]++] = (int32_t)e;
    const int32_t base = (int32_t)(C * nv2);
    for (int64_t e = 0; e < B * nvb2; e++) centry[pos[bnd_slot[e]]++] = base + (int32_t)e;
    diag.resize(m.n);
    for (int64_t r = 0; r < m.n; r++) diag[r] = find_slot(m, (int32_t)r, (int32_t)r);
}

// Per-slot lists of the extension entries, each list in the order the
// entries were given, so that their sum after the domain and boundary terms
// rounds as the reference's additions into its map matrix do.
void build_extension_map(const MeshData &m, std::vector<int32_t> &ptr, std::vector<double> &val) {
    const size_t nx = m.ext_rows.size();
    ptr.assign(m.nnz + 1, 0);
    val.clear();
    if (nx == 0) return;
    std::vector<int32_t> slot(nx);
    for (size_t q = 0; q < nx; q++) {
        slot[q] = find_slot(m, m.ext_rows[q], m.ext_cols[q]);
        ptr[slot[q] + 1]++;
    }
    for (int64_t i = 0; i < m.nnz; i++) ptr[i + 1] += ptr[i];
    val.assign(nx, 0.0);
    std::vector<int32_t> pos(ptr.begin(), ptr.end() - 1);
    for (size_t q = 0; q < nx; q++) val[pos[slot[q]]++] = m.ext_vals[q];
}

// Lower-triangular pattern of A (the FSAI factor G) and its transpose:
//   L: rows of A restricted to columns <= row (diagonal last), with the A slot
//      of every entry;
//   U: the transpose of L (row j lists the rows i >= j that have column j),
//      with the L slot of every entry, so G^T values are a gather of G.
void build_lower_pattern(MeshData &m) {
    const int64_t n = m.n;
    m.Lrowptr.assign(n + 1, 0);
    m.Lcolidx.clear();
    m.LtoA.clear();
    for (int64_t r = 0; r < n; r++) {
        for (int32_t s = m.rowptr[r]; s < m.rowptr[r + 1]; s++) {
            if (m.colidx[s] <= r) {
                m.Lcolidx.push_back(m.colidx[s]);
                m.LtoA.push_back(s);
            }
        }
        m.Lrowptr[r + 1] = (int32_t)m.Lcolidx.size();
    }
    const int64_t nL = (int64_t)m.Lcolidx.size();
    m.Urowptr.assign(n + 1, 0);
    for (int64_t q = 0; q < nL; q++) m.Urowptr[m.Lcolidx[q] + 1]++;
    for (int64_t i = 0; i < n; i++) m.Urowptr[i + 1] += m.Urowptr[i];
    m.Ucolidx.assign(nL, 0);
    m.UtoL.assign(nL, 0);
    std::vector<int32_t> pos(m.Urowptr.begin(), m.Urowptr.end() - 1);
    for (int64_t r = 0; r < n; r++)
        for (int32_t q = m.Lrowptr[r]; q < m.Lrowptr[r + 1]; q++) {
            const int32_t cidx = m.Lcolidx[q];
            m.Ucolidx[pos[cidx]] = (int32_t)r;
            m.UtoL[pos[cidx]] = q;
            pos[cidx]++;
        }
}

}  // namespace ertgb
