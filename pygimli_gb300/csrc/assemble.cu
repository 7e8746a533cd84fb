// FP64 kernels of the ERT forward operator around the solve:
//   element matrices      per cell gradient (K) and mass (M) matrices
//   boundary coefficients mixed (Robin) boundary alpha per wavenumber
//   primary potentials    analytic unit-current potentials per (k, electrode)
//   assembly              S = sum_cells (M k^2 + K)/rho + sum_bnd u2 alpha/rho
//                         as a gather over the per-slot contribution lists
//   source resistivity    geometric mean of the cells at each electrode
//   SR right-hand side    b = S1 prim / rho_s - S prim, prim = rho_s u_p
//   potentials            u = x + prim
//   collect / response    electrode potential matrix, ABMN voltages,
//                         reciprocity mean apparent resistivity
//
// Reference (paths in pyGIMLi):
//   core/src/elementmatrix.cpp:683-796, 798-870, 1036-1041
//   core/src/bert/dcfemmodelling.cpp:163-228 (domain), 243-299 and 430-506
//   (mixed boundary), 2152-2296 (SR calculateK), 1697-1729 (k-sum),
//   1139-1196 (response); core/src/bert/bertMisc.cpp:186-271
//   (exactDCSolution); core/src/bert/electrode.cpp:102-197;
//   core/src/bert/datamap.cpp:57-98, 159-231.
#include <cfloat>
#include <cmath>

#include "bessel.cuh"
#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

constexpr double kTol = 1e-12;  // TOLERANCE of the reference (gimli.h)
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr int kThreads = 256;

inline unsigned grid1(int64_t n, int threads = kThreads, int64_t cap = 1 << 20) {
    int64_t g = ceil_div(n, threads);
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// ---------------------------------------------------------------- geometry
__global__ void k_element_matrices(int64_t C, int dim, const double *__restrict__ xyz,
                                   const int32_t *__restrict__ cells, double *__restrict__ K,
                                   double *__restrict__ M) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
         c += (int64_t)gridDim.x * blockDim.x) {
        if (dim == 2) {
            const int32_t *cn = cells + c * 3;
            const double x1 = xyz[3 * cn[0]], y1 = xyz[3 * cn[0] + 1];
            const double x2 = xyz[3 * cn[1]], y2 = xyz[3 * cn[1] + 1];
            const double x3 = xyz[3 * cn[2]], y3 = xyz[3 * cn[2] + 1];
            // closed form of the reference's triangle gradient matrix, J = 2 * area
            const double J = fabs((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1));
            const double a = ((x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1)) / J;
            const double b = -((x3 - x1) * (x2 - x1) + (y3 - y1) * (y2 - y1)) / J;
            const double cc = ((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1)) / J;
            double *k = K + c * 9;
            k[0] = a * 0.5 + b + cc * 0.5;
            k[3] = a * -0.5 + b * -0.5;
            k[6] = b * -0.5 + cc * -0.5;
            k[4] = a * 0.5;
            k[7] = b * 0.5;
            k[8] = cc * 0.5;
            k[1] = k[3];
            k[2] = k[6];
            k[5] = k[7];
            const double m0 = (J / 2.0) / 12.0;
            double *m = M + c * 9;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) m[i * 3 + j] = (i == j) ? 2.0 * m0 : m0;
        } else {
            const int32_t *cn = cells + c * 4;
            double p[4][3];
            for (int i = 0; i < 4; i++)
                for (int d = 0; d < 3; d++) p[i][d] = xyz[3 * cn[i] + d];
            double e1[3], e2[3], e3[3];
            for (int d = 0; d < 3; d++) {
                e1[d] = p[1][d] - p[0][d];
                e2[d] = p[2][d] - p[0][d];
                e3[d] = p[3][d] - p[0][d];
            }
            // gradients of the barycentric coordinates: rows of inv([e1 e2 e3])
            double g[4][3];
            const double c23[3] = {e2[1] * e3[2] - e2[2] * e3[1], e2[2] * e3[0] - e2[0] * e3[2],
                                   e2[0] * e3[1] - e2[1] * e3[0]};
            const double c31[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2],
                                   e3[0] * e1[1] - e3[1] * e1[0]};
            const double c12[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                   e1[0] * e2[1] - e1[1] * e2[0]};
            const double det = e1[0] * c23[0] + e1[1] * c23[1] + e1[2] * c23[2];
            for (int d = 0; d < 3; d++) {
                g[1][d] = c23[d] / det;
                g[2][d] = c31[d] / det;
                g[3][d] = c12[d] / det;
                g[0][d] = -(g[1][d] + g[2][d] + g[3][d]);
            }
            const double V = fabs(det) / 6.0;
            double *k = K + c * 16;
            double *m = M + c * 16;
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) {
                    k[i * 4 + j] = V * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
                    m[i * 4 + j] = (i == j) ? 2.0 * (V / 20.0) : (V / 20.0);
                }
        }
    }
}

// ------------------------------------------------------- quadratic cells
// Quadrature in barycentric coordinates, weights summing to 1 (multiplied by
// the cell size).  Gradient products of P2 functions are quadratic: the
// degree-2 rules are exact (tetrahedron: 4 points, a = (5 + 3 sqrt 5)/20,
// b = (5 - sqrt 5)/20; triangle: the three edge midpoints).  Products of P2
// functions are quartic: Keast's 11-point tetrahedron rule and the 6-point
// Dunavant triangle rule are exact for degree 4.  The reference integrates
// with the same degrees (core/src/integration.cpp:302-440, used by
// core/src/elementmatrix.cpp:780-781 and 1043-1096), so both agree to rounding.
__device__ inline void p2_shape(int dim, const double *l, double *N) {
    if (dim == 3) {
        for (int i = 0; i < 4; i++) N[i] = l[i] * (2.0 * l[i] - 1.0);
        N[4] = 4.0 * l[0] * l[1];
        N[5] = 4.0 * l[0] * l[2];
        N[6] = 4.0 * l[0] * l[3];
        N[7] = 4.0 * l[1] * l[2];
        N[8] = 4.0 * l[2] * l[3];
        N[9] = 4.0 * l[3] * l[1];
    } else {
        for (int i = 0; i < 3; i++) N[i] = l[i] * (2.0 * l[i] - 1.0);
        N[3] = 4.0 * l[0] * l[1];
        N[4] = 4.0 * l[1] * l[2];
        N[5] = 4.0 * l[2] * l[0];
    }
}

// gradients of the P2 functions at l given the barycentric gradients g[k][3]
__device__ inline void p2_grad(int dim, const double *l, const double (*g)[3], double (*dN)[3]) {
    const int nvx = dim + 1;
    for (int i = 0; i < nvx; i++)
        for (int d = 0; d < 3; d++) dN[i][d] = (4.0 * l[i] - 1.0) * g[i][d];
    const int e3[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {2, 3}, {3, 1}};
    const int e2[3][2] = {{0, 1}, {1, 2}, {2, 0}};
    const int ne = dim == 3 ? 6 : 3;
    for (int e = 0; e < ne; e++) {
        const int a = dim == 3 ? e3[e][0] : e2[e][0], b = dim == 3 ? e3[e][1] : e2[e][1];
        for (int d = 0; d < 3; d++) dN[nvx + e][d] = 4.0 * (l[b] * g[a][d] + l[a] * g[b][d]);
    }
}

__global__ void k_element_matrices_p2(int64_t C, int dim, const double *__restrict__ xyz,
                                      const int32_t *__restrict__ cells, double *__restrict__ K,
                                      double *__restrict__ M) {
    const int nv = dim == 3 ? 10 : 6, nvx = dim + 1;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x) {
        const int32_t *cn = cells + c * nv;
        double g[4][3] = {{0}};
        double V;
        if (dim == 3) {
            double p[4][3];
            for (int i = 0; i < 4; i++)
                for (int d = 0; d < 3; d++) p[i][d] = xyz[3 * cn[i] + d];
            double e1[3], e2[3], e3[3];
            for (int d = 0; d < 3; d++) {
                e1[d] = p[1][d] - p[0][d];
                e2[d] = p[2][d] - p[0][d];
                e3[d] = p[3][d] - p[0][d];
            }
            const double c23[3] = {e2[1] * e3[2] - e2[2] * e3[1], e2[2] * e3[0] - e2[0] * e3[2], e2[0] * e3[1] - e2[1] * e3[0]};
            const double c31[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
            const double c12[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            const double det = e1[0] * c23[0] + e1[1] * c23[1] + e1[2] * c23[2];
            for (int d = 0; d < 3; d++) {
                g[1][d] = c23[d] / det;
                g[2][d] = c31[d] / det;
                g[3][d] = c12[d] / det;
                g[0][d] = -(g[1][d] + g[2][d] + g[3][d]);
            }
            V = fabs(det) / 6.0;
        } else {
            const double x1 = xyz[3 * cn[0]], y1 = xyz[3 * cn[0] + 1];
            const double x2 = xyz[3 * cn[1]], y2 = xyz[3 * cn[1] + 1];
            const double x3 = xyz[3 * cn[2]], y3 = xyz[3 * cn[2] + 1];
            const double det = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
            g[1][0] = (y3 - y1) / det;
            g[1][1] = -(x3 - x1) / det;
            g[2][0] = -(y2 - y1) / det;
            g[2][1] = (x2 - x1) / det;
            g[0][0] = -(g[1][0] + g[2][0]);
            g[0][1] = -(g[1][1] + g[2][1]);
            V = fabs(det) / 2.0;
        }
        double Kc[10][10] = {{0}}, Mc[10][10] = {{0}};
        double l[4], N[10], dN[10][3];
        // stiffness: degree-2 rule
        const int nq2 = dim == 3 ? 4 : 3;
        for (int q = 0; q < nq2; q++) {
            if (dim == 3) {
                const double a = 0.58541019662496845446, b = 0.13819660112501051518;
                for (int i = 0; i < 4; i++) l[i] = (i == q) ? a : b;
            } else {
                l[0] = l[1] = l[2] = 0.5;
                l[q] = 0.0;
            }
            p2_grad(dim, l, g, dN);
            const double wq = 1.0 / nq2;
            for (int i = 0; i < nv; i++)
                for (int j = 0; j < nv; j++)
                    Kc[i][j] += wq * (dN[i][0] * dN[j][0] + dN[i][1] * dN[j][1] + dN[i][2] * dN[j][2]);
        }
        // mass: degree-4 rule
        if (dim == 3) {
            const double sq = sqrt(5.0 / 14.0);
            const double ca = (1.0 + sq) / 4.0, cb = (1.0 - sq) / 4.0;
            const int pairs[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
            for (int q = 0; q < 11; q++) {
                double wq;
                if (q == 0) {
                    l[0] = l[1] = l[2] = l[3] = 0.25;
                    wq = -74.0 / 5625.0 * 6.0;
                } else if (q < 5) {
                    for (int i = 0; i < 4; i++) l[i] = (i == q - 1) ? 11.0 / 14.0 : 1.0 / 14.0;
                    wq = 343.0 / 45000.0 * 6.0;
                } else {
                    for (int i = 0; i < 4; i++) l[i] = cb;
                    l[pairs[q - 5][0]] = ca;
                    l[pairs[q - 5][1]] = ca;
                    wq = 56.0 / 2250.0 * 6.0;
                }
                p2_shape(3, l, N);
                for (int i = 0; i < nv; i++)
                    for (int j = 0; j < nv; j++) Mc[i][j] += wq * N[i] * N[j];
            }
        } else {
            const double A1 = 0.816847572980458513080, B1 = 0.091576213509770743460;
            const double A2 = 0.108103018168070227360, B2 = 0.445948490915964886320;
            const double W1 = 0.109951743655321868504, W2 = 0.223381589678011464830;
            for (int q = 0; q < 6; q++) {
                const double a = q < 3 ? A1 : A2, b = q < 3 ? B1 : B2;
                for (int i = 0; i < 3; i++) l[i] = (i == q % 3) ? a : b;
                p2_shape(2, l, N);
                const double wq = q < 3 ? W1 : W2;
                for (int i = 0; i < nv; i++)
                    for (int j = 0; j < nv; j++) Mc[i][j] += wq * N[i] * N[j];
            }
        }
        double *kk = K + c * nv * nv;
        double *mm = M + c * nv * nv;
        for (int i = 0; i < nv; i++)
            for (int j = 0; j < nv; j++) {
                kk[i * nv + j] = V * Kc[i][j];
                mm[i * nv + j] = V * Mc[i][j];
            }
        (void)nvx;
    }
}

__global__ void k_boundary_geometry(int64_t B, int dim, const double *__restrict__ xyz,
                                    const int32_t *__restrict__ bnd, double *__restrict__ mass,
                                    double *__restrict__ center, double *__restrict__ normal, int nvb) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < B;
         b += (int64_t)gridDim.x * blockDim.x) {
        if (nvb == 3 && dim == 2) {
            // Edge3 (nodes v0, v1, midpoint): exact mass L/30 [4 -1 2; -1 4 2; 2 2 16]
            const int32_t *bn = bnd + b * 3;
            const double tx = xyz[3 * bn[1]] - xyz[3 * bn[0]], ty = xyz[3 * bn[1] + 1] - xyz[3 * bn[0] + 1];
            const double L = sqrt(tx * tx + ty * ty);
            const double m30[9] = {4, -1, 2, -1, 4, 2, 2, 2, 16};
            for (int i = 0; i < 9; i++) mass[b * 9 + i] = L / 30.0 * m30[i];
            for (int d = 0; d < 3; d++)
                center[b * 3 + d] = (xyz[3 * bn[0] + d] + xyz[3 * bn[1] + d] + xyz[3 * bn[2] + d]) / 3.0;
            normal[b * 3 + 0] = ty / L;
            normal[b * 3 + 1] = -tx / L;
            normal[b * 3 + 2] = 0.0;
        } else if (nvb == 6) {
            // Triangle6 face: 6-point degree-4 rule on the P2 functions
            const int32_t *bn = bnd + b * 6;
            double p[3][3];
            for (int i = 0; i < 3; i++)
                for (int d = 0; d < 3; d++) p[i][d] = xyz[3 * bn[i] + d];
            const double u[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
            const double v[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
            const double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
            const double nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            const double A = 0.5 * nl;
            const double A1 = 0.816847572980458513080, B1 = 0.091576213509770743460;
            const double A2 = 0.108103018168070227360, B2 = 0.445948490915964886320;
            const double W1 = 0.109951743655321868504, W2 = 0.223381589678011464830;
            double Mf[6][6] = {{0}};
            double l[3], N[6];
            for (int q = 0; q < 6; q++) {
                const double a = q < 3 ? A1 : A2, bb = q < 3 ? B1 : B2;
                for (int i = 0; i < 3; i++) l[i] = (i == q % 3) ? a : bb;
                p2_shape(2, l, N);
                const double wq = q < 3 ? W1 : W2;
                for (int i = 0; i < 6; i++)
                    for (int j = 0; j < 6; j++) Mf[i][j] += wq * N[i] * N[j];
            }
            for (int i = 0; i < 6; i++)
                for (int j = 0; j < 6; j++) mass[b * 36 + i * 6 + j] = A * Mf[i][j];
            for (int d = 0; d < 3; d++) {
                double sum = 0.0;
                for (int i = 0; i < 6; i++) sum += xyz[3 * bn[i] + d];
                center[b * 3 + d] = sum / 6.0;
                normal[b * 3 + d] = n[d] / nl;
            }
        } else if (dim == 2) {
            const int32_t *bn = bnd + b * 2;
            const double x0 = xyz[3 * bn[0]], y0 = xyz[3 * bn[0] + 1], z0 = xyz[3 * bn[0] + 2];
            const double x1 = xyz[3 * bn[1]], y1 = xyz[3 * bn[1] + 1], z1 = xyz[3 * bn[1] + 2];
            const double tx = x1 - x0, ty = y1 - y0;
            const double L = sqrt(tx * tx + ty * ty + (z1 - z0) * (z1 - z0));
            const double m0 = L / 6.0;
            mass[b * 4 + 0] = 2.0 * m0;
            mass[b * 4 + 1] = m0;
            mass[b * 4 + 2] = m0;
            mass[b * 4 + 3] = 2.0 * m0;
            center[b * 3 + 0] = (x0 + x1) / 2.0;
            center[b * 3 + 1] = (y0 + y1) / 2.0;
            center[b * 3 + 2] = (z0 + z1) / 2.0;
            const double tl = sqrt(tx * tx + ty * ty);
            normal[b * 3 + 0] = ty / tl;
            normal[b * 3 + 1] = -tx / tl;
            normal[b * 3 + 2] = 0.0;
        } else {
            const int32_t *bn = bnd + b * 3;
            double p[3][3];
            for (int i = 0; i < 3; i++)
                for (int d = 0; d < 3; d++) p[i][d] = xyz[3 * bn[i] + d];
            const double u[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
            const double v[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
            const double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
            const double nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            const double m0 = (0.5 * nl) / 12.0;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) mass[b * 9 + i * 3 + j] = (i == j) ? 2.0 * m0 : m0;
            for (int d = 0; d < 3; d++) {
                center[b * 3 + d] = (p[0][d] + p[1][d] + p[2][d]) / 3.0;
                normal[b * 3 + d] = n[d] / nl;
            }
        }
    }
}

// mixedBoundaryCondition: mirror source through the plane 0 on axis dim-1
// (y for k > 0, z for k == 0), source = mean electrode position.
__global__ void k_boundary_alpha(int64_t B, int nK, const double *__restrict__ kv, double sx, double sy,
                                 double sz, const double *__restrict__ center,
                                 const double *__restrict__ normal, double *__restrict__ alpha) {
    const int64_t total = B * nK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int ki = (int)(t / B);
        const int64_t b = t - (int64_t)ki * B;
        const double k = kv[ki];
        double src[3] = {sx, sy, sz};
        double mir[3] = {sx, sy, sz};
        const int ax = (k > 0.0) ? 1 : 2;
        mir[ax] = 2.0 * 0.0 - src[ax];
        double r[3], rm[3];
        for (int d = 0; d < 3; d++) {
            r[d] = src[d] - center[b * 3 + d];
            rm[d] = mir[d] - center[b * 3 + d];
        }
        const double ra = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        const double rma = sqrt(rm[0] * rm[0] + rm[1] * rm[1] + rm[2] * rm[2]);
        const double *n = normal + b * 3;
        const double rn = fabs(r[0] * n[0] + r[1] * n[1] + r[2] * n[2]);
        const double rmn = fabs(rm[0] * n[0] + rm[1] * n[1] + rm[2] * n[2]);
        double res;
        if (k == 0.0) {
            res = ((rma * rma) * rn / ra + (ra * ra) * rmn / rma) / (rma * ra * (ra + rma));
        } else {
            const double k0a = as_k0(ra * k), k0m = as_k0(rma * k);
            if (fabs(k0a) < kTol || fabs(k0m) < kTol) {
                res = 0.0;
            } else {
                res = k * (rn / ra * as_k1(ra * k) + rmn / rma * as_k1(rma * k)) / (k0a + k0m);
            }
        }
        alpha[(int64_t)ki * B + b] = res;
    }
}

// Unit-current half-space potential at node (vx, vy, vz) of a source at s
// whose node is snode (exactDCSolution with the singular value at that node,
// radius mr).
__device__ double unit_potential(int64_t node, double vx, double vy, double vz, const double *s, int64_t snode,
                                 double mr, double k, double surface_z, int fullspace) {
    if (node == snode) return (k > 0.0) ? as_k0(mr / 6.0 * k) / kPi : 1.0 / (2.0 * kPi * mr / 2.0);
    const double dx = vx - s[0], dy = vy - s[1], dz = vz - s[2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    if (r < kTol) return 0.0;
    const int ax = (k > 0.0) ? 1 : 2;
    double m[3] = {s[0], s[1], s[2]};
    m[ax] = 2.0 * surface_z - s[ax];
    if (fullspace) return (k == 0.0) ? 1.0 / (4.0 * kPi * r) : as_k0(r * k) / (2.0 * kPi);
    const double mx = vx - m[0], my = vy - m[1], mz = vz - m[2];
    const double rm = sqrt(mx * mx + my * my + mz * mz);
    if (k == 0.0) return (1.0 / r + 1.0 / rm) / (4.0 * kPi);
    if (m[0] == s[0] && m[1] == s[1] && m[2] == s[2]) return as_k0(r * k) / kPi;
    return (as_k0(r * k) + as_k0(rm * k)) / (2.0 * kPi);
}

// Where the current returns: electrode ref_e (>= 0), else a node (rnode >= 0,
// at rpos with singular radius rmr), else nowhere (infinity).
struct RefSource {
    int ref_e;
    int64_t rnode;
    double rpos[3];
    double rmr;
};

// Primary potential of the unit-current pattern of column t = k*nE + e at
// every node: the source at electrode e minus the reference electrode's
// (checkPrimpotentials_, core/src/bert/dcfemmodelling.cpp:2085-2090).
__global__ void k_primary(int64_t n, int nE, int nK, int64_t Rpad, const double *__restrict__ xyz,
                          const double *__restrict__ epos, const int32_t *__restrict__ enode,
                          const double *__restrict__ emin_r, const double *__restrict__ kv,
                          double surface_z, int fullspace, RefSource ref, double *__restrict__ up) {
    const int64_t R = (int64_t)nE * nK;
    const int64_t total = n * Rpad;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t node = idx / Rpad;
        const int64_t t = idx - node * Rpad;
        if (t >= R) {
            up[idx] = 0.0;
            continue;
        }
        const int ki = (int)(t / nE);
        const int e = (int)(t - (int64_t)ki * nE);
        const double k = kv[ki];
        const double vx = xyz[3 * node], vy = xyz[3 * node + 1], vz = xyz[3 * node + 2];
        double val = unit_potential(node, vx, vy, vz, epos + 3 * e, enode[e], emin_r[e], k, surface_z, fullspace);
        if (ref.ref_e >= 0)
            val -= unit_potential(node, vx, vy, vz, epos + 3 * ref.ref_e, enode[ref.ref_e], emin_r[ref.ref_e], k,
                                  surface_z, fullspace);
        else if (ref.rnode >= 0)
            val -= unit_potential(node, vx, vy, vz, ref.rpos, ref.rnode, ref.rmr, k, surface_z, fullspace);
        up[idx] = val;
    }
}

// ---------------------------------------------------------------- assembly
// One thread per (slot, wavenumber).  Contributions are summed in the
// reference's order: cells ascending, then mixed boundaries ascending.
// 1/rho per cell (0 for a cell whose |rho| <= kTol, which adds nothing): one
// FP64 division per cell instead of one per element entry in k_assemble
__global__ void k_inv_rho(int64_t C, const double *__restrict__ rho, double *__restrict__ inv) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
         c += (int64_t)gridDim.x * blockDim.x) {
        const double r = rho[c];
        inv[c] = fabs(r) > kTol ? 1.0 / r : 0.0;
    }
}

__global__ void k_assemble(int64_t nnz, const int32_t *__restrict__ cptr, const int32_t *__restrict__ centry,
                           const double *__restrict__ K, const double *__restrict__ M,
                           const double *__restrict__ bmass, const double *__restrict__ alpha,
                           const int32_t *__restrict__ bcell, const double *__restrict__ rho,
                           const double *__restrict__ inv_rho,
                           const double *__restrict__ kv, int nv2, int nvb2, int64_t C, int64_t B,
                           const int32_t *__restrict__ xptr, const double *__restrict__ xval,
                           double *__restrict__ vals) {
    const int ki = blockIdx.y;
    const double k = kv[ki];
    const double kk = k * k;
    const int64_t cbase = C * nv2;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nnz;
         s += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        const int32_t q1 = cptr[s + 1];
        for (int32_t q = cptr[s]; q < q1; q++) {
            const int64_t e = centry[q];
            if (e < cbase) {
                const double ir = inv_rho ? inv_rho[e / nv2] : 1.0;
                const double se = (k > 0.0) ? M[e] * kk + K[e] : K[e];
                acc += ir * se;
            } else {
                const int64_t eb = e - cbase;
                const int64_t b = eb / nvb2;
                const double r = rho ? rho[bcell[b]] : 1.0;
                acc += (alpha[(int64_t)ki * B + b] / r) * bmass[eb];
            }
        }
        if (xptr) {  // constant extension (CEM, bypass), in the order given
            const int32_t x1 = xptr[s + 1];
            for (int32_t q = xptr[s]; q < x1; q++) acc += xval[q];
        }
        vals[(int64_t)ki * nnz + s] = acc;
    }
}

__global__ void k_dinv(int64_t n, int nK, int64_t nnz, const int32_t *__restrict__ diag,
                       const double *__restrict__ vals, double *__restrict__ dinv) {
    const int64_t total = n * nK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ki = t / n, r = t - ki * n;
        dinv[t] = 1.0 / vals[ki * nnz + diag[r]];
    }
}

__device__ double geo_mean(const int32_t *__restrict__ lst, int a, int b, const double *__restrict__ rho) {
    double s = 0.0;
    for (int q = a; q < b; q++) s += log(rho[lst[q]]);
    return exp(s / (double)(b - a));
}

// Source resistivity of electrode e's pattern: the geometric mean of the
// cells around the electrode, averaged with the reference electrode's
// (electrode ref_e, or the nrc cells around the reference node) over those
// above the tolerance (calculateK, core/src/bert/dcfemmodelling.cpp:2236-2266).
__global__ void k_source_rho(int nE, const int32_t *__restrict__ ptr, const int32_t *__restrict__ ecell,
                             const double *__restrict__ rho, int ref_e, const int32_t *__restrict__ rcell, int nrc,
                             double *__restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
    double rs = geo_mean(ecell, ptr[e], ptr[e + 1], rho);
    if (ref_e >= 0 || nrc > 0) {
        const double rr = ref_e >= 0 ? geo_mean(ecell, ptr[ref_e], ptr[ref_e + 1], rho) : geo_mean(rcell, 0, nrc, rho);
        double sum = 0.0;
        int cnt = 0;
        if (rs > kTol) sum += rs, cnt++;
        if (rr > kTol) sum += rr, cnt++;
        if (cnt) rs = sum / cnt;
    }
    out[e] = rs;
}

__global__ void k_check_rho(int64_t C, const double *__restrict__ rho, int32_t *__restrict__ bad) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
         c += (int64_t)gridDim.x * blockDim.x) {
        const double r = rho[c];
        if (!(r >= kTol) || isinf(r)) atomicAdd(bad, 1);
    }
}

// SR right-hand side, one warp per row, lanes over columns t = k*nE + e:
// b = (S1 prim) / rho_s - S prim with prim = rho_s * u_p.
__global__ void k_rhs(int64_t n, int64_t nnz, int nE, int64_t R, int64_t Rpad,
                      const int32_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
                      const double *__restrict__ S, const double *__restrict__ S1,
                      const double *__restrict__ up, const double *__restrict__ rhos,
                      double *__restrict__ b) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = warp; row < n; row += nwarps) {
        const int32_t s0 = rowptr[row], s1 = rowptr[row + 1];
        for (int64_t t = lane; t < Rpad; t += 32) {
            double out = 0.0;
            if (t < R) {
                const int64_t ki = t / nE;
                const int e = (int)(t - ki * nE);
                const double rs = rhos[e];
                const double *Sk = S + ki * nnz;
                const double *S1k = S1 + ki * nnz;
                double a1 = 0.0, a2 = 0.0;
                for (int32_t s = s0; s < s1; s++) {
                    const double prim = up[(int64_t)colidx[s] * Rpad + t] * rs;
                    a1 += S1k[s] * prim;
                    a2 += Sk[s] * prim;
                }
                out = a1 / rs - a2;
            }
            b[row * Rpad + t] = out;
        }
    }
}

// column partials of ||S1 u_p / rho_s||^2 = ||S1 up||^2 (rho_s cancels): block
// (32, 8) over (columns, rows), partial row per blockIdx.y
__global__ void k_pnorm_part(int64_t n, int64_t nnz, int nE, int64_t R, int64_t Rpad,
                             const int32_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
                             const double *__restrict__ S1, const double *__restrict__ up, double *__restrict__ part) {
    __shared__ double red[8][32];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    double acc = 0.0;
    if (t < R) {
        const double *S1k = S1 + (t / nE) * nnz;
        for (int64_t row = (int64_t)blockIdx.y * 8 + threadIdx.y; row < n; row += (int64_t)gridDim.y * 8) {
            double a = 0.0;
            for (int32_t s = rowptr[row]; s < rowptr[row + 1]; s++) a += S1k[s] * up[(int64_t)colidx[s] * Rpad + t];
            acc = fma(a, a, acc);
        }
    }
    red[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; w++) s += red[w][threadIdx.x];
        part[(int64_t)blockIdx.y * Rpad + t] = s;
    }
}

__global__ void k_pnorm_sum(int64_t Rpad, int NB, const double *__restrict__ part, double *__restrict__ out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= Rpad) return;
    double s = 0.0;
    for (int b = 0; b < NB; b++) s += part[(int64_t)b * Rpad + t];
    out[t] = s;
}

__global__ void k_finish_pot(int64_t n, int nE, int64_t R, int64_t Rpad, const double *__restrict__ up,
                             const double *__restrict__ rhos, double *__restrict__ x) {
    const int64_t total = n * Rpad;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = idx % Rpad;
        if (t < R) {
            const int e = (int)(t % nE);
            x[idx] += up[idx] * rhos[e];
        }
    }
}

// U[e][f] = sum_k w_k u_k[e](node of electrode f), summed like the
// reference's k loop (first term a product, then accumulate).
// last_k: the last wavenumber's potential, unweighted (the complete
// electrode model's collect, core/src/bert/dcfemmodelling.cpp:1829, 1912).
// U[e][f]: potential at electrode f for the source at electrode e, the
// k-summed solution at f's rows weighted by f's weights (a node electrode: its
// row with weight 1; an electrode inside a cell: the cell's shape functions
// there, ElectrodeShapeEntity::pot, core/src/bert/electrode.cpp:273-275)
__global__ void k_collect(int nE, int nK, int64_t Rpad, const int32_t *__restrict__ ew_ptr,
                          const int32_t *__restrict__ ew_row, const double *__restrict__ ew_w,
                          const double *__restrict__ w, const double *__restrict__ x,
                          double *__restrict__ U, int last_k) {
    const int64_t total = (int64_t)nE * nE;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t / nE), f = (int)(t % nE);
        double u = 0.0;
        for (int q = ew_ptr[f]; q < ew_ptr[f + 1]; q++) {
            const double *row = x + (int64_t)ew_row[q] * Rpad;
            double acc;
            if (last_k) {
                acc = row[(int64_t)(nK - 1) * nE + e];
            } else {
                acc = row[e] * w[0];
                for (int ki = 1; ki < nK; ki++) acc += row[(int64_t)ki * nE + e] * w[ki];
            }
            u = q == ew_ptr[f] ? ew_w[q] * acc : fma(ew_w[q], acc, u);
        }
        U[t] = u;
    }
}

// Total potential: column t = k * nE + e carries a unit current at electrode
// e: its source row (ElectrodeShapeNode / ElectrodeShapeDomain::assembleRHS,
// core/src/bert/electrode.cpp:133-150, 341-355) or the shape functions of
// the cell holding it (ElectrodeShapeEntity::assembleRHS, 278-290), and the
// reference electrode's rows with the weights negated (calculateK_,
// core/src/bert/dcfemmodelling.cpp:1862-1864); b is zeroed before.
__global__ void k_rhs_total(int nE, int64_t R, int64_t Rpad, const int32_t *__restrict__ ew_ptr,
                            const int32_t *__restrict__ ew_row, const double *__restrict__ ew_w, int n_sink,
                            const int32_t *__restrict__ sink_row, const double *__restrict__ sink_w,
                            double *__restrict__ b) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= R) return;
    const int e = (int)(t % nE);
    for (int q = ew_ptr[e]; q < ew_ptr[e + 1]; q++) b[(int64_t)ew_row[q] * Rpad + t] += ew_w[q];
    for (int q = 0; q < n_sink; q++) b[(int64_t)sink_row[q] * Rpad + t] -= sink_w[q];
}

// Homogeneous Dirichlet rows (assembleStiffnessMatrixHomogenDirichletBC,
// core/src/bert/dcfemmodelling.cpp:141-154): on a fixed row every entry 0
// but the diagonal 1, on a fixed column every entry 0; one warp per row.
__global__ void k_clean_fixed(int64_t n, int nK, int64_t nnz, const int32_t *__restrict__ rowptr,
                              const int32_t *__restrict__ colidx, const uint8_t *__restrict__ fixed,
                              double *__restrict__ vals) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = warp; row < n; row += nwarps) {
        const bool fr = fixed[row] != 0;
        for (int32_t q = rowptr[row] + lane; q < rowptr[row + 1]; q += 32) {
            const int32_t col = colidx[q];
            if (!fr && !fixed[col]) continue;
            const double v = (fr && col == row) ? 1.0 : 0.0;
            for (int ki = 0; ki < nK; ki++) vals[(int64_t)ki * nnz + q] = v;
        }
    }
}

// Singularity removal: zero right-hand side on the calibration rows
// (calculateK, core/src/bert/dcfemmodelling.cpp:2281-2283).
__global__ void k_zero_rows(int n_rows, const int32_t *__restrict__ rows, int64_t Rpad, double *__restrict__ b) {
    const int64_t total = (int64_t)n_rows * Rpad;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        b[(int64_t)rows[i / Rpad] * Rpad + i % Rpad] = 0.0;
}

__device__ inline double abmn_u(const double *U, int nE, int a, int b, int m, int n) {
    double uAM = 0.0, uAN = 0.0, uBM = 0.0, uBN = 0.0;
    if (a != -1 && m != -1) uAM = U[(int64_t)a * nE + m];
    if (a != -1 && n != -1) uAN = U[(int64_t)a * nE + n];
    if (b != -1 && m != -1) uBM = U[(int64_t)b * nE + m];
    if (b != -1 && n != -1) uBN = U[(int64_t)b * nE + n];
    return (uAM - uAN) - (uBM - uBN);
}

__global__ void k_response(int64_t D, int nE, const int32_t *__restrict__ abmn, const double *__restrict__ kfac,
                           const double *__restrict__ U, double *__restrict__ rhoa) {
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < D;
         d += (int64_t)gridDim.x * blockDim.x) {
        const int a = abmn[4 * d], b = abmn[4 * d + 1], m = abmn[4 * d + 2], n = abmn[4 * d + 3];
        double r = abmn_u(U, nE, a, b, m, n);
        double rr = abmn_u(U, nE, m, n, a, b);
        r = rint(r / 1e-10) * 1e-10;
        rr = rint(rr / 1e-10) * 1e-10;
        r *= kfac[d];
        rr *= kfac[d];
        rhoa[d] = sqrt(fabs(r * rr));
    }
}

}  // namespace

// ----------------------------------------------------------------- drivers
void build_mesh_device(Context &c) {
    MeshData &m = c.mesh;
    cudaStream_t s = c.stream;
    m.d_xyz.upload(m.xyz, s);
    m.d_cells.upload(m.cells, s);
    m.d_rowptr.upload(m.rowptr, s);
    m.d_colidx.upload(m.colidx, s);
    std::vector<int32_t> cptr, centry, diag;
    build_assembly_map(m, cptr, centry, diag);
    m.d_cptr.upload(cptr, s);
    m.d_centry.upload(centry, s);
    m.d_diag.upload(diag, s);
    {
        std::vector<int32_t> xptr;
        std::vector<double> xval;
        build_extension_map(m, xptr, xval);
        if (xval.empty()) {
            m.d_ext_ptr.release();
            m.d_ext_val.release();
        } else {
            m.d_ext_ptr.upload(xptr, s);
            m.d_ext_val.upload(xval, s);
        }
    }
    build_lower_pattern(m);
    m.d_Lrowptr.upload(m.Lrowptr, s);
    m.d_Lcolidx.upload(m.Lcolidx, s);
    m.d_LtoA.upload(m.LtoA, s);
    m.d_Urowptr.upload(m.Urowptr, s);
    m.d_Ucolidx.upload(m.Ucolidx, s);
    m.d_UtoL.upload(m.UtoL, s);
    m.d_K.alloc((size_t)m.C * m.nv * m.nv);
    m.d_M.alloc((size_t)m.C * m.nv * m.nv);
    if (m.order == 1)
        k_element_matrices<<<grid1(m.C), kThreads, 0, s>>>(m.C, m.dim, m.d_xyz.p, m.d_cells.p, m.d_K.p, m.d_M.p);
    else
        k_element_matrices_p2<<<grid1(m.C, 128), 128, 0, s>>>(m.C, m.dim, m.d_xyz.p, m.d_cells.p, m.d_K.p, m.d_M.p);
    ERTGB_CUDA(cudaGetLastError());
    m.d_bnd_nodes.upload(m.bnd_nodes, s);
    m.d_bnd_cell.upload(m.bnd_cell, s);
    m.d_bnd_mass.alloc((size_t)m.B * m.nvb * m.nvb);
    m.d_bnd_center.alloc((size_t)m.B * 3);
    m.d_bnd_normal.alloc((size_t)m.B * 3);
    if (m.B) {
        k_boundary_geometry<<<grid1(m.B), kThreads, 0, s>>>(m.B, m.dim, m.d_xyz.p, m.d_bnd_nodes.p,
                                                             m.d_bnd_mass.p, m.d_bnd_center.p,
                                                             m.d_bnd_normal.p, m.nvb);
        ERTGB_CUDA(cudaGetLastError());
    }
    // host copies of large maps are not kept
    ERTGB_CUDA(cudaStreamSynchronize(s));
}

void compute_boundary_alpha(Context &c) {
    MeshData &m = c.mesh;
    c.d_alpha.alloc((size_t)std::max<int64_t>(m.B, 1) * c.nK);
    if (m.B) {
        k_boundary_alpha<<<grid1(m.B * c.nK), kThreads, 0, c.stream>>>(
            m.B, c.nK, c.d_k.p, c.src_center[0], c.src_center[1], c.src_center[2], m.d_bnd_center.p,
            m.d_bnd_normal.p, c.d_alpha.p);
        ERTGB_CUDA(cudaGetLastError());
    }
}

static RefSource ref_source(const Context &c) {
    RefSource r{};
    r.ref_e = c.ref_elec;
    r.rnode = c.ref_elec < 0 ? c.ref_node : -1;
    for (int d = 0; d < 3; d++) r.rpos[d] = c.ref_pos[d];
    r.rmr = c.ref_minr;
    return r;
}

void compute_primary(Context &c) {
    MeshData &m = c.mesh;
    c.d_up.alloc((size_t)m.n * c.Rpad);
    const int fullspace = (c.surface_z == -DBL_MAX || std::isnan(c.surface_z)) ? 1 : 0;
    k_primary<<<grid1(m.n * c.Rpad, kThreads, 1 << 16), kThreads, 0, c.stream>>>(
        m.n, c.nE, c.nK, c.Rpad, m.d_xyz.p, c.d_epos.p, c.d_enode.p, c.d_emin_r.p, c.d_k.p, c.surface_z,
        fullspace, ref_source(c), c.d_up.p);
    ERTGB_CUDA(cudaGetLastError());
}

__global__ void k_scale(int64_t total, double f, double *__restrict__ x) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= f;
}

void analytic_potentials(Context &c, double rho, double *out) {
    MeshData &m = c.mesh;
    const int fullspace = (c.surface_z == -DBL_MAX || std::isnan(c.surface_z)) ? 1 : 0;
    const int64_t total = m.n * c.Rpad;
    k_primary<<<grid1(total, kThreads, 1 << 16), kThreads, 0, c.stream>>>(
        m.n, c.nE, c.nK, c.Rpad, m.d_xyz.p, c.d_epos.p, c.d_enode.p, c.d_emin_r.p, c.d_k.p, c.surface_z, fullspace,
        ref_source(c), out);
    ERTGB_CUDA(cudaGetLastError());
    k_scale<<<grid1(total, kThreads, 1 << 16), kThreads, 0, c.stream>>>(total, rho, out);
    ERTGB_CUDA(cudaGetLastError());
}

void build_electrode_weights(Context &c) {
    const bool total = c.formulation == ERTGB_FORMULATION_TOTAL_POTENTIAL;
    const int nv = c.mesh.nv;
    std::vector<int32_t> ptr(1, 0), row;
    std::vector<double> wt;
    for (int e = 0; e < c.nE; e++) {
        const int32_t cell = e < (int)c.ent_cell.size() ? c.ent_cell[e] : -1;
        if (cell >= 0) {
            for (int i = 0; i < nv; i++) {
                row.push_back(c.mesh.cells[(size_t)cell * nv + i]);
                wt.push_back(c.ent_w[(size_t)e * nv + i]);
            }
        } else {
            row.push_back(total ? c.src_row[e] : c.enode[e]);
            wt.push_back(1.0);
        }
        ptr.push_back((int32_t)row.size());
    }
    c.d_ew_ptr.upload(ptr, c.stream);
    c.d_ew_row.upload(row, c.stream);
    c.d_ew_w.upload(wt, c.stream);
    // the reference electrode's rows and weights (negated in the right-hand side)
    std::vector<int32_t> srow;
    std::vector<double> sw;
    if (c.ref_elec >= 0) {
        srow.assign(row.begin() + ptr[c.ref_elec], row.begin() + ptr[c.ref_elec + 1]);
        sw.assign(wt.begin() + ptr[c.ref_elec], wt.begin() + ptr[c.ref_elec + 1]);
    } else if (c.ref_node >= 0) {
        srow.push_back(c.ref_node);
        sw.push_back(1.0);
    }
    c.n_sink = (int)srow.size();
    c.d_sink_row.upload(srow, c.stream);
    c.d_sink_w.upload(sw, c.stream);
    c.d_ref_cells.upload(c.ref_cells, c.stream);
    // fixed rows: Dirichlet boundary nodes and calibration nodes
    const MeshData &m = c.mesh;
    c.have_fixed = !m.dir_nodes.empty() || !c.calib.empty();
    if (c.have_fixed) {
        std::vector<uint8_t> fixed((size_t)m.n, 0);
        for (int32_t v : m.dir_nodes) fixed[v] = 1;
        for (int32_t v : c.calib) fixed[v] = 1;
        c.d_fixed.upload(fixed, c.stream);
    } else {
        c.d_fixed.release();
    }
    c.d_calib.upload(c.calib, c.stream);
    ERTGB_CUDA(cudaStreamSynchronize(c.stream));
}

void clean_fixed_rows(Context &c, double *vals, cudaStream_t s) {
    if (!c.have_fixed) return;
    MeshData &m = c.mesh;
    k_clean_fixed<<<grid1(m.n * 32, kThreads, 1 << 14), kThreads, 0, s>>>(m.n, c.nK, m.nnz, m.d_rowptr.p,
                                                                          m.d_colidx.p, c.d_fixed.p, vals);
    ERTGB_CUDA(cudaGetLastError());
}

void upload_primary(Context &c) {
    MeshData &m = c.mesh;
    const int64_t n = m.n;
    std::vector<double> tmp((size_t)n * c.Rpad, 0.0);
    for (int ki = 0; ki < c.nK; ki++)
        for (int e = 0; e < c.nE; e++) {
            const double *src = c.up_user.data() + ((size_t)ki * c.nE + e) * n;
            const int64_t t = (int64_t)ki * c.nE + e;
            for (int64_t i = 0; i < n; i++) tmp[(size_t)i * c.Rpad + t] = src[i];
        }
    c.d_up.alloc((size_t)n * c.Rpad);
    ERTGB_CUDA(cudaMemcpyAsync(c.d_up.p, tmp.data(), sizeof(double) * tmp.size(), cudaMemcpyHostToDevice, c.stream));
    ERTGB_CUDA(cudaStreamSynchronize(c.stream));
}

void assemble_all(Context &c, const double *rho_cell, double *vals, cudaStream_t s) {
    MeshData &m = c.mesh;
    if (rho_cell) {
        c.d_inv_rho.alloc((size_t)m.C);
        k_inv_rho<<<grid1(m.C, kThreads, 4096), kThreads, 0, s>>>(m.C, rho_cell, c.d_inv_rho.p);
        ERTGB_CUDA(cudaGetLastError());
    }
    dim3 grid(grid1(m.nnz, kThreads, 1 << 16), c.nK);
    k_assemble<<<grid, kThreads, 0, s>>>(m.nnz, m.d_cptr.p, m.d_centry.p, m.d_K.p, m.d_M.p, m.d_bnd_mass.p,
                                         c.d_alpha.p, m.d_bnd_cell.p, rho_cell, rho_cell ? c.d_inv_rho.p : nullptr,
                                         c.d_k.p, m.nv * m.nv, m.nvb * m.nvb, m.C, m.B, m.d_ext_ptr.p,
                                         m.d_ext_val.p, vals);
    ERTGB_CUDA(cudaGetLastError());
    clean_fixed_rows(c, vals, s);
    if (rho_cell) {
        c.d_dinv.alloc((size_t)m.n * c.nK);
        k_dinv<<<grid1(m.n * c.nK), kThreads, 0, s>>>(m.n, c.nK, m.nnz, m.d_diag.p, vals, c.d_dinv.p);
        ERTGB_CUDA(cudaGetLastError());
    }
}

void assemble_unit(Context &c, cudaStream_t s) {
    c.d_S1.alloc((size_t)c.nK * c.mesh.nnz);
    assemble_all(c, nullptr, c.d_S1.p, s);
}

void check_rho(Context &c, const double *rho_cell, cudaStream_t s) {
    DBuf<int32_t> bad;
    bad.alloc(1);
    bad.zero(s);
    k_check_rho<<<grid1(c.mesh.C, kThreads, 4096), kThreads, 0, s>>>(c.mesh.C, rho_cell, bad.p);
    ERTGB_CUDA(cudaGetLastError());
    int32_t h = 0;
    ERTGB_CUDA(cudaMemcpyAsync(&h, bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    if (h) throw Error(ERTGB_BAD_INPUT, "response for model with negative or zero resistivity is not defined (" +
                                            std::to_string(h) + " cells)");
}

void compute_source_rho(Context &c, const double *rho_cell, cudaStream_t s) {
    c.d_rhos.alloc(c.nE);
    const int nrc = c.ref_elec < 0 && c.ref_node >= 0 ? (int)c.ref_cells.size() : 0;
    k_source_rho<<<(unsigned)ceil_div(c.nE, 128), 128, 0, s>>>(c.nE, c.d_ecell_ptr.p, c.d_ecell.p, rho_cell,
                                                              c.ref_elec, c.d_ref_cells.p, nrc, c.d_rhos.p);
    ERTGB_CUDA(cudaGetLastError());
}

void build_rhs(Context &c, cudaStream_t s) {
    MeshData &m = c.mesh;
    k_rhs<<<grid1(m.n * 32, kThreads, 1 << 16), kThreads, 0, s>>>(m.n, m.nnz, c.nE, c.R, c.Rpad, m.d_rowptr.p,
                                                                  m.d_colidx.p, c.d_S.p, c.d_S1.p, c.d_up.p,
                                                                  c.d_rhos.p, c.d_r.p);
    ERTGB_CUDA(cudaGetLastError());
    if (!c.calib.empty()) {
        k_zero_rows<<<grid1((int64_t)c.calib.size() * c.Rpad), kThreads, 0, s>>>((int)c.calib.size(), c.d_calib.p,
                                                                                 c.Rpad, c.d_r.p);
        ERTGB_CUDA(cudaGetLastError());
    }
}

void build_rhs_total(Context &c, cudaStream_t s) {
    MeshData &m = c.mesh;
    ERTGB_CUDA(cudaMemsetAsync(c.d_r.p, 0, sizeof(double) * (size_t)m.n * c.Rpad, s));
    k_rhs_total<<<(unsigned)ceil_div(c.R, kThreads), kThreads, 0, s>>>(c.nE, c.R, c.Rpad, c.d_ew_ptr.p, c.d_ew_row.p,
                                                                       c.d_ew_w.p, c.n_sink, c.d_sink_row.p,
                                                                       c.d_sink_w.p, c.d_r.p);
    ERTGB_CUDA(cudaGetLastError());
    c.d_pnorm2.release();  // no primary field: the reference norm is ||b||
}

void compute_rhs_scale(Context &c, cudaStream_t s) {
    MeshData &m = c.mesh;
    const int NB = (int)std::min<int64_t>(ceil_div(m.n, 8), 256);
    DBuf<double> part;
    part.alloc((size_t)NB * c.Rpad);
    c.d_pnorm2.alloc((size_t)c.Rpad);
    k_pnorm_part<<<dim3((unsigned)(c.Rpad / 32), (unsigned)NB), dim3(32, 8), 0, s>>>(
        m.n, m.nnz, c.nE, c.R, c.Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S1.p, c.d_up.p, part.p);
    k_pnorm_sum<<<(unsigned)ceil_div(c.Rpad, 128), 128, 0, s>>>(c.Rpad, NB, part.p, c.d_pnorm2.p);
    ERTGB_CUDA(cudaGetLastError());
    ERTGB_CUDA(cudaStreamSynchronize(s));
}

void finish_potentials(Context &c, cudaStream_t s) {
    MeshData &m = c.mesh;
    k_finish_pot<<<grid1(m.n * c.Rpad, kThreads, 1 << 16), kThreads, 0, s>>>(m.n, c.nE, c.R, c.Rpad, c.d_up.p,
                                                                             c.d_rhos.p, c.d_x.p);
    ERTGB_CUDA(cudaGetLastError());
}

void collect_potentials(Context &c, cudaStream_t s) {
    c.d_U.alloc((size_t)c.nE * c.nE);
    const bool total = c.formulation == ERTGB_FORMULATION_TOTAL_POTENTIAL;
    k_collect<<<grid1((int64_t)c.nE * c.nE), kThreads, 0, s>>>(c.nE, c.nK, c.Rpad, c.d_ew_ptr.p, c.d_ew_row.p,
                                                               c.d_ew_w.p, c.d_w.p, c.d_x.p, c.d_U.p,
                                                               total && c.collect_last_k ? 1 : 0);
    ERTGB_CUDA(cudaGetLastError());
}

void collect_response(Context &c, double *rhoa, cudaStream_t s) {
    collect_potentials(c, s);
    k_response<<<grid1(c.D), kThreads, 0, s>>>(c.D, c.nE, c.d_abmn.p, c.d_kfac.p, c.d_U.p, rhoa);
    ERTGB_CUDA(cudaGetLastError());
}

void profile_assemble(Context &c, int reps, double *ms, double *bytes, double *flops) {
    MeshData &m = c.mesh;
    if (c.d_S.n < (size_t)c.nK * m.nnz || !c.d_rho_last) throw Error(ERTGB_STATE, "profile needs a completed response");
    cudaStream_t s = c.stream;
    dim3 grid(grid1(m.nnz, kThreads, 1 << 16), c.nK);
    c.d_inv_rho.alloc((size_t)m.C);
    k_inv_rho<<<grid1(m.C, kThreads, 4096), kThreads, 0, s>>>(m.C, c.d_rho_last, c.d_inv_rho.p);
    ERTGB_CUDA(cudaGetLastError());
    auto go = [&] {
        k_assemble<<<grid, kThreads, 0, s>>>(m.nnz, m.d_cptr.p, m.d_centry.p, m.d_K.p, m.d_M.p, m.d_bnd_mass.p,
                                             c.d_alpha.p, m.d_bnd_cell.p, c.d_rho_last, c.d_inv_rho.p, c.d_k.p,
                                             m.nv * m.nv, m.nvb * m.nvb, m.C, m.B, m.d_ext_ptr.p, m.d_ext_val.p,
                                             c.d_S.p);
    };
    go();
    ERTGB_CUDA(cudaEventRecord(c.ev[0], s));
    for (int r = 0; r < reps; r++) go();
    ERTGB_CUDA(cudaEventRecord(c.ev[1], s));
    ERTGB_CUDA(cudaEventSynchronize(c.ev[1]));
    float t = 0.f;
    ERTGB_CUDA(cudaEventElapsedTime(&t, c.ev[0], c.ev[1]));
    *ms = (double)t / reps;
    const double entries = (double)m.C * m.nv * m.nv + (double)m.B * m.nvb * m.nvb;
    // slot lists, element values (K, and M where a wavenumber is positive: the
    // 3-D operator has k = 0 and reads K alone), resistivity per cell, boundary
    // terms, matrix values written per wavenumber
    bool any_k = false;
    for (double kv : c.k) any_k = any_k || kv > 0.0;
    *bytes = (double)(m.nnz + 1) * 4.0 + entries * 4.0 + (double)m.C * m.nv * m.nv * (any_k ? 16.0 : 8.0) + m.C * 8.0 +
             (double)m.B * (m.nvb * m.nvb * 8.0 + c.nK * 8.0 + 4.0) + (double)c.nK * m.nnz * 8.0;
    *flops = entries * c.nK * 3.0;
}

}  // namespace ertgb
