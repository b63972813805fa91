// Curvature and the surface-tension source on the GPU, once per time step
// (SEMO calls calcSourceSurfaceTension before its outer loop,
// src/solvers/pressureBased.cpp:142).
//
// Stages (reference function, file:line):
//   k_sft_init     interface cells and the 0.5-shifted level set
//                  src/solvers/source/curvature.cpp (calcCurvature: smoothAi = VF,
//                  the face values of VF, a cell is on the interface when the 0.5
//                  level lies between it and one of its faces)
//   k_sft_norm     LSQ gradient of the level set; on interface cells with
//                  |grad|^2 > 1 the level set is divided by it; the pseudo
//                  time step tau and the sign speed vel0
//   k_sft_reinit   four sweeps of upwind-weighted least-squares
//                  re-initialisation: a 3x3 normal matrix per cell from its faces,
//                  pseudo-inverted by SVD (src/math/math.cpp:372-585, Golub-Reinsch),
//                  the level set of cells off the interface moved towards |grad| = 1
//   k_sft_normals  unit normals of the re-initialised level set (LSQ gradient)
//   k_sft_kappa    kappa = -div(n) from an unweighted stencil least squares on
//                  the normals' own components (d_q (n_jq - n_iq))
//   k_sft_source   src/solvers/source/surfaceTension.cpp:7-120: Gauss-Green
//                  gradient of VF (skew-corrected face values, the LSQ gradient of
//                  VF of the stencil pass), src = sigma kappa grad VF and
//                  sigma kappa grad VF . U
//
// Cells gather over their faces in ascending face order and over their
// stencils in stored order (the reference's accumulation order), without
// atomics.  The product path is compiled with FMA contraction, so values
// agree with the reference to rounding, not bit for bit.  Outputs (RCM order,
// planes of n_cells in c->sft): 0 kappa, 1 ls, 2-5 src (x, y, z, .U).
#include <cuda_runtime.h>

#include <cmath>

#include "face_common.cuh"
#include "semo_internal.h"

namespace {

using namespace semo::face;

// LSQ gradient of phi at cell i from its vertex stencil (w_k d_k weights in
// stw, normal-matrix inverse in minv); boundary faces contribute nothing
// (zero-gradient values: phi_b - phi_i = 0).
__device__ __forceinline__ void lsq1(int i, int nc, const int* __restrict__ stp, const int* __restrict__ sti,
                                     const double* __restrict__ stw, int64_t stn, const double* __restrict__ minv,
                                     const double* __restrict__ phi, double g[3]) {
    const double pi = phi[i];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = stp[i]; k < stp[i + 1]; ++k) {
        const double d = __ldg(phi + __ldg(sti + k)) - pi;
        s0 += __ldg(stw + k) * d;
        s1 += __ldg(stw + stn + k) * d;
        s2 += __ldg(stw + 2 * stn + k) * d;
    }
    const double m0 = minv[i], m1 = minv[nc + i], m2 = minv[2 * nc + i];
    const double m3 = minv[3 * nc + i], m4 = minv[4 * nc + i], m5 = minv[5 * nc + i];
    g[0] = m0 * s0 + m1 * s1 + m2 * s2;
    g[1] = m1 * s0 + m3 * s1 + m4 * s2;
    g[2] = m2 * s0 + m4 * s1 + m5 * s2;
}

__device__ __forceinline__ double hyp2(double a, double b) {
    const double x = fabs(a), y = fabs(b);
    if (x > y) { const double r = y / x; return x * sqrt(1.0 + r * r); }
    if (y == 0.0) return 0.0;
    const double r = x / y;
    return y * sqrt(1.0 + r * r);
}

// Singular value decomposition a = U diag(w) V^T of a 3x3 matrix
// (Householder bidiagonalisation, implicit-shift QR; Golub & Reinsch 1970),
// a replaced by U.  At most 30 QR sweeps per singular value.
__device__ void svd3(double a[3][3], double w[3], double v[3][3]) {
    const int n = 3;
    double rv1[3] = {0.0, 0.0, 0.0};
    double g = 0.0, scale = 0.0, anorm = 0.0, s, f, h, c, x, y, z;
    int l = 0, nm = 0;
    for (int i = 0; i < n; i++) {
        l = i + 1;
        rv1[i] = scale * g;
        g = s = scale = 0.0;
        for (int k = i; k < n; k++) scale += fabs(a[k][i]);
        if (scale != 0.0) {
            for (int k = i; k < n; k++) { a[k][i] /= scale; s += a[k][i] * a[k][i]; }
            f = a[i][i];
            g = (f > 0.0) ? -sqrt(s) : sqrt(s);
            h = f * g - s;
            a[i][i] = f - g;
            for (int j = l; j < n; j++) {
                s = 0.0;
                for (int k = i; k < n; k++) s += a[k][i] * a[k][j];
                f = s / h;
                for (int k = i; k < n; k++) a[k][j] += f * a[k][i];
            }
            for (int k = i; k < n; k++) a[k][i] *= scale;
        }
        w[i] = scale * g;
        g = s = scale = 0.0;
        if (i != n - 1) {
            for (int k = l; k < n; k++) scale += fabs(a[i][k]);
            if (scale != 0.0) {
                for (int k = l; k < n; k++) { a[i][k] /= scale; s += a[i][k] * a[i][k]; }
                f = a[i][l];
                g = (f > 0.0) ? -sqrt(s) : sqrt(s);
                h = f * g - s;
                a[i][l] = f - g;
                for (int k = l; k < n; k++) rv1[k] = a[i][k] / h;
                for (int j = l; j < n; j++) {
                    s = 0.0;
                    for (int k = l; k < n; k++) s += a[j][k] * a[i][k];
                    for (int k = l; k < n; k++) a[j][k] += s * rv1[k];
                }
                for (int k = l; k < n; k++) a[i][k] *= scale;
            }
        }
        anorm = smax(anorm, fabs(w[i]) + fabs(rv1[i]));
    }
    for (int i = n - 1; i >= 0; i--) {
        if (i < n - 1) {
            if (g != 0.0) {
                for (int j = l; j < n; j++) v[j][i] = (a[i][j] / a[i][l]) / g;
                for (int j = l; j < n; j++) {
                    s = 0.0;
                    for (int k = l; k < n; k++) s += a[i][k] * v[k][j];
                    for (int k = l; k < n; k++) v[k][j] += s * v[k][i];
                }
            }
            for (int j = l; j < n; j++) v[i][j] = v[j][i] = 0.0;
        }
        v[i][i] = 1.0;
        g = rv1[i];
        l = i;
    }
    for (int i = n - 1; i >= 0; i--) {
        l = i + 1;
        g = w[i];
        for (int j = l; j < n; j++) a[i][j] = 0.0;
        if (g != 0.0) {
            g = 1.0 / g;
            for (int j = l; j < n; j++) {
                s = 0.0;
                for (int k = l; k < n; k++) s += a[k][i] * a[k][j];
                f = (s / a[i][i]) * g;
                for (int k = i; k < n; k++) a[k][j] += f * a[k][i];
            }
            for (int j = i; j < n; j++) a[j][i] *= g;
        } else {
            for (int j = i; j < n; j++) a[j][i] = 0.0;
        }
        a[i][i] += 1.0;
    }
    for (int k = n - 1; k >= 0; k--) {
        for (int its = 0; its < 30; its++) {
            bool split = true;
            for (l = k; l >= 0; l--) {
                nm = l - 1;
                // rv1[0] is always 0, so l = 0 always stops here
                if (l == 0 || (fabs(rv1[l]) + anorm) == anorm) { split = false; break; }
                if ((fabs(w[nm]) + anorm) == anorm) break;
            }
            if (split) {
                c = 0.0;
                s = 1.0;
                for (int i = l; i <= k; i++) {
                    f = s * rv1[i];
                    rv1[i] = c * rv1[i];
                    if ((fabs(f) + anorm) == anorm) break;
                    g = w[i];
                    h = hyp2(f, g);
                    w[i] = h;
                    h = 1.0 / h;
                    c = g * h;
                    s = -f * h;
                    for (int j = 0; j < n; j++) {
                        y = a[j][nm];
                        z = a[j][i];
                        a[j][nm] = y * c + z * s;
                        a[j][i] = z * c - y * s;
                    }
                }
            }
            z = w[k];
            if (l == k) {
                if (z < 0.0) {
                    w[k] = -z;
                    for (int j = 0; j < n; j++) v[j][k] = -v[j][k];
                }
                break;
            }
            x = w[l];
            nm = k - 1;
            y = w[nm];
            g = rv1[nm];
            h = rv1[k];
            f = ((y - z) * (y + z) + (g - h) * (g + h)) / (2.0 * h * y);
            g = hyp2(f, 1.0);
            f = ((x - z) * (x + z) + h * ((y / (f + (f > 0.0 ? fabs(g) : -fabs(g)))) - h)) / x;
            c = s = 1.0;
            for (int j = l; j <= nm; j++) {
                const int i = j + 1;
                g = rv1[i];
                y = w[i];
                h = s * g;
                g = c * g;
                z = hyp2(f, h);
                rv1[j] = z;
                c = f / z;
                s = h / z;
                f = x * c + g * s;
                g = g * c - x * s;
                h = y * s;
                y *= c;
                for (int jj = 0; jj < n; jj++) {
                    x = v[jj][j];
                    z = v[jj][i];
                    v[jj][j] = x * c + z * s;
                    v[jj][i] = z * c - x * s;
                }
                z = hyp2(f, h);
                w[j] = z;
                if (z != 0.0) {
                    z = 1.0 / z;
                    c = f * z;
                    s = h * z;
                }
                f = c * g + s * y;
                x = c * y - s * g;
                for (int jj = 0; jj < n; jj++) {
                    y = a[jj][j];
                    z = a[jj][i];
                    a[jj][j] = y * c + z * s;
                    a[jj][i] = z * c - y * s;
                }
            }
            rv1[l] = 0.0;
            rv1[k] = f;
            w[k] = x;
        }
    }
}

// face f's distance vector: neighbour centre - owner centre, or face centre -
// owner centre on the boundary (pf holds fc - cc[owner])
__device__ __forceinline__ void face_dist(int f, int ni, int nf, int nc, const int* __restrict__ own,
                                          const int* __restrict__ nei, const double* __restrict__ cc,
                                          const double* __restrict__ pf, double d[3]) {
    if (f < ni) {
        const int o = own[f], q = nei[f];
        d[0] = cc[q] - cc[o];
        d[1] = cc[nc + q] - cc[nc + o];
        d[2] = cc[2 * nc + q] - cc[2 * nc + o];
    } else {
        d[0] = pf[f];
        d[1] = pf[nf + f];
        d[2] = pf[2 * nf + f];
    }
}

__global__ void k_sft_init(int nc, int ni, const int* __restrict__ cfp, const int* __restrict__ cfi,
                           const int* __restrict__ own, const int* __restrict__ nei, const double* __restrict__ wc,
                           const double* __restrict__ fa, const double* __restrict__ vol,
                           const double* __restrict__ VF, double* __restrict__ ls0, int* __restrict__ iface,
                           double* __restrict__ tau) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double a = VF[i] - 0.5;
    int on = 0;
    double maxA = 0.0;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int f = cfi[k] & kFaceMask;
        double fv;
        if (f < ni) {
            const double wL = wc[f], wR = 1.0 - wL;
            fv = __dadd_rn(__dmul_rn(wL, VF[own[f]]), __dmul_rn(wR, VF[nei[f]]));
        } else {
            fv = VF[i];
        }
        if (__dmul_rn(a, fv - 0.5) <= 0.0) on = 1;
        maxA = smax(maxA, fa[f]);
    }
    ls0[i] = a;
    iface[i] = on;
    const double v = vol[i];
    tau[i] = smin(v / maxA, pow(v, 0.3));
}

__global__ void k_sft_norm(int nc, const int* __restrict__ stp, const int* __restrict__ sti,
                           const double* __restrict__ stw, int64_t stn, const double* __restrict__ minv,
                           const double* __restrict__ vol, const int* __restrict__ iface,
                           const double* __restrict__ ls0, double* __restrict__ ls1, double* __restrict__ vel0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double g[3];
    lsq1(i, nc, stp, sti, stw, stn, minv, ls0, g);
    double var = ls0[i];
    if (iface[i]) {
        const double mg = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
        if (mg > 1.0) var = var / mg;
    }
    ls1[i] = var;
    const double t = fabs(var) * pow(vol[i], 0.333);
    vel0[i] = var / sqrt(var * var + t * t);
}

// One re-initialisation sweep, ls_in -> ls_out (Jacobi: every cell reads ls_in).
__global__ void __launch_bounds__(128) k_sft_reinit(int nc, int ni, int nf, const int* __restrict__ stp,
                                                    const int* __restrict__ sti, const double* __restrict__ stw,
                                                    int64_t stn, const double* __restrict__ minv,
                                                    const int* __restrict__ cfp, const int* __restrict__ cfi,
                                                    const int* __restrict__ own, const int* __restrict__ nei,
                                                    const double* __restrict__ cc, const double* __restrict__ pf,
                                                    const int* __restrict__ iface, const double* __restrict__ tau,
                                                    const double* __restrict__ vel0,
                                                    const double* __restrict__ ls_in, double* __restrict__ ls_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double g[3];
    lsq1(i, nc, stp, sti, stw, stn, minv, ls_in, g);
    const double m = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    double nv[3];
    for (int q = 0; q < 3; ++q) nv[q] = (m != 0.0) ? g[q] / m : 0.0;
    const double sgn = (vel0[i] > 0.0) ? 1.0 : -1.0;
    double vs[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    double gt[3] = {0.0, 0.0, 0.0};
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int e = cfi[k], f = e & kFaceMask;
        const double side = (e >> 30) ? 1.0 : -1.0;   // the owner looks along -d
        double d[3];
        face_dist(f, ni, nf, nc, own, nei, cc, pf, d);
        double wk = sgn * nv[0] * (side * d[0]) + sgn * nv[1] * (side * d[1]) + sgn * nv[2] * (side * d[2]);
        wk = smax(1.e-5, wk);
        vs[0] += wk * d[0] * d[0]; vs[1] += wk * d[0] * d[1]; vs[2] += wk * d[0] * d[2];
        vs[3] += wk * d[1] * d[1]; vs[4] += wk * d[1] * d[2]; vs[5] += wk * d[2] * d[2];
        const double dv = (f < ni) ? __ldg(ls_in + nei[f]) - __ldg(ls_in + own[f]) : 0.0;
        gt[0] += wk * d[0] * dv; gt[1] += wk * d[1] * dv; gt[2] += wk * d[2] * dv;
    }
    double out = ls_in[i];
    if (!iface[i]) {
        double U[3][3] = {{vs[0], vs[1], vs[2]}, {vs[1], vs[3], vs[4]}, {vs[2], vs[4], vs[5]}};
        double D[3], V[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        svd3(U, D, V);
        // pseudo-inverse V diag(1/D) U^T (singular values below 1e-25 dropped)
        double iD[3];
        for (int q = 0; q < 3; ++q) iD[q] = (fabs(D[q]) > 1.e-25) ? 1.0 / D[q] : 0.0;
        double P[3][3];
        for (int r = 0; r < 3; ++r)
            for (int s = 0; s < 3; ++s) P[r][s] = V[r][0] * (iD[0] * U[s][0]) + V[r][1] * (iD[1] * U[s][1]) +
                                                  V[r][2] * (iD[2] * U[s][2]);
        // the upper triangle of P is applied as a symmetric matrix
        const double t0 = P[0][0] * gt[0] + P[0][1] * gt[1] + P[0][2] * gt[2];
        const double t1 = P[0][1] * gt[0] + P[1][1] * gt[1] + P[1][2] * gt[2];
        const double t2 = P[0][2] * gt[0] + P[1][2] * gt[1] + P[2][2] * gt[2];
        const double mg = sqrt(t0 * t0 + t1 * t1 + t2 * t2);
        out += 0.1 * tau[i] * vel0[i] * (1.0 - mg);
    }
    ls_out[i] = out;
}

__global__ void k_sft_normals(int nc, const int* __restrict__ stp, const int* __restrict__ sti,
                              const double* __restrict__ stw, int64_t stn, const double* __restrict__ minv,
                              const double* __restrict__ ls, double* __restrict__ nrm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double g[3];
    lsq1(i, nc, stp, sti, stw, stn, minv, ls, g);
    const double m = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    for (int q = 0; q < 3; ++q) nrm[(size_t)q * nc + i] = (m > 1.e-15) ? g[q] / m : 0.0;
}

__global__ void k_sft_kappa(int nc, int ni, int nf, const int* __restrict__ stp, const int* __restrict__ sti,
                            const int* __restrict__ cfp, const int* __restrict__ cfi,
                            const double* __restrict__ cc, const double* __restrict__ pf,
                            const double* __restrict__ nrm, double* __restrict__ kappa) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const size_t N = nc;
    const double cx = cc[i], cy = cc[N + i], cz = cc[2 * N + i];
    const double ni0 = nrm[i], ni1 = nrm[N + i], ni2 = nrm[2 * N + i];
    double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    double t[3] = {0.0, 0.0, 0.0};
    for (int k = stp[i]; k < stp[i + 1]; ++k) {
        const int j = __ldg(sti + k);
        const double d0 = __ldg(cc + j) - cx, d1 = __ldg(cc + N + j) - cy, d2 = __ldg(cc + 2 * N + j) - cz;
        v[0] += d0 * d0; v[1] += d0 * d1; v[2] += d0 * d2; v[3] += d1 * d1; v[4] += d1 * d2; v[5] += d2 * d2;
        t[0] += d0 * (__ldg(nrm + j) - ni0);
        t[1] += d1 * (__ldg(nrm + N + j) - ni1);
        t[2] += d2 * (__ldg(nrm + 2 * N + j) - ni2);
    }
    // boundary faces (ascending, the last entries of the cell's face list) add
    // to the normal matrix only
    int kb = cfp[i + 1];
    while (kb > cfp[i] && (cfi[kb - 1] & kFaceMask) >= ni) --kb;
    for (int k = kb; k < cfp[i + 1]; ++k) {
        const int f = cfi[k] & kFaceMask;
        const double d0 = pf[f], d1 = pf[nf + f], d2 = pf[2 * nf + f];
        v[0] += d0 * d0; v[1] += d0 * d1; v[2] += d0 * d2; v[3] += d1 * d1; v[4] += d1 * d2; v[5] += d2 * d2;
    }
    const double det = v[0] * v[3] * v[5] + v[1] * v[4] * v[2] + v[2] * v[1] * v[4] - v[0] * v[4] * v[4] -
                       v[2] * v[3] * v[2] - v[1] * v[1] * v[5];
    const double m0 = (v[3] * v[5] - v[4] * v[4]) / det, m1 = (v[2] * v[4] - v[1] * v[5]) / det;
    const double m2 = (v[1] * v[4] - v[2] * v[3]) / det, m3 = (v[0] * v[5] - v[2] * v[2]) / det;
    const double m4 = (v[2] * v[1] - v[0] * v[4]) / det, m5 = (v[0] * v[3] - v[1] * v[1]) / det;
    const double r0 = m0 * t[0] + m1 * t[1] + m2 * t[2];
    const double r1 = m1 * t[0] + m3 * t[1] + m4 * t[2];
    const double r2 = m2 * t[0] + m4 * t[1] + m5 * t[2];
    kappa[i] = -(r0 + r1 + r2);
}

// Gauss-Green gradient of VF (face values skew-corrected with the LSQ
// gradient gvf, 3 planes of nc; boundary values by the VF condition), then
// the source planes sigma kappa grad VF and sigma kappa grad VF . U.
__global__ void k_sft_source(int nc, int ni, int nf, int nb, const int* __restrict__ cfp,
                             const int* __restrict__ cfi, const int* __restrict__ own, const int* __restrict__ nei,
                             const int* __restrict__ bpatch, const int* __restrict__ bct,
                             const double* __restrict__ bcv, const double* __restrict__ wc,
                             const double* __restrict__ skew, const double* __restrict__ fn,
                             const double* __restrict__ fa, const double* __restrict__ pf,
                             const double* __restrict__ vol, const double* __restrict__ VF,
                             const double* __restrict__ gvf, const double* __restrict__ bface,
                             const double* __restrict__ U, const double* __restrict__ V,
                             const double* __restrict__ W, const double* __restrict__ kappa, double sigma,
                             double* __restrict__ src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const size_t N = nc;
    const double iv = 1.0 / vol[i];
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int e = cfi[k], f = e & kFaceMask;
        double vf;
        if (f < ni) {
            const int o = own[f], q = nei[f];
            const double wL = wc[f], wR = 1.0 - wL;
            const double s0 = skew[f], s1 = skew[nf + f], s2 = skew[2 * nf + f];
            vf = wL * VF[o] + wR * VF[q];
            vf += wL * (gvf[o] * s0 + gvf[N + o] * s1 + gvf[2 * N + o] * s2);
            vf += wR * (gvf[q] * s0 + gvf[N + q] * s1 + gvf[2 * N + q] * s2);
        } else {
            const int b = f - ni, p = bpatch[b], t = bct[3 * p + 2];
            if (t == SEMO_BC_FIXED_VALUE) vf = bcv[5 * p + 4];
            else if (t == SEMO_BC_ZERO_GRADIENT)
                vf = VF[i] + gvf[i] * pf[f] + gvf[N + i] * pf[nf + f] + gvf[2 * N + i] * pf[2 * nf + f];
            else vf = 0.5 * (VF[i] + bface[4 * (size_t)nb + b]);
        }
        const double w = ((e >> 30) ? -vf : vf) * fa[f] * iv;
        g0 += w * fn[f]; g1 += w * fn[nf + f]; g2 += w * fn[2 * nf + f];
    }
    const double sk = sigma * kappa[i];
    src[i] = sk * g0;
    src[N + i] = sk * g1;
    src[2 * N + i] = sk * g2;
    src[3 * N + i] = sk * (g0 * U[i] + g1 * V[i] + g2 * W[i]);
}

}  // namespace

namespace semo {

// Needs the face values (assemble_face_values: clamped VF, boundary values)
// and a full stencil pass (the LSQ gradient of VF in grad planes 12-14).
void assemble_surface_tension(semo_ctx* c) {
    const double sigma = c->phys.sigma;
    c->sft_current = false;
    if (sigma == 0.0) return;
    const int T = 128;
    cudaStream_t s = c->stream;
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    const size_t N = nc;
    StageScope sc(c, ST_SFT);
    // planes: 0 kappa, 1 ls, 2-5 src, 6 ls scratch, 7 tau, 8 vel0, 9-11 normals
    c->sft.alloc(12 * N, s);
    c->sft_iface.alloc(N, s);
    double* kap = c->sft.p;
    double* ls = c->sft.p + N;
    double* src = c->sft.p + 2 * N;
    double* lsb = c->sft.p + 6 * N;
    double* tau = c->sft.p + 7 * N;
    double* vel0 = c->sft.p + 8 * N;
    double* nrm = c->sft.p + 9 * N;
    const int B = blocks(nc, T);
    k_sft_init<<<B, T, 0, s>>>(nc, ni, c->cf_ptr, c->cf_idx, c->own, c->nei, c->wc, c->fa, c->vol, c->VF, lsb,
                               c->sft_iface, tau);
    SEMO_CHECK_LAUNCH();
    k_sft_norm<<<B, T, 0, s>>>(nc, c->st_ptr, c->st_idx, c->stw, c->st_nnz, c->minv, c->vol, c->sft_iface, lsb, ls,
                               vel0);
    SEMO_CHECK_LAUNCH();
    for (int it = 0; it < 4; ++it) {   // ls -> lsb -> ls -> lsb -> ls
        const double* in = (it & 1) ? lsb : ls;
        double* out = (it & 1) ? ls : lsb;
        k_sft_reinit<<<B, T, 0, s>>>(nc, ni, nf, c->st_ptr, c->st_idx, c->stw, c->st_nnz, c->minv, c->cf_ptr,
                                     c->cf_idx, c->own, c->nei, c->cc, c->pf, c->sft_iface, tau, vel0, in, out);
        SEMO_CHECK_LAUNCH();
    }
    k_sft_normals<<<B, T, 0, s>>>(nc, c->st_ptr, c->st_idx, c->stw, c->st_nnz, c->minv, ls, nrm);
    SEMO_CHECK_LAUNCH();
    k_sft_kappa<<<B, T, 0, s>>>(nc, ni, nf, c->st_ptr, c->st_idx, c->cf_ptr, c->cf_idx, c->cc, c->pf, nrm, kap);
    SEMO_CHECK_LAUNCH();
    k_sft_source<<<B, T, 0, s>>>(nc, ni, nf, nb, c->cf_ptr, c->cf_idx, c->own, c->nei, c->bpatch, c->bc_type,
                                 c->bc_value, c->wc, c->skew, c->fn, c->fa, c->pf, c->vol, c->VF,
                                 c->grad.p + 12 * N, c->bface, c->U, c->V, c->W, kap, sigma, src);
    SEMO_CHECK_LAUNCH();
    c->sft_current = true;
}

}  // namespace semo
