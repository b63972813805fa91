// Per-outer-iteration pressure-correction assembly on the GPU.
//
// Stages (reference function, file:line):
//   k_cell_eos        calcIncomCellEOSVF            src/solvers/eos.cpp:10-151
//   k_bface_values    reconIncomZeroOrder + face EOS src/solvers/reconIncom.cpp:501-1035, :440-496
//   k_grav_face/cell  calcSourceGravity             src/solvers/source/gravity.cpp:7-75
//   k_stencil         setCellVarMinMax x4 + calcLeastSquare("cellVertex","1st") x5
//                                                   src/solvers/cellVarMinMax.cpp:8-23,
//                                                   src/math/gradient.cpp:761-816, :997-1050, :1136-1159
//   k_pface           calcPressureEq face loop      src/solvers/eqPressure.cpp:246-564
//                     + Rhie-Chow helpers           src/solvers/surfaceNormalVelocity.cpp:125-187
//   k_pbface          calcPressureEq boundary loop  src/solvers/eqPressure.cpp:570-673
//   k_pcell           diagonal and RHS gather       (the += into A_vals[diag] / B of the two loops)
//   k_gg_face/cell    Gauss-Green grad p', 2 sweeps src/solvers/eqPressure.cpp:686-809
//   k_update          P/U/V/W update + norms        src/solvers/eqPressure.cpp:823-883
//
// Everything is atomic-free: faces write per-face results, cells gather them
// through the cell->face list in ascending face order (the order SEMO's face
// loop accumulates them), so results are deterministic run to run.  Cells are
// in RCM order, faces in the caller's order; all arrays are SoA planes.
#include <cuda_runtime.h>

#include <cmath>

#include "face_common.cuh"
#include "semo_internal.h"

namespace {

using namespace semo::face;

// EOS (eos.cpp:10-151) and, when mu is given, the laminar viscosity of
// calcCellTransport (transport.cpp:9-98): mu = VF mu0 + (1 - VF) mu1 on the
// clamped VF, with its reciprocal in a second plane.
__global__ void k_cell_eos(int nc, double r0, double r1, double m0, double m1, double* __restrict__ VF,
                           double* __restrict__ rho, double* __restrict__ irho, double* __restrict__ mu) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double mf = clamp01(VF[i]);
    const double v0 = clamp01(mf), v1 = clamp01(1.0 - mf);
    // unfused, as the reference rounds it (rho feeds every coefficient)
    double r = 0.0;
    r = __dadd_rn(r, __dmul_rn(v0, r0));
    r = __dadd_rn(r, __dmul_rn(v1, r1));
    rho[i] = r;
    irho[i] = 1.0 / r;
    VF[i] = v0;
    if (mu) {
        const double m = __dadd_rn(__dmul_rn(v0, m0), __dmul_rn(__dsub_rn(1.0, v0), m1));
        mu[i] = m;
        mu[nc + i] = 1.0 / m;
    }
}

// boundary-face values (left == right for every supported condition);
// planes of nb: 0 p, 1 u, 2 v, 3 w, 4 vf, 5 rho
__global__ void k_bface_values(int nb, int ni, int nf, const int* __restrict__ own, const int* __restrict__ bpatch,
                               const int* __restrict__ bct, const double* __restrict__ bcv,
                               const double* __restrict__ fn, const double* __restrict__ P,
                               const double* __restrict__ U, const double* __restrict__ V,
                               const double* __restrict__ W, const double* __restrict__ VF, double r0, double r1,
                               double* __restrict__ bf) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int f = ni + b, o = own[f], p = bpatch[b];
    const int tp = bct[3 * p], tu = bct[3 * p + 1], tv = bct[3 * p + 2];
    bf[b] = (tp == SEMO_BC_FIXED_VALUE) ? bcv[5 * p] : P[o];
    double u, v, w;
    if (tu == SEMO_BC_FIXED_VALUE) { u = bcv[5 * p + 1]; v = bcv[5 * p + 2]; w = bcv[5 * p + 3]; }
    else if (tu == SEMO_BC_NO_SLIP) { u = 0.0; v = 0.0; w = 0.0; }
    else if (tu == SEMO_BC_SLIP) {
        const double n0 = fn[f], n1 = fn[nf + f], n2 = fn[2 * nf + f];
        const double un = U[o] * n0 + V[o] * n1 + W[o] * n2;
        u = U[o] - un * n0; v = V[o] - un * n1; w = W[o] - un * n2;
    } else { u = U[o]; v = V[o]; w = W[o]; }
    bf[nb + b] = u; bf[2 * nb + b] = v; bf[3 * nb + b] = w;
    const double vf = (tv == SEMO_BC_FIXED_VALUE) ? bcv[5 * p + 4] : VF[o];
    bf[4 * nb + b] = vf;
    const double a0 = clamp01(vf), a1 = clamp01(1.0 - vf);
    double r = 0.0;
    r = __dadd_rn(r, __dmul_rn(a0, r0));
    r = __dadd_rn(r, __dmul_rn(a1, r1));
    bf[5 * nb + b] = r;
}

// gravity source, face part: (RhoF*g.PF, RhoF*g.NF, UnF) per face
__global__ void k_grav_face(int nf, int ni, int nc, int nb, const int* __restrict__ own, const int* __restrict__ nei,
                            const double* __restrict__ fn, const double* __restrict__ wc,
                            const double* __restrict__ pf, const double* __restrict__ nfv,
                            const double* __restrict__ U, const double* __restrict__ V,
                            const double* __restrict__ W, const double* __restrict__ irho,
                            const double* __restrict__ bf, double g0, double g1, double g2,
                            double* __restrict__ out) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int o = own[f];
    const double n0 = fn[f], n1 = fn[nf + f], n2 = fn[2 * nf + f];
    const double wL = wc[f], wR = 1.0 - wL;
    double uL, vL, wwL, uR, vR, wwR, irL, irR;
    if (f < ni) {
        const int q = nei[f];
        uL = U[o]; vL = V[o]; wwL = W[o]; uR = U[q]; vR = V[q]; wwR = W[q];
        irL = irho[o]; irR = irho[q];   // face densities equal the cells' (same EOS of the same VF)
    } else {
        const int b = f - ni;
        uL = uR = bf[nb + b]; vL = vR = bf[2 * nb + b]; wwL = wwR = bf[3 * nb + b];
        irL = irR = 1.0 / bf[5 * nb + b];
    }
    const double UnL = uL * n0 + vL * n1 + wwL * n2;
    const double UnR = uR * n0 + vR * n1 + wwR * n2;
    const double UnF = wL * UnL + wR * UnR;
    const double RhoF = 1.0 / (wL * irL + wR * irR);
    double gL = 0.0, gR = 0.0;
    gL += g0 * pf[f]; gL += g1 * pf[nf + f]; gL += g2 * pf[2 * nf + f];
    gR += g0 * nfv[f]; gR += g1 * nfv[nf + f]; gR += g2 * nfv[2 * nf + f];
    out[f] = RhoF * gL;
    out[nf + f] = RhoF * gR;
    out[2 * nf + f] = UnF;
}

__global__ void k_grav_cell(int nc, int nf, const int* __restrict__ cfp, const int* __restrict__ cfi,
                            const double* __restrict__ fn, const double* __restrict__ fa,
                            const double* __restrict__ vol, const double* __restrict__ gf, double* __restrict__ sg) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    // one reciprocal per cell instead of four divisions per face (FP64 division
    // is the bottleneck here on GB300); agrees with SEMO's x*n*A/V to rounding
    const double iv = 1.0 / vol[i];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int e = cfi[k], f = e & kFaceMask;
        const double n0 = fn[f], n1 = fn[nf + f], n2 = fn[2 * nf + f], a = fa[f];
        const double un = gf[2 * nf + f];
        if (e >> 30) {
            const double w = gf[nf + f] * a * iv;
            s0 -= w * n0; s1 -= w * n1; s2 -= w * n2; s3 -= w * un;
        } else {
            const double w = gf[f] * a * iv;
            s0 += w * n0; s1 += w * n1; s2 += w * n2; s3 += w * un;
        }
    }
    sg[i] = s0; sg[nc + i] = s1; sg[2 * nc + i] = s2; sg[3 * nc + i] = s3;
}

// One pass over each cell's vertex stencil: LSQ gradients of P,U,V,W,VF and
// stencil min/max of U,V,W,VF,P (mm planes maxU,minU,maxV,minV,maxW,minW,
// maxVF,minVF,maxP,minP).  Stencil weights w_k*d_k are precomputed, and so is
// their per-cell sum S (stencil and boundary faces): the gradient's sum
// sum_k w_k (phi_k - phi_i) is formed as sum_k w_k phi_k - phi_i S, three FMAs
// an entry and field instead of a difference and three FMAs (FP64 issue bounds
// this kernel on GB300).  With kPVF false only the U,V,W parts are computed
// and the P and VF planes are left as they are (they are still current: see
// assemble_gravity_stencil).
template <bool kPVF>
__global__ void __launch_bounds__(128) k_stencil(int nc, int nf, int ni, int nb, const int* __restrict__ stp,
                                                 const int* __restrict__ sti, const double* __restrict__ stw,
                                                 int64_t stn, const int* __restrict__ cfp,
                                                 const int* __restrict__ cfi, const double* __restrict__ bfw,
                                                 const double* __restrict__ stws,
                                                 const double* __restrict__ minv, const double* __restrict__ P,
                                                 const double* __restrict__ U, const double* __restrict__ V,
                                                 const double* __restrict__ W, const double* __restrict__ VF,
                                                 const double* __restrict__ bf, double* __restrict__ grad,
                                                 double* __restrict__ mm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double pi = P[i], ui = U[i], vi = V[i], wi = W[i], fi = VF[i];
    double g[5][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    long long kmaxu = okey(ui), kminu = kmaxu, kmaxv = okey(vi), kminv = kmaxv;
    long long kmaxw = okey(wi), kminw = kmaxw, kmaxf = okey(fi), kminf = kmaxf;
    long long kmaxp = okey(pi), kminp = kmaxp;
    const int kb = stp[i], ke = stp[i + 1];
    for (int k = kb; k < ke; ++k) {
        const int j = __ldg(sti + k);
        const double wx = __ldg(stw + k), wy = __ldg(stw + stn + k), wz = __ldg(stw + 2 * stn + k);
        const double uj = __ldg(U + j), vj = __ldg(V + j), wj = __ldg(W + j);
        long long t;
        if constexpr (kPVF) {
            const double pj = __ldg(P + j), fj = __ldg(VF + j);
            g[0][0] = fma(wx, pj, g[0][0]); g[0][1] = fma(wy, pj, g[0][1]); g[0][2] = fma(wz, pj, g[0][2]);
            g[4][0] = fma(wx, fj, g[4][0]); g[4][1] = fma(wy, fj, g[4][1]); g[4][2] = fma(wz, fj, g[4][2]);
            t = okey(fj); kmaxf = (kmaxf < t) ? t : kmaxf; kminf = (t < kminf) ? t : kminf;
            t = okey(pj); kmaxp = (kmaxp < t) ? t : kmaxp; kminp = (t < kminp) ? t : kminp;
        }
        g[1][0] = fma(wx, uj, g[1][0]); g[1][1] = fma(wy, uj, g[1][1]); g[1][2] = fma(wz, uj, g[1][2]);
        g[2][0] = fma(wx, vj, g[2][0]); g[2][1] = fma(wy, vj, g[2][1]); g[2][2] = fma(wz, vj, g[2][2]);
        g[3][0] = fma(wx, wj, g[3][0]); g[3][1] = fma(wy, wj, g[3][1]); g[3][2] = fma(wz, wj, g[3][2]);
        t = okey(uj); kmaxu = (kmaxu < t) ? t : kmaxu; kminu = (t < kminu) ? t : kminu;
        t = okey(vj); kmaxv = (kmaxv < t) ? t : kmaxv; kminv = (t < kminv) ? t : kminv;
        t = okey(wj); kmaxw = (kmaxw < t) ? t : kmaxw; kminw = (t < kminw) ? t : kminw;
    }
    // boundary faces (face index >= ni) come last in the ascending list
    {
        int kfirst = cfp[i + 1];
        while (kfirst > cfp[i] && (cfi[kfirst - 1] & kFaceMask) >= ni) --kfirst;
        for (int k = kfirst; k < cfp[i + 1]; ++k) {
            const int b = (cfi[k] & kFaceMask) - ni;
            const double wx = bfw[b], wy = bfw[nb + b], wz = bfw[2 * nb + b];
            double d;
            if constexpr (kPVF) { d = bf[b]; g[0][0] += wx * d; g[0][1] += wy * d; g[0][2] += wz * d; }
            d = bf[nb + b]; g[1][0] += wx * d; g[1][1] += wy * d; g[1][2] += wz * d;
            d = bf[2 * nb + b]; g[2][0] += wx * d; g[2][1] += wy * d; g[2][2] += wz * d;
            d = bf[3 * nb + b]; g[3][0] += wx * d; g[3][1] += wy * d; g[3][2] += wz * d;
            if constexpr (kPVF) { d = bf[4 * nb + b]; g[4][0] += wx * d; g[4][1] += wy * d; g[4][2] += wz * d; }
        }
    }
    const double sx = stws[i], sy = stws[nc + i], sz = stws[2 * nc + i];
    const double phi_i[5] = {pi, ui, vi, wi, fi};
    const double m0 = minv[i], m1 = minv[nc + i], m2 = minv[2 * nc + i];
    const double m3 = minv[3 * nc + i], m4 = minv[4 * nc + i], m5 = minv[5 * nc + i];
#pragma unroll
    for (int q = kPVF ? 0 : 1; q < (kPVF ? 5 : 4); ++q) {
        const double a0 = fma(-phi_i[q], sx, g[q][0]);
        const double a1 = fma(-phi_i[q], sy, g[q][1]);
        const double a2 = fma(-phi_i[q], sz, g[q][2]);
        double t0 = 0.0; t0 += m0 * a0; t0 += m1 * a1; t0 += m2 * a2;
        double t1 = 0.0; t1 += m1 * a0; t1 += m3 * a1; t1 += m4 * a2;
        double t2 = 0.0; t2 += m2 * a0; t2 += m4 * a1; t2 += m5 * a2;
        grad[(3 * q + 0) * (size_t)nc + i] = t0;
        grad[(3 * q + 1) * (size_t)nc + i] = t1;
        grad[(3 * q + 2) * (size_t)nc + i] = t2;
    }
    mm[i] = ounkey(kmaxu); mm[nc + i] = ounkey(kminu);
    mm[2 * (size_t)nc + i] = ounkey(kmaxv); mm[3 * (size_t)nc + i] = ounkey(kminv);
    mm[4 * (size_t)nc + i] = ounkey(kmaxw); mm[5 * (size_t)nc + i] = ounkey(kminw);
    if constexpr (kPVF) {
        mm[6 * (size_t)nc + i] = ounkey(kmaxf); mm[7 * (size_t)nc + i] = ounkey(kminf);
        mm[8 * (size_t)nc + i] = ounkey(kmaxp); mm[9 * (size_t)nc + i] = ounkey(kminp);
    }
}

// SEMO's clamp sequence (if x <= lo: x = lo; if x >= hi: x = hi) on the
// integer pipes
__device__ __forceinline__ double clamp_seq(double x, double lo, double hi) {
    long long k = okey(x);
    const long long kl = okey(lo), kh = okey(hi);
    if (k <= kl) k = kl;
    if (k >= kh) k = kh;
    return ounkey(k);
}

// Pressure-matrix coefficients, written with explicit roundings so that the
// early matrix (pressure_matrix) and the pass's own assembly agree bit for bit.
// Internal face: kA dt (wR/rhoL + wR/rhoR), SEMO's rho* = 1/(wCR/rhoL + wCR/rhoR)
// (wCR twice, eqPressure.cpp:396).
__device__ __forceinline__ double pcoef_face(double kA, double dt, double wR, double iRL, double iRR) {
    return __dmul_rn(kA, __dmul_rn(dt, __dadd_rn(__dmul_rn(wR, iRL), __dmul_rn(wR, iRR))));
}
// Boundary face (eqPressure.cpp:570-673): fixedValue pressure alpha tmp1/dPN
// area with tmp1 = dt/rhoF; zeroGradient 0 x the same
__device__ __forceinline__ double pcoef_bface(bool fixed, double alpha, double tmp1, double dPN, double area) {
    const double t = alpha * tmp1 / dPN * area;
    return fixed ? 1.0 * t : 0.0 * t;
}

// Internal faces of calcPressureEq (UnF as face_unf).  With a.val null the
// matrix values are left as they are (built beforehand by pressure_matrix).
__global__ void __launch_bounds__(256) k_pface(FaceArgs a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.ni) return;
    const int o = a.own[f], q = a.nei[f];
    const FaceGeo g = load_geo(a, f);
    const double UnF = face_unf(a, g, o, q);
    const double iRL = __ldg(a.irho + o), iRR = __ldg(a.irho + q);
    const double area = g.area;
    const double coef = pcoef_face(g.kA, a.dt, g.wR, iRL, iRR);
    if (a.val) {
        a.val[a.lr[f]] = -coef;
        a.val[a.rl[f]] = -coef;
    }
    a.coef[f] = coef;
    a.flux[f] = UnF * area;
    a.unf[f] = UnF;
}

__global__ void k_pbface(int nb, int ni, int nf, int nc, const int* __restrict__ own, const int* __restrict__ bpatch,
                         const int* __restrict__ bct, const double* __restrict__ fn, const double* __restrict__ fa,
                         const double* __restrict__ mpn, const double* __restrict__ alf,
                         const double* __restrict__ epn, const double* __restrict__ P,
                         const double* __restrict__ grad, const double* __restrict__ bf, double dt,
                         double* __restrict__ coef, double* __restrict__ flux, double* __restrict__ unf) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int f = ni + b, o = own[f];
    const double n0 = fn[f], n1 = fn[nf + f], n2 = fn[2 * nf + f], area = fa[f];
    const double u = bf[nb + b], v = bf[2 * nb + b], w = bf[3 * nb + b];
    const double UnL = u * n0 + v * n1 + w * n2;
    double UnF = 0.5 * UnL + 0.5 * UnL;
    const double tmp1 = 1.0 / bf[5 * nb + b] * dt;
    const bool fixed = bct[3 * bpatch[b]] == SEMO_BC_FIXED_VALUE;
    const double dPN = 0.5 * mpn[f], alpha = alf[f];
    if (fixed) {
        UnF -= alpha * tmp1 * (bf[b] - P[o]) / dPN;
        UnF += alpha * tmp1 * grad[o] * epn[f];
        UnF += alpha * tmp1 * grad[nc + o] * epn[nf + f];
        UnF += alpha * tmp1 * grad[2 * (size_t)nc + o] * epn[2 * nf + f];
    }
    coef[f] = pcoef_bface(fixed, alpha, tmp1, dPN, area);
    flux[f] = UnF * area;
    unf[f] = UnF;
}

__global__ void k_pcell(int nc, int ni, const int* __restrict__ cfp, const int* __restrict__ cfi,
                        const int* __restrict__ dig, const double* __restrict__ coef,
                        const double* __restrict__ flux, const double* __restrict__ src,
                        const double* __restrict__ vol, double* __restrict__ val, double* __restrict__ b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double d = 0.0, s = 0.0;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int e = cfi[k], f = e & kFaceMask;
        d += coef[f];
        if (e >> 30) s += flux[f]; else s -= flux[f];
    }
    if (src) s += src[i] * vol[i];
    if (val) val[dig[i]] = d;
    b[i] = s;
}

// The matrix part of the three kernels above alone (values only, the same
// roundings): face coefficients, off-diagonals, then the diagonal gather.
__global__ void k_pmat_face(int nf, int ni, int nb, const int* __restrict__ own, const int* __restrict__ nei,
                            const int* __restrict__ lr, const int* __restrict__ rl, const double* __restrict__ fk,
                            const double* __restrict__ irho, const int* __restrict__ bpatch,
                            const int* __restrict__ bct, const double* __restrict__ mpn,
                            const double* __restrict__ alf, const double* __restrict__ fa,
                            const double* __restrict__ bf, double dt, double* __restrict__ coef,
                            double* __restrict__ val) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    if (f < ni) {
        const double kA = fk[f], wR = 1.0 - fk[3 * ni + f];
        const double c = pcoef_face(kA, dt, wR, __ldg(irho + own[f]), __ldg(irho + nei[f]));
        val[lr[f]] = -c;
        val[rl[f]] = -c;
        coef[f] = c;
    } else {
        const int b = f - ni;
        const double tmp1 = 1.0 / bf[5 * nb + b] * dt;
        const bool fixed = bct[3 * bpatch[b]] == SEMO_BC_FIXED_VALUE;
        coef[f] = pcoef_bface(fixed, alf[f], tmp1, 0.5 * mpn[f], fa[f]);
    }
}

__global__ void k_pmat_cell(int nc, const int* __restrict__ cfp, const int* __restrict__ cfi,
                            const int* __restrict__ dig, const double* __restrict__ coef, double* __restrict__ val) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double d = 0.0;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) d += coef[cfi[k] & kFaceMask];
    val[dig[i]] = d;
}

// Gauss-Green sweep, face part: interpolated p' with skewness correction
__global__ void k_gg_face(int nf, int ni, int nc, int nb, const int* __restrict__ own, const int* __restrict__ nei,
                          const int* __restrict__ bpatch, const int* __restrict__ bct,
                          const double* __restrict__ wc, const double* __restrict__ skew,
                          const double* __restrict__ x, const double* __restrict__ g, double* __restrict__ vF) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int o = own[f];
    if (f < ni) {
        const int q = nei[f];
        const double wL = wc[f], wR = 1.0 - wL;
        double v = wL * x[o] + wR * x[q];
        for (int k = 0; k < 3; ++k) {
            const double s = skew[(size_t)k * nf + f];
            v += wL * g[(size_t)k * nc + o] * s;
            v += wR * g[(size_t)k * nc + q] * s;
        }
        vF[f] = v;
    } else {
        vF[f] = (bct[3 * bpatch[f - ni]] == SEMO_BC_FIXED_VALUE) ? 0.0 : x[o];
    }
}

__global__ void k_gg_cell(int nc, int nf, const int* __restrict__ cfp, const int* __restrict__ cfi,
                          const double* __restrict__ fn, const double* __restrict__ fa,
                          const double* __restrict__ vol, const double* __restrict__ vF, double* __restrict__ g) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double iv = 1.0 / vol[i];   // one reciprocal per cell, not three divisions per face
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int e = cfi[k], f = e & kFaceMask;
        const double w = vF[f] * fa[f] * iv;
        const double c0 = w * fn[f], c1 = w * fn[nf + f], c2 = w * fn[2 * nf + f];
        if (e >> 30) { g0 -= c0; g1 -= c1; g2 -= c2; }
        else { g0 += c0; g1 += c1; g2 += c2; }
    }
    g[i] = g0; g[nc + i] = g1; g[2 * (size_t)nc + i] = g2;
}

// The divisions dt/rho use the EOS's reciprocal density (one FP64 division a
// cell is ~20 FP64 instructions on this part); the clamps compare
// order-preserving integer images.  Both agree with SEMO's expressions to
// rounding (the clamps up to the sign of a zero).
__global__ void __launch_bounds__(kRedThreads) k_update(int nc, double urf_p, double urf_u, double dt,
                                                        const double* __restrict__ x,
                                                        const double* __restrict__ g,
                                                        const double* __restrict__ irho, double* __restrict__ P,
                                                        double* __restrict__ U, double* __restrict__ V,
                                                        double* __restrict__ W, double pmin, double pmax,
                                                        double umin, double umax, double vmin, double vmax,
                                                        double wmin, double wmax, double* __restrict__ part) {
    __shared__ double sh[32];
    double nd = 0.0, np = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
        const double xi = x[i];
        double p = P[i] + urf_p * xi;
        const double t = dt * irho[i];
        const double ru = urf_u * t * g[i], rv = urf_u * t * g[nc + i], rw = urf_u * t * g[2 * (size_t)nc + i];
        double u = U[i] - ru, v = V[i] - rv, w = W[i] - rw;
        p = clamp_seq(p, pmin, pmax);
        u = clamp_seq(u, umin, umax);
        v = clamp_seq(v, vmin, vmax);
        w = clamp_seq(w, wmin, wmax);
        P[i] = p; U[i] = u; V[i] = v; W[i] = w;
        nd += xi * xi + ru * ru + rv * rv + rw * rw;
        np += p * p + u * u + v * v + w * w;
    }
    nd = block_sum(nd, sh);
    np = block_sum(np, sh);
    if (threadIdx.x == 0) { part[blockIdx.x] = nd; part[kRedBlocks + blockIdx.x] = np; }
}

// caller order <-> RCM order for up to 5 cell planes
struct Planes5 {
    double* p[5];
};
struct CPlanes5 {
    const double* p[5];
};
__global__ void k_from_caller(int nc, int planes, const int* __restrict__ perm, const double* __restrict__ src,
                              Planes5 dst, int* __restrict__ bad) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nc) return;
    const int o = perm[r];
    bool ok = true;
    for (int q = 0; q < planes; ++q) {
        const double v = src[(size_t)q * nc + o];
        ok &= isfinite(v);
        dst.p[q][r] = v;
    }
    if (!ok) atomicExch(bad, 1);
}
__global__ void k_to_caller(int nc, int planes, const int* __restrict__ perm, CPlanes5 src,
                            double* __restrict__ dst) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nc) return;
    const int o = perm[r];
    for (int q = 0; q < planes; ++q) dst[(size_t)q * nc + o] = src.p[q][r];
}
__global__ void k_cell_product(int nc, const double* __restrict__ a, const double* __restrict__ b,
                               double* __restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nc) out[r] = a[r] * b[r];
}

}  // namespace

namespace semo {
namespace face {
__global__ void k_finish2(const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[32];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < kRedBlocks; i += blockDim.x) { a += part[i]; b += part[kRedBlocks + i]; }
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    if (threadIdx.x == 0) { out[0] = a; out[1] = b; }
}
}  // namespace face

bool fields_from_caller_order(semo_ctx* c, const double* src, double* const* dst, int planes) {
    Planes5 d{};
    for (int q = 0; q < planes; ++q) d.p[q] = dst[q];
    SEMO_CUDA(cudaMemsetAsync(c->flag.p + 8, 0, sizeof(int), c->stream));
    k_from_caller<<<blocks(c->nc, 256), 256, 0, c->stream>>>(c->nc, planes, c->dperm, src, d, c->flag.p + 8);
    SEMO_CHECK_LAUNCH();
    int* const bad = c->hpin_scan + 1;
    SEMO_CUDA(cudaMemcpyAsync(bad, c->flag.p + 8, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SEMO_CUDA(cudaStreamSynchronize(c->stream));
    return *bad == 0;
}

void cellwise_product(semo_ctx* c, const double* a, const double* b, double* out) {
    k_cell_product<<<blocks(c->nc, 256), 256, 0, c->stream>>>(c->nc, a, b, out);
    SEMO_CHECK_LAUNCH();
}

void fields_to_caller_order(semo_ctx* c, const double* const* src, double* dst, int planes) {
    CPlanes5 s{};
    for (int q = 0; q < planes; ++q) s.p[q] = src[q];
    k_to_caller<<<blocks(c->nc, 256), 256, 0, c->stream>>>(c->nc, planes, c->dperm, s, dst);
    SEMO_CHECK_LAUNCH();
}

void assemble_face_values(semo_ctx* c, bool with_mu) {
    const int T = 256;
    cudaStream_t s = c->stream;
    StageScope sc(c, ST_FACE_VALUES);
    if (with_mu) c->mu.alloc(2 * (size_t)c->nc, s);
    k_cell_eos<<<blocks(c->nc, T), T, 0, s>>>(c->nc, c->phys.rho[0], c->phys.rho[1], c->phys.mu[0], c->phys.mu[1],
                                               c->VF, c->rho, c->irho, with_mu ? c->mu.p : nullptr);
    SEMO_CHECK_LAUNCH();
    if (c->nb > 0) {
        k_bface_values<<<blocks(c->nb, T), T, 0, s>>>(c->nb, c->ni, c->nf, c->own, c->bpatch, c->bc_type, c->bc_value,
                                                       c->fn, c->P, c->U, c->V, c->W, c->VF, c->phys.rho[0],
                                                       c->phys.rho[1], c->bface);
        SEMO_CHECK_LAUNCH();
    }
}

// Gravity source and the stencil pass, shared by the pressure and momentum
// assemblies.  The momentum pass leaves P and VF unchanged, so after it
// (c->pvf_current) the pressure pass keeps the P and VF gradients and limits
// and the gravity source -- SEMO too computes that source once per time step,
// before its outer loop (src/solvers/pressureBased.cpp:141) -- and recomputes
// only what depends on U, V, W.
void assemble_gravity(semo_ctx* c) {
    const int T = 256;
    cudaStream_t s = c->stream;
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    if (c->phys.use_gravity) {
        StageScope sc(c, ST_GRAVITY);
        k_grav_face<<<blocks(nf, T), T, 0, s>>>(nf, ni, nc, nb, c->own, c->nei, c->fn, c->wc, c->pf, c->nfv, c->U, c->V,
                                                 c->W, c->irho, c->bface, c->phys.gravity[0], c->phys.gravity[1],
                                                 c->phys.gravity[2], c->fscr);
        SEMO_CHECK_LAUNCH();
        k_grav_cell<<<blocks(nc, T), T, 0, s>>>(nc, nf, c->cf_ptr, c->cf_idx, c->fn, c->fa, c->vol, c->fscr, c->sg);
        SEMO_CHECK_LAUNCH();
    } else {
        c->sg.zero();
    }
    c->sg_current = true;
}

void stencil_pass(semo_ctx* c, bool full) {
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    cudaStream_t s = c->stream;
    StageScope sc(c, full ? ST_STENCIL : ST_STENCIL_UVW);
    auto launch = [&](auto kern) {
        kern<<<blocks(nc, 128), 128, 0, s>>>(nc, nf, ni, nb, c->st_ptr, c->st_idx, c->stw, c->st_nnz, c->cf_ptr,
                                             c->cf_idx, c->bfw, c->stws, c->minv, c->P, c->U, c->V, c->W, c->VF, c->bface,
                                             c->grad, c->mm);
    };
    if (full) launch(k_stencil<true>);
    else launch(k_stencil<false>);
    SEMO_CHECK_LAUNCH();
}

void lsq_gradients5(semo_ctx* c, const double* f0, const double* f1, const double* f2, const double* f3,
                    const double* f4, const double* bf, double* grad, double* mm) {
    k_stencil<true><<<blocks(c->nc, 128), 128, 0, c->stream>>>(c->nc, c->nf, c->ni, c->nb, c->st_ptr, c->st_idx,
                                                               c->stw, c->st_nnz, c->cf_ptr, c->cf_idx, c->bfw,
                                                               c->stws, c->minv, f0, f1, f2, f3, f4, bf, grad, mm);
    SEMO_CHECK_LAUNCH();
}

void assemble_gravity_stencil(semo_ctx* c) {
    const bool keep = c->pvf_current;
    if (!keep) assemble_gravity(c);   // else the gravity source is kept
    stencil_pass(c, !keep);
    // the surface-tension source is kept with the gravity source
    if (!keep || (c->phys.sigma != 0.0 && !c->sft_current)) assemble_surface_tension(c);
}

void assemble_pressure(semo_ctx* c) {
    const int T = 256;
    cudaStream_t s = c->stream;
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    assemble_face_values(c, false);
    assemble_gravity_stencil(c);
    double* coef = c->fscr.p;
    double* flux = c->fscr.p + nf;
    if (ni > 0) {
        FaceArgs a;
        a.ni = ni; a.nf = nf; a.nc = nc;
        a.own = c->own; a.nei = c->nei; a.lr = c->A_lr; a.rl = c->A_rl;
        a.fn = c->fn; a.epn = c->epn; a.skew = c->skew; a.alf = c->alf; a.fk = c->fk;
        a.P = c->P; a.U = c->U; a.V = c->V; a.W = c->W; a.irho = c->irho; a.grad = c->grad; a.mm = c->mm; a.sg = c->sg;
        a.dt = c->phys.dt; a.g0 = c->phys.gravity[0]; a.g1 = c->phys.gravity[1]; a.g2 = c->phys.gravity[2];
        a.use_gravity = c->phys.use_gravity;
        set_sft_args(c, a);
        a.val = c->matrix_prebuilt ? nullptr : c->A_val.p;
        a.coef = coef; a.flux = flux; a.unf = c->unf;
        StageScope sc(c, ST_PFACE);
        k_pface<<<blocks(ni, 256), 256, 0, s>>>(a);
        SEMO_CHECK_LAUNCH();
    }
    if (nb > 0) {
        StageScope sc(c, ST_PBFACE);
        k_pbface<<<blocks(nb, T), T, 0, s>>>(nb, ni, nf, nc, c->own, c->bpatch, c->bc_type, c->fn, c->fa, c->mpn,
                                              c->alf, c->epn, c->P, c->grad, c->bface, c->phys.dt, coef, flux, c->unf);
        SEMO_CHECK_LAUNCH();
    }
    StageScope sc(c, ST_PCELL);
    k_pcell<<<blocks(nc, T), T, 0, s>>>(nc, ni, c->cf_ptr, c->cf_idx, c->A_dig, coef, flux,
                                         c->has_src ? c->src.p : nullptr, c->vol,
                                         c->matrix_prebuilt ? nullptr : c->A_val.p, c->b);
    SEMO_CHECK_LAUNCH();
}

void pressure_matrix(semo_ctx* c, cudaStream_t s) {
    const int T = 256;
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    c->pm_coef.alloc(std::max(nf, 1), s);
    if (nf > 0) {
        k_pmat_face<<<blocks(nf, T), T, 0, s>>>(nf, ni, nb, c->own, c->nei, c->A_lr, c->A_rl, c->fk, c->irho,
                                                 c->bpatch, c->bc_type, c->mpn, c->alf, c->fa, c->bface,
                                                 c->phys.dt, c->pm_coef, c->A_val);
        SEMO_CHECK_LAUNCH();
    }
    k_pmat_cell<<<blocks(nc, T), T, 0, s>>>(nc, c->cf_ptr, c->cf_idx, c->A_dig, c->pm_coef, c->A_val);
    SEMO_CHECK_LAUNCH();
}

double pressure_update(semo_ctx* c) {
    c->pvf_current = false;   // P changes below
    const int T = 256;
    cudaStream_t s = c->stream;
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    c->gx.zero();
    double* vF = c->fscr.p;
    for (int it = 0; it < 2; ++it) {
        StageScope sg(c, ST_GG);
        k_gg_face<<<blocks(nf, T), T, 0, s>>>(nf, ni, nc, nb, c->own, c->nei, c->bpatch, c->bc_type, c->wc, c->skew,
                                               c->x, c->gx, vF);
        SEMO_CHECK_LAUNCH();
        k_gg_cell<<<blocks(nc, T), T, 0, s>>>(nc, nf, c->cf_ptr, c->cf_idx, c->fn, c->fa, c->vol, vF, c->gx);
        SEMO_CHECK_LAUNCH();
    }
    c->red.alloc(4 * kRedBlocks + 32, s);
    const semo_physics& p = c->phys;
    StageScope su(c, ST_UPDATE);
    k_update<<<kRedBlocks, kRedThreads, 0, s>>>(nc, p.urf_p, p.urf_u, p.dt, c->x, c->gx, c->irho, c->P, c->U, c->V,
                                                c->W, p.p_min, p.p_max, p.u_min, p.u_max, p.v_min, p.v_max, p.w_min,
                                                p.w_max, c->red);
    SEMO_CHECK_LAUNCH();
    k_finish2<<<1, 256, 0, s>>>(c->red, c->red.p + 2 * kRedBlocks);
    SEMO_CHECK_LAUNCH();
    double* const h = c->hpin;
    SEMO_CUDA(cudaMemcpyAsync(h, c->red.p + 2 * kRedBlocks, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    return std::sqrt(h[0]) / std::sqrt(h[1]);
}

}  // namespace semo
