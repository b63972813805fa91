// Momentum equation assembly and update on the GPU.
//
// Stages (reference function, file:line):
//   k_cell_eos (mu)   calcCellTransport, laminar   src/solvers/transport.cpp:9-98
//   k_stencil         setCellVarMinMax P,U,V,W + calcLeastSquare x5 (shared with the pressure pass)
//                                                  src/solvers/eqMomentum.cpp:40-105
//   k_mface           internal-face loop           src/solvers/eqMomentum.cpp:331-787
//   k_mbface          boundary-face loop           src/solvers/eqMomentum.cpp:795-1008
//   k_mcell           BDF2 diagonal and RHS + gather of the face terms
//                                                  src/solvers/eqMomentum.cpp:223-326
//   k_mupdate         U,V,W += urf x, clamps, norm src/solvers/eqMomentum.cpp:1029-1119
//
// One matrix serves the three velocity components.  It lives on the pressure
// system's CSR pattern (RCM rows, SEMO in-row order): the face kernel writes
// each internal face's two off-diagonals straight into their slots, with the
// value 0 where SEMO leaves the entry out (|a| < DBL_MIN, eqMomentum.cpp:
// 699-711).  The diagonal and the three right-hand sides are gathered per cell
// from per-face terms in ascending face order, SEMO's accumulation order,
// without atomics.  Face terms (8 planes of n_faces):
//   internal face: 0 owner diagonal +=, 1 neighbour diagonal -=,
//                  2-4 owner RHS -= (x,y,z), 5-7 neighbour RHS += (x,y,z)
//   boundary face: 0 and 1 owner diagonal += (convective, viscous),
//                  2-4 owner RHS -= (x,y,z)
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>

#include "face_common.cuh"
#include "semo_internal.h"

namespace {

using namespace semo::face;

struct MomArgs {
    FaceArgs a;                 // a.mm has 10 planes (P limits in 8, 9); a.val = momentum values
    const double *rho, *mu;
    double* sc;
};

__device__ __forceinline__ double kept(double a) { return (fabs(a) < DBL_MIN) ? 0.0 : a; }

__global__ void __launch_bounds__(256) k_mface(MomArgs m) {
    const FaceArgs& a = m.a;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.ni) return;
    const int o = a.own[f], q = a.nei[f];
    const FaceGeo g = load_geo(a, f);
    const double UnF = face_unf(a, g, o, q);
    const size_t N = a.nc, NF = a.nf;
    const double* G = a.grad;
    const double* M = a.mm;
    const double RhoL = __ldg(m.rho + o), RhoR = __ldg(m.rho + q);
    // harmonic viscosity (eqMomentum.cpp:373) from the cells' reciprocals (plane 1 of mu)
    const double muF = 1.0 / (g.wL * __ldg(m.mu + N + o) + g.wR * __ldg(m.mu + N + q));
    // first-order upwind on UnF (eqMomentum.cpp:613-620)
    // face pressure, skew-corrected and limited by both cells (eqMomentum.cpp:617-659)
    double PF = g.wL * __ldg(a.P + o) + g.wR * __ldg(a.P + q);
    PF += g.wL * __ldg(G + o) * g.s0;
    PF += g.wR * __ldg(G + q) * g.s0;
    PF += g.wL * __ldg(G + N + o) * g.s1;
    PF += g.wR * __ldg(G + N + q) * g.s1;
    PF += g.wL * __ldg(G + 2 * N + o) * g.s2;
    PF += g.wR * __ldg(G + 2 * N + q) * g.s2;
    PF = clamp_k(PF, __ldg(M + 9 * N + o), __ldg(M + 8 * N + o));
    PF = clamp_k(PF, __ldg(M + 9 * N + q), __ldg(M + 8 * N + q));
    const double UL = __ldg(a.U + o), VL = __ldg(a.V + o), WL = __ldg(a.W + o);
    const double UR = __ldg(a.U + q), VR = __ldg(a.V + q), WR = __ldg(a.W + q);
    // the upwind weights are 0 or 1: selections, not FP64 arithmetic
    const bool up = UnF > 0.0;
    const double UF = up ? UL : UR, VFh = up ? VL : VR, WFh = up ? WL : WR;
    const double area = g.area, mf = UnF * area;
    const double ad = muF * g.kA;   // alpha muF / |PN| * area
    const double rlm = RhoL * mf, rrm = RhoR * mf;
    // coefficients (eqMomentum.cpp:694-712)
    const double dO = up ? rlm + ad : ad;
    const double dN = up ? -ad : rrm - ad;
    a.val[a.lr[f]] = kept(up ? -ad : rlm - ad);
    a.val[a.rl[f]] = kept(up ? -(rrm + ad) : -ad);
    // convection + pressure, over-relaxed diffusion with its non-orthogonal
    // part on (n - alpha e), and SEMO's extra grad.n term (eqMomentum.cpp:739-779)
    const double t0 = g.n0 - g.ae0, t1 = g.n1 - g.ae1, t2 = g.n2 - g.ae2;
    const double ma = muF * area, pa = PF * area;
    double* sc = m.sc;
    sc[f] = dO;
    sc[NF + f] = dN;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double* Gc = G + (size_t)(3 + 3 * c) * N;   // grad U, V, W
        const double gl0 = __ldg(Gc + o), gl1 = __ldg(Gc + N + o), gl2 = __ldg(Gc + 2 * N + o);
        const double gr0 = __ldg(Gc + q), gr1 = __ldg(Gc + N + q), gr2 = __ldg(Gc + 2 * N + q);
        const double uf = (c == 0) ? UF : (c == 1 ? VFh : WFh);
        const double dl = (c == 0) ? UR - UL : (c == 1 ? VR - VL : WR - WL);
        const double nc = (c == 0) ? g.n0 : (c == 1 ? g.n1 : g.n2);
        const double pn = pa * nc;
        // (wL gL + wR gR).t = wL (gL.t) + wR (gR.t): the projections serve both terms
        const double glt = gl0 * t0 + gl1 * t1 + gl2 * t2, grt = gr0 * t0 + gr1 * t1 + gr2 * t2;
        const double diff = ad * dl + ma * (g.wL * glt + g.wR * grt);
        const double dLn = ma * (gl0 * g.n0 + gl1 * g.n1 + gl2 * g.n2);
        const double dRn = ma * (gr0 * g.n0 + gr1 * g.n1 + gr2 * g.n2);
        sc[(2 + c) * NF + f] = (rlm * uf + pn) - diff - dLn;
        sc[(5 + c) * NF + f] = (rrm * uf + pn) - diff - dRn;
    }
}

__global__ void k_mbface(int nb, int ni, int nf, int nc, const int* __restrict__ own, const int* __restrict__ bpatch,
                         const int* __restrict__ bct, const double* __restrict__ fn, const double* __restrict__ fa,
                         const double* __restrict__ mpn, const double* __restrict__ alf,
                         const double* __restrict__ epn, const double* __restrict__ P, const double* __restrict__ U,
                         const double* __restrict__ V, const double* __restrict__ W, const double* __restrict__ mu,
                         const double* __restrict__ grad, const double* __restrict__ bf, double dt,
                         double* __restrict__ sc) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int f = ni + b, o = own[f], p = bpatch[b];
    const size_t N = nc;
    const double n[3] = {fn[f], fn[nf + f], fn[2 * nf + f]};
    const double e[3] = {epn[f], epn[nf + f], epn[2 * nf + f]};
    const double area = fa[f];
    // boundary values: left == right for every supported condition
    const double ub[3] = {bf[nb + b], bf[2 * nb + b], bf[3 * nb + b]};
    const double uc[3] = {U[o], V[o], W[o]};
    const double UnL = ub[0] * n[0] + ub[1] * n[1] + ub[2] * n[2];
    double UnF = 0.5 * UnL + 0.5 * UnL;
    const double RhoL = bf[5 * nb + b];
    const double tmp1 = 1.0 / RhoL * dt;
    const double PF = 0.5 * bf[b] + 0.5 * bf[b];
    const int tu = bct[3 * p + 1];
    double cU, cUd;
    if (tu == SEMO_BC_FIXED_VALUE) { cU = 0.0; cUd = 1.0; }
    else if (tu == SEMO_BC_ZERO_GRADIENT) { cU = 1.0; cUd = 0.0; }
    else if (tu == SEMO_BC_SLIP) { cU = 0.0; cUd = 0.0; }
    else { cU = 0.0; cUd = 1.0; }   // noSlip
    const double muF = 0.5 * mu[o] + 0.5 * mu[o];
    const double dPN = 0.5 * mpn[f], alpha = alf[f];
    if (bct[3 * p] == SEMO_BC_FIXED_VALUE) {
        UnF -= alpha * tmp1 * (bf[b] - P[o]) / dPN;
        for (int k = 0; k < 3; ++k) UnF += alpha * tmp1 * grad[k * N + o] * e[k];
    }
    sc[f] = cU * (RhoL * UnF * area);
    sc[nf + f] = cUd * (muF * alpha / dPN * area);
    for (int c = 0; c < 3; ++c) {
        const double* Gc = grad + (size_t)(3 + 3 * c) * N;
        double d = alpha * (ub[c] - uc[c]) / dPN;
        for (int k = 0; k < 3; ++k) d += Gc[k * N + o] * (n[k] - alpha * e[k]);
        for (int k = 0; k < 3; ++k) d += Gc[k * N + o] * n[k];
        sc[(2 + c) * (size_t)nf + f] = RhoL * ub[c] * UnF * area + PF * n[c] * area - muF * d * area;
    }
}

__global__ void k_mcell(int nc, int ni, int nf, double dt, const int* __restrict__ cfp, const int* __restrict__ cfi,
                        const int* __restrict__ dig, const double* __restrict__ rho, const double* __restrict__ vol,
                        const double* __restrict__ U, const double* __restrict__ V, const double* __restrict__ W,
                        const double* __restrict__ old, int has_old, const double* __restrict__ sg,
                        const double* __restrict__ sft, const double* __restrict__ sc, double* __restrict__ val,
                        double* __restrict__ bm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const size_t N = nc, NF = nf;
    const double r = rho[i], v = vol[i];
    const double cur[3] = {U[i], V[i], W[i]};
    double d = r * 1.5 * v / dt;
    double b[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double o1 = has_old ? old[c * N + i] : cur[c];
        const double o2 = has_old ? old[(3 + c) * N + i] : cur[c];
        b[c] = -r * (1.5 * cur[c] - 2.0 * o1 + 0.5 * o2) * v / dt;
        b[c] += v * sg[c * N + i];
        if (sft) b[c] += v * sft[c * N + i];   // surface tension (eqMomentum.cpp:320-322)
    }
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int e = cfi[k], f = e & kFaceMask;
        if (f < ni) {
            if (e >> 30) {
                d -= sc[NF + f];
                b[0] += sc[5 * NF + f]; b[1] += sc[6 * NF + f]; b[2] += sc[7 * NF + f];
            } else {
                d += sc[f];
                b[0] -= sc[2 * NF + f]; b[1] -= sc[3 * NF + f]; b[2] -= sc[4 * NF + f];
            }
        } else {
            d += sc[f];
            d += sc[NF + f];
            b[0] -= sc[2 * NF + f]; b[1] -= sc[3 * NF + f]; b[2] -= sc[4 * NF + f];
        }
    }
    val[dig[i]] = d;
    bm[i] = b[0]; bm[N + i] = b[1]; bm[2 * N + i] = b[2];
}

__global__ void __launch_bounds__(kRedThreads) k_mupdate(int nc, double urf, const double* __restrict__ x,
                                                         double* __restrict__ U, double* __restrict__ V,
                                                         double* __restrict__ W, double umin, double umax,
                                                         double vmin, double vmax, double wmin, double wmax,
                                                         double* __restrict__ part) {
    __shared__ double sh[32];
    const size_t N = nc;
    double nd = 0.0, np = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
        const double x0 = x[i], x1 = x[N + i], x2 = x[2 * N + i];
        double u = U[i] + urf * x0, v = V[i] + urf * x1, w = W[i] + urf * x2;
        if (u <= umin) u = umin;
        if (u >= umax) u = umax;
        if (v <= vmin) v = vmin;
        if (v >= vmax) v = vmax;
        if (w <= wmin) w = wmin;
        if (w >= wmax) w = wmax;
        U[i] = u; V[i] = v; W[i] = w;
        nd += x0 * x0 + x1 * x1 + x2 * x2;
        np += u * u + v * v + w * w;
    }
    nd = block_sum(nd, sh);
    np = block_sum(np, sh);
    if (threadIdx.x == 0) { part[blockIdx.x] = nd; part[kRedBlocks + blockIdx.x] = np; }
}

}  // namespace

namespace semo {

void assemble_momentum(semo_ctx* c, bool face_values_done) {
    const int T = 256;
    cudaStream_t s = c->stream;
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    if (!face_values_done) assemble_face_values(c, true);
    c->pvf_current = false;
    assemble_gravity_stencil(c);
    c->pvf_current = true;
    c->Am_val.alloc(c->nnz, s);
    c->bm.alloc(3 * (size_t)nc, s);
    c->msc.alloc(8 * (size_t)nf, s);
    if (ni > 0) {
        MomArgs m;
        FaceArgs& a = m.a;
        a.ni = ni; a.nf = nf; a.nc = nc;
        a.own = c->own; a.nei = c->nei; a.lr = c->A_lr; a.rl = c->A_rl;
        a.fn = c->fn; a.epn = c->epn; a.skew = c->skew; a.alf = c->alf; a.fk = c->fk;
        a.P = c->P; a.U = c->U; a.V = c->V; a.W = c->W; a.irho = c->irho; a.grad = c->grad; a.mm = c->mm; a.sg = c->sg;
        a.dt = c->phys.dt; a.g0 = c->phys.gravity[0]; a.g1 = c->phys.gravity[1]; a.g2 = c->phys.gravity[2];
        a.use_gravity = c->phys.use_gravity;
        set_sft_args(c, a);
        a.val = c->Am_val; a.coef = nullptr; a.flux = nullptr; a.unf = nullptr;
        m.rho = c->rho; m.mu = c->mu; m.sc = c->msc;
        StageScope sc(c, ST_MFACE);
        k_mface<<<blocks(ni, 256), 256, 0, s>>>(m);
        SEMO_CHECK_LAUNCH();
    }
    if (nb > 0) {
        StageScope sc(c, ST_MBFACE);
        k_mbface<<<blocks(nb, T), T, 0, s>>>(nb, ni, nf, nc, c->own, c->bpatch, c->bc_type, c->fn, c->fa, c->mpn,
                                              c->alf, c->epn, c->P, c->U, c->V, c->W, c->mu, c->grad, c->bface,
                                              c->phys.dt, c->msc);
        SEMO_CHECK_LAUNCH();
    }
    StageScope sc(c, ST_MCELL);
    k_mcell<<<blocks(nc, T), T, 0, s>>>(nc, ni, nf, c->phys.dt, c->cf_ptr, c->cf_idx, c->A_dig, c->rho, c->vol,
                                         c->U, c->V, c->W, c->has_old ? c->old.p : nullptr, c->has_old ? 1 : 0,
                                         c->sg, (c->phys.sigma != 0.0 && c->sft_current) ? c->sft.p + 2 * (size_t)nc : nullptr,
                                         c->msc, c->Am_val, c->bm);
    SEMO_CHECK_LAUNCH();
}

double momentum_update(semo_ctx* c) {
    cudaStream_t s = c->stream;
    c->red.alloc(4 * kRedBlocks + 32, s);
    const semo_physics& p = c->phys;
    StageScope su(c, ST_MUPDATE);
    k_mupdate<<<kRedBlocks, kRedThreads, 0, s>>>(c->nc, p.urf_mom, c->xm, c->U, c->V, c->W, p.u_min, p.u_max,
                                                 p.v_min, p.v_max, p.w_min, p.w_max, c->red);
    SEMO_CHECK_LAUNCH();
    face::k_finish2<<<1, 256, 0, s>>>(c->red, c->red.p + 2 * kRedBlocks);
    SEMO_CHECK_LAUNCH();
    double* const h = c->hpin;
    SEMO_CUDA(cudaMemcpyAsync(h, c->red.p + 2 * kRedBlocks, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    return std::sqrt(h[0]) / std::sqrt(h[1]);
}

}  // namespace semo
