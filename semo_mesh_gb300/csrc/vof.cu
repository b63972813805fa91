// Volume-fraction sub-iteration on the GPU.
//
// Stages (reference function, file:line):
//   k_cell_eos + k_bface_values + k_stencil  reconIncomZeroOrder, LSQ grad VF and the
//                                            gradients/limits calcVolfracEq forms
//                                            (src/solvers/reconIncom.cpp:345-372,
//                                            src/solvers/eqVolfrac.cpp:27-110)
//   k_courant         cell Courant number    src/solvers/NVD.cpp:1112-1130
//   k_mstacs          MSTACS face values     src/solvers/NVD.cpp:1160-1790
//   k_vface           internal-face loop     src/solvers/eqVolfrac.cpp:262-606
//   k_vbface          boundary-face loop     src/solvers/eqVolfrac.cpp:611-755
//   k_vcell           BDF2 diagonal and RHS + gather of the face terms
//                                            src/solvers/eqVolfrac.cpp:222-260
//   k_vupdate         VF += urf x, clamp to [0,1], norm
//                                            src/solvers/eqVolfrac.cpp:770-793
//
// The matrix lives on the pressure system's CSR pattern like the momentum
// matrix; first-order upwind leaves one off-diagonal per internal face (the
// other is exactly 0 and is dropped, eqVolfrac.cpp:528-545).  Face terms for
// the gather (3 planes of n_faces): internal face: 0 owner diagonal +=,
// 1 neighbour diagonal -=, 2 flux (owner RHS -=, neighbour RHS +=); boundary
// face: 0 owner diagonal +=, 2 owner RHS -=.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>

#include "face_common.cuh"
#include "semo_internal.h"

namespace {

using namespace semo::face;

// |u| dt max(face area) / V per cell (the reference's 1/tmpCFL is 1)
__global__ void k_courant(int nc, double dt, const int* __restrict__ cfp, const int* __restrict__ cfi,
                          const double* __restrict__ fa, const double* __restrict__ vol,
                          const double* __restrict__ U, const double* __restrict__ V,
                          const double* __restrict__ W, double* __restrict__ co) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double magVel = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(U[i], U[i]), __dmul_rn(V[i], V[i])), __dmul_rn(W[i], W[i])));
    double maxA = 0.0;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) maxA = smax(maxA, fa[cfi[k] & kFaceMask]);
    co[i] = magVel * dt * maxA / vol[i];
}

// x^4 rounded once: x^2 = hi + lo exactly (FMA residual), then
// (hi + lo)^2 = hi^2 + 2 hi lo + lo^2 with the last term below half an ulp.
__device__ __forceinline__ double pow4(double x) {
    const double hi = x * x, lo = fma(x, x, -hi);
    const double p = hi * hi, pe = fma(hi, hi, -p);
    return p + (pe + 2.0 * hi * lo);
}

// MSTACS face values of the internal faces (the boundary faces keep their
// zero-order values), written as planes left | right of length ni.
__global__ void __launch_bounds__(256) k_mstacs(int ni, int nf, int nc, const int* __restrict__ own,
                                                const int* __restrict__ nei, const double* __restrict__ VF,
                                                const double* __restrict__ gvf, const double* __restrict__ cc,
                                                const double* __restrict__ wc, const double* __restrict__ fn,
                                                const double* __restrict__ skew, const double* __restrict__ co,
                                                double* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= ni) return;
    const size_t N = nc;
    const int o = own[f], q = nei[f];
    const double eps = 1.e-12;
    const double wCL = wc[f], wCR = 1.0 - wCL;
    const double L1 = VF[o], R1 = VF[q];
    const double dL[3] = {gvf[o], gvf[N + o], gvf[2 * N + o]};
    const double dR[3] = {gvf[q], gvf[N + q], gvf[2 * N + q]};
    const double pn[3] = {cc[q] - cc[o], cc[N + q] - cc[N + o], cc[2 * N + q] - cc[2 * N + o]};
    double L2 = 0.0, R2 = 0.0;
    for (int k = 0; k < 3; ++k) { L2 += dL[k] * pn[k]; R2 += dR[k] * pn[k]; }
    L2 = smax(0.0, smin(1.0, R1 - 2.0 * L2));
    R2 = smax(0.0, smin(1.0, L1 + 2.0 * R2));
    const double coDD = smax(co[o], co[q]);
    const double n[3] = {fn[f], fn[nf + f], fn[2 * nf + f]};
    const double s[3] = {skew[f], skew[nf + f], skew[2 * nf + f]};
    // the blended gradient direction is the same for both sides
    double m[3] = {wCL * dL[0] + wCR * dR[0], wCL * dL[1] + wCR * dR[1], wCL * dL[2] + wCR * dR[2]};
    double mag = m[0] * m[0];
    mag += m[1] * m[1];
    mag += m[2] * m[2];
    mag = sqrt(mag);
    for (int k = 0; k < 3; ++k) m[k] = m[k] / (mag + 1.e-200);
    double cosTheta = m[0] * n[0];
    cosTheta += m[1] * n[1];
    cosTheta += m[2] * n[2];
    const double gamF = smin(pow4(fabs(cosTheta)), 1.0);
    double vf[2] = {L1, R1};
    for (int LR = 0; LR < 2; ++LR) {
        const double own_vf = LR ? R1 : L1;
        if (own_vf > 1.0 - eps || own_vf < eps) continue;
        const double alpU = LR ? R2 : L2, alpD = LR ? R1 : L1, alpA = LR ? L1 : R1;
        const double tildeCd = (alpD - alpU) / (fabs(alpA - alpU) + 1.e-200) * (alpA > alpU ? 1.0 : -1.0);
        const double side = 2.0 * (LR ? wCL : wCR);
        // compressive branch
        double g = 0.0;
        if (tildeCd >= 0.0 && tildeCd < 1.0) {
            if (coDD > 0.0 && coDD <= 0.33) g = (smin(1.0, tildeCd / coDD) - tildeCd) / (1.0 - tildeCd);
            else if (coDD > 0.33 && coDD <= 1.0) g = (smin(1.0, 3.0 * tildeCd) - tildeCd) / (1.0 - tildeCd);
        }
        g = smax(0.0, smin(1.0, g * side));
        double vfC = alpD + g * (alpA - alpD);
        for (int k = 0; k < 3; ++k) vfC += wCL * dL[k] * s[k];
        for (int k = 0; k < 3; ++k) vfC += wCR * dR[k] * s[k];
        vfC = smax(0.0, smin(1.0, vfC));
        // diffusive branch
        double gd;
        if (tildeCd >= 0.0 && tildeCd < 0.2) gd = (smin(1.0, 3.0 * tildeCd) - tildeCd) / (1.0 - tildeCd);
        else if (tildeCd >= 0.2 && tildeCd < 0.5) gd = (0.5 + 0.5 * tildeCd - tildeCd) / (1.0 - tildeCd);
        else if (tildeCd >= 0.5 && tildeCd < 0.8333) gd = (0.375 + 0.75 * tildeCd - tildeCd) / (1.0 - tildeCd);
        else if (tildeCd >= 0.8333 && tildeCd < 1.0) gd = (1.0 - tildeCd) / (1.0 - tildeCd);
        else gd = 0.0;
        gd = smax(0.0, smin(1.0, gd * side));
        double vfD = alpD + gd * (alpA - alpD);
        for (int k = 0; k < 3; ++k) vfD += wCL * dL[k] * s[k];
        for (int k = 0; k < 3; ++k) vfD += wCR * dR[k] * s[k];
        vfD = smax(0.0, smin(1.0, vfD));
        vf[LR] = gamF * vfC + (1.0 - gamF) * vfD;
    }
    out[f] = vf[0];
    out[ni + f] = vf[1];
}

__device__ __forceinline__ double kept(double a) { return (fabs(a) < DBL_MIN) ? 0.0 : a; }

struct VofArgs {
    FaceArgs a;                 // a.val = VOF matrix values
    const double* fvf;          // MSTACS face values, planes left | right of ni
    double* sc;                 // 3 planes of nf
};

__global__ void __launch_bounds__(256) k_vface(VofArgs m) {
    const FaceArgs& a = m.a;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.ni) return;
    const int o = a.own[f], q = a.nei[f];
    const FaceGeo g = load_geo(a, f);
    const double UnF = face_unf(a, g, o, q);
    const double wLu = (UnF > 0.0) ? 1.0 : 0.0, wRu = 1.0 - wLu;
    const double vff = wLu * m.fvf[f] + wRu * m.fvf[a.ni + f];
    const double mf = UnF * g.area;
    a.val[a.lr[f]] = kept(wRu * mf);
    a.val[a.rl[f]] = kept(-(wLu * mf));
    const size_t NF = a.nf;
    m.sc[f] = wLu * mf;
    m.sc[NF + f] = wRu * mf;
    m.sc[2 * NF + f] = vff * mf;
}

__global__ void k_vbface(int nb, int ni, int nf, int nc, const int* __restrict__ own, const int* __restrict__ bpatch,
                         const int* __restrict__ bct, const double* __restrict__ fn, const double* __restrict__ fa,
                         const double* __restrict__ mpn, const double* __restrict__ alf,
                         const double* __restrict__ epn, const double* __restrict__ P,
                         const double* __restrict__ grad, const double* __restrict__ bf, double dt,
                         double* __restrict__ sc) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int f = ni + b, o = own[f], p = bpatch[b];
    const double n0 = fn[f], n1 = fn[nf + f], n2 = fn[2 * nf + f], area = fa[f];
    const double u = bf[nb + b], v = bf[2 * nb + b], w = bf[3 * nb + b];
    const double UnL = u * n0 + v * n1 + w * n2;
    double UnF = 0.5 * UnL + 0.5 * UnL;
    const double tmp1 = 1.0 / bf[5 * nb + b] * dt;
    const double vff = 0.5 * bf[4 * nb + b] + 0.5 * bf[4 * nb + b];
    const double coeff = (bct[3 * p + 2] == SEMO_BC_FIXED_VALUE) ? 0.0 : 1.0;
    const double dPN = 0.5 * mpn[f], alpha = alf[f];
    if (bct[3 * p] == SEMO_BC_FIXED_VALUE) {
        UnF -= alpha * tmp1 * (bf[b] - P[o]) / dPN;
        UnF += alpha * tmp1 * grad[o] * epn[f];
        UnF += alpha * tmp1 * grad[nc + o] * epn[nf + f];
        UnF += alpha * tmp1 * grad[2 * (size_t)nc + o] * epn[2 * nf + f];
    }
    sc[f] = coeff * (UnF * area);
    sc[2 * (size_t)nf + f] = vff * UnF * area;
}

__global__ void k_vcell(int nc, int ni, int nf, double dt, const int* __restrict__ cfp, const int* __restrict__ cfi,
                        const int* __restrict__ dig, const double* __restrict__ vol, const double* __restrict__ VF,
                        const double* __restrict__ old, int has_old, const double* __restrict__ sc,
                        double* __restrict__ val, double* __restrict__ bv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const size_t N = nc, NF = nf;
    const double v = vol[i], cur = VF[i];
    const double o1 = has_old ? old[i] : cur, o2 = has_old ? old[N + i] : cur;
    double d = 1.5 * v / dt;
    double b = -(1.5 * cur - 2.0 * o1 + 0.5 * o2) * v / dt;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int e = cfi[k], f = e & kFaceMask;
        if (f < ni && (e >> 30)) {
            d -= sc[NF + f];
            b += sc[2 * NF + f];
        } else {
            d += sc[f];
            b -= sc[2 * NF + f];
        }
    }
    val[dig[i]] = d;
    bv[i] = b;
}

__global__ void __launch_bounds__(kRedThreads) k_vupdate(int nc, double urf, const double* __restrict__ x,
                                                         double* __restrict__ VF, double* __restrict__ part) {
    __shared__ double sh[32];
    double nd = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
        const double xi = x[i];
        VF[i] = smax(0.0, smin(1.0, VF[i] + urf * xi));
        nd += xi * xi;
    }
    nd = block_sum(nd, sh);
    if (threadIdx.x == 0) { part[blockIdx.x] = nd; part[kRedBlocks + blockIdx.x] = 0.0; }
}

}  // namespace

namespace semo {

void assemble_vof(semo_ctx* c) {
    const int T = 256;
    cudaStream_t s = c->stream;
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    assemble_face_values(c, false);
    // the gravity and surface-tension sources are the time step's (computed
    // once, as SEMO does before its outer loop)
    const bool fresh = !c->sg_current;
    if (fresh) assemble_gravity(c);
    stencil_pass(c, true);
    if (fresh || (c->phys.sigma != 0.0 && !c->sft_current)) assemble_surface_tension(c);
    c->co.alloc(nc, s);
    c->fvf.alloc(2 * (size_t)std::max(ni, 1), s);
    c->Av_val.alloc(c->nnz, s);
    c->bvf.alloc(nc, s);
    c->vsc.alloc(3 * (size_t)nf, s);
    {
        StageScope sc(c, ST_MSTACS);
        k_courant<<<blocks(nc, T), T, 0, s>>>(nc, c->phys.dt, c->cf_ptr, c->cf_idx, c->fa, c->vol, c->U, c->V, c->W,
                                               c->co);
        SEMO_CHECK_LAUNCH();
        if (ni > 0) {
            k_mstacs<<<blocks(ni, 256), 256, 0, s>>>(ni, nf, nc, c->own, c->nei, c->VF, c->grad.p + 12 * (size_t)nc,
                                                      c->cc, c->wc, c->fn, c->skew, c->co, c->fvf);
            SEMO_CHECK_LAUNCH();
        }
    }
    StageScope sc(c, ST_VFACE);
    if (ni > 0) {
        VofArgs m;
        FaceArgs& a = m.a;
        a.ni = ni; a.nf = nf; a.nc = nc;
        a.own = c->own; a.nei = c->nei; a.lr = c->A_lr; a.rl = c->A_rl;
        a.fn = c->fn; a.epn = c->epn; a.skew = c->skew; a.alf = c->alf; a.fk = c->fk;
        a.P = c->P; a.U = c->U; a.V = c->V; a.W = c->W; a.irho = c->irho; a.grad = c->grad; a.mm = c->mm; a.sg = c->sg;
        a.dt = c->phys.dt; a.g0 = c->phys.gravity[0]; a.g1 = c->phys.gravity[1]; a.g2 = c->phys.gravity[2];
        a.use_gravity = c->phys.use_gravity;
        set_sft_args(c, a);
        a.val = c->Av_val; a.coef = nullptr; a.flux = nullptr; a.unf = nullptr;
        m.fvf = c->fvf; m.sc = c->vsc;
        k_vface<<<blocks(ni, 256), 256, 0, s>>>(m);
        SEMO_CHECK_LAUNCH();
    }
    if (nb > 0) {
        k_vbface<<<blocks(nb, T), T, 0, s>>>(nb, ni, nf, nc, c->own, c->bpatch, c->bc_type, c->fn, c->fa, c->mpn,
                                              c->alf, c->epn, c->P, c->grad, c->bface, c->phys.dt, c->vsc);
        SEMO_CHECK_LAUNCH();
    }
    k_vcell<<<blocks(nc, T), T, 0, s>>>(nc, ni, nf, c->phys.dt, c->cf_ptr, c->cf_idx, c->A_dig, c->vol, c->VF,
                                         c->has_oldvf ? c->oldvf.p : nullptr, c->has_oldvf ? 1 : 0, c->vsc, c->Av_val,
                                         c->bvf);
    SEMO_CHECK_LAUNCH();
}

double vof_update(semo_ctx* c) {
    cudaStream_t s = c->stream;
    c->red.alloc(4 * kRedBlocks + 32, s);
    StageScope su(c, ST_VUPDATE);
    k_vupdate<<<kRedBlocks, kRedThreads, 0, s>>>(c->nc, c->phys.urf_vof, c->xvf, c->VF, c->red);
    SEMO_CHECK_LAUNCH();
    face::k_finish2<<<1, 256, 0, s>>>(c->red, c->red.p + 2 * kRedBlocks);
    SEMO_CHECK_LAUNCH();
    double* const h = c->hpin;
    SEMO_CUDA(cudaMemcpyAsync(h, c->red.p + 2 * kRedBlocks, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    c->pvf_current = false;   // VF changed
    c->assembled = c->mom_assembled = false;
    return std::sqrt(h[0]);
}

}  // namespace semo
