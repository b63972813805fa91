// Device helpers shared by the pressure (assemble.cu) and momentum
// (momentum.cu) face kernels: value ordering for min/max, std::min/max
// semantics, and the face-normal velocity UnF that both equations build the
// same way (skew-corrected, stencil-limited interpolation plus the pressure and
// gravity Rhie-Chow terms of src/solvers/surfaceNormalVelocity.cpp:100-187).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace semo {
namespace face {

constexpr int kFaceMask = 0x3FFFFFFF;   // cell->face list entry: face index; bit 30 = neighbour side
inline int blocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

// Order-preserving int64 image of a double (for min/max on the integer
// pipes instead of the FP64 unit); the map is its own inverse.
__device__ __forceinline__ long long okey(double x) {
    long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ double ounkey(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL));
}
// std::max(a,b) = (a<b)?b:a ; std::min(a,b) = (b<a)?b:a
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double clamp01(double x) { return smax(0.0, smin(1.0, x)); }
// std::max(lo, std::min(hi, x)) with the comparisons on the integer pipes
// (order-preserving keys); the FP64 pipe is the bottleneck of the face kernels.
// Differs from the double compares only in the sign of a zero result.
__device__ __forceinline__ double clamp_k(double x, double lo, double hi) {
    long long k = okey(x);
    const long long kh = okey(hi), kl = okey(lo);
    k = (k < kh) ? k : kh;
    k = (kl < k) ? k : kl;
    return ounkey(k);
}

// Fixed-grid reductions: kRedBlocks partial sums summed by one block, so
// every sum has the same order run to run.
constexpr int kRedBlocks = 608;   // 4 x 152 SMs
constexpr int kRedThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = 0.0;
    if (threadIdx.x < 32) {
        v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;
}

// out[0] = sum of part[0..kRedBlocks), out[1] = sum of the next kRedBlocks (one block)
__global__ void k_finish2(const double* __restrict__ part, double* __restrict__ out);

// Inputs of the internal-face velocity.  Cells in RCM order, faces in stored
// order; grad holds 15 planes (P,U,V,W,VF x xyz) and mm the stencil limits
// (maxU,minU,maxV,minV,maxW,minW,... planes of nc); fk 4 planes of ni:
// alpha*area/|PN|, alpha/|PN|, area, wC.
struct FaceArgs {
    int ni, nf, nc;
    const int *own, *nei, *lr, *rl;
    const double *fn, *epn, *skew, *alf, *fk;
    const double *P, *U, *V, *W, *irho, *grad, *mm, *sg;
    const double *VF, *kap, *ss;   // surface tension: cell VF, curvature, source (4 planes of nc)
    double dt, g0, g1, g2, sigma;
    int use_gravity, use_sft;
    double *val, *coef, *flux, *unf;
};

// Surface-tension inputs of the face velocity from a context (semo_ctx):
// cell VF, curvature and source planes, used when sigma != 0.
template <class Ctx>
inline void set_sft_args(const Ctx* c, FaceArgs& a) {
    a.sigma = c->phys.sigma;
    a.use_sft = (c->phys.sigma != 0.0 && c->sft_current) ? 1 : 0;
    a.VF = c->VF.p;
    a.kap = a.use_sft ? c->sft.p : nullptr;
    a.ss = a.use_sft ? c->sft.p + 2 * (size_t)c->nc : nullptr;
}

struct FaceGeo {
    double n0, n1, n2, s0, s1, s2, alpha, ae0, ae1, ae2, kA, kP, area, wL, wR;
};

__device__ __forceinline__ FaceGeo load_geo(const FaceArgs& a, int f) {
    FaceGeo g;
    const int nf = a.nf, ni = a.ni;
    g.n0 = a.fn[f]; g.n1 = a.fn[nf + f]; g.n2 = a.fn[2 * nf + f];
    g.s0 = a.skew[f]; g.s1 = a.skew[nf + f]; g.s2 = a.skew[2 * nf + f];
    g.alpha = a.alf[f];
    g.ae0 = g.alpha * a.epn[f]; g.ae1 = g.alpha * a.epn[nf + f]; g.ae2 = g.alpha * a.epn[2 * nf + f];
    g.kA = a.fk[f]; g.kP = a.fk[ni + f]; g.area = a.fk[2 * ni + f]; g.wL = a.fk[3 * ni + f];
    g.wR = 1.0 - g.wL;
    return g;
}

// UnF of internal face (o, q): skew-corrected velocities clamped to the
// stencil limits (eqPressure.cpp:416-451, eqMomentum.cpp:519-553), weighted
// by wC, then the pressure (surfaceNormalVelocity.cpp:125-155) and gravity
// (:156-187) Rhie-Chow terms.  Those are evaluated in reduced form:
// (dt/rho*)*rho* = dt, and the (n - alpha e) and n pieces of the
// non-orthogonal correction combine to alpha e; agreement with SEMO's
// operation order is to rounding (a few ulp), not bit-for-bit.  With sigma
// != 0 the surface-tension terms (:190-221) follow, reduced the same way:
// alpha (dt/rho*) sigma (wL kL + wR kR) (VF_R - VF_L)/|PN| and the source's
// non-orthogonal part.
__device__ __forceinline__ double face_unf(const FaceArgs& a, const FaceGeo& g, int o, int q) {
    const size_t N = a.nc;
    const double* G = a.grad;
    const double iRL = __ldg(a.irho + o), iRR = __ldg(a.irho + q);
    double ul = __ldg(a.U + o) + __ldg(G + 3 * N + o) * g.s0 + __ldg(G + 4 * N + o) * g.s1 + __ldg(G + 5 * N + o) * g.s2;
    double vl = __ldg(a.V + o) + __ldg(G + 6 * N + o) * g.s0 + __ldg(G + 7 * N + o) * g.s1 + __ldg(G + 8 * N + o) * g.s2;
    double wl = __ldg(a.W + o) + __ldg(G + 9 * N + o) * g.s0 + __ldg(G + 10 * N + o) * g.s1 + __ldg(G + 11 * N + o) * g.s2;
    double ur = __ldg(a.U + q) + __ldg(G + 3 * N + q) * g.s0 + __ldg(G + 4 * N + q) * g.s1 + __ldg(G + 5 * N + q) * g.s2;
    double vr = __ldg(a.V + q) + __ldg(G + 6 * N + q) * g.s0 + __ldg(G + 7 * N + q) * g.s1 + __ldg(G + 8 * N + q) * g.s2;
    double wr = __ldg(a.W + q) + __ldg(G + 9 * N + q) * g.s0 + __ldg(G + 10 * N + q) * g.s1 + __ldg(G + 11 * N + q) * g.s2;
    const double* M = a.mm;
    ul = clamp_k(ul, __ldg(M + N + o), __ldg(M + o));
    ur = clamp_k(ur, __ldg(M + N + q), __ldg(M + q));
    vl = clamp_k(vl, __ldg(M + 3 * N + o), __ldg(M + 2 * N + o));
    vr = clamp_k(vr, __ldg(M + 3 * N + q), __ldg(M + 2 * N + q));
    wl = clamp_k(wl, __ldg(M + 5 * N + o), __ldg(M + 4 * N + o));
    wr = clamp_k(wr, __ldg(M + 5 * N + q), __ldg(M + 4 * N + q));
    const double UnL = ul * g.n0 + vl * g.n1 + wl * g.n2;
    const double UnR = ur * g.n0 + vr * g.n1 + wr * g.n2;
    double UnF = g.wL * UnL + g.wR * UnR;
    const double tt = a.dt * (g.wL * iRL + g.wR * iRR);
    UnF -= tt * g.kP * (__ldg(a.P + q) - __ldg(a.P + o));
    const double aL = a.dt * g.wL * iRL, aR = a.dt * g.wR * iRR;
    UnF += aL * (__ldg(G + o) * g.ae0 + __ldg(G + N + o) * g.ae1 + __ldg(G + 2 * N + o) * g.ae2);
    UnF += aR * (__ldg(G + q) * g.ae0 + __ldg(G + N + q) * g.ae1 + __ldg(G + 2 * N + q) * g.ae2);
    const double t0 = g.n0 - g.ae0 - g.alpha * g.n0, t1 = g.n1 - g.ae1 - g.alpha * g.n1;
    const double t2 = g.n2 - g.ae2 - g.alpha * g.n2;
    if (a.use_gravity) {
        UnF += a.dt * g.alpha * (a.g0 * g.ae0 + a.g1 * g.ae1 + a.g2 * g.ae2);
        const double* S = a.sg;
        UnF += aL * (__ldg(S + o) * t0 + __ldg(S + N + o) * t1 + __ldg(S + 2 * N + o) * t2);
        UnF += aR * (__ldg(S + q) * t0 + __ldg(S + N + q) * t1 + __ldg(S + 2 * N + q) * t2);
    }
    if (a.use_sft) {
        const double kf = g.wL * __ldg(a.kap + o) + g.wR * __ldg(a.kap + q);
        UnF += tt * g.kP * a.sigma * kf * (__ldg(a.VF + q) - __ldg(a.VF + o));
        const double* S = a.ss;
        UnF += aL * (__ldg(S + o) * t0 + __ldg(S + N + o) * t1 + __ldg(S + 2 * N + o) * t2);
        UnF += aR * (__ldg(S + q) * t0 + __ldg(S + N + q) * t1 + __ldg(S + 2 * N + q) * t2);
    }
    return UnF;
}

}  // namespace face
}  // namespace semo
