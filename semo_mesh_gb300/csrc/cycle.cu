// Applying the AMG hierarchy: V-cycle and the outer flexible CG.
//
// Replaces the solve half of SEMO's solveAMGCL (src/solvers/solveAMGCL.cpp:
// 974-980, AMGCL's V-cycle lib/amgcl/mpi/amg.hpp:343-380 and its Krylov
// loop).  The hierarchy is built by amg_setup.cu.
//
// Layout and kernels, GB300-first:
//  * the finest level and the FP64 outer operator are stored SELL-32 (slices
//    of 32 rows, column-major inside a slice, padded to the slice's longest
//    row): one thread per row, every load coalesced.  Rows there have ~7
//    entries, so a warp-per-row or sub-warp CSR kernel is latency-bound;
//    coarse levels (27-60 entries a row) stay CSR with 4-32 lanes a row;
//  * degree-2 Chebyshev smoothing is fused: pre-smoothing from a zero guess
//    is one kernel (the first iterate D^-1 b / theta is formed on the fly
//    for the neighbours), post-smoothing is two, with no separate x += d;
//  * the CG update uses q = A z + beta q (so p and q update in place) and
//    the dot products are folded into the kernels that produce their
//    operands; one CG iteration is ~30 launches, captured as a CUDA graph.
// FP32 V-cycle arithmetic stays on the FP32 pipes (FP64 is 1/58 of FP32
// on GB300); dot products and the outer residual are FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "semo_internal.h"

namespace semo {
namespace {

// Grid of the kernels that end in a reduction (dot products fused into the
// SpMVs and vector updates), grid-stride: a fixed 608-way partition of the
// rows, one partial sum per block, summed in a fixed order.  608 is 4 blocks
// of 256 per multiprocessor on GB300's 152 (measured faster here than 16 a
// multiprocessor); it is not taken from the device so that the partition,
// and with it every sum's bits, is the same on any GPU.
constexpr int kRedBlocks = 608;
constexpr int kRedThreads = 256;
inline int blocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = 0.0;
    if (threadIdx.x < 32) {
        v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
        v = warp_sum(v);
    }
    __syncthreads();
    return v;
}

// ------------------------------------------------------------ matrix views
// CSR with VS lanes per row.
template <class V, int VS>
struct CsrView {
    static constexpr int kVS = VS;
    const int* __restrict__ ptr;
    const int* __restrict__ col;
    const V* __restrict__ val;
    int n;
    template <class F>
    __device__ __forceinline__ V dot(int row, int lane, const F& x) const {
        V s = V(0);
        if (row < n) {
            const int e = ptr[row + 1];
            for (int k = ptr[row] + lane; k < e; k += VS) s += val[k] * x(col[k]);
        }
#pragma unroll
        for (int o = VS / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, VS);
        return s;
    }
};

// SELL-32: slice s holds rows 32s..32s+31; entry j of row 32s+l at
// sptr[s] + 32j + l; padding entries point at column 0 with value 0.
template <class V>
struct SellView {
    static constexpr int kVS = 1;
    const int* __restrict__ sptr;
    const int* __restrict__ col;
    const V* __restrict__ val;
    int n;
    template <class F>
    __device__ __forceinline__ V dot(int row, int, const F& x) const {
        V s = V(0);
        if (row < n) {
            const int sl = row >> 5, l = row & 31;
            const int b = sptr[sl], w = (sptr[sl + 1] - b) >> 5;
            int k = b + l;
            int j = 0;
            for (; j + 1 < w; j += 2, k += 64) {   // two independent loads in flight
                const int c0 = col[k], c1 = col[k + 32];
                const V v0 = val[k], v1 = val[k + 32];
                s += v0 * x(c0);
                s += v1 * x(c1);
            }
            if (j < w) s += val[k] * x(col[k]);
        }
        return s;
    }
};

// SELL-32 with 16-bit columns.  Each slice of 32 rows picks one of three
// encodings (smode[s]), a choice that is uniform across the warp that walks it:
//  0  a signed offset from the row (every |col - row| <= 32767: an RCM-ordered
//     mesh matrix up to ~200^3 cells has all its slices so);
//  1  an unsigned offset from a base column of its (slice, j) group,
//     gbase[(sptr[s] >> 5) + j]: consecutive rows of an RCM order have their
//     j-th entries next to one another (median spread 31 columns), so this
//     holds at any bandwidth unless a group spans more than 65,535 columns;
//  2  32-bit columns in wcol[wptr[s] ..] (values stay in val).
// An FP32 entry moves 6 bytes instead of 8 in modes 0 and 1.  Padding entries
// point at the row (mode 0) or at the group's base (1, 2) with value 0.
template <class V>
struct Sell16View {
    static constexpr int kVS = 1;
    const int* __restrict__ sptr;
    const int* __restrict__ smode;
    const int* __restrict__ gbase;
    const int* __restrict__ wptr;
    const unsigned short* __restrict__ dcol;
    const int* __restrict__ wcol;
    const V* __restrict__ val;
    int n;
    template <class F>
    __device__ __forceinline__ V dot(int row, int, const F& x) const {
        V s = V(0);
        if (row < n) {
            const int sl = row >> 5, l = row & 31;
            const int b = sptr[sl], w = (sptr[sl + 1] - b) >> 5;
            const int mode = smode[sl];
            int k = b + l;
            int j = 0;
            if (sizeof(V) == 4 && mode == 0 && w <= 8) {
                // short FP32 rows (the finest mesh level): every entry load,
                // then every gather, then the products in entry order -- two
                // memory round trips a slice instead of one per pair of
                // entries (measured 11 % faster at 2.1M rows; the FP64 copy
                // of this path loses more to its register count than it gains)
                int cj[8];
                V vj[8], xj[8];
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (q < w) { cj[q] = row + (short)dcol[k + 32 * q]; vj[q] = val[k + 32 * q]; }
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (q < w) xj[q] = x(cj[q]);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (q < w) s += vj[q] * xj[q];
            } else if (mode == 0) {
                if (sizeof(V) == 4)   // longer FP32 rows (coarse levels): four entries in flight
                    for (; j + 3 < w; j += 4, k += 128) {
                        const int c0 = row + (short)dcol[k], c1 = row + (short)dcol[k + 32];
                        const int c2 = row + (short)dcol[k + 64], c3 = row + (short)dcol[k + 96];
                        const V v0 = val[k], v1 = val[k + 32], v2 = val[k + 64], v3 = val[k + 96];
                        const V x0 = x(c0), x1 = x(c1), x2 = x(c2), x3 = x(c3);
                        s += v0 * x0;
                        s += v1 * x1;
                        s += v2 * x2;
                        s += v3 * x3;
                    }
                for (; j + 1 < w; j += 2, k += 64) {   // two independent loads in flight
                    const int c0 = row + (short)dcol[k], c1 = row + (short)dcol[k + 32];
                    const V v0 = val[k], v1 = val[k + 32];
                    s += v0 * x(c0);
                    s += v1 * x(c1);
                }
                if (j < w) s += val[k] * x(row + (short)dcol[k]);
            } else if (mode == 1) {
                const int* __restrict__ gb = gbase + (b >> 5);
                for (; j + 1 < w; j += 2, k += 64) {
                    const int c0 = __ldg(gb + j) + dcol[k], c1 = __ldg(gb + j + 1) + dcol[k + 32];
                    const V v0 = val[k], v1 = val[k + 32];
                    s += v0 * x(c0);
                    s += v1 * x(c1);
                }
                if (j < w) s += val[k] * x(__ldg(gb + j) + dcol[k]);
            } else {
                const int* __restrict__ wc = wcol + wptr[sl] + l;
                for (; j + 1 < w; j += 2, k += 64) {
                    const int c0 = wc[32 * j], c1 = wc[32 * j + 32];
                    const V v0 = val[k], v1 = val[k + 32];
                    s += v0 * x(c0);
                    s += v1 * x(c1);
                }
                if (j < w) s += val[k] * x(wc[32 * j]);
            }
        }
        return s;
    }
};

template <class V, class X>
struct Vec {
    const X* __restrict__ p;
    __device__ __forceinline__ V operator()(int j) const { return (V)__ldg(p + j); }
};
// the first Chebyshev iterate from zero, D^-1 b / theta, formed on the fly
template <class V>
struct FirstIterate {
    const V* __restrict__ dinv;
    const V* __restrict__ b;
    V inv_theta;
    __device__ __forceinline__ V operator()(int j) const { return __ldg(dinv + j) * __ldg(b + j) * inv_theta; }
};

// ------------------------------------------- programmatic dependent launch
// The ~30 kernels of a CG iteration each depend on the one before and are
// short, so the gap between one kernel's last block and the next one's first
// is a real share of an iteration.  They are launched with programmatic
// stream serialisation: a kernel's launch is processed while its predecessor
// drains (the predecessor's blocks signal it implicitly as they exit), and
// the kernel waits at pdl_enter() -- its first statement: nothing is read
// before it -- until the predecessor has finished and its writes are
// visible.  Measured at 128^3: 0.42 -> 0.40 ms a CG iteration.  Signalling
// early instead (griddepcontrol.launch_dependents after the wait) put the
// waiting successor's blocks on the multiprocessors beside the running
// kernel and made the iteration 8 % slower than plain launches.  Without a
// programmatic predecessor the wait returns at once, so the kernels stay
// correct under plain launches.
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
template <class... P, class... A>
void launch_pdl(void (*k)(P...), int grid, int block, cudaStream_t s, A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SEMO_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...));
    SEMO_CHECK_LAUNCH();
}

// ------------------------------------------------------- V-cycle kernels
// pre-smoothing, degree 2 from x = 0:  x = d0 + c1 d0 + c2 D^-1 (b - A d0),  d0 = D^-1 b / theta
template <class M, class V>
__global__ void __launch_bounds__(256) k_pre2(M A, const V* __restrict__ dinv, const V* __restrict__ b,
                                              V inv_theta, V c1, V c2, V* __restrict__ x) {
    pdl_enter();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / M::kVS, lane = g % M::kVS;
    const V s = A.dot(row, lane, FirstIterate<V>{dinv, b, inv_theta});
    if (row < A.n && lane == 0) {
        const V di = dinv[row], bi = b[row];
        const V d0 = di * bi * inv_theta;
        x[row] = d0 + c1 * d0 + c2 * (di * (bi - s));
    }
}
// r = b - A x
template <class M, class V>
__global__ void __launch_bounds__(256) k_res(M A, const V* __restrict__ x, const V* __restrict__ b,
                                             V* __restrict__ r) {
    pdl_enter();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / M::kVS, lane = g % M::kVS;
    const V s = A.dot(row, lane, Vec<V, V>{x});
    if (row < A.n && lane == 0) r[row] = b[row] - s;
}
// y = A x (restriction with R, or any plain product)
template <class M, class V>
__global__ void __launch_bounds__(256) k_mv(M A, const V* __restrict__ x, V* __restrict__ y) {
    pdl_enter();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / M::kVS, lane = g % M::kVS;
    const V s = A.dot(row, lane, Vec<V, V>{x});
    if (row < A.n && lane == 0) y[row] = s;
}
// x += P xc
template <class M, class V>
__global__ void __launch_bounds__(256) k_prolong_add(M P, const V* __restrict__ xc, V* __restrict__ x) {
    pdl_enter();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / M::kVS, lane = g % M::kVS;
    const V s = P.dot(row, lane, Vec<V, V>{xc});
    if (row < P.n && lane == 0) x[row] += s;
}
// post-smoothing step 0 from x:  d = D^-1 (b - A x) / theta ;  y = x + d
template <class M, class V>
__global__ void __launch_bounds__(256) k_post0(M A, const V* __restrict__ dinv, const V* __restrict__ b,
                                               V inv_theta, const V* __restrict__ x, V* __restrict__ d,
                                               V* __restrict__ y) {
    pdl_enter();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / M::kVS, lane = g % M::kVS;
    const V s = A.dot(row, lane, Vec<V, V>{x});
    if (row < A.n && lane == 0) {
        const V dv = dinv[row] * (b[row] - s) * inv_theta;
        d[row] = dv;
        y[row] = x[row] + dv;
    }
}
// post-smoothing step 1:  x = y + c1 d + c2 D^-1 (b - A y)
template <class M, class V>
__global__ void __launch_bounds__(256) k_post1(M A, const V* __restrict__ dinv, const V* __restrict__ b, V c1, V c2,
                                               const V* __restrict__ y, const V* __restrict__ d,
                                               V* __restrict__ x) {
    pdl_enter();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / M::kVS, lane = g % M::kVS;
    const V s = A.dot(row, lane, Vec<V, V>{y});
    if (row < A.n && lane == 0) x[row] = y[row] + c1 * d[row] + c2 * (dinv[row] * (b[row] - s));
}
// finest-level post-smoothing step 1 (SELL), also folding in the CG dots
// z.r and z.q (q = A p of the previous iteration); grid-stride, fixed grid
template <class M, class V>
__global__ void __launch_bounds__(kRedThreads) k_post1_dots(M A, const V* __restrict__ dinv,
                                                            const V* __restrict__ b, V c1, V c2,
                                                            const V* __restrict__ y, const V* __restrict__ d,
                                                            V* __restrict__ z, const double* __restrict__ r,
                                                            const double* __restrict__ q,
                                                            double* __restrict__ part) {
    pdl_enter();
    __shared__ double sh[32];
    double zr = 0.0, zq = 0.0;
    const int per_block = blockDim.x / M::kVS, lane = threadIdx.x % M::kVS;
    for (int row0 = blockIdx.x * per_block; row0 < A.n; row0 += gridDim.x * per_block) {
        const int row = row0 + threadIdx.x / M::kVS;   // every lane runs the dot's shuffles
        const V s = A.dot(row, lane, Vec<V, V>{y});
        if (row < A.n && lane == 0) {
            const V zi = y[row] + c1 * d[row] + c2 * (dinv[row] * (b[row] - s));
            z[row] = zi;
            zr += (double)zi * r[row];
            zq += (double)zi * q[row];
        }
    }
    zr = block_sum(zr, sh);
    zq = block_sum(zq, sh);
    if (threadIdx.x == 0) { part[blockIdx.x] = zr; part[kRedBlocks + blockIdx.x] = zq; }
}

// generic Chebyshev pieces for degrees other than 2 (CSR)
template <class M, class V>
__global__ void __launch_bounds__(256) k_cheb_d(M A, const V* __restrict__ dinv, const V* __restrict__ b,
                                                const V* __restrict__ x, V c1, V c2, V* __restrict__ d) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / M::kVS, lane = g % M::kVS;
    const V s = A.dot(row, lane, Vec<V, V>{x});
    if (row < A.n && lane == 0) d[row] = c1 * d[row] + c2 * (dinv[row] * (b[row] - s));
}
template <class V>
__global__ void k_axpy1(int n, const V* __restrict__ d, V* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += d[i];
}
template <class V>
__global__ void k_zero(int n, V* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = V(0);
}
template <class V>
__global__ void k_copy_t(int n, const V* __restrict__ a, V* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

// coarsest level: x = A^-1 b with the explicit FP64 inverse, one block
template <class V>
__global__ void k_coarse_solve(int n, const double* __restrict__ inv, const V* __restrict__ b, V* __restrict__ x) {
    pdl_enter();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += inv[(size_t)i * n + k] * (double)b[k];
        x[i] = (V)s;
    }
}

// ---------------------------------------------------------- CG kernels
// device scalars: 0 rz, 1 zq, 2 pq, 3 rr, 4 alpha_prev, 5 beta, 6 alpha,
// 7 rz_prev, 8/9 scratch, 10 iteration count
__device__ __forceinline__ double sum_parts(const double* part, double* sh) {
    double s = 0.0;
    for (int i = threadIdx.x; i < kRedBlocks; i += blockDim.x) s += part[i];
    return block_sum(s, sh);
}
__global__ void k_fin_beta(const double* __restrict__ part, double* __restrict__ scal) {
    pdl_enter();
    __shared__ double sh[32];
    const double rz = sum_parts(part, sh);
    const double zq = sum_parts(part + kRedBlocks, sh);
    if (threadIdx.x == 0) {
        scal[0] = rz;
        scal[1] = zq;
        // Polak-Ribiere: beta = z.(r_k - r_{k-1}) / (z_{k-1}.r_{k-1}) = -alpha_{k-1} z.q_{k-1} / rz_prev
        scal[5] = (scal[10] == 0.0) ? 0.0 : (-scal[4] * zq / scal[7]);
        scal[7] = rz;
        scal[10] += 1.0;
    }
}
// w = A z;  q = w + beta q;  p = z + beta p;  part = p.q   (FP64 SELL operator)
template <class M, class Z>
__global__ void __launch_bounds__(kRedThreads) k_outer_mv(M A, const Z* __restrict__ z,
                                                          double* __restrict__ p, double* __restrict__ q,
                                                          const double* __restrict__ scal,
                                                          double* __restrict__ part) {
    pdl_enter();
    __shared__ double sh[32];
    const double beta = scal[5];
    double pq = 0.0;
    const int stride = gridDim.x * blockDim.x;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += stride) {
        const double w = A.dot(row, 0, Vec<double, Z>{z});
        const double qi = w + beta * q[row];
        const double pi = (double)z[row] + beta * p[row];
        q[row] = qi;
        p[row] = pi;
        pq += pi * qi;
    }
    pq = block_sum(pq, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = pq;
}
__global__ void k_fin_alpha(const double* __restrict__ part, double* __restrict__ scal) {
    pdl_enter();
    __shared__ double sh[32];
    const double pq = sum_parts(part, sh);
    if (threadIdx.x == 0) {
        scal[2] = pq;
        scal[6] = scal[7] / pq;
        scal[4] = scal[6];
    }
}
// x += alpha p;  r -= alpha q;  rv = r in the V-cycle's type;  part = r.r
template <class V>
__global__ void __launch_bounds__(kRedThreads) k_xr(int n, double* __restrict__ x, double* __restrict__ r,
                                                    V* __restrict__ rv, const double* __restrict__ p,
                                                    const double* __restrict__ q, const double* __restrict__ scal,
                                                    double* __restrict__ part) {
    pdl_enter();
    __shared__ double sh[32];
    const double alpha = scal[6];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * q[i];
        r[i] = ri;
        rv[i] = (V)ri;
        s += ri * ri;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void k_fin_rr(const double* __restrict__ part, double* __restrict__ scal) {
    pdl_enter();
    __shared__ double sh[32];
    const double rr = sum_parts(part, sh);
    if (threadIdx.x == 0) scal[3] = rr;
}
// generic dots for the non-fused path: part = a.b, part+R = a.c
template <class A>
__global__ void __launch_bounds__(kRedThreads) k_dot2(int n, const A* __restrict__ a, const double* __restrict__ b,
                                                      const double* __restrict__ c, double* __restrict__ part) {
    __shared__ double sh[32];
    double s = 0.0, t = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double ai = (double)a[i];
        s += ai * b[i];
        t += ai * c[i];
    }
    s = block_sum(s, sh);
    t = block_sum(t, sh);
    if (threadIdx.x == 0) { part[blockIdx.x] = s; part[kRedBlocks + blockIdx.x] = t; }
}
__global__ void __launch_bounds__(kRedThreads) k_dot(int n, const double* __restrict__ a, const double* __restrict__ b,
                                                     double* __restrict__ part) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += a[i] * b[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
template <class A, class B>
__global__ void k_conv(int n, const A* __restrict__ a, B* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (B)a[i];
}
// r = b - A x in FP64 (CSR, 8 lanes a row)
__global__ void __launch_bounds__(256) k_res64(CsrView<double, 8> A, const double* __restrict__ x,
                                               const double* __restrict__ b, double* __restrict__ r) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / 8, lane = g % 8;
    const double s = A.dot(row, lane, Vec<double, double>{x});
    if (row < A.n && lane == 0) r[row] = b[row] - s;
}

// --------------------------------------------------------------- SELL build
__global__ void k_sell_width(int n, const int* __restrict__ ptr, int* __restrict__ slice_len) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    const int len = (row < n) ? ptr[row + 1] - ptr[row] : 0;
    const int w = __reduce_max_sync(0xffffffffu, len);
    if ((threadIdx.x & 31) == 0 && row < ((n + 31) & ~31)) slice_len[row >> 5] = 32 * w;
}
template <class V, class W>
__global__ void k_sell_fill(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                            const V* __restrict__ val, const int* __restrict__ sptr, int* __restrict__ scol,
                            W* __restrict__ sval) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= ((n + 31) & ~31)) return;
    const int sl = row >> 5, l = row & 31;
    const int b = sptr[sl], w = (sptr[sl + 1] - b) >> 5;
    const int rb = (row < n) ? ptr[row] : 0, len = (row < n) ? ptr[row + 1] - rb : 0;
    for (int j = 0; j < w; ++j) {
        const int k = b + 32 * j + l;
        // padding reads column 0, which exists for every operator (P and R are not square)
        if (j < len) { scol[k] = col[rb + j]; sval[k] = (W)val[rb + j]; }
        else { scol[k] = 0; sval[k] = W(0); }
    }
}

// ------------------------------------------------------------ host side
template <class V>
struct Sell {
    int n = 0, nslices = 0;
    DBuf<int> sptr, col;
    DBuf<V> val;
    SellView<V> view() const { return SellView<V>{sptr.p, col.p, val.p, n}; }
};

template <class V>
CsrView<V, 4> csr4(const DCsr<V>& A) { return CsrView<V, 4>{A.ptr.p, A.col.p, A.val.p, A.n}; }

template <class V>
int pick_vs(const DCsr<V>& A) {
    const double avg = A.n ? (double)A.nnz / A.n : 1.0;
    return avg <= 6 ? 4 : (avg <= 12 ? 8 : (avg <= 24 ? 16 : 32));
}

// launch a row kernel on a CSR matrix with the lanes-per-row that suits it
template <class V, class F>
void with_csr(const DCsr<V>& A, F&& f) {
    switch (pick_vs(A)) {
        case 4: f(CsrView<V, 4>{A.ptr.p, A.col.p, A.val.p, A.n}); break;
        case 8: f(CsrView<V, 8>{A.ptr.p, A.col.p, A.val.p, A.n}); break;
        case 16: f(CsrView<V, 16>{A.ptr.p, A.col.p, A.val.p, A.n}); break;
        default: f(CsrView<V, 32>{A.ptr.p, A.col.p, A.val.p, A.n}); break;
    }
}
template <class M>
int grid_for(const M& A) { return blocks((int64_t)A.n * M::kVS, 256); }

// SELL-32 copy of a CSR matrix's structure and values (value type W); hpin:
// a pinned int of the calling thread for the slice scan's total
template <class V, class W>
void build_sell(cudaStream_t s, const int* ptr, const int* col, const V* val, int n, Sell<W>& S, int* hpin) {
    S.n = n;
    S.nslices = (n + 31) / 32;
    S.sptr.alloc(S.nslices + 1, s);
    SEMO_CUDA(cudaMemsetAsync(S.sptr.p + S.nslices, 0, sizeof(int), s));
    const int rows_pad = S.nslices * 32;
    k_sell_width<<<blocks(rows_pad, 256), 256, 0, s>>>(n, ptr, S.sptr.p);
    SEMO_CHECK_LAUNCH();
    const int total = device_scan(s, S.sptr.p, S.nslices + 1, hpin);
    S.col.alloc(std::max(total, 1), s);
    S.val.alloc(std::max(total, 1), s);
    k_sell_fill<V, W><<<blocks(rows_pad, 256), 256, 0, s>>>(n, ptr, col, val, S.sptr.p, S.col.p, S.val.p);
    SEMO_CHECK_LAUNCH();
}

// One warp per slice (blocks of whole warps): the slice's encoding, the base
// column (smallest column) of every (slice, j) group and the slice's 32-bit
// column count in wsz (0 unless its encoding is 2).
__global__ void k_sell16_groups(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                const int* __restrict__ sptr, int* __restrict__ smode, int* __restrict__ gbase,
                                int* __restrict__ wsz) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    const int sl = row >> 5;
    if (sl >= ((n + 31) >> 5)) return;   // whole warps: the test is uniform in a warp
    const int b = sptr[sl], w = (sptr[sl + 1] - b) >> 5;
    const int rb = (row < n) ? ptr[row] : 0, len = (row < n) ? ptr[row + 1] - rb : 0;
    bool wide = false, near = true;
    for (int j = 0; j < w; ++j) {
        const int c = (j < len) ? col[rb + j] : -1;
        const int mn = __reduce_min_sync(0xffffffffu, (c >= 0) ? c : INT_MAX);
        const int mx = __reduce_max_sync(0xffffffffu, c);
        wide |= (long long)mx - (long long)mn > 65535;
        near &= (c < 0) || (c - row >= -32768 && c - row <= 32767);
        if ((threadIdx.x & 31) == 0) gbase[(b >> 5) + j] = mn;
    }
    near = __all_sync(0xffffffffu, near);
    const int mode = near ? 0 : (wide ? 2 : 1);
    if ((threadIdx.x & 31) == 0) {
        smode[sl] = mode;
        wsz[sl] = (mode == 2) ? 32 * w : 0;
    }
}

__global__ void k_sell16_cols(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                              const int* __restrict__ sptr, const int* __restrict__ smode,
                              const int* __restrict__ gbase, const int* __restrict__ wptr,
                              unsigned short* __restrict__ dcol, int* __restrict__ wcol) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= ((n + 31) & ~31)) return;
    const int sl = row >> 5, l = row & 31;
    const int b = sptr[sl], w = (sptr[sl + 1] - b) >> 5;
    const int mode = smode[sl];
    const int rb = (row < n) ? ptr[row] : 0, len = (row < n) ? ptr[row + 1] - rb : 0;
    for (int j = 0; j < w; ++j) {
        const int k = b + 32 * j + l;
        const int base = (mode == 0) ? row : gbase[(b >> 5) + j];
        const int c = (j < len) ? col[rb + j] : base;
        dcol[k] = (mode == 2) ? (unsigned short)0 : (unsigned short)(c - base);
        if (mode == 2) wcol[wptr[sl] + 32 * j + l] = c;
    }
}
// the values into a layout's slots (padding slots 0)
template <class V, class W>
__global__ void k_sell16_vals(int n, const int* __restrict__ ptr, const V* __restrict__ val,
                              const int* __restrict__ sptr, W* __restrict__ sval) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= ((n + 31) & ~31)) return;
    const int sl = row >> 5, l = row & 31;
    const int b = sptr[sl], w = (sptr[sl + 1] - b) >> 5;
    const int rb = (row < n) ? ptr[row] : 0, len = (row < n) ? ptr[row + 1] - rb : 0;
    for (int j = 0; j < w; ++j) sval[b + 32 * j + l] = (j < len) ? (W)val[rb + j] : W(0);
}

// The structure of a SELL-32 layout with 16-bit columns (slice pointers,
// per-slice encodings, group bases, 16- and 32-bit columns).  It depends on
// the pattern only, so the FP64 outer operator and the finest level of the
// pressure hierarchy, both on the mesh's pattern, share one, built once per
// mesh; a setup then only writes the two value arrays.
struct Sell16Struct {
    int n = 0, nslices = 0;
    int slots = 0;   // padded entries (sptr[nslices])
    DBuf<int> sptr, smode, gbase, wptr, wcol;
    DBuf<unsigned short> dcol;
};
template <class V>
struct Sell16 {
    std::shared_ptr<Sell16Struct> st;
    DBuf<V> val;
    Sell16View<V> view() const {
        return Sell16View<V>{st->sptr.p, st->smode.p, st->gbase.p, st->wptr.p, st->dcol.p, st->wcol.p, val.p,
                             st->n};
    }
};

// SELL-32 structure with 16-bit columns of a square CSR pattern (slices that
// fit no 16-bit encoding keep 32-bit columns)
std::shared_ptr<Sell16Struct> build_sell16_struct(cudaStream_t s, const int* ptr, const int* col, int n,
                                                  int* hpin) {
    auto S = std::make_shared<Sell16Struct>();
    S->n = n;
    S->nslices = (n + 31) / 32;
    S->sptr.alloc(S->nslices + 1, s);
    S->wptr.alloc(S->nslices + 1, s);
    S->smode.alloc(S->nslices, s);
    SEMO_CUDA(cudaMemsetAsync(S->sptr.p + S->nslices, 0, sizeof(int), s));
    SEMO_CUDA(cudaMemsetAsync(S->wptr.p + S->nslices, 0, sizeof(int), s));
    const int rows_pad = S->nslices * 32;
    k_sell_width<<<blocks(rows_pad, 256), 256, 0, s>>>(n, ptr, S->sptr.p);
    SEMO_CHECK_LAUNCH();
    S->slots = device_scan(s, S->sptr.p, S->nslices + 1, hpin);
    S->gbase.alloc(std::max(S->slots / 32, 1), s);
    k_sell16_groups<<<blocks(rows_pad, 256), 256, 0, s>>>(n, ptr, col, S->sptr.p, S->smode.p, S->gbase.p,
                                                          S->wptr.p);
    SEMO_CHECK_LAUNCH();
    const int wide = device_scan(s, S->wptr.p, S->nslices + 1, hpin);
    S->dcol.alloc(std::max(S->slots, 1), s);
    S->wcol.alloc(std::max(wide, 1), s);
    k_sell16_cols<<<blocks(rows_pad, 256), 256, 0, s>>>(n, ptr, col, S->sptr.p, S->smode.p, S->gbase.p, S->wptr.p,
                                                         S->dcol.p, S->wcol.p);
    SEMO_CHECK_LAUNCH();
    return S;
}
// the values of a CSR operator on the structure's pattern into S (type W)
template <class V, class W>
void fill_sell16(cudaStream_t s, const int* ptr, const V* val, const std::shared_ptr<Sell16Struct>& st,
                 Sell16<W>& S) {
    S.st = st;
    S.val.alloc(std::max(st->slots, 1), s);
    k_sell16_vals<V, W><<<blocks((int64_t)st->nslices * 32, 256), 256, 0, s>>>(st->n, ptr, val, st->sptr.p,
                                                                              S.val.p);
    SEMO_CHECK_LAUNCH();
}
template <class V, class W>
bool build_sell16(cudaStream_t s, const int* ptr, const int* col, const V* val, int n, Sell16<W>& S, int* hpin) {
    fill_sell16<V, W>(s, ptr, val, build_sell16_struct(s, ptr, col, n, hpin), S);
    return true;
}

// The FP64 outer operator: 16-bit column offsets when they fit, else SELL-32
struct OuterOp {
    Sell<double> s32;
    Sell16<double> s16;
    bool use16 = false;
    template <class F>
    void with(F&& f) const {
        if (use16) f(s16.view());
        else f(s32.view());
    }
};

struct ChebCoef {
    double inv_theta, c1, c2;
};
ChebCoef cheb2(double lam) {
    const double hi = lam, lo = lam / 30.0;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
    const double sigma = theta / delta, rho0 = 1.0 / sigma;
    const double rho1 = 1.0 / (2.0 * sigma - rho0);
    return ChebCoef{1.0 / theta, rho1 * rho0, 2.0 * rho1 / delta};
}

// Everything the V-cycle needs beyond the hierarchy: SELL copies of the
// operators it pays for.  SELL runs one thread per row, so it needs enough
// rows to fill the GPU (65536 rows = 2048 warps, ~13 per SM) unless rows are
// short; a few thousand long rows (a coarse level, ~60 entries each) would
// leave ~2 warps per SM walking 60 dependent loads, and run faster as CSR
// with 32 lanes a row.  Small operators are launch-latency bound either way
// and stay CSR.
constexpr int kSellMinRows = 4096;
constexpr int kSellFullRows = 65536;
constexpr double kSellMaxAvgRow = 12.0;
template <class V>
bool sell_pays(const DCsr<V>& M) {
    if (M.n < kSellMinRows) return false;
    return M.n >= kSellFullRows || (double)M.nnz <= kSellMaxAvgRow * (double)M.n;
}
template <class V>
struct LevelMats {
    Sell<V> A, P, R;
    Sell16<V> A16;
    bool a = false, p = false, r = false, a16 = false;
    // multicolour Gauss-Seidel (semo_params.smoother == 1): the level's rows
    // grouped by colour, colour k at crow[cptr[k] .. cptr[k + 1])
    bool gs = false;
    DBuf<int> crow;
    std::vector<int> cptr;
};
template <class V>
struct Cycle {
    std::vector<LevelMats<V>> lev;
};

// run f on the SELL view of a level operator if it has one, else on CSR
template <class V, class F>
void with_op(const Sell<V>& S, bool use_sell, const DCsr<V>& M, F&& f) {
    if (use_sell) f(S.view());
    else with_csr(M, f);
}
// the level's A: 16-bit-offset SELL, SELL, or CSR
template <class V, class F>
void with_A(const LevelMats<V>& M, const DCsr<V>& A, F&& f) {
    if (M.a16) f(M.A16.view());
    else with_op(M.A, M.a, A, f);
}

// ---------------------------------------------- multicolour Gauss-Seidel
__device__ __forceinline__ uint32_t color_hash(uint32_t x) {
    // integer avalanche mixer (public-domain "lowbias32" constants), as the MIS uses
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
// One synchronous Jones-Plassmann round on the pattern of A: an uncoloured row
// whose (hash, index) key is larger than every uncoloured neighbour's takes
// the smallest colour no neighbour coloured in an earlier round holds (the
// rows coloured in one round are independent, so they never clash).  Reads
// cold, writes cnew (a copy of cold); counts the rows still uncoloured and
// flags a row that would need a colour beyond 127.
__global__ void k_color_round(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                              const int* __restrict__ cold, int* __restrict__ cnew, int* __restrict__ left,
                              int* __restrict__ overflow) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || cold[i] >= 0) return;
    const unsigned long long ki = ((unsigned long long)color_hash((uint32_t)i) << 32) | (unsigned)i;
    unsigned long long used0 = 0, used1 = 0;
    bool top = true;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        const int j = col[k];
        if (j == i) continue;
        const int cj = cold[j];
        if (cj < 0) {
            const unsigned long long kj = ((unsigned long long)color_hash((uint32_t)j) << 32) | (unsigned)j;
            if (kj > ki) { top = false; break; }
        } else if (cj < 64) {
            used0 |= 1ull << cj;
        } else if (cj < 128) {
            used1 |= 1ull << (cj - 64);
        }
    }
    if (!top) { atomicAdd(left, 1); return; }
    int c = -1;
    if (~used0) c = __ffsll((long long)~used0) - 1;
    else if (~used1) c = 64 + __ffsll((long long)~used1) - 1;
    if (c < 0) { atomicExch(overflow, 1); c = 127; }
    cnew[i] = c;
}

// One colour of a Gauss-Seidel sweep: x_i += (b_i - (A x)_i) / a_ii for the
// rows of that colour (no two of them are coupled, so the order is free)
template <class M, class V>
__global__ void __launch_bounds__(256) k_gs_color(M A, const int* __restrict__ rows, int nrows,
                                                  const V* __restrict__ dinv, const V* __restrict__ b,
                                                  V* __restrict__ x) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = g / M::kVS, lane = g % M::kVS;
    const int row = (t < nrows) ? rows[t] : A.n;   // rows past the list: an empty dot
    const V s = A.dot(row, lane, Vec<V, V>{x});
    if (t < nrows && lane == 0) x[row] += dinv[row] * (b[row] - s);
}
// Under the Gauss-Seidel option only the finest level, when it has more than
// this many rows, is swept by colours; the coarser levels keep Chebyshev.
// A sweep is one launch per colour: the finest mesh graph needs a handful of
// colours, a coarse level (denser rows) 20-40, each colour a launch of a few
// thousand rows, and there the sweeps cost launch latency, not bandwidth
// (measured at 128^3: 50 extra launches per V-cycle, twice the solve time).
constexpr int kGsMinRows = 16384;

template <class V>
void color_level(semo_ctx* c, cudaStream_t s, const DCsr<V>& A, LevelMats<V>& M) {
    const int n = A.n;
    DBuf<int> c0, c1, cnt;
    c0.alloc(n, s);
    c1.alloc(n, s);
    cnt.alloc(2, s);
    SEMO_CUDA(cudaMemsetAsync(c0.p, 0xff, sizeof(int) * n, s));   // -1: uncoloured
    int h[2] = {1, 0};
    int* cold = c0.p;
    int* cnew = c1.p;
    // rounds in batches of 4 between host checks (a round over a fully
    // coloured graph changes nothing)
    for (int batch = 0; h[0] > 0; ++batch) {
        if (batch > 1024) throw Error(SEMO_ERR_CUDA, "graph colouring did not finish");
        for (int r = 0; r < 4; ++r) {
            SEMO_CUDA(cudaMemcpyAsync(cnew, cold, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
            SEMO_CUDA(cudaMemsetAsync(cnt.p, 0, 2 * sizeof(int), s));
            k_color_round<<<blocks(n, 256), 256, 0, s>>>(n, A.ptr, A.col, cold, cnew, cnt.p, cnt.p + 1);
            SEMO_CHECK_LAUNCH();
            std::swap(cold, cnew);
        }
        SEMO_CUDA(cudaMemcpyAsync(h, cnt.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
        if (h[1]) throw Error(SEMO_ERR_CUDA, "graph colouring needs more than 128 colours");
    }
    // rows grouped by colour (counting sort on the host; the order inside a colour is free)
    std::vector<int> hc(n);
    SEMO_CUDA(cudaMemcpyAsync(hc.data(), cold, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    int ncol = 0;
    for (int v : hc) ncol = std::max(ncol, v + 1);
    M.cptr.assign(ncol + 1, 0);
    for (int v : hc) M.cptr[v + 1]++;
    for (int k = 0; k < ncol; ++k) M.cptr[k + 1] += M.cptr[k];
    std::vector<int> fill(M.cptr.begin(), M.cptr.end() - 1), rows(n);
    for (int i = 0; i < n; ++i) rows[fill[hc[i]]++] = i;
    M.crow.upload(rows.data(), n, s);
    SEMO_CUDA(cudaStreamSynchronize(s));   // the host vector above is freed on return
    M.gs = true;
}

// one Gauss-Seidel sweep of level L (forward: colours ascending)
template <class V>
void gs_sweep(cudaStream_t s, AmgLevel<V>& L, const LevelMats<V>& M, bool backward, bool zero_start) {
    const int n = L.A.n;
    const int ncol = (int)M.cptr.size() - 1;
    if (zero_start) {
        k_zero<V><<<blocks(n, 256), 256, 0, s>>>(n, L.x.p);
        SEMO_CHECK_LAUNCH();
    }
    for (int q = 0; q < ncol; ++q) {
        const int k = backward ? ncol - 1 - q : q;
        const int nr = M.cptr[k + 1] - M.cptr[k];
        if (nr == 0) continue;
        with_csr(L.A, [&](auto A) {
            using MV = decltype(A);
            k_gs_color<<<blocks((int64_t)nr * MV::kVS, 256), 256, 0, s>>>(A, M.crow.p + M.cptr[k], nr, L.dinv.p,
                                                                          L.b.p, L.x.p);
        });
        SEMO_CHECK_LAUNCH();
    }
}

template <class V>
void chebyshev_generic(cudaStream_t s, AmgLevel<V>& L, int degree, bool zero_start) {
    const int n = L.A.n;
    const double hi = L.lam_max, lo = hi / 30.0;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
    const double sigma = theta / delta;
    double rho = 1.0 / sigma;
    V* x = L.x.p;
    V* d = L.t.p;
    if (zero_start) {
        k_zero<V><<<blocks(n, 256), 256, 0, s>>>(n, x);
        SEMO_CHECK_LAUNCH();
    }
    k_zero<V><<<blocks(n, 256), 256, 0, s>>>(n, d);
    SEMO_CHECK_LAUNCH();
    // d = D^-1 (b - A x) / theta ; x += d
    with_csr(L.A, [&](auto M) {
        k_cheb_d<<<grid_for(M), 256, 0, s>>>(M, L.dinv.p, L.b.p, x, V(0), (V)(1.0 / theta), d);
    });
    SEMO_CHECK_LAUNCH();
    k_axpy1<V><<<blocks(n, 256), 256, 0, s>>>(n, d, x);
    SEMO_CHECK_LAUNCH();
    for (int k = 1; k < degree; ++k) {
        const double rho_new = 1.0 / (2.0 * sigma - rho);
        const V c1 = (V)(rho_new * rho), c2 = (V)(2.0 * rho_new / delta);
        with_csr(L.A, [&](auto M) { k_cheb_d<<<grid_for(M), 256, 0, s>>>(M, L.dinv.p, L.b.p, x, c1, c2, d); });
        SEMO_CHECK_LAUNCH();
        k_axpy1<V><<<blocks(n, 256), 256, 0, s>>>(n, d, x);
        SEMO_CHECK_LAUNCH();
        rho = rho_new;
    }
}

// V-cycle from level l down, input L.b, output L.x
template <class V>
void vcycle_from(semo_ctx* c, Amg<V>& h, Cycle<V>& cy, int l) {
    cudaStream_t s = c->stream;
    AmgLevel<V>& L = h.lev[l];
    if (l == (int)h.lev.size() - 1) {
        launch_pdl(k_coarse_solve<V>, 1, 256, s, h.coarse_n, h.cinv.p, L.b.p, L.x.p);
        return;
    }
    const LevelMats<V>& M = cy.lev[l];
    const int degree = c->prm.cheb_degree;
    const ChebCoef cc = cheb2(L.lam_max);
    if (M.gs) {
        gs_sweep(s, L, M, false, true);   // forward sweep from x = 0
    } else if (degree == 2) {
        with_A(M, L.A, [&](auto A) {
            launch_pdl(k_pre2<decltype(A), V>, grid_for(A), 256, s, A, L.dinv.p, L.b.p, (V)cc.inv_theta, (V)cc.c1,
                       (V)cc.c2, L.x.p);
        });
    } else {
        chebyshev_generic(s, L, degree, true);
    }
    with_A(M, L.A, [&](auto A) { launch_pdl(k_res<decltype(A), V>, grid_for(A), 256, s, A, L.x.p, L.b.p, L.r.p); });
    AmgLevel<V>& C = h.lev[l + 1];
    with_op(M.R, M.r, L.R, [&](auto R) { launch_pdl(k_mv<decltype(R), V>, grid_for(R), 256, s, R, L.r.p, C.b.p); });
    vcycle_from(c, h, cy, l + 1);
    with_op(M.P, M.p, L.P,
            [&](auto P) { launch_pdl(k_prolong_add<decltype(P), V>, grid_for(P), 256, s, P, C.x.p, L.x.p); });
    if (M.gs) {
        gs_sweep(s, L, M, true, false);   // backward sweep: the cycle stays symmetric
    } else if (degree == 2) {
        with_A(M, L.A, [&](auto A) {
            launch_pdl(k_post0<decltype(A), V>, grid_for(A), 256, s, A, L.dinv.p, L.b.p, (V)cc.inv_theta, L.x.p,
                       L.t.p, L.r.p);
        });
        if (l > 0) {
            with_A(M, L.A, [&](auto A) {
                launch_pdl(k_post1<decltype(A), V>, grid_for(A), 256, s, A, L.dinv.p, L.b.p, (V)cc.c1, (V)cc.c2,
                           L.r.p, L.t.p, L.x.p);
            });
        }
        // on the finest level the last step is fused with the CG dot products (cg_iteration)
    } else {
        chebyshev_generic(s, L, degree, false);
    }
}

struct Red {
    double* part;
    double* scal;
};
Red red_area(semo_ctx* c) {
    c->red.alloc(4 * kRedBlocks + 32, c->stream);
    return Red{c->red.p, c->red.p + 4 * kRedBlocks + 8};
}

// One preconditioned CG iteration.  In: r (FP64) and its copy L0.b in V; out: x, r, L0.b updated.
template <class V>
void cg_iteration(semo_ctx* c, Amg<V>& h, Cycle<V>& cy, const OuterOp& outer, double* x, const Red& R) {
    cudaStream_t s = c->stream;
    AmgLevel<V>& L = h.lev[0];
    const int n = L.A.n;
    double* r = c->kr.p;
    double* p = c->kp.p;
    double* q = c->kq.p;
    const int degree = c->prm.cheb_degree;
    const bool single = h.lev.size() == 1;
    if (single) {
        k_coarse_solve<V><<<1, 256, 0, s>>>(h.coarse_n, h.cinv, L.b, L.x);
        SEMO_CHECK_LAUNCH();
        k_dot2<V><<<kRedBlocks, kRedThreads, 0, s>>>(n, L.x.p, r, q, R.part);
        SEMO_CHECK_LAUNCH();
    } else if (degree == 2 && !cy.lev[0].gs) {
        const ChebCoef cc = cheb2(L.lam_max);
        vcycle_from(c, h, cy, 0);   // everything but the last smoothing step of the finest level
        // z lands in L.x; z.r and z.q folded in
        with_A(cy.lev[0], L.A, [&](auto A) {
            launch_pdl(k_post1_dots<decltype(A), V>, kRedBlocks, kRedThreads, s, A, L.dinv.p, L.b.p, (V)cc.c1,
                       (V)cc.c2, L.r.p, L.t.p, L.x.p, r, q, R.part);
        });
    } else {
        vcycle_from(c, h, cy, 0);
        k_dot2<V><<<kRedBlocks, kRedThreads, 0, s>>>(n, L.x.p, r, q, R.part);
        SEMO_CHECK_LAUNCH();
    }
    launch_pdl(k_fin_beta, 1, 256, s, R.part, R.scal);
    outer.with([&](auto A) {
        launch_pdl(k_outer_mv<decltype(A), V>, kRedBlocks, kRedThreads, s, A, L.x.p, p, q, R.scal, R.part);
    });
    launch_pdl(k_fin_alpha, 1, 256, s, R.part, R.scal);
    launch_pdl(k_xr<V>, kRedBlocks, kRedThreads, s, n, x, r, L.b.p, p, q, R.scal, R.part);
    launch_pdl(k_fin_rr, 1, 256, s, R.part, R.scal);
}

struct GraphGuard {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    ~GraphGuard() {
        if (e) cudaGraphExecDestroy(e);
        if (g) cudaGraphDestroy(g);
    }
};

// The loop's stopping threshold on r.r: (tol |b|)^2, |b| = 1 for b = 0
// (scal[11] = b.b)
__device__ __forceinline__ double cg_stop_rr(const double* scal, double tol) {
    const double bn = sqrt(scal[11]);
    const double bnorm = (bn > 0.0) ? bn : 1.0;
    return (tol * bnorm) * (tol * bnorm);
}
// Before the loop: iterate at all? (no when r0 already meets the tolerance,
// or b or r0 is not finite -- the host reports that after the graph)
__global__ void k_cg_begin(cudaGraphConditionalHandle h, const double* __restrict__ scal, double tol, int max_iter) {
    const double bn = sqrt(scal[11]), rn = sqrt(scal[12]);
    const double bnorm = (bn > 0.0) ? bn : 1.0;
    const bool go = isfinite(bn) && isfinite(rn) && rn > tol * bnorm && max_iter > 0;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}
// End of one CG iteration on the device: count it and decide whether the
// loop goes on (scal[13] iterations, scal[14] status: 1 NaN/Inf, 2 p.q <= 0).
// The loop is a conditional WHILE node, so no iteration waits for the host;
// max_iter bounds it.
__global__ void k_cg_check(cudaGraphConditionalHandle h, double* __restrict__ scal, double tol, int max_iter) {
    pdl_enter();
    const double stop_rr = cg_stop_rr(scal, tol);
    const double it = scal[13] + 1.0;
    scal[13] = it;
    const double pq = scal[2], rr = scal[3];
    unsigned go = 1;
    if (!isfinite(rr) || !isfinite(pq)) { scal[14] = 1.0; go = 0; }
    else if (!(pq > 0.0)) { scal[14] = 2.0; go = 0; }
    else if (!(rr > stop_rr) || it >= (double)max_iter) go = 0;
    cudaGraphSetConditional(h, go);
}

template <class V>
void pcg(semo_ctx* c, Amg<V>& h, Cycle<V>& cy, const OuterOp& outer, const int* ptr, const int* col,
         const double* val, int n, const double* b, double* x, bool zero_guess, semo_solve_info* info) {
    cudaStream_t s = c->stream;
    Red R = red_area(c);
    c->kr.alloc(n, s); c->kp.alloc(n, s); c->kq.alloc(n, s);
    double* h2 = c->hpin;
    double* r = c->kr.p;
    const CsrView<double, 8> A8{ptr, col, val, n};
    if (zero_guess) {
        SEMO_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        SEMO_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    } else {
        k_res64<<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(A8, x, b, r);
        SEMO_CHECK_LAUNCH();
    }
    k_conv<double, V><<<blocks(n, 256), 256, 0, s>>>(n, r, h.lev[0].b.p);
    SEMO_CHECK_LAUNCH();
    SEMO_CUDA(cudaMemsetAsync(c->kq.p, 0, sizeof(double) * n, s));
    SEMO_CUDA(cudaMemsetAsync(c->kp.p, 0, sizeof(double) * n, s));
    SEMO_CUDA(cudaMemsetAsync(R.scal, 0, sizeof(double) * 16, s));
    k_dot<<<kRedBlocks, kRedThreads, 0, s>>>(n, b, b, R.part);
    SEMO_CHECK_LAUNCH();
    k_dot<<<kRedBlocks, kRedThreads, 0, s>>>(n, r, r, R.part + kRedBlocks);
    SEMO_CHECK_LAUNCH();
    k_fin_rr<<<1, 256, 0, s>>>(R.part, R.scal + 8);   // ||b||^2 -> scal[11]
    SEMO_CHECK_LAUNCH();
    k_fin_rr<<<1, 256, 0, s>>>(R.part + kRedBlocks, R.scal + 9);   // ||r0||^2 -> scal[12]
    SEMO_CHECK_LAUNCH();
    // The loop is one graph: k_cg_begin, then a conditional WHILE node whose
    // body is one CG iteration (~30 kernels) plus k_cg_check, which decides on
    // the device whether to go on.  It is captured and instantiated while the
    // kernels above run, and the host waits once, after the true residual.
    GraphGuard gg;
    SEMO_CUDA(cudaGraphCreate(&gg.g, 0));
    cudaGraphConditionalHandle handle;
    SEMO_CUDA(cudaGraphConditionalHandleCreate(&handle, gg.g, 0, cudaGraphCondAssignDefault));
    cudaKernelNodeParams kb = {};
    const double tol = c->prm.tol;
    const int max_iter = c->prm.max_iter;
    const double* scal_c = R.scal;
    void* kb_args[] = {(void*)&handle, (void*)&scal_c, (void*)&tol, (void*)&max_iter};
    kb.func = (void*)k_cg_begin;
    kb.gridDim = dim3(1);
    kb.blockDim = dim3(1);
    kb.kernelParams = kb_args;
    cudaGraphNode_t begin;
    SEMO_CUDA(cudaGraphAddKernelNode(&begin, gg.g, nullptr, 0, &kb));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loop;
    SEMO_CUDA(cudaGraphAddNode(&loop, gg.g, &begin, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const long long before = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
    SEMO_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    try {
        cg_iteration(c, h, cy, outer, x, R);
        launch_pdl(k_cg_check, 1, 1, s, handle, R.scal, tol, max_iter);
    } catch (...) {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(s, &junk);
        throw;
    }
    cudaGraph_t captured = nullptr;
    SEMO_CUDA(cudaStreamEndCapture(s, &captured));
    size_t body_nodes = 0;
    SEMO_CUDA(cudaGraphGetNodes(body, nullptr, &body_nodes));
    __atomic_store_n(&g_kernel_launches, before, __ATOMIC_RELAXED);
    SEMO_CUDA(cudaGraphInstantiate(&gg.e, gg.g, 0));
    SEMO_CUDA(cudaGraphLaunch(gg.e, s));
    // true FP64 residual of the returned solution -> scal[16]
    k_res64<<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(A8, x, b, r);
    SEMO_CHECK_LAUNCH();
    k_dot<<<kRedBlocks, kRedThreads, 0, s>>>(n, r, r, R.part);
    SEMO_CHECK_LAUNCH();
    k_fin_rr<<<1, 256, 0, s>>>(R.part, R.scal + 13);
    SEMO_CHECK_LAUNCH();
    SEMO_CUDA(cudaMemcpyAsync(h2, R.scal, sizeof(double) * 17, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    const double bn = std::sqrt(h2[11]), rn0 = std::sqrt(h2[12]);
    if (!std::isfinite(bn) || !std::isfinite(rn0)) throw Error(SEMO_ERR_NAN, "non-finite right-hand side");
    const int it = (int)h2[13];
    __atomic_add_fetch(&g_kernel_launches, 1LL + (long long)body_nodes * it, __ATOMIC_RELAXED);
    if (h2[14] == 1.0) throw Error(SEMO_ERR_NAN, "NaN/Inf in the Krylov residual");
    if (h2[14] == 2.0) throw Error(SEMO_ERR_BREAKDOWN, "CG breakdown: p.Ap <= 0 (matrix not SPD?)");
    info->iterations = it;
    info->rel_residual = (bn > 0.0) ? std::sqrt(h2[16]) / bn : 0.0;
}

template <class V>
void fill_info(const Amg<V>& h, int64_t nnz, semo_solve_info* info) {
    info->levels = (int)h.lev.size();
    info->coarse_size = h.coarse_n;
    info->operator_complexity = (double)h.total_nnz / (double)std::max<int64_t>(nnz, 1);
}

// per-context apply state (kept for the adjoint solve on the same hierarchy)
struct ApplyState {
    Cycle<float> cy32;
    Cycle<double> cy64;
    OuterOp outer;
    // the SELL-32/16-bit structure of the context's mesh pattern (A_ptr, A_col)
    // and the mesh generation it was built for
    std::shared_ptr<Sell16Struct> pat16;
    int pat16_gen = 0;
    // the matrix values the current hierarchy was built from (pressure path only)
    DBuf<double> src_val;
    int src_n = 0;
    int64_t src_nnz = 0;
    int src_prec = -1;
};

// flag[0] = 1 if a and b differ anywhere (bit patterns)
__global__ void k_differs(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                          int* __restrict__ flag) {
    bool d = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d |= __double_as_longlong(a[i]) != __double_as_longlong(b[i]);
    if (__any_sync(0xffffffffu, d) && (threadIdx.x & 31) == 0) flag[0] = 1;
}
ApplyState& apply_state(semo_ctx* c) {
    if (!c->apply) c->apply = std::shared_ptr<void>(new ApplyState(), [](void* p) { delete (ApplyState*)p; });
    return *(ApplyState*)c->apply.get();
}

template <class V>
void prepare_cycle(semo_ctx* c, Amg<V>& h, Cycle<V>& cy, const std::shared_ptr<Sell16Struct>& lev0 = nullptr) {
    cudaStream_t s = setup_stream(c);
    const int nl = (int)h.lev.size();
    cy.lev.resize(std::max(nl - 1, 0));
    for (int l = 0; l + 1 < nl; ++l) {
        AmgLevel<V>& L = h.lev[l];
        LevelMats<V>& M = cy.lev[l];
        M.a = sell_pays(L.A);
        M.p = sell_pays(L.P);
        M.r = sell_pays(L.R);
        int* const hp = c->hpin_int + 4;
        if (l == 0 && M.a && lev0 && lev0->n == L.A.n) {   // the mesh pattern's structure, shared
            fill_sell16<V, V>(s, L.A.ptr, L.A.val, lev0, M.A16);
            M.a16 = true;
        } else {
            M.a16 = M.a && build_sell16<V, V>(s, L.A.ptr, L.A.col, L.A.val, L.A.n, M.A16, hp);
        }
        if (M.a16) M.a = false;
        if (M.a) build_sell<V, V>(s, L.A.ptr, L.A.col, L.A.val, L.A.n, M.A, hp);
        if (M.p) build_sell<V, V>(s, L.P.ptr, L.P.col, L.P.val, L.P.n, M.P, hp);
        if (M.r) build_sell<V, V>(s, L.R.ptr, L.R.col, L.R.val, L.R.n, M.R, hp);
        M.gs = false;
        if (c->prm.smoother == 1 && l == 0 && L.A.n > kGsMinRows) color_level(c, s, L.A, M);
    }
}

// ---------------------------------- momentum and VOF: batched BiCGStab
// NR right-hand sides (3 for the velocity components, 1 for the volume
// fraction) share one matrix: every kernel walks the rows once and serves all
// of them, so the operator is read once per product for the NR systems.  Right preconditioning by D^-1 (the momentum
// matrix is dominated by its BDF2 diagonal at the time steps of interest).
// Per system j the scalars live at scal[16 j + k]:
//   0 rho, 1 alpha, 2 omega, 3 beta, 4 (rh,v), 5 (t,s), 6 (t,t), 7 (r,r),
//   8 (b,b), 9 active, 10 breakdown, 11 iterations
constexpr int kMomScal = 16;
__device__ __forceinline__ bool mom_active(const double* scal, int j) { return scal[kMomScal * j + 9] != 0.0; }

template <int NR>
__device__ __forceinline__ void sell_mv(const SellView<double>& A, int row, const double* __restrict__ x, size_t N,
                                       double* y) {
#pragma unroll
    for (int j = 0; j < NR; ++j) y[j] = 0.0;
    const int sl = row >> 5, l = row & 31;
    const int b = A.sptr[sl], w = (A.sptr[sl + 1] - b) >> 5;
    if (NR == 1 && w <= 8) {
        // one right-hand side, short rows (the mesh's): every entry load
        // first, then the gathers, so a row costs about two memory round
        // trips instead of one per entry; the products are summed in entry
        // order as below (0.85 -> 0.73 ms for the volume-fraction solve at
        // 128^3; with three right-hand sides the batch's registers cost more
        // than it gains: 1.63 -> 1.67 ms for the momentum solve)
        int cj[8];
        double vj[8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q < w) { cj[q] = A.col[b + l + 32 * q]; vj[q] = A.val[b + l + 32 * q]; }
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q < w) {
#pragma unroll
                for (int j = 0; j < NR; ++j) y[j] += vj[q] * __ldg(x + j * N + cj[q]);
            }
        return;
    }
    for (int e = 0, k = b + l; e < w; ++e, k += 32) {
        const int c = A.col[k];
        const double v = A.val[k];
#pragma unroll
        for (int j = 0; j < NR; ++j) y[j] += v * __ldg(x + j * N + c);
    }
}

// x = 0, r = rh = b, p = v = 0;  part = (b,b) per system
template <int NR>
__global__ void __launch_bounds__(kRedThreads) k_bi_init(int n, const double* __restrict__ b, double* __restrict__ x,
                                                         double* __restrict__ r, double* __restrict__ rh,
                                                         double* __restrict__ p, double* __restrict__ v,
                                                         double* __restrict__ part) {
    __shared__ double sh[32];
    double bb[NR] = {};
    const size_t N = n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int j = 0; j < NR; ++j) {
            const double bi = b[j * N + i];
            x[j * N + i] = 0.0; r[j * N + i] = bi; rh[j * N + i] = bi; p[j * N + i] = 0.0; v[j * N + i] = 0.0;
            bb[j] += bi * bi;
        }
    for (int j = 0; j < NR; ++j) {
        const double t = block_sum(bb[j], sh);
        if (threadIdx.x == 0) part[j * kRedBlocks + blockIdx.x] = t;
    }
}
template <int NR>
__global__ void k_bi_fin0(const double* __restrict__ part, double* __restrict__ scal, double tol2) {
    __shared__ double sh[32];
    for (int j = 0; j < NR; ++j) {
        const double bb = sum_parts(part + j * kRedBlocks, sh);
        if (threadIdx.x == 0) {
            double* S = scal + kMomScal * j;
            for (int k = 0; k < kMomScal; ++k) S[k] = 0.0;
            S[0] = bb; S[1] = 1.0; S[2] = 1.0; S[3] = 0.0; S[7] = bb; S[8] = bb;
            S[9] = (bb > 0.0 && !(bb <= tol2 * bb)) ? 1.0 : 0.0;
        }
    }
}
// p = r + beta (p - omega v);  ph = D^-1 p
template <int NR>
__global__ void k_bi_p(int n, const double* __restrict__ dinv, const double* __restrict__ r, double* __restrict__ p,
                       const double* __restrict__ v, double* __restrict__ ph, const double* __restrict__ scal) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = n;
    const double di = dinv[i];
    for (int j = 0; j < NR; ++j) {
        if (!mom_active(scal, j)) continue;
        const double beta = scal[kMomScal * j + 3], omega = scal[kMomScal * j + 2];
        const double pi = r[j * N + i] + beta * (p[j * N + i] - omega * v[j * N + i]);
        p[j * N + i] = pi;
        ph[j * N + i] = di * pi;
    }
}
// y = A x for the three systems;  part = (rh, y) per system
template <int NR>
__global__ void __launch_bounds__(kRedThreads) k_bi_mv1(SellView<double> A, const double* __restrict__ x,
                                                        double* __restrict__ y, const double* __restrict__ rh,
                                                        const double* __restrict__ scal, double* __restrict__ part) {
    __shared__ double sh[32];
    const size_t N = A.n;
    double d[NR] = {};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x) {
        double s[NR];
        sell_mv<NR>(A, row, x, N, s);
        for (int j = 0; j < NR; ++j) {
            if (!mom_active(scal, j)) continue;
            y[j * N + row] = s[j];
            d[j] += rh[j * N + row] * s[j];
        }
    }
    for (int j = 0; j < NR; ++j) {
        const double t = block_sum(d[j], sh);
        if (threadIdx.x == 0) part[j * kRedBlocks + blockIdx.x] = t;
    }
}
template <int NR>
__global__ void k_bi_fin1(const double* __restrict__ part, double* __restrict__ scal) {
    __shared__ double sh[32];
    for (int j = 0; j < NR; ++j) {
        const double rv = sum_parts(part + j * kRedBlocks, sh);
        if (threadIdx.x == 0) {
            double* S = scal + kMomScal * j;
            if (S[9] != 0.0) {
                S[4] = rv;
                if (rv == 0.0 || !isfinite(rv)) { S[10] = 1.0; S[9] = 0.0; }
                else S[1] = S[0] / rv;
            }
        }
    }
}
// s = r - alpha v (in place in r);  sh = D^-1 s
template <int NR>
__global__ void k_bi_s(int n, const double* __restrict__ dinv, double* __restrict__ r, const double* __restrict__ v,
                       double* __restrict__ shv, const double* __restrict__ scal) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = n;
    const double di = dinv[i];
    for (int j = 0; j < NR; ++j) {
        if (!mom_active(scal, j)) continue;
        const double si = r[j * N + i] - scal[kMomScal * j + 1] * v[j * N + i];
        r[j * N + i] = si;
        shv[j * N + i] = di * si;
    }
}
// t = A sh;  part = (t,s), (t,t) per system
template <int NR>
__global__ void __launch_bounds__(kRedThreads) k_bi_mv2(SellView<double> A, const double* __restrict__ x,
                                                        double* __restrict__ t, const double* __restrict__ s,
                                                        const double* __restrict__ scal, double* __restrict__ part) {
    __shared__ double sh[32];
    const size_t N = A.n;
    double ts[NR] = {}, tt[NR] = {};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x) {
        double y[NR];
        sell_mv<NR>(A, row, x, N, y);
        for (int j = 0; j < NR; ++j) {
            if (!mom_active(scal, j)) continue;
            t[j * N + row] = y[j];
            ts[j] += y[j] * s[j * N + row];
            tt[j] += y[j] * y[j];
        }
    }
    for (int j = 0; j < NR; ++j) {
        const double a = block_sum(ts[j], sh);
        const double b = block_sum(tt[j], sh);
        if (threadIdx.x == 0) { part[(2 * j) * kRedBlocks + blockIdx.x] = a; part[(2 * j + 1) * kRedBlocks + blockIdx.x] = b; }
    }
}
template <int NR>
__global__ void k_bi_fin2(const double* __restrict__ part, double* __restrict__ scal) {
    __shared__ double sh[32];
    for (int j = 0; j < NR; ++j) {
        const double ts = sum_parts(part + (2 * j) * kRedBlocks, sh);
        const double tt = sum_parts(part + (2 * j + 1) * kRedBlocks, sh);
        if (threadIdx.x == 0) {
            double* S = scal + kMomScal * j;
            if (S[9] != 0.0) { S[5] = ts; S[6] = tt; S[2] = (tt > 0.0) ? ts / tt : 0.0; }
        }
    }
}
// x += alpha ph + omega sh;  r = s - omega t;  part = (rh,r), (r,r)
template <int NR>
__global__ void __launch_bounds__(kRedThreads) k_bi_xr(int n, double* __restrict__ x, const double* __restrict__ ph,
                                                       const double* __restrict__ shv, double* __restrict__ r,
                                                       const double* __restrict__ t, const double* __restrict__ rh,
                                                       const double* __restrict__ scal, double* __restrict__ part) {
    __shared__ double sh[32];
    const size_t N = n;
    double a[NR] = {}, b[NR] = {};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int j = 0; j < NR; ++j) {
            if (!mom_active(scal, j)) continue;
            const double alpha = scal[kMomScal * j + 1], omega = scal[kMomScal * j + 2];
            x[j * N + i] += alpha * ph[j * N + i] + omega * shv[j * N + i];
            const double ri = r[j * N + i] - omega * t[j * N + i];
            r[j * N + i] = ri;
            a[j] += rh[j * N + i] * ri;
            b[j] += ri * ri;
        }
    for (int j = 0; j < NR; ++j) {
        const double u = block_sum(a[j], sh);
        const double w = block_sum(b[j], sh);
        if (threadIdx.x == 0) { part[(2 * j) * kRedBlocks + blockIdx.x] = u; part[(2 * j + 1) * kRedBlocks + blockIdx.x] = w; }
    }
}
template <int NR>
__global__ void k_bi_fin3(const double* __restrict__ part, double* __restrict__ scal, double tol2) {
    __shared__ double sh[32];
    for (int j = 0; j < NR; ++j) {
        const double rho1 = sum_parts(part + (2 * j) * kRedBlocks, sh);
        const double rr = sum_parts(part + (2 * j + 1) * kRedBlocks, sh);
        if (threadIdx.x == 0) {
            double* S = scal + kMomScal * j;
            if (S[9] != 0.0) {
                S[11] += 1.0;                                        // iterations of this system
                S[7] = rr;
                if (rr <= tol2 * S[8]) {
                    S[9] = 0.0;                                     // converged
                } else if (rho1 == 0.0 || S[2] == 0.0 || !isfinite(rr)) {
                    S[10] = 1.0; S[9] = 0.0;                        // breakdown
                } else {
                    S[3] = (rho1 / S[0]) * (S[1] / S[2]);
                    S[0] = rho1;
                }
            }
        }
    }
}
// r = b - A x;  part = (r,r) per system
template <int NR>
__global__ void __launch_bounds__(kRedThreads) k_bi_res(SellView<double> A, const double* __restrict__ x,
                                                        const double* __restrict__ b, double* __restrict__ part) {
    __shared__ double sh[32];
    const size_t N = A.n;
    double d[NR] = {};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x) {
        double y[NR];
        sell_mv<NR>(A, row, x, N, y);
        for (int j = 0; j < NR; ++j) { const double ri = b[j * N + row] - y[j]; d[j] += ri * ri; }
    }
    for (int j = 0; j < NR; ++j) {
        const double t = block_sum(d[j], sh);
        if (threadIdx.x == 0) part[j * kRedBlocks + blockIdx.x] = t;
    }
}
template <int NR>
__global__ void k_bi_fin_res(const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[32];
    for (int j = 0; j < NR; ++j) {
        const double rr = sum_parts(part + j * kRedBlocks, sh);
        if (threadIdx.x == 0) out[j] = rr;
    }
}
__global__ void k_dinv_dig(int n, const int* __restrict__ dig, const double* __restrict__ val,
                           double* __restrict__ dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dinv[i] = 1.0 / val[dig[i]];
}

// The instantiated iteration graph of a batched BiCGStab, kept while every
// pointer and scalar baked into its kernels stays the same (the buffers below
// are reused from call to call, so the momentum and volume-fraction solves of
// successive outer iterations launch it without capturing it again).
struct BiGraphKey {
    int nr = 0, n = 0, max_iter = 0;
    double tol2 = 0.0;
    const void* ptrs[8] = {};
    bool operator==(const BiGraphKey& o) const {
        if (nr != o.nr || n != o.n || max_iter != o.max_iter || tol2 != o.tol2) return false;
        for (int k = 0; k < 8; ++k)
            if (ptrs[k] != o.ptrs[k]) return false;
        return true;
    }
};
struct BiGraph {
    BiGraphKey key;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    void reset() {
        if (e) cudaGraphExecDestroy(e);
        if (g) cudaGraphDestroy(g);
        e = nullptr;
        g = nullptr;
        key = BiGraphKey{};
    }
    BiGraph() = default;
    BiGraph(const BiGraph&) = delete;
    BiGraph& operator=(const BiGraph&) = delete;
    ~BiGraph() { reset(); }
};
struct MomState {
    Sell<double> A;
    int gen = -1;                 // mesh generation the SELL layout was built for
    DBuf<double> dinv, vec, part, scal;
    BiGraph graph[2];             // NR = 1, NR = 3
};

// end of one batched BiCGStab iteration on the device: go on while a system
// is active and the cap is not reached (scal[3*16+0] counts iterations)
template <int NR>
__global__ void k_bi_check(cudaGraphConditionalHandle h, double* __restrict__ scal, int max_iter) {
    double* it = scal + 3 * kMomScal;
    it[0] += 1.0;
    bool any = false;
    for (int j = 0; j < NR; ++j) any |= scal[kMomScal * j + 9] != 0.0;
    cudaGraphSetConditional(h, (any && it[0] < (double)max_iter) ? 1u : 0u);
}
MomState& mom_state(semo_ctx* c) {
    if (!c->mom_apply) c->mom_apply = std::shared_ptr<void>(new MomState(), [](void* p) { delete (MomState*)p; });
    return *(MomState*)c->mom_apply.get();
}

}  // namespace

void pressure_setup(semo_ctx* c, const int* ptr, const int* col, const double* val, int n, int64_t nnz,
                    bool may_reuse, semo_solve_info* info) {
    cudaStream_t s = setup_stream(c);
    ApplyState& st = apply_state(c);
    c->sflag.alloc(16, s);
    SEMO_CUDA(cudaMemsetAsync(c->sflag.p, 0, 16 * sizeof(int), s));
    SEMO_CUDA(cudaEventRecord(c->setup_ev[0], s));
    {
        StageScope sc(c, ST_AMG_SETUP);
        // The hierarchy is a deterministic function of the matrix: when the
        // values are bit-identical to the ones it was built from (the pressure
        // matrix depends only on geometry, dt and the densities, so it repeats
        // across the outer iterations of a time step), rebuilding would give
        // the same hierarchy bit for bit, and it is kept instead.
        bool reuse = false;
        const Amg<float>& h32 = c->amg32;
        const Amg<double>& h64 = c->amg64;
        const bool have = (c->prm.precision == SEMO_PREC_MIXED) ? h32.ready : h64.ready;
        if (may_reuse && c->prm.reuse_hierarchy && have && st.src_prec == c->prm.precision && st.src_n == n &&
            st.src_nnz == nnz) {
            k_differs<<<kRedBlocks, kRedThreads, 0, s>>>(nnz, val, st.src_val, c->sflag.p + 10);
            SEMO_CHECK_LAUNCH();
            int* const differs = c->hpin_int + 13;
            SEMO_CUDA(cudaMemcpyAsync(differs, c->sflag.p + 10, sizeof(int), cudaMemcpyDeviceToHost, s));
            SEMO_CUDA(cudaStreamSynchronize(s));
            reuse = *differs == 0;
        }
        if (!reuse) {
            if (c->prm.precision == SEMO_PREC_MIXED) {
                c->amg64.clear();
                build_hierarchy<float>(c, c->amg32, ptr, col, val, n, nnz);
            } else {
                c->amg32.clear();
                build_hierarchy<double>(c, c->amg64, ptr, col, val, n, nnz);
            }
            StageScope scy(c, ST_SETUP_CYCLE);
            // on the mesh's own pattern the layout structure is built once per mesh
            std::shared_ptr<Sell16Struct> pat;
            if (ptr == c->A_ptr.p && col == c->A_col.p) {
                if (!st.pat16 || st.pat16_gen != c->mesh_gen || st.pat16->n != n)
                    st.pat16 = build_sell16_struct(s, ptr, col, n, c->hpin_int + 4);
                st.pat16_gen = c->mesh_gen;
                pat = st.pat16;
            } else {
                pat = build_sell16_struct(s, ptr, col, n, c->hpin_int + 4);
            }
            if (c->prm.precision == SEMO_PREC_MIXED)
                prepare_cycle(c, c->amg32, st.cy32, pat);
            else
                prepare_cycle(c, c->amg64, st.cy64, pat);
            fill_sell16<double, double>(s, ptr, val, pat, st.outer.s16);
            st.outer.use16 = true;
            st.src_prec = -1;
            if (may_reuse && c->prm.reuse_hierarchy) {
                st.src_val.alloc(nnz, s);
                SEMO_CUDA(cudaMemcpyAsync(st.src_val.p, val, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, s));
                st.src_n = n;
                st.src_nnz = nnz;
                st.src_prec = c->prm.precision;
            }
        }
    }
    SEMO_CUDA(cudaEventRecord(c->setup_ev[1], s));   // setup_ms is read from setup_ev after the solve
    (void)info;
}

void solve_system(semo_ctx* c, const int* ptr, const int* col, const double* val, int n, int64_t nnz,
                  const double* b, double* x, semo_solve_info* info, bool zero_guess, bool may_reuse) {
    cudaStream_t s = c->stream;
    // with matrix_prebuilt the hierarchy is being built beside this thread's
    // work; before_solve joins that setup and makes this stream wait for it
    if (c->before_solve) {
        auto f = std::move(c->before_solve);
        c->before_solve = nullptr;
        f();
    }
    ApplyState& st = apply_state(c);
    c->flag.zero();
    if (!c->matrix_prebuilt) pressure_setup(c, ptr, col, val, n, nnz, may_reuse, info);
    SEMO_CUDA(cudaEventRecord(c->ev[2], s));
    {
        StageScope sc(c, ST_PCG);
        if (c->prm.precision == SEMO_PREC_MIXED) {
            pcg<float>(c, c->amg32, st.cy32, st.outer, ptr, col, val, n, b, x, zero_guess, info);
            fill_info(c->amg32, nnz, info);
        } else {
            pcg<double>(c, c->amg64, st.cy64, st.outer, ptr, col, val, n, b, x, zero_guess, info);
            fill_info(c->amg64, nnz, info);
        }
    }
    SEMO_CUDA(cudaEventRecord(c->ev[3], s));
    SEMO_CUDA(cudaEventSynchronize(c->ev[3]));
    float t0 = 0, t1 = 0;
    if (c->matrix_prebuilt) {
        t0 = (float)c->side_setup_ms;   // the setup shared the GPU with the momentum pass
    } else {
        SEMO_CUDA(cudaEventSynchronize(c->setup_ev[1]));
        SEMO_CUDA(cudaEventElapsedTime(&t0, c->setup_ev[0], c->setup_ev[1]));
    }
    SEMO_CUDA(cudaEventElapsedTime(&t1, c->ev[2], c->ev[3]));
    info->setup_ms = t0;
    info->solve_ms = t1;
}

namespace {

// The CSR pattern a batched BiCGStab solve runs on: the context's mesh
// pattern (gen = the mesh generation, so its SELL layout is kept across
// solves) or a caller's matrix (gen < 0: the layout is built for this solve).
struct KrylovPattern {
    int n;
    const int* ptr;
    const int* col;
    const int* dig;   // position of each row's diagonal
    int gen;
};
KrylovPattern mesh_pattern(semo_ctx* c) { return KrylovPattern{c->nc, c->A_ptr, c->A_col, c->A_dig, c->mesh_gen}; }

// Jacobi-preconditioned BiCGStab on NR right-hand sides (planes of b, x) of
// the matrix with values val on the pattern pat, from x = 0.
template <int NR>
semo_status bicgstab_jacobi(semo_ctx* c, int stage, const KrylovPattern& pat, const double* val, const double* b,
                            double* x, semo_solve_info* info) {
    StageScope scope(c, stage);
    cudaStream_t s = c->stream;
    const int n = pat.n;
    const size_t N = n;
    MomState& st = mom_state(c);
    st.dinv.alloc(N, s);
    st.vec.alloc(7 * 3 * N, s);       // r, rh, p, v, ph, sh, t (room for 3 systems)
    st.part.alloc(6 * kRedBlocks, s);
    st.scal.alloc(4 * kMomScal, s);
    double* r = st.vec.p;
    double* rh = r + NR * N;
    double* p = rh + NR * N;
    double* v = p + NR * N;
    double* ph = v + NR * N;
    double* shv = ph + NR * N;
    double* t = shv + NR * N;
    // the recurrence residual is driven to half the tolerance so that the true
    // residual, checked at the end, lands under it
    const double tol2 = 0.25 * c->prm.mom_tol * c->prm.mom_tol;
    SEMO_CUDA(cudaEventRecord(c->ev[0], s));
    if (pat.gen < 0 || st.gen != pat.gen) {
        build_sell<double, double>(s, pat.ptr, pat.col, val, n, st.A, c->hpin_scan);
        st.gen = pat.gen;
    } else {   // same pattern (the mesh's): refill the values into the kept layout
        k_sell_fill<double, double><<<blocks((int64_t)st.A.nslices * 32, 256), 256, 0, s>>>(
            n, pat.ptr, pat.col, val, st.A.sptr, st.A.col, st.A.val);
        SEMO_CHECK_LAUNCH();
    }
    k_dinv_dig<<<blocks(n, 256), 256, 0, s>>>(n, pat.dig, val, st.dinv);
    SEMO_CHECK_LAUNCH();
    SEMO_CUDA(cudaEventRecord(c->ev[1], s));
    const SellView<double> A = st.A.view();
    k_bi_init<NR><<<kRedBlocks, kRedThreads, 0, s>>>(n, b, x, r, rh, p, v, st.part);
    SEMO_CHECK_LAUNCH();
    k_bi_fin0<NR><<<1, 256, 0, s>>>(st.part, st.scal, tol2);
    SEMO_CHECK_LAUNCH();
    // The iterations run as one graph: a conditional WHILE node around one
    // iteration (8 kernels + k_bi_check), launched without a host round trip
    // first: systems whose right-hand side is zero, already converged or not
    // finite start inactive (k_bi_fin0), every kernel skips them, and the
    // host reads the outcome once, after the true residuals.
    BiGraph& G = st.graph[NR == 1 ? 0 : 1];
    BiGraphKey key;
    key.nr = NR;
    key.n = n;
    key.max_iter = c->prm.mom_max_iter;
    key.tol2 = tol2;
    const void* kp[8] = {A.sptr, A.col, A.val, st.dinv.p, st.vec.p, st.part.p, st.scal.p, x};
    std::copy(kp, kp + 8, key.ptrs);
    if (!G.e || !(G.key == key)) {
        G.reset();
        SEMO_CUDA(cudaGraphCreate(&G.g, 0));
        cudaGraphConditionalHandle handle;
        SEMO_CUDA(cudaGraphConditionalHandleCreate(&handle, G.g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t loop;
        SEMO_CUDA(cudaGraphAddNode(&loop, G.g, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        const long long before = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
        SEMO_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        try {
            k_bi_p<NR><<<blocks(n, 256), 256, 0, s>>>(n, st.dinv, r, p, v, ph, st.scal);
            SEMO_CHECK_LAUNCH();
            k_bi_mv1<NR><<<kRedBlocks, kRedThreads, 0, s>>>(A, ph, v, rh, st.scal, st.part);
            SEMO_CHECK_LAUNCH();
            k_bi_fin1<NR><<<1, 256, 0, s>>>(st.part, st.scal);
            SEMO_CHECK_LAUNCH();
            k_bi_s<NR><<<blocks(n, 256), 256, 0, s>>>(n, st.dinv, r, v, shv, st.scal);
            SEMO_CHECK_LAUNCH();
            k_bi_mv2<NR><<<kRedBlocks, kRedThreads, 0, s>>>(A, shv, t, r, st.scal, st.part);
            SEMO_CHECK_LAUNCH();
            k_bi_fin2<NR><<<1, 256, 0, s>>>(st.part, st.scal);
            SEMO_CHECK_LAUNCH();
            k_bi_xr<NR><<<kRedBlocks, kRedThreads, 0, s>>>(n, x, ph, shv, r, t, rh, st.scal, st.part);
            SEMO_CHECK_LAUNCH();
            k_bi_fin3<NR><<<1, 256, 0, s>>>(st.part, st.scal, tol2);
            SEMO_CHECK_LAUNCH();
            k_bi_check<NR><<<1, 1, 0, s>>>(handle, st.scal, c->prm.mom_max_iter);
            SEMO_CHECK_LAUNCH();
        } catch (...) {
            cudaGraph_t junk = nullptr;
            cudaStreamEndCapture(s, &junk);
            G.reset();
            throw;
        }
        cudaGraph_t captured = nullptr;
        SEMO_CUDA(cudaStreamEndCapture(s, &captured));
        __atomic_store_n(&g_kernel_launches, before, __ATOMIC_RELAXED);
        SEMO_CUDA(cudaGraphInstantiate(&G.e, G.g, 0));
        G.key = key;
    }
    SEMO_CUDA(cudaMemsetAsync(st.scal.p + 3 * kMomScal, 0, sizeof(double) * kMomScal, s));
    SEMO_CUDA(cudaGraphLaunch(G.e, s));
    // true FP64 residuals of the returned solutions
    k_bi_res<NR><<<kRedBlocks, kRedThreads, 0, s>>>(A, x, b, st.part);
    SEMO_CHECK_LAUNCH();
    k_bi_fin_res<NR><<<1, 256, 0, s>>>(st.part, st.scal.p + 3 * kMomScal - 3);
    SEMO_CHECK_LAUNCH();
    // pinned: the systems' scalars and the iteration count hpin[0, 64), the
    // true residuals hpin[64, 64 + NR)
    double* const hs = c->hpin;
    double* const tr = c->hpin + 4 * kMomScal;
    SEMO_CUDA(cudaMemcpyAsync(hs, st.scal.p, sizeof(double) * 4 * kMomScal, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaMemcpyAsync(tr, st.scal.p + 3 * kMomScal - 3, sizeof(double) * NR, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaEventRecord(c->ev[2], s));
    SEMO_CUDA(cudaEventSynchronize(c->ev[2]));
    const int it = (int)hs[3 * kMomScal];
    __atomic_add_fetch(&g_kernel_launches, 9LL * it, __ATOMIC_RELAXED);
    int iters[NR] = {};
    for (int j = 0; j < NR; ++j) {
        if (!std::isfinite(hs[kMomScal * j + 8])) throw Error(SEMO_ERR_NAN, "non-finite right-hand side");
        if (!std::isfinite(hs[kMomScal * j + 7])) throw Error(SEMO_ERR_NAN, "NaN/Inf in the BiCGStab residual");
        // systems converge one after another; each counts the iterations it was active
        iters[j] = (int)hs[kMomScal * j + 11];
    }
    float t0 = 0, t1 = 0;
    SEMO_CUDA(cudaEventElapsedTime(&t0, c->ev[0], c->ev[1]));
    SEMO_CUDA(cudaEventElapsedTime(&t1, c->ev[1], c->ev[2]));
    semo_status worst = SEMO_OK;
    for (int j = 0; j < NR; ++j) {
        const double bb = hs[kMomScal * j + 8];
        const double rel = (bb > 0.0) ? std::sqrt(tr[j] / bb) : 0.0;
        if (info) {
            info[j] = semo_solve_info{};
            info[j].iterations = iters[j];
            info[j].rel_residual = rel;
            info[j].levels = 1;
            info[j].coarse_size = n;
            info[j].operator_complexity = 1.0;
            info[j].setup_ms = t0;
            info[j].solve_ms = t1;
        }
        if (hs[kMomScal * j + 10] != 0.0 && !(rel <= c->prm.mom_tol)) worst = SEMO_ERR_BREAKDOWN;
        else if (!(rel <= c->prm.mom_tol) && worst == SEMO_OK) worst = SEMO_ERR_NOT_CONVERGED;
    }
    return worst;
}

}  // namespace

semo_status solve_momentum(semo_ctx* c, semo_solve_info* info) {
    c->xm.alloc(3 * (size_t)c->nc, c->stream);
    return bicgstab_jacobi<3>(c, ST_MSOLVE, mesh_pattern(c), c->Am_val, c->bm, c->xm, info);
}

semo_status solve_vof(semo_ctx* c, semo_solve_info* info) {
    c->xvf.alloc((size_t)c->nc, c->stream);
    return bicgstab_jacobi<1>(c, ST_VSOLVE, mesh_pattern(c), c->Av_val, c->bvf, c->xvf, info);
}

semo_status solve_csr_multi(semo_ctx* c, int n, const int* ptr, const int* col, const int* dig, const double* val,
                            int nrhs, const double* b, double* x, bool guess, semo_solve_info* info) {
    cudaStream_t s = c->stream;
    const size_t N = n;
    const KrylovPattern pat{n, ptr, col, dig, -1};
    // with an initial guess x0: solve A d = b - A x0 from d = 0, then x = x0 + d
    DBuf<double> rb, d;
    const double* rhs = b;
    double* sol = x;
    if (guess) {
        rb.alloc(N * nrhs, s);
        d.alloc(N * nrhs, s);
        const CsrView<double, 8> A8{ptr, col, val, n};
        for (int j = 0; j < nrhs; ++j) {
            k_res64<<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(A8, x + j * N, b + j * N, rb.p + j * N);
            SEMO_CHECK_LAUNCH();
        }
        rhs = rb.p;
        sol = d.p;
    }
    semo_status worst = SEMO_OK;
    auto merge = [&](semo_status st) {
        if (st == SEMO_ERR_BREAKDOWN || (st != SEMO_OK && worst == SEMO_OK)) worst = st;
    };
    if (nrhs == 3) {
        merge(bicgstab_jacobi<3>(c, ST_MSOLVE, pat, val, rhs, sol, info));
    } else {
        for (int j = 0; j < nrhs; ++j)
            merge(bicgstab_jacobi<1>(c, ST_MSOLVE, pat, val, rhs + j * N, sol + j * N, info ? info + j : nullptr));
    }
    if (guess) {
        k_axpy1<double><<<blocks((int64_t)N * nrhs, 256), 256, 0, s>>>((int)(N * nrhs), d.p, x);
        SEMO_CHECK_LAUNCH();
    }
    SEMO_CUDA(cudaStreamSynchronize(s));
    return worst;
}

// Adjoint solve on the hierarchy of the last forward solve (the pressure
// matrix is symmetric, so A^T = A and the same preconditioner applies).
void solve_transpose_reuse(semo_ctx* c, const double* g, double* lam, semo_solve_info* info) {
    const int n = c->nc;
    ApplyState& st = apply_state(c);
    SEMO_CUDA(cudaEventRecord(c->ev[1], c->stream));
    if (c->prm.precision == SEMO_PREC_MIXED) {
        if (!c->amg32.ready) throw Error(SEMO_ERR_STATE, "no hierarchy: run a forward solve first");
        pcg<float>(c, c->amg32, st.cy32, st.outer, c->A_ptr, c->A_col, c->A_val, n, g, lam, true, info);
        fill_info(c->amg32, c->nnz, info);
    } else {
        if (!c->amg64.ready) throw Error(SEMO_ERR_STATE, "no hierarchy: run a forward solve first");
        pcg<double>(c, c->amg64, st.cy64, st.outer, c->A_ptr, c->A_col, c->A_val, n, g, lam, true, info);
        fill_info(c->amg64, c->nnz, info);
    }
    SEMO_CUDA(cudaEventRecord(c->ev[2], c->stream));
    SEMO_CUDA(cudaEventSynchronize(c->ev[2]));
    float t1 = 0;
    SEMO_CUDA(cudaEventElapsedTime(&t1, c->ev[1], c->ev[2]));
    info->setup_ms = 0.0;
    info->solve_ms = t1;
}

// ---- measurement hooks on the last pressure hierarchy ----------------------
namespace {
template <class V>
Amg<V>& pressure_amg(semo_ctx* c);
template <> Amg<float>& pressure_amg<float>(semo_ctx* c) { return c->amg32; }
template <> Amg<double>& pressure_amg<double>(semo_ctx* c) { return c->amg64; }
template <class V>
Cycle<V>& pressure_cycle(ApplyState& st);
template <> Cycle<float>& pressure_cycle<float>(ApplyState& st) { return st.cy32; }
template <> Cycle<double>& pressure_cycle<double>(ApplyState& st) { return st.cy64; }

// reps launches of y = A x with A the finest level's operator in the layout
// the V-cycle uses (which = 0) or the FP64 outer operator (which = 1)
template <class V>
double time_spmv(semo_ctx* c, int which, int reps) {
    ApplyState& st = apply_state(c);
    Amg<V>& h = pressure_amg<V>(c);
    if (!h.ready || h.lev.empty()) throw Error(SEMO_ERR_STATE, "no pressure hierarchy: run a pressure solve first");
    cudaStream_t s = c->stream;
    const int n = h.lev[0].A.n;
    if (which == 0 && h.lev.size() < 2) throw Error(SEMO_ERR_STATE, "single-level hierarchy: no V-cycle operator");
    if (which == 1 && (c->kp.n < (size_t)n || c->kq.n < (size_t)n)) throw Error(SEMO_ERR_STATE, "no Krylov vectors");
    cudaEvent_t e0, e1;
    SEMO_CUDA(cudaEventCreate(&e0));
    SEMO_CUDA(cudaEventCreate(&e1));
    float ms = 0.f;
    try {
        SEMO_CUDA(cudaEventRecord(e0, s));
        for (int k = 0; k < reps; ++k) {
            if (which == 0) {
                AmgLevel<V>& L = h.lev[0];
                with_A(pressure_cycle<V>(st).lev[0], L.A,
                       [&](auto A) { k_mv<<<grid_for(A), 256, 0, s>>>(A, L.x.p, L.t.p); });
            } else {
                st.outer.with([&](auto A) { k_mv<<<grid_for(A), 256, 0, s>>>(A, c->kp.p, c->kq.p); });
            }
            SEMO_CHECK_LAUNCH();
        }
        SEMO_CUDA(cudaEventRecord(e1, s));
        SEMO_CUDA(cudaEventSynchronize(e1));
        SEMO_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / reps;
}

template <class V>
int levels_of(semo_ctx* c, int64_t* out, int max_levels) {
    ApplyState& st = apply_state(c);
    Amg<V>& h = pressure_amg<V>(c);
    if (!h.ready) throw Error(SEMO_ERR_STATE, "no pressure hierarchy: run a pressure solve first");
    const int nl = (int)h.lev.size();
    Cycle<V>& cy = pressure_cycle<V>(st);
    for (int l = 0; l < nl && l < max_levels; ++l) {
        const AmgLevel<V>& L = h.lev[l];
        int64_t* o = out + 6 * l;
        o[0] = L.A.n;
        o[1] = L.A.nnz;
        o[2] = L.P.nnz;
        o[3] = L.R.nnz;
        o[4] = (l + 1 < nl && l < (int)cy.lev.size()) ? (cy.lev[l].a16 ? 2 : (cy.lev[l].a ? 1 : 0)) : -1;
        o[5] = (int64_t)sizeof(V);
    }
    return nl;
}
}  // namespace

double time_pressure_spmv(semo_ctx* c, int which, int reps) {
    return c->prm.precision == SEMO_PREC_MIXED ? time_spmv<float>(c, which, reps) : time_spmv<double>(c, which, reps);
}

int pressure_levels(semo_ctx* c, int64_t* out, int max_levels) {
    return c->prm.precision == SEMO_PREC_MIXED ? levels_of<float>(c, out, max_levels)
                                               : levels_of<double>(c, out, max_levels);
}

// ---- AMG on the pressure equation of the coupled system (first stage of its
// two-stage preconditioner).  A hierarchy of its own, so the pressure
// equation's hierarchy is left as it is.
struct CprState {
    Amg<float> h32;
    Cycle<float> cy32;
    Amg<double> h64;
    Cycle<double> cy64;
};
CprState& cpr_state(semo_ctx* c) {
    if (!c->cpr) c->cpr = std::shared_ptr<void>(new CprState(), [](void* p) { delete (CprState*)p; });
    return *(CprState*)c->cpr.get();
}
template <class V> Amg<V>& cpr_h(CprState& S);
template <> Amg<float>& cpr_h<float>(CprState& S) { return S.h32; }
template <> Amg<double>& cpr_h<double>(CprState& S) { return S.h64; }
template <class V> Cycle<V>& cpr_cy(CprState& S);
template <> Cycle<float>& cpr_cy<float>(CprState& S) { return S.cy32; }
template <> Cycle<double>& cpr_cy<double>(CprState& S) { return S.cy64; }

template <class V>
void cpr_setup(semo_ctx* c, const int* ptr, const int* col, const double* val, int n, int64_t nnz) {
    CprState& S = cpr_state(c);
    build_hierarchy<V>(c, cpr_h<V>(S), ptr, col, val, n, nnz);
    prepare_cycle(c, cpr_h<V>(S), cpr_cy<V>(S));
}

// x = one V-cycle (zero start, both smoothing sweeps on every level) applied to b
template <class V>
void cpr_vcycle(semo_ctx* c, const V* b, V* x) {
    CprState& S = cpr_state(c);
    Amg<V>& h = cpr_h<V>(S);
    Cycle<V>& cy = cpr_cy<V>(S);
    cudaStream_t s = c->stream;
    AmgLevel<V>& L = h.lev[0];
    const int n = L.A.n;
    SEMO_CUDA(cudaMemcpyAsync(L.b.p, b, sizeof(V) * n, cudaMemcpyDeviceToDevice, s));
    vcycle_from(c, h, cy, 0);
    if (h.lev.size() > 1 && c->prm.cheb_degree == 2 && !cy.lev[0].gs) {
        // the last step vcycle_from leaves to the fused CG kernels on the finest level
        const ChebCoef cc = cheb2(L.lam_max);
        with_A(cy.lev[0], L.A, [&](auto A) {
            k_post1<<<grid_for(A), 256, 0, s>>>(A, L.dinv.p, L.b.p, (V)cc.c1, (V)cc.c2, L.r.p, L.t.p, L.x.p);
        });
        SEMO_CHECK_LAUNCH();
    }
    SEMO_CUDA(cudaMemcpyAsync(x, L.x.p, sizeof(V) * n, cudaMemcpyDeviceToDevice, s));
}
template void cpr_setup<float>(semo_ctx*, const int*, const int*, const double*, int, int64_t);
template void cpr_setup<double>(semo_ctx*, const int*, const int*, const double*, int, int64_t);
template void cpr_vcycle<float>(semo_ctx*, const float*, float*);
template void cpr_vcycle<double>(semo_ctx*, const double*, double*);

}  // namespace semo
