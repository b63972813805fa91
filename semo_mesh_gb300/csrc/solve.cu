// AMG-preconditioned Krylov solve on the GPU.
//
// Replaces SEMO's solveAMGCL (src/solvers/solveAMGCL.cpp:179-1108), which
// builds AMGCL's smoothed-aggregation hierarchy and runs an OpenMP Krylov
// solver.  The coarsening keeps AMGCL's smoothed-aggregation semantics
// (lib/amgcl/coarsening/smoothed_aggregation.hpp:130-215,
// lib/amgcl/coarsening/plain_aggregates.hpp:120-140):
//   strong(i,j)  <=>  j != i  and  eps^2 * a_ii * a_jj < a_ij^2,  eps = 0.08 halved per level
//   P = (I - w D_f^-1 A_f) P_tent,  w = 2/3,  D_f = diag + weak off-diagonals
//   A_c = P^T A P
// but the aggregation is a deterministic parallel MIS(2) over the strong graph
// (synchronous max-propagation of (state, hash(i), i) tuples, after Bell,
// Dalton & Olson 2012) instead of AMGCL's serial greedy sweep.  Smoothing is
// Chebyshev on D^-1 A over [lambda/30, lambda] with a Gershgorin lambda; the
// coarsest level is solved with an explicit FP64 inverse.  The outer solver is
// flexible (Polak-Ribiere) CG in FP64; in mixed mode the whole hierarchy and
// V-cycle are FP32 while residuals, dot products and the solution stay FP64.
//
// All reductions use a fixed grid and a fixed-order final sum; the Galerkin
// SpGEMM accumulates products in a fixed order; so the solve is
// deterministic run to run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "semo_internal.h"

namespace semo {
namespace {

constexpr int kRedBlocks = 608;
constexpr int kRedThreads = 256;
inline int blocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ uint32_t hash_u32(uint32_t x) {
    // integer avalanche mixer (public-domain "lowbias32" constants)
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

// ------------------------------------------------------------------ reductions
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

// part[blockIdx] = sum a_i b_i over a grid-stride slice
template <class A, class B>
__global__ void __launch_bounds__(kRedThreads) k_dot(int n, const A* __restrict__ a, const B* __restrict__ b,
                                                     double* __restrict__ part) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s += (double)a[i] * (double)b[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// two dots at once: part[blk] = a.b, part[kRedBlocks+blk] = a.c
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

// sum `count` partial arrays (each kRedBlocks long) in fixed order -> out[0..count)
__global__ void k_finish(const double* __restrict__ part, int count, double* __restrict__ out) {
    __shared__ double sh[32];
    for (int c = 0; c < count; ++c) {
        double s = 0.0;
        for (int i = threadIdx.x; i < kRedBlocks; i += blockDim.x) s += part[c * kRedBlocks + i];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) out[c] = s;
    }
}

// --------------------------------------------------------------------- scans
constexpr int kScanT = 256, kScanItems = 8, kScanTile = kScanT * kScanItems;

__global__ void k_scan_tile(int n, const int* __restrict__ in, int* __restrict__ out, int* __restrict__ tile_sum) {
    __shared__ int sh[kScanT];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) { v[k] = (base + k < n) ? in[base + k] : 0; s += v[k]; }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < kScanT; o <<= 1) {
        int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    int run = sh[threadIdx.x] - s;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanT - 1) tile_sum[blockIdx.x] = sh[kScanT - 1];
}
__global__ void k_scan_add(int n, int* __restrict__ out, const int* __restrict__ tile_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_off[i / kScanTile];
}

// exclusive scan of d[0..n) in place; returns the total (host sync)
int scan_exclusive(cudaStream_t s, int* d, int n) {
    if (n <= 0) return 0;
    const int tiles = blocks(n, kScanTile);
    DBuf<int> ts;
    ts.alloc(tiles + 1, s);
    k_scan_tile<<<tiles, kScanT, 0, s>>>(n, d, d, ts.p);
    SEMO_CHECK_LAUNCH();
    int total = 0;
    if (tiles > 1) {
        // scan the tile sums (recursively) and add them back
        DBuf<int> tot;
        tot.alloc(tiles + 1, s);
        SEMO_CUDA(cudaMemcpyAsync(tot.p, ts.p, sizeof(int) * tiles, cudaMemcpyDeviceToDevice, s));
        int last = 0;
        SEMO_CUDA(cudaMemcpyAsync(&last, ts.p + tiles - 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        int sum_before_last = scan_exclusive(s, tot.p, tiles);  // syncs
        total = sum_before_last;
        (void)last;
        k_scan_add<<<blocks(n, 256), 256, 0, s>>>(n, d, tot.p);
        SEMO_CHECK_LAUNCH();
    } else {
        SEMO_CUDA(cudaMemcpyAsync(&total, ts.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
    }
    return total;
}

// ------------------------------------------------------------------ SpMV etc.
// Sub-warp CSR row dot product: VS lanes per row (rows are short, ~7 entries
// on the finest level).  Accumulates in the matrix's own type, so the FP32
// V-cycle runs on the FP32 pipes; every lane takes part in the shuffles,
// rows past n contribute zero.
template <class V, class X, int VS>
__device__ __forceinline__ V row_dot(int row, int n, int lane, const int* __restrict__ ptr,
                                     const int* __restrict__ col, const V* __restrict__ val,
                                     const X* __restrict__ x) {
    V s = V(0);
    if (row < n) {
        const int e = ptr[row + 1];
        for (int k = ptr[row] + lane; k < e; k += VS) s += val[k] * (V)__ldg(x + col[k]);
    }
#pragma unroll
    for (int o = VS / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, VS);
    return s;
}

// y = A x
template <class V, class X, int VS>
__global__ void __launch_bounds__(256) k_spmv(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                              const V* __restrict__ val, const X* __restrict__ x,
                                              X* __restrict__ y) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / VS, lane = g % VS;
    const V s = row_dot<V, X, VS>(row, n, lane, ptr, col, val, x);
    if (row < n && lane == 0) y[row] = (X)s;
}

// q = A p (FP64) and part = p.q
template <int VS>
__global__ void __launch_bounds__(256) k_spmv_dot(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                  const double* __restrict__ val, const double* __restrict__ p,
                                                  double* __restrict__ q, double* __restrict__ part) {
    __shared__ double sh[32];
    double acc = 0.0;
    const int rows_per_block = blockDim.x / VS;
    const int lane = threadIdx.x % VS;
    for (int row0 = blockIdx.x * rows_per_block; row0 < n; row0 += gridDim.x * rows_per_block) {
        const int row = row0 + threadIdx.x / VS;
        const double s = row_dot<double, double, VS>(row, n, lane, ptr, col, val, p);
        if (lane == 0 && row < n) { q[row] = s; acc += s * p[row]; }
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// r = b - A x
template <class V, int VS>
__global__ void __launch_bounds__(256) k_residual(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                  const V* __restrict__ val, const V* __restrict__ x,
                                                  const V* __restrict__ b, V* __restrict__ r) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / VS, lane = g % VS;
    const V s = row_dot<V, V, VS>(row, n, lane, ptr, col, val, x);
    if (row < n && lane == 0) r[row] = b[row] - s;
}

// Chebyshev first step from x = 0: d = D^-1 b / theta ; x = d
template <class V>
__global__ void k_cheb_first(int n, const V* __restrict__ dinv, const V* __restrict__ b, V inv_theta,
                             V* __restrict__ x, V* __restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V v = dinv[i] * b[i] * inv_theta;
    d[i] = v;
    x[i] = v;
}
// Chebyshev first step from a given x: d = D^-1 (b - A x) / theta (x += d by k_add:
// other rows of this launch still read x)
template <class V, int VS>
__global__ void __launch_bounds__(256) k_cheb_start(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                    const V* __restrict__ val, const V* __restrict__ dinv,
                                                    const V* __restrict__ b, V inv_theta, const V* __restrict__ x,
                                                    V* __restrict__ d) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / VS, lane = g % VS;
    const V s = row_dot<V, V, VS>(row, n, lane, ptr, col, val, x);
    if (row < n && lane == 0) d[row] = dinv[row] * (b[row] - s) * inv_theta;
}
template <class V>
__global__ void k_add(int n, const V* __restrict__ d, V* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += d[i];
}
// Chebyshev recurrence step: z = D^-1 (b - A x); d = c1 d + c2 z  (x += d by k_add)
template <class V, int VS>
__global__ void __launch_bounds__(256) k_cheb_step(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                   const V* __restrict__ val, const V* __restrict__ dinv,
                                                   const V* __restrict__ b, const V* __restrict__ x, V c1, V c2,
                                                   V* __restrict__ d) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / VS, lane = g % VS;
    const V s = row_dot<V, V, VS>(row, n, lane, ptr, col, val, x);
    if (row < n && lane == 0) d[row] = c1 * d[row] + c2 * (dinv[row] * (b[row] - s));
}
// x += P xc (prolongation and correction)
template <class V, int VS>
__global__ void __launch_bounds__(256) k_prolong(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const V* __restrict__ val, const V* __restrict__ xc,
                                                 V* __restrict__ x) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / VS, lane = g % VS;
    const V s = row_dot<V, V, VS>(row, n, lane, ptr, col, val, xc);
    if (row < n && lane == 0) x[row] += s;
}

// coarse solve x = Ainv b (dense FP64 inverse), one block
template <class V>
__global__ void k_coarse_solve(int n, const double* __restrict__ inv, const V* __restrict__ b, V* __restrict__ x) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += inv[(size_t)i * n + k] * (double)b[k];
        x[i] = (V)s;
    }
}

template <class A, class B>
__global__ void k_convert(int n, const A* __restrict__ a, B* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (B)a[i];
}

// ----------------------------------------------------------- Krylov updates
// scal[0..] live on the device: 0 rz, 1 zq, 2 pq, 3 rr, 4 alpha_prev, 5 beta, 6 alpha, 7 rz_prev
// scal[10] counts iterations (0 on the first), so one captured iteration
// serves every iteration of the loop
__global__ void k_cg_beta(double* scal) {
    if (threadIdx.x != 0) return;
    // Polak-Ribiere: beta = z.(r_k - r_{k-1}) / (z_{k-1}.r_{k-1}) = -alpha_{k-1} z.q_{k-1} / rz_prev
    scal[5] = (scal[10] == 0.0) ? 0.0 : (-scal[4] * scal[1] / scal[7]);
    scal[7] = scal[0];
    scal[10] += 1.0;
}
__global__ void k_p_update(int n, const double* __restrict__ z, double* __restrict__ p, const double* scal) {
    const double beta = scal[5];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i] + beta * p[i];
}
template <class Z>
__global__ void k_p_update_t(int n, const Z* __restrict__ z, double* __restrict__ p, const double* scal) {
    const double beta = scal[5];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (double)z[i] + beta * p[i];
}
__global__ void k_cg_alpha(double* scal) {
    if (threadIdx.x != 0) return;
    scal[6] = scal[7] / scal[2];
    scal[4] = scal[6];
}
__global__ void __launch_bounds__(kRedThreads) k_xr_update(int n, double* __restrict__ x, double* __restrict__ r,
                                                           const double* __restrict__ p,
                                                           const double* __restrict__ q, const double* scal,
                                                           double* __restrict__ part) {
    __shared__ double sh[32];
    const double alpha = scal[6];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * q[i];
        r[i] = ri;
        s += ri * ri;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
template <class R>
__global__ void k_copy_residual(int n, const double* __restrict__ r, R* __restrict__ rr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rr[i] = (R)r[i];
}

// --------------------------------------------------------------- AMG setup
template <class V>
__global__ void k_diag(int n, const int* __restrict__ ptr, const int* __restrict__ col, const V* __restrict__ val,
                       V* __restrict__ dia, V* __restrict__ dinv, double* __restrict__ ratio, int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 0.0, rs = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        const double v = (double)val[k];
        if (col[k] == i) d = v;
        rs += fabs(v);
    }
    if (!(d > 0.0) && !(d < 0.0)) atomicExch(flag + 2, 1);   // zero diagonal
    if (!isfinite(d) || !isfinite(rs)) atomicExch(flag + 3, 1);
    dia[i] = (V)d;
    dinv[i] = (V)(1.0 / d);
    ratio[i] = rs / fabs(d);
}

__global__ void __launch_bounds__(kRedThreads) k_max(int n, const double* __restrict__ a, double* __restrict__ part) {
    __shared__ double sh[32];
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, a[i]);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, sh[w]);
        part[blockIdx.x] = r;
    }
}

template <class V>
__global__ void k_strength(int n, const int* __restrict__ ptr, const int* __restrict__ col, const V* __restrict__ val,
                           const V* __restrict__ dia, double eps2, unsigned char* __restrict__ strong,
                           int* __restrict__ state) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V ed = (V)(eps2 * (double)dia[i]);
    int has = 0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        const int j = col[k];
        const V v = val[k];
        const unsigned char s = (j != i) && (ed * dia[j] < v * v);
        strong[k] = s;
        has |= s;
    }
    state[i] = has ? 1 : -1;   // -1: no strong connection, never aggregated
}

__device__ __forceinline__ unsigned long long mis_key(int st, int i) {
    const unsigned long long s = (st < 0) ? 0ull : (unsigned long long)st;
    return (s << 62) | ((unsigned long long)hash_u32((uint32_t)i) << 30) | (unsigned long long)i;
}

__global__ void k_mis_max1(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                           const unsigned char* __restrict__ strong, const int* __restrict__ state,
                           unsigned long long* __restrict__ m1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long m = mis_key(state[i], i);
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
        if (strong[k]) {
            const int j = col[k];
            const unsigned long long t = mis_key(state[j], j);
            m = (t > m) ? t : m;
        }
    m1[i] = m;
}
__global__ void k_mis_max2(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                           const unsigned char* __restrict__ strong, const unsigned long long* __restrict__ m1,
                           int* __restrict__ state, int* __restrict__ undecided) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long m = m1[i];
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
        if (strong[k]) { const unsigned long long t = m1[col[k]]; m = (t > m) ? t : m; }
    const int st = state[i];
    if (st != 1) return;
    // decided from the round's snapshot (m1 was computed before any update)
    if (m == mis_key(1, i)) state[i] = 2;
    else if ((m >> 62) == 2ull) state[i] = 0;
    else atomicAdd(undecided, 1);
}
// state update must not be seen by other threads of the same round: k_mis_max2
// reads only m1 (fixed for the round) and writes only its own state.

__global__ void k_root_flags(int n, const int* __restrict__ state, int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = (state[i] == 2) ? 1 : 0;
}
__global__ void k_root_ids(int n, const int* __restrict__ state, const int* __restrict__ scanned, int* __restrict__ agg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) agg[i] = (state[i] == 2) ? scanned[i] : -1;
}
__global__ void k_agg_join(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                           const unsigned char* __restrict__ strong, const int* __restrict__ state,
                           const int* __restrict__ agg_in, int* __restrict__ agg_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int a = agg_in[i];
    if (a < 0 && state[i] >= 0) {
        unsigned long long best = 0;
        int ba = -1;
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
            const int j = col[k];
            if (!strong[k] || agg_in[j] < 0) continue;
            const unsigned long long kj = ((unsigned long long)hash_u32((uint32_t)j) << 32) | (unsigned long long)j;
            if (ba < 0 || kj > best) { best = kj; ba = agg_in[j]; }
        }
        a = ba;
    }
    agg_out[i] = a;
}

// prolongation row i: (1-w) e_agg(i) + sum over strong j of (-w/df_i) a_ij e_agg(j), merged, sorted
template <class V>
__global__ void k_prolong_count(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                const unsigned char* __restrict__ strong, const int* __restrict__ agg,
                                int* __restrict__ cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = 0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        const int j = col[k];
        if (j != i && !strong[k]) continue;
        const int g = agg[j];
        if (g < 0) continue;
        bool seen = false;
        for (int t = ptr[i]; t < k; ++t) {
            const int jt = col[t];
            if (jt != i && !strong[t]) continue;
            if (agg[jt] == g) { seen = true; break; }
        }
        if (!seen) ++c;
    }
    cnt[i] = c;
}
template <class V>
__global__ void k_prolong_fill(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                               const V* __restrict__ val, const unsigned char* __restrict__ strong,
                               const int* __restrict__ agg, double omega, const int* __restrict__ pptr,
                               int* __restrict__ pcol, V* __restrict__ pval) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double df = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
        if (col[k] == i || !strong[k]) df += (double)val[k];
    df = -omega * (1.0 / df);
    const int rb = pptr[i];
    int m = rb;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        const int j = col[k];
        if (j != i && !strong[k]) continue;
        const int g = agg[j];
        if (g < 0) continue;
        const double v = (j == i) ? (1.0 - omega) : df * (double)val[k];
        int t = rb;
        while (t < m && pcol[t] != g) ++t;
        if (t < m) pval[t] = (V)((double)pval[t] + v);
        else { pcol[m] = g; pval[m] = (V)v; ++m; }
    }
    for (int s = rb + 1; s < m; ++s) {   // insertion sort by column
        const int cv = pcol[s];
        const V vv = pval[s];
        int t = s - 1;
        while (t >= rb && pcol[t] > cv) { pcol[t + 1] = pcol[t]; pval[t + 1] = pval[t]; --t; }
        pcol[t + 1] = cv;
        pval[t + 1] = vv;
    }
}

// transpose: count per column, then place, then sort each row by column
__global__ void k_col_count(int64_t nnz, const int* __restrict__ col, int* __restrict__ cnt) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) atomicAdd(cnt + col[k], 1);
}
template <class V>
__global__ void k_transpose_fill(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                 const V* __restrict__ val, int* __restrict__ fill, int* __restrict__ tcol,
                                 V* __restrict__ tval) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        const int d = atomicAdd(fill + col[k], 1);
        tcol[d] = i;
        tval[d] = val[k];
    }
}
// Sort each row by column into a second buffer, one warp per row: an entry's
// place is the number of smaller columns in its row (columns are unique).
template <class V>
__global__ void k_sort_rows(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                            const V* __restrict__ val, int* __restrict__ ocol, V* __restrict__ oval) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int rb = ptr[warp], re = ptr[warp + 1];
    for (int e = rb + lane; e < re; e += 32) {
        const int ce = col[e];
        int rank = 0;
        for (int u = rb; u < re; ++u) rank += (__ldg(col + u) < ce);
        ocol[rb + rank] = ce;
        oval[rb + rank] = val[e];
    }
}

__global__ void k_max_int(int n, const int* __restrict__ a, int* __restrict__ out) {
    __shared__ int sh[32];
    int m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = max(m, a[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int r = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = max(r, sh[w]);
        atomicMax(out, r);
    }
}

// Row-wise SpGEMM C = A * B, one warp per row, open-addressing hash table in
// shared memory.  Pass 0 counts distinct columns (flagging rows that fill
// more than 3/4 of the table); pass 1 fills.  Products are consumed in a fixed
// order (A entries in row order, B entries in chunks of 32); lanes that hit
// the same column are combined in lane order by the lowest lane, so every sum
// has a fixed association.  Occupied slots are compacted and ranked by
// column, so output rows are sorted.
constexpr int kGemmWarps = 4;
template <class V, int HT>
__global__ void __launch_bounds__(32 * kGemmWarps) k_spgemm(int n, const int* __restrict__ aptr,
                                                            const int* __restrict__ acol, const V* __restrict__ aval,
                                                            const int* __restrict__ bptr, const int* __restrict__ bcol,
                                                            const V* __restrict__ bval, int pass,
                                                            int* __restrict__ cnt, const int* __restrict__ cptr,
                                                            int* __restrict__ ccol, V* __restrict__ cval,
                                                            int* __restrict__ overflow) {
    extern __shared__ unsigned char smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // per warp: keys[HT] int, ckeys[HT] int, vals[HT] double, cvals[HT] double
    int* keys = reinterpret_cast<int*>(smem) + wid * 2 * HT;
    int* ckeys = keys + HT;
    double* vals = reinterpret_cast<double*>(smem + sizeof(int) * 2 * HT * kGemmWarps) + wid * 2 * HT;
    double* cvals = vals + HT;
    for (int row = blockIdx.x * kGemmWarps + wid; row < n; row += gridDim.x * kGemmWarps) {
        for (int t = lane; t < HT; t += 32) { keys[t] = -1; vals[t] = 0.0; }
        __syncwarp();
        int distinct = 0;
        bool full = false;
        for (int ka = aptr[row]; ka < aptr[row + 1] && !full; ++ka) {
            const int a = acol[ka];
            const double av = (double)aval[ka];
            const int bb = bptr[a], be = bptr[a + 1];
            for (int q0 = bb; q0 < be; q0 += 32) {
                const int q = q0 + lane;
                const bool act = q < be;
                const int c = act ? bcol[q] : -1;
                int slot = -1;
                bool fresh = false;
                if (act) {
                    uint32_t h = hash_u32((uint32_t)c) & (HT - 1);
                    for (int probe = 0; probe < HT; ++probe) {
                        const int prev = atomicCAS(keys + h, -1, c);
                        if (prev == -1) { slot = (int)h; fresh = true; break; }
                        if (prev == c) { slot = (int)h; break; }
                        h = (h + 1) & (HT - 1);
                    }
                }
                distinct += __popc(__ballot_sync(0xffffffffu, fresh));
                const bool lost = __any_sync(0xffffffffu, act && slot < 0);
                // the lanes of one chunk hold distinct columns of one B row, so
                // no two lanes share a slot; chunks are applied in order
                if (pass == 1 && !lost && act) vals[slot] += av * (double)bval[q];
                __syncwarp();
                if (lost || distinct > (HT * 3) / 4) { full = true; break; }
            }
        }
        if (full) {
            if (lane == 0) atomicExch(overflow, 1);
            if (pass == 0 && lane == 0) cnt[row] = 0;
            __syncwarp();
            continue;
        }
        if (pass == 0) {
            if (lane == 0) cnt[row] = distinct;
        } else {
            // compact occupied slots (slot order), then rank by column
            int base_c = 0;
            for (int t0 = 0; t0 < HT; t0 += 32) {
                const int t = t0 + lane;
                const bool occ = keys[t] >= 0;
                const unsigned bal = __ballot_sync(0xffffffffu, occ);
                if (occ) {
                    const int pos = base_c + __popc(bal & ((1u << lane) - 1u));
                    ckeys[pos] = keys[t];
                    cvals[pos] = vals[t];
                }
                base_c += __popc(bal);
            }
            __syncwarp();
            const int out = cptr[row];
            for (int e = lane; e < base_c; e += 32) {
                const int ce = ckeys[e];
                int rank = 0;
                for (int u = 0; u < base_c; ++u) rank += (ckeys[u] < ce);
                ccol[out + rank] = ce;
                cval[out + rank] = (V)cvals[e];
            }
        }
        __syncwarp();
    }
}

// dense copy and Gauss-Jordan inverse (partial pivoting) of the coarsest matrix, one block
template <class V>
__global__ void k_dense(int n, const int* __restrict__ ptr, const int* __restrict__ col, const V* __restrict__ val,
                        double* __restrict__ a) {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) a[t] = 0.0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) a[(size_t)i * n + col[k]] = (double)val[k];
}
__global__ void k_gauss_jordan(int n, double* __restrict__ a, double* __restrict__ inv, int* __restrict__ flag) {
    __shared__ int piv;
    __shared__ double pval;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) inv[t] = ((t / n) == (t % n)) ? 1.0 : 0.0;
    __syncthreads();
    for (int c = 0; c < n; ++c) {
        if (threadIdx.x == 0) {
            int p = c;
            double best = fabs(a[(size_t)c * n + c]);
            for (int r = c + 1; r < n; ++r) {
                const double v = fabs(a[(size_t)r * n + c]);
                if (v > best) { best = v; p = r; }
            }
            piv = p;
            pval = a[(size_t)p * n + c];
            if (!(best > 0.0)) flag[4] = 1;
        }
        __syncthreads();
        if (pval == 0.0) return;
        if (piv != c)
            for (int t = threadIdx.x; t < n; t += blockDim.x) {
                double x = a[(size_t)c * n + t]; a[(size_t)c * n + t] = a[(size_t)piv * n + t]; a[(size_t)piv * n + t] = x;
                x = inv[(size_t)c * n + t]; inv[(size_t)c * n + t] = inv[(size_t)piv * n + t]; inv[(size_t)piv * n + t] = x;
            }
        __syncthreads();
        const double ip = 1.0 / pval;
        for (int t = threadIdx.x; t < n; t += blockDim.x) { a[(size_t)c * n + t] *= ip; inv[(size_t)c * n + t] *= ip; }
        __syncthreads();
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
            const int r = t / n, k = t % n;
            if (r == c) continue;
            const double f = a[(size_t)r * n + c];
            if (k != c) a[(size_t)r * n + k] -= f * a[(size_t)c * n + k];
            inv[(size_t)r * n + k] -= f * inv[(size_t)c * n + k];
        }
        __syncthreads();
        for (int r = threadIdx.x; r < n; r += blockDim.x)
            if (r != c) a[(size_t)r * n + c] = 0.0;
        __syncthreads();
    }
}

// ------------------------------------------------------------- host helpers
double finish_dot(semo_ctx* c, double* part, int count, double* out_host) {
    cudaStream_t s = c->stream;
    k_finish<<<1, 256, 0, s>>>(part, count, part + 4 * kRedBlocks);
    SEMO_CHECK_LAUNCH();
    SEMO_CUDA(cudaMemcpyAsync(out_host, part + 4 * kRedBlocks, sizeof(double) * count, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    return out_host[0];
}

template <class V>
int pick_vs(const DCsr<V>& A) {
    const double avg = A.n ? (double)A.nnz / A.n : 1.0;
    return avg <= 6 ? 4 : (avg <= 12 ? 8 : (avg <= 24 ? 16 : 32));
}

template <class V>
void spmv(cudaStream_t s, const DCsr<V>& A, const V* x, V* y) {
    switch (pick_vs(A)) {
        case 4: k_spmv<V, V, 4><<<blocks((int64_t)A.n * 4, 256), 256, 0, s>>>(A.n, A.ptr, A.col, A.val, x, y); break;
        case 8: k_spmv<V, V, 8><<<blocks((int64_t)A.n * 8, 256), 256, 0, s>>>(A.n, A.ptr, A.col, A.val, x, y); break;
        case 16: k_spmv<V, V, 16><<<blocks((int64_t)A.n * 16, 256), 256, 0, s>>>(A.n, A.ptr, A.col, A.val, x, y); break;
        default: k_spmv<V, V, 32><<<blocks((int64_t)A.n * 32, 256), 256, 0, s>>>(A.n, A.ptr, A.col, A.val, x, y); break;
    }
    SEMO_CHECK_LAUNCH();
}

// C = A * B (rows of A, cols of B = m)
template <class V>
void spgemm_pass(cudaStream_t s, int ht, int pass, const DCsr<V>& A, const DCsr<V>& B, DCsr<V>& C, int* cnt,
                 int* overflow) {
    const int n = A.n;
    const size_t shm = (size_t)kGemmWarps * ht * 2 * (sizeof(int) + sizeof(double));
    const int grid = std::max(1, std::min(blocks(n, kGemmWarps), 152 * 32));
#define SEMO_GEMM_CASE(H)                                                                                        \
    case H:                                                                                                      \
        if (shm > 48 * 1024)                                                                                     \
            SEMO_CUDA(cudaFuncSetAttribute(k_spgemm<V, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm)); \
        k_spgemm<V, H><<<grid, 32 * kGemmWarps, shm, s>>>(n, A.ptr, A.col, A.val, B.ptr, B.col, B.val, pass, cnt,  \
                                                           C.ptr, C.col.p, C.val.p, overflow);                   \
        break;
    switch (ht) {
        SEMO_GEMM_CASE(64)
        SEMO_GEMM_CASE(128)
        SEMO_GEMM_CASE(256)
        SEMO_GEMM_CASE(512)
        SEMO_GEMM_CASE(1024)
        default:
        SEMO_GEMM_CASE(2048)
    }
#undef SEMO_GEMM_CASE
    SEMO_CHECK_LAUNCH();
}

template <class V>
void spgemm(cudaStream_t s, semo_ctx* c, const DCsr<V>& A, const DCsr<V>& B, DCsr<V>& C) {
    const int n = A.n;
    C.n = n;
    C.m = B.m;
    C.ptr.alloc(n + 1, s);
    DBuf<int> flags;
    flags.alloc(2, s);
    // pass 0 with a growing table until no row overflows; counts land in C.ptr
    int ht = 256, of = 0;
    for (;;) {
        flags.zero();
        SEMO_CUDA(cudaMemsetAsync(C.ptr.p + n, 0, sizeof(int), s));
        spgemm_pass(s, ht, 0, A, B, C, C.ptr.p, flags.p);
        SEMO_CUDA(cudaMemcpyAsync(&of, flags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
        if (!of) break;
        if (ht >= 2048) throw Error(SEMO_ERR_CUDA, "SpGEMM row has more than 1536 distinct columns");
        ht <<= 1;
    }
    // pass 1 with the smallest table that holds the densest row at <= 3/4 load
    DBuf<int> mx;
    mx.alloc(1, s);
    mx.zero();
    k_max_int<<<std::min(blocks(n, 256), 1024), 256, 0, s>>>(n, C.ptr, mx);
    SEMO_CHECK_LAUNCH();
    int maxd = 0;
    SEMO_CUDA(cudaMemcpyAsync(&maxd, mx.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    const int nnz = scan_exclusive(s, C.ptr.p, n + 1);   // syncs
    int ht1 = 64;
    while (ht1 * 3 / 4 < maxd + 32 && ht1 < ht) ht1 <<= 1;
    C.nnz = nnz;
    C.col.alloc(std::max(nnz, 1), s);
    C.val.alloc(std::max(nnz, 1), s);
    flags.zero();
    spgemm_pass(s, ht1, 1, A, B, C, nullptr, flags.p);
    SEMO_CUDA(cudaMemcpyAsync(&of, flags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    if (of) throw Error(SEMO_ERR_CUDA, "SpGEMM numeric pass overflowed its table");
    (void)c;
}

template <class V>
void transpose(cudaStream_t s, const DCsr<V>& A, DCsr<V>& T) {
    T.n = A.m;
    T.m = A.n;
    T.nnz = A.nnz;
    T.ptr.alloc(T.n + 1, s);
    T.ptr.zero();
    DBuf<int> tcol;
    DBuf<V> tval;
    tcol.alloc(std::max<int64_t>(A.nnz, 1), s);
    tval.alloc(std::max<int64_t>(A.nnz, 1), s);
    T.col.alloc(std::max<int64_t>(A.nnz, 1), s);
    T.val.alloc(std::max<int64_t>(A.nnz, 1), s);
    if (A.nnz) {
        k_col_count<<<blocks(A.nnz, 256), 256, 0, s>>>(A.nnz, A.col, T.ptr);
        SEMO_CHECK_LAUNCH();
    }
    scan_exclusive(s, T.ptr.p, T.n + 1);
    DBuf<int> fill;
    fill.alloc(T.n + 1, s);
    SEMO_CUDA(cudaMemcpyAsync(fill.p, T.ptr.p, sizeof(int) * (T.n + 1), cudaMemcpyDeviceToDevice, s));
    k_transpose_fill<V><<<blocks(A.n, 256), 256, 0, s>>>(A.n, A.ptr, A.col, A.val, fill, tcol, tval);
    SEMO_CHECK_LAUNCH();
    k_sort_rows<V><<<blocks((int64_t)T.n * 32, 256), 256, 0, s>>>(T.n, T.ptr, tcol, tval, T.col, T.val);
    SEMO_CHECK_LAUNCH();
}

template <class V>
void level_prepare(semo_ctx* c, AmgLevel<V>& L, DBuf<V>& dia) {
    cudaStream_t s = c->stream;
    const int n = L.A.n;
    L.dinv.alloc(n, s);
    dia.alloc(n, s);
    DBuf<double> ratio, part;
    ratio.alloc(n, s);
    part.alloc(kRedBlocks, s);
    k_diag<V><<<blocks(n, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, dia, L.dinv, ratio, c->flag);
    SEMO_CHECK_LAUNCH();
    k_max<<<kRedBlocks, kRedThreads, 0, s>>>(n, ratio, part);
    SEMO_CHECK_LAUNCH();
    std::vector<double> h(kRedBlocks);
    SEMO_CUDA(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * kRedBlocks, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    double lam = 0.0;
    for (double v : h) lam = std::max(lam, v);
    L.lam_max = lam;
    L.x.alloc(n, s); L.b.alloc(n, s); L.r.alloc(n, s); L.t.alloc(n, s);
}

template <class V>
void amg_setup(semo_ctx* c, Amg<V>& h, const int* ptr, const int* col, const double* val64, int n, int64_t nnz) {
    cudaStream_t s = c->stream;
    h.clear();
    h.lev.reserve(c->prm.max_levels + 1);
    h.lev.emplace_back();
    {
        AmgLevel<V>& L0 = h.lev[0];
        L0.A.n = n; L0.A.m = n; L0.A.nnz = nnz;
        L0.A.ptr.alloc(n + 1, s);
        L0.A.col.alloc(nnz, s);
        L0.A.val.alloc(nnz, s);
        SEMO_CUDA(cudaMemcpyAsync(L0.A.ptr.p, ptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToDevice, s));
        SEMO_CUDA(cudaMemcpyAsync(L0.A.col.p, col, sizeof(int) * nnz, cudaMemcpyDeviceToDevice, s));
        k_convert<double, V><<<blocks(nnz, 256), 256, 0, s>>>((int)nnz, val64, L0.A.val.p);
        SEMO_CHECK_LAUNCH();
    }
    float eps = (float)c->prm.eps_strong;
    const double omega = 2.0 / 3.0;
    for (int l = 0;; ++l) {
        AmgLevel<V>& L = h.lev[l];
        DBuf<V> dia;
        level_prepare(c, L, dia);
        h.total_nnz += L.A.nnz;
        const int nl = L.A.n;
        if (nl <= c->prm.coarse_enough || l == c->prm.max_levels - 1) break;
        // strength + MIS(2) aggregation
        DBuf<unsigned char> strong;
        DBuf<int> state, agg, agg2, undec;
        DBuf<unsigned long long> m1;
        strong.alloc(std::max<int64_t>(L.A.nnz, 1), s);
        state.alloc(nl, s); agg.alloc(nl + 1, s); agg2.alloc(nl, s); undec.alloc(1, s);
        m1.alloc(nl, s);
        const double eps2 = (double)(eps * eps);
        eps *= 0.5f;
        k_strength<V><<<blocks(nl, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, L.A.val, dia, eps2, strong, state);
        SEMO_CHECK_LAUNCH();
        for (int round = 0; round < 200; ++round) {
            undec.zero();
            k_mis_max1<<<blocks(nl, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, strong, state, m1);
            SEMO_CHECK_LAUNCH();
            k_mis_max2<<<blocks(nl, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, strong, m1, state, undec);
            SEMO_CHECK_LAUNCH();
            int u = 0;
            SEMO_CUDA(cudaMemcpyAsync(&u, undec.p, sizeof(int), cudaMemcpyDeviceToHost, s));
            SEMO_CUDA(cudaStreamSynchronize(s));
            if (u == 0) break;
            if (round == 199) throw Error(SEMO_ERR_CUDA, "MIS(2) aggregation did not terminate");
        }
        k_root_flags<<<blocks(nl, 256), 256, 0, s>>>(nl, state, agg2);
        SEMO_CHECK_LAUNCH();
        const int nagg = scan_exclusive(s, agg2.p, nl);
        if (nagg == 0 || nagg >= nl) break;
        k_root_ids<<<blocks(nl, 256), 256, 0, s>>>(nl, state, agg2, agg);
        SEMO_CHECK_LAUNCH();
        for (int pass = 0; pass < 2; ++pass) {
            k_agg_join<<<blocks(nl, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, strong, state, agg, agg2);
            SEMO_CHECK_LAUNCH();
            std::swap(agg.p, agg2.p);
        }
        L.nagg = nagg;
        // smoothed prolongation
        L.P.n = nl; L.P.m = nagg;
        L.P.ptr.alloc(nl + 1, s);
        SEMO_CUDA(cudaMemsetAsync(L.P.ptr.p + nl, 0, sizeof(int), s));
        k_prolong_count<V><<<blocks(nl, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, strong, agg, L.P.ptr);
        SEMO_CHECK_LAUNCH();
        L.P.nnz = scan_exclusive(s, L.P.ptr.p, nl + 1);
        L.P.col.alloc(std::max<int64_t>(L.P.nnz, 1), s);
        L.P.val.alloc(std::max<int64_t>(L.P.nnz, 1), s);
        k_prolong_fill<V><<<blocks(nl, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, L.A.val, strong, agg, omega, L.P.ptr,
                                                          L.P.col, L.P.val);
        SEMO_CHECK_LAUNCH();
        transpose(s, L.P, L.R);
        DCsr<V> AP;
        spgemm(s, c, L.A, L.P, AP);
        h.lev.emplace_back();
        AmgLevel<V>& Lc = h.lev.back();
        AmgLevel<V>& Lf = h.lev[h.lev.size() - 2];
        spgemm(s, c, Lf.R, AP, Lc.A);
        Lc.A.m = Lc.A.n;
    }
    // coarsest level: explicit FP64 inverse (Gauss-Jordan, partial pivoting)
    AmgLevel<V>& Lc = h.lev.back();
    const int m = Lc.A.n;
    if (m > 4096) throw Error(SEMO_ERR_CUDA, "AMG coarsening stalled above 4096 rows");
    h.coarse_n = m;
    DBuf<double> dense;
    dense.alloc((size_t)m * m, s);
    h.cinv.alloc((size_t)m * m, s);
    k_dense<V><<<1, 1024, 0, s>>>(m, Lc.A.ptr, Lc.A.col, Lc.A.val, dense);
    SEMO_CHECK_LAUNCH();
    k_gauss_jordan<<<1, 1024, 0, s>>>(m, dense, h.cinv, c->flag);
    SEMO_CHECK_LAUNCH();
    int hf[5] = {0, 0, 0, 0, 0};
    SEMO_CUDA(cudaMemcpyAsync(hf, c->flag.p, sizeof(hf), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    if (hf[2]) throw Error(SEMO_ERR_ARGUMENT, "matrix has a zero diagonal entry");
    if (hf[3]) throw Error(SEMO_ERR_NAN, "non-finite matrix entry");
    if (hf[4]) throw Error(SEMO_ERR_BREAKDOWN, "coarsest AMG matrix is singular");
    h.ready = true;
}

// ------------------------------------------------------------------ V-cycle
template <class V>
void chebyshev(cudaStream_t s, AmgLevel<V>& L, int degree, bool zero_start) {
    const int n = L.A.n;
    const double hi = L.lam_max, lo = hi / 30.0;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
    const double sigma = theta / delta;
    double rho = 1.0 / sigma;
    const int vs = pick_vs(L.A);
    V* x = L.x.p;
    V* d = L.t.p;
    if (zero_start) {
        k_cheb_first<V><<<blocks(n, 256), 256, 0, s>>>(n, L.dinv, L.b, (V)(1.0 / theta), x, d);
        SEMO_CHECK_LAUNCH();
    } else {
        switch (vs) {
            case 4: k_cheb_start<V, 4><<<blocks((int64_t)n * 4, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.dinv, L.b, (V)(1.0 / theta), x, d); break;
            case 8: k_cheb_start<V, 8><<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.dinv, L.b, (V)(1.0 / theta), x, d); break;
            case 16: k_cheb_start<V, 16><<<blocks((int64_t)n * 16, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.dinv, L.b, (V)(1.0 / theta), x, d); break;
            default: k_cheb_start<V, 32><<<blocks((int64_t)n * 32, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.dinv, L.b, (V)(1.0 / theta), x, d); break;
        }
        SEMO_CHECK_LAUNCH();
        k_add<V><<<blocks(n, 256), 256, 0, s>>>(n, d, x);
        SEMO_CHECK_LAUNCH();
    }
    for (int k = 1; k < degree; ++k) {
        const double rho_new = 1.0 / (2.0 * sigma - rho);
        const double c1 = rho_new * rho, c2 = 2.0 * rho_new / delta;
        switch (vs) {
            case 4: k_cheb_step<V, 4><<<blocks((int64_t)n * 4, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.dinv, L.b, x, (V)c1, (V)c2, d); break;
            case 8: k_cheb_step<V, 8><<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.dinv, L.b, x, (V)c1, (V)c2, d); break;
            case 16: k_cheb_step<V, 16><<<blocks((int64_t)n * 16, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.dinv, L.b, x, (V)c1, (V)c2, d); break;
            default: k_cheb_step<V, 32><<<blocks((int64_t)n * 32, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.dinv, L.b, x, (V)c1, (V)c2, d); break;
        }
        SEMO_CHECK_LAUNCH();
        k_add<V><<<blocks(n, 256), 256, 0, s>>>(n, d, x);
        SEMO_CHECK_LAUNCH();
        rho = rho_new;
    }
}

template <class V>
void vcycle(cudaStream_t s, Amg<V>& h, int l, int degree) {
    AmgLevel<V>& L = h.lev[l];
    const int n = L.A.n;
    if (l == (int)h.lev.size() - 1) {
        k_coarse_solve<V><<<1, 256, 0, s>>>(h.coarse_n, h.cinv, L.b, L.x);
        SEMO_CHECK_LAUNCH();
        return;
    }
    chebyshev(s, L, degree, true);
    const int vs = pick_vs(L.A);
    switch (vs) {
        case 4: k_residual<V, 4><<<blocks((int64_t)n * 4, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.x, L.b, L.r); break;
        case 8: k_residual<V, 8><<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.x, L.b, L.r); break;
        case 16: k_residual<V, 16><<<blocks((int64_t)n * 16, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.x, L.b, L.r); break;
        default: k_residual<V, 32><<<blocks((int64_t)n * 32, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, L.x, L.b, L.r); break;
    }
    SEMO_CHECK_LAUNCH();
    AmgLevel<V>& C = h.lev[l + 1];
    spmv(s, L.R, L.r.p, C.b.p);
    vcycle(s, h, l + 1, degree);
    const int pvs = pick_vs(L.P);
    switch (pvs) {
        case 4: k_prolong<V, 4><<<blocks((int64_t)n * 4, 256), 256, 0, s>>>(n, L.P.ptr, L.P.col, L.P.val, C.x, L.x); break;
        case 8: k_prolong<V, 8><<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(n, L.P.ptr, L.P.col, L.P.val, C.x, L.x); break;
        case 16: k_prolong<V, 16><<<blocks((int64_t)n * 16, 256), 256, 0, s>>>(n, L.P.ptr, L.P.col, L.P.val, C.x, L.x); break;
        default: k_prolong<V, 32><<<blocks((int64_t)n * 32, 256), 256, 0, s>>>(n, L.P.ptr, L.P.col, L.P.val, C.x, L.x); break;
    }
    SEMO_CHECK_LAUNCH();
    chebyshev(s, L, degree, false);
}

// scalars on the device, inside c->red: [0,4R) partials, [4R, 4R+16) scalars
struct Red {
    double* part;
    double* scal;
};
Red red_area(semo_ctx* c) {
    c->red.alloc(4 * kRedBlocks + 32, c->stream);
    return Red{c->red.p, c->red.p + 4 * kRedBlocks + 8};
}

template <class V>
void precondition(semo_ctx* c, Amg<V>& h, const double* r) {
    cudaStream_t s = c->stream;
    AmgLevel<V>& L0 = h.lev[0];
    const int n = L0.A.n;
    k_convert<double, V><<<blocks(n, 256), 256, 0, s>>>(n, r, L0.b.p);
    SEMO_CHECK_LAUNCH();
    vcycle(s, h, 0, c->prm.cheb_degree);
}

// One flexible-CG iteration, every scalar kept on the device.
template <class V>
void cg_iteration(semo_ctx* c, Amg<V>& h, const int* ptr, const int* col, const double* val, int n, double* x,
                  const Red& R) {
    cudaStream_t s = c->stream;
    double* r = c->kr.p;
    double* p = c->kp.p;
    double* q = c->kq.p;
    AmgLevel<V>& L0 = h.lev[0];
    precondition(c, h, r);
    k_dot2<V><<<kRedBlocks, kRedThreads, 0, s>>>(n, L0.x.p, r, q, R.part);
    SEMO_CHECK_LAUNCH();
    k_finish<<<1, 256, 0, s>>>(R.part, 2, R.scal + 0);
    SEMO_CHECK_LAUNCH();
    k_cg_beta<<<1, 32, 0, s>>>(R.scal);
    SEMO_CHECK_LAUNCH();
    k_p_update_t<V><<<blocks(n, 256), 256, 0, s>>>(n, L0.x.p, p, R.scal);
    SEMO_CHECK_LAUNCH();
    k_spmv_dot<8><<<kRedBlocks, 256, 0, s>>>(n, ptr, col, val, p, q, R.part);
    SEMO_CHECK_LAUNCH();
    k_finish<<<1, 256, 0, s>>>(R.part, 1, R.scal + 2);
    SEMO_CHECK_LAUNCH();
    k_cg_alpha<<<1, 32, 0, s>>>(R.scal);
    SEMO_CHECK_LAUNCH();
    k_xr_update<<<kRedBlocks, kRedThreads, 0, s>>>(n, x, r, p, q, R.scal, R.part);
    SEMO_CHECK_LAUNCH();
    k_finish<<<1, 256, 0, s>>>(R.part, 1, R.scal + 3);
    SEMO_CHECK_LAUNCH();
}

struct GraphGuard {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    ~GraphGuard() {
        if (e) cudaGraphExecDestroy(e);
        if (g) cudaGraphDestroy(g);
    }
};

template <class V>
void pcg(semo_ctx* c, Amg<V>& h, const int* ptr, const int* col, const double* val, int n, const double* b,
         double* x, bool zero_guess, semo_solve_info* info) {
    cudaStream_t s = c->stream;
    Red R = red_area(c);
    c->kr.alloc(n, s); c->kp.alloc(n, s); c->kq.alloc(n, s);
    if (!c->hpin) SEMO_CUDA(cudaMallocHost((void**)&c->hpin, 16 * sizeof(double)));
    double* h2 = c->hpin;
    double* r = c->kr.p;
    // r = b - A x
    if (zero_guess) {
        SEMO_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        SEMO_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    } else {
        k_residual<double, 8><<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(n, ptr, col, val, x, b, r);
        SEMO_CHECK_LAUNCH();
    }
    SEMO_CUDA(cudaMemsetAsync(c->kq.p, 0, sizeof(double) * n, s));
    SEMO_CUDA(cudaMemsetAsync(c->kp.p, 0, sizeof(double) * n, s));
    SEMO_CUDA(cudaMemsetAsync(R.scal, 0, sizeof(double) * 16, s));
    k_dot<double, double><<<kRedBlocks, kRedThreads, 0, s>>>(n, b, b, R.part);
    SEMO_CHECK_LAUNCH();
    k_dot<double, double><<<kRedBlocks, kRedThreads, 0, s>>>(n, r, r, R.part + kRedBlocks);
    SEMO_CHECK_LAUNCH();
    k_finish<<<1, 256, 0, s>>>(R.part, 2, R.scal + 8);
    SEMO_CHECK_LAUNCH();
    SEMO_CUDA(cudaMemcpyAsync(h2, R.scal + 8, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    const double bn = std::sqrt(h2[0]);
    double rn = std::sqrt(h2[1]);
    if (!std::isfinite(bn) || !std::isfinite(rn)) throw Error(SEMO_ERR_NAN, "non-finite right-hand side");
    const double bnorm = (bn > 0.0) ? bn : 1.0;
    int it = 0;
    // The iteration body is captured once per hierarchy and replayed: the
    // coarse levels are launch-latency bound, the graph removes the per-kernel
    // host overhead.  Convergence is read back after every iteration.
    GraphGuard gg;
    size_t graph_nodes = 0;
    if (rn > c->prm.tol * bnorm && c->prm.max_iter > 0) {
        // launches recorded during capture do not run; replays are counted below
        const long long launches_before = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
        SEMO_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
            cg_iteration(c, h, ptr, col, val, n, x, R);
        } catch (...) {
            cudaGraph_t junk = nullptr;
            cudaStreamEndCapture(s, &junk);
            if (junk) cudaGraphDestroy(junk);
            throw;
        }
        SEMO_CUDA(cudaStreamEndCapture(s, &gg.g));
        SEMO_CUDA(cudaGraphInstantiate(&gg.e, gg.g, 0));
        SEMO_CUDA(cudaGraphGetNodes(gg.g, nullptr, &graph_nodes));
        __atomic_store_n(&g_kernel_launches, launches_before, __ATOMIC_RELAXED);
    }
    while (it < c->prm.max_iter && rn > c->prm.tol * bnorm) {
        SEMO_CUDA(cudaGraphLaunch(gg.e, s));
        __atomic_add_fetch(&g_kernel_launches, (long long)graph_nodes, __ATOMIC_RELAXED);
        SEMO_CUDA(cudaMemcpyAsync(h2, R.scal, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
        ++it;
        if (!std::isfinite(h2[3]) || !std::isfinite(h2[2])) throw Error(SEMO_ERR_NAN, "NaN/Inf in the Krylov residual");
        if (!(h2[2] > 0.0)) throw Error(SEMO_ERR_BREAKDOWN, "CG breakdown: p.Ap <= 0 (matrix not SPD?)");
        rn = std::sqrt(h2[3]);
    }
    // true FP64 residual of the returned solution
    k_residual<double, 8><<<blocks((int64_t)n * 8, 256), 256, 0, s>>>(n, ptr, col, val, x, b, r);
    SEMO_CHECK_LAUNCH();
    k_dot<double, double><<<kRedBlocks, kRedThreads, 0, s>>>(n, r, r, R.part);
    SEMO_CHECK_LAUNCH();
    k_finish<<<1, 256, 0, s>>>(R.part, 1, R.scal + 8);
    SEMO_CHECK_LAUNCH();
    SEMO_CUDA(cudaMemcpyAsync(h2, R.scal + 8, sizeof(double), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    info->iterations = it;
    info->rel_residual = (bn > 0.0) ? std::sqrt(h2[0]) / bn : 0.0;
}

template <class V>
void fill_info(const Amg<V>& h, int64_t nnz, semo_solve_info* info) {
    info->levels = (int)h.lev.size();
    info->coarse_size = h.coarse_n;
    info->operator_complexity = (double)h.total_nnz / (double)std::max<int64_t>(nnz, 1);
}

}  // namespace

void solve_system(semo_ctx* c, const int* ptr, const int* col, const double* val, int n, int64_t nnz,
                  const double* b, double* x, semo_solve_info* info, bool zero_guess) {
    cudaStream_t s = c->stream;
    c->flag.zero();
    SEMO_CUDA(cudaEventRecord(c->ev[0], s));
    {
        StageScope sc(c, ST_AMG_SETUP);
        if (c->prm.precision == SEMO_PREC_MIXED) {
            c->amg64.clear();
            amg_setup<float>(c, c->amg32, ptr, col, val, n, nnz);
        } else {
            c->amg32.clear();
            amg_setup<double>(c, c->amg64, ptr, col, val, n, nnz);
        }
    }
    SEMO_CUDA(cudaEventRecord(c->ev[1], s));
    {
        StageScope sc(c, ST_PCG);
        if (c->prm.precision == SEMO_PREC_MIXED) {
            pcg<float>(c, c->amg32, ptr, col, val, n, b, x, zero_guess, info);
            fill_info(c->amg32, nnz, info);
        } else {
            pcg<double>(c, c->amg64, ptr, col, val, n, b, x, zero_guess, info);
            fill_info(c->amg64, nnz, info);
        }
    }
    SEMO_CUDA(cudaEventRecord(c->ev[2], s));
    SEMO_CUDA(cudaEventSynchronize(c->ev[2]));
    float t0 = 0, t1 = 0;
    SEMO_CUDA(cudaEventElapsedTime(&t0, c->ev[0], c->ev[1]));
    SEMO_CUDA(cudaEventElapsedTime(&t1, c->ev[1], c->ev[2]));
    info->setup_ms = t0;
    info->solve_ms = t1;
}

// Adjoint solve on the hierarchy of the last forward solve (the pressure
// matrix is symmetric, so A^T = A and the same preconditioner applies).
void solve_transpose_reuse(semo_ctx* c, const double* g, double* lam, semo_solve_info* info) {
    const int n = c->nc;
    SEMO_CUDA(cudaEventRecord(c->ev[1], c->stream));
    if (c->prm.precision == SEMO_PREC_MIXED) {
        if (!c->amg32.ready) throw Error(SEMO_ERR_STATE, "no hierarchy: run a forward solve first");
        pcg<float>(c, c->amg32, c->A_ptr, c->A_col, c->A_val, n, g, lam, true, info);
        fill_info(c->amg32, c->nnz, info);
    } else {
        if (!c->amg64.ready) throw Error(SEMO_ERR_STATE, "no hierarchy: run a forward solve first");
        pcg<double>(c, c->amg64, c->A_ptr, c->A_col, c->A_val, n, g, lam, true, info);
        fill_info(c->amg64, c->nnz, info);
    }
    SEMO_CUDA(cudaEventRecord(c->ev[2], c->stream));
    SEMO_CUDA(cudaEventSynchronize(c->ev[2]));
    float t1 = 0;
    SEMO_CUDA(cudaEventElapsedTime(&t1, c->ev[1], c->ev[2]));
    info->setup_ms = 0.0;
    info->solve_ms = t1;
}

}  // namespace semo
