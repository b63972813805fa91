// Smoothed-aggregation AMG setup on the GPU (the hierarchy; cycle.cu applies it).
//
// Replaces the setup half of SEMO's solveAMGCL (src/solvers/solveAMGCL.cpp:
// 974-976), which builds AMGCL's smoothed-aggregation hierarchy on the CPU
// every call.  The coarsening keeps AMGCL's smoothed-aggregation semantics
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

#include <type_traits>

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

// exclusive scan of d[0..n) in place, all on the stream; *total_dev (if
// given) receives the total on the device
void scan_async(cudaStream_t s, int* d, int n, int* total_dev) {
    if (n <= 0) {
        if (total_dev) SEMO_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(int), s));
        return;
    }
    const int tiles = blocks(n, kScanTile);
    DBuf<int> ts;
    ts.alloc(tiles + 1, s);
    k_scan_tile<<<tiles, kScanT, 0, s>>>(n, d, d, ts.p);
    SEMO_CHECK_LAUNCH();
    if (tiles > 1) {
        // scan the tile sums (recursively) and add them back
        scan_async(s, ts.p, tiles, total_dev);
        k_scan_add<<<blocks(n, 256), 256, 0, s>>>(n, d, ts.p);
        SEMO_CHECK_LAUNCH();
    } else if (total_dev) {
        SEMO_CUDA(cudaMemcpyAsync(total_dev, ts.p, sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
}

// exclusive scan of d[0..n) in place; returns the total, read back through
// the pinned int *hpin (one host sync).  Extra D2H copies enqueued before the
// call land by the time it returns.
int scan_exclusive(cudaStream_t s, int* d, int n, int* hpin) {
    if (n <= 0) return 0;
    DBuf<int> tot;
    tot.alloc(1, s);
    scan_async(s, d, n, tot.p);
    SEMO_CUDA(cudaMemcpyAsync(hpin, tot.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    return *hpin;
}

template <class A, class B>
__global__ void k_convert(int n, const A* __restrict__ a, B* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (B)a[i];
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

// The per-row setup kernels below run VS lanes per row (VS = 1: a thread per
// row).  Fine levels have ~7 entries a row and use one thread; coarse levels
// (tens to hundreds of entries a row, few rows) use 8 or 32 lanes so that a
// row is not one thread walking hundreds of dependent loads.  Lanes of a row
// are consecutive within a warp; every lane reaches the group shuffles.
constexpr unsigned kFull = 0xffffffffu;
template <int VS>
__device__ __forceinline__ void row_lane(int& i, int& lane) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    i = g / VS;
    lane = g % VS;
}
template <int VS>
__device__ __forceinline__ unsigned long long grp_max(unsigned long long v) {
#pragma unroll
    for (int o = VS / 2; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(kFull, v, o, VS);
        v = (t > v) ? t : v;
    }
    return v;
}
template <int VS>
__device__ __forceinline__ int grp_sum(int v) {
#pragma unroll
    for (int o = VS / 2; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o, VS);
    return v;
}

template <class V, int VS>
__global__ void k_strength(int n, const int* __restrict__ ptr, const int* __restrict__ col, const V* __restrict__ val,
                           const V* __restrict__ dia, double eps2, unsigned char* __restrict__ strong,
                           int* __restrict__ state) {
    int i, lane;
    row_lane<VS>(i, lane);
    int has = 0;
    if (i < n) {
        const V ed = (V)(eps2 * (double)dia[i]);
        for (int k = ptr[i] + lane; k < ptr[i + 1]; k += VS) {
            const int j = col[k];
            const V v = val[k];
            const unsigned char s = (j != i) && (ed * dia[j] < v * v);
            strong[k] = s;
            has |= s;
        }
    }
    has = grp_sum<VS>(has);
    if (i < n && lane == 0) state[i] = has ? 1 : -1;   // -1: no strong connection, never aggregated
}

__device__ __forceinline__ unsigned long long mis_key(int st, int i) {
    const unsigned long long s = (st < 0) ? 0ull : (unsigned long long)st;
    return (s << 62) | ((unsigned long long)hash_u32((uint32_t)i) << 30) | (unsigned long long)i;
}

// need[i] marks the rows whose m1 an undecided row reads in the next round
// (the undecided rows and their strong neighbours); every other m1 is left as
// it is, so late rounds, with few undecided rows, touch little of the graph.
// The keys read are the same as with a full recomputation.
template <int VS>
__global__ void k_mis_max1(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                           const unsigned char* __restrict__ strong, const int* __restrict__ state,
                           unsigned char* __restrict__ need, unsigned long long* __restrict__ m1) {
    int i, lane;
    row_lane<VS>(i, lane);
    const bool go = i < n && need[i];
    unsigned long long m = 0;
    if (go) {
        if (lane == 0) m = mis_key(state[i], i);
        for (int k = ptr[i] + lane; k < ptr[i + 1]; k += VS)
            if (strong[k]) {
                const int j = col[k];
                const unsigned long long t = mis_key(state[j], j);
                m = (t > m) ? t : m;
            }
    }
    m = grp_max<VS>(m);
    if (go && lane == 0) { m1[i] = m; need[i] = 0; }
}
template <int VS>
__global__ void k_mis_max2(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                           const unsigned char* __restrict__ strong, const unsigned long long* __restrict__ m1,
                           int* __restrict__ state, unsigned char* __restrict__ need, int* __restrict__ undecided) {
    int i, lane;
    row_lane<VS>(i, lane);
    const bool active = i < n && state[i] == 1;
    unsigned long long m = 0;
    if (active) {
        if (lane == 0) m = m1[i];
        for (int k = ptr[i] + lane; k < ptr[i + 1]; k += VS)
            if (strong[k]) { const unsigned long long t = m1[col[k]]; m = (t > m) ? t : m; }
    }
    m = grp_max<VS>(m);
    if (!active) return;
    // decided from the round's snapshot (m1 was computed before any update)
    const bool root = m == mis_key(1, i);
    const bool covered = !root && (m >> 62) == 2ull;
    if (lane == 0) {
        if (root) state[i] = 2;
        else if (covered) state[i] = 0;
        else atomicAdd(undecided, 1);
    }
    if (root || covered) return;
    if (lane == 0) need[i] = 1;
    for (int k = ptr[i] + lane; k < ptr[i + 1]; k += VS)
        if (strong[k]) need[col[k]] = 1;
}
// state update must not be seen by other threads of the same round: k_mis_max2
// reads only m1 (fixed for the round) and writes only its own state; the need
// flags it sets are read by the next round's k_mis_max1.

__global__ void k_root_flags(int n, const int* __restrict__ state, int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = (state[i] == 2) ? 1 : 0;
}
__global__ void k_root_ids(int n, const int* __restrict__ state, const int* __restrict__ scanned, int* __restrict__ agg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) agg[i] = (state[i] == 2) ? scanned[i] : -1;
}
// an undecided node joins the aggregate of its strong neighbour with the
// largest (hash, index) key; keys are unique, so the choice is order-free
template <int VS>
__global__ void k_agg_join(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                           const unsigned char* __restrict__ strong, const int* __restrict__ state,
                           const int* __restrict__ agg_in, int* __restrict__ agg_out) {
    int i, lane;
    row_lane<VS>(i, lane);
    const bool look = i < n && agg_in[i] < 0 && state[i] >= 0;
    unsigned long long best = 0;   // key + 1; 0 = none
    if (look)
        for (int k = ptr[i] + lane; k < ptr[i + 1]; k += VS) {
            const int j = col[k];
            if (!strong[k] || agg_in[j] < 0) continue;
            const unsigned long long kj = (((unsigned long long)hash_u32((uint32_t)j) << 32) | (unsigned long long)j) + 1;
            best = (kj > best) ? kj : best;
        }
    best = grp_max<VS>(best);
    if (i >= n || lane != 0) return;
    agg_out[i] = look ? (best ? agg_in[(int)((best - 1) & 0xffffffffull)] : -1) : agg_in[i];
}

// prolongation row i: (1-w) e_agg(i) + sum over strong j of (-w/df_i) a_ij e_agg(j), merged, sorted
__device__ __forceinline__ bool p_eligible(int i, int k, const int* col, const unsigned char* strong,
                                           const int* agg) {
    const int j = col[k];
    return (j == i || strong[k]) && agg[j] >= 0;
}
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
// the same rows with VS lanes: first[k] marks an entry whose aggregate has not
// appeared earlier in its row; a row's output is its first entries ranked by
// aggregate, each summing its aggregate's contributions in entry order -- the
// same values and order as the one-thread kernels above.
template <int VS>
__global__ void k_prolong_count_vs(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                   const unsigned char* __restrict__ strong, const int* __restrict__ agg,
                                   unsigned char* __restrict__ first, int* __restrict__ cnt) {
    int i, lane;
    row_lane<VS>(i, lane);
    int c = 0;
    if (i < n)
        for (int k = ptr[i] + lane; k < ptr[i + 1]; k += VS) {
            bool f = p_eligible(i, k, col, strong, agg);
            if (f) {
                const int g = agg[col[k]];
                for (int t = ptr[i]; t < k; ++t)
                    if (p_eligible(i, t, col, strong, agg) && agg[col[t]] == g) { f = false; break; }
            }
            first[k] = f;
            c += f;
        }
    c = grp_sum<VS>(c);
    if (i < n && lane == 0) cnt[i] = c;
}
template <class V, int VS>
__global__ void k_prolong_fill_vs(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                  const V* __restrict__ val, const unsigned char* __restrict__ strong,
                                  const int* __restrict__ agg, const unsigned char* __restrict__ first, double omega,
                                  const int* __restrict__ pptr, int* __restrict__ pcol, V* __restrict__ pval) {
    int i, lane;
    row_lane<VS>(i, lane);
    if (i >= n) return;   // no group collectives below
    const int kb = ptr[i], ke = ptr[i + 1];
    double df = 0.0;
    for (int k = kb; k < ke; ++k)
        if (col[k] == i || !strong[k]) df += (double)val[k];
    df = -omega * (1.0 / df);
    for (int k = kb + lane; k < ke; k += VS) {
        if (!first[k]) continue;
        const int g = agg[col[k]];
        int rank = 0;
        double sum = 0.0;
        bool started = false;
        for (int t = kb; t < ke; ++t) {
            if (first[t] && agg[col[t]] < g) ++rank;
            if (t >= k && p_eligible(i, t, col, strong, agg) && agg[col[t]] == g) {
                const double v = (col[t] == i) ? (1.0 - omega) : df * (double)val[t];
                sum = started ? (double)(V)(sum + v) : (double)(V)v;
                started = true;
            }
        }
        pcol[pptr[i] + rank] = g;
        pval[pptr[i] + rank] = (V)sum;
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


// products of row i of A*B (sum of the B-row lengths it touches); out[n] stays 0
__global__ void k_row_products(int n, const int* __restrict__ aptr, const int* __restrict__ acol,
                               const int* __restrict__ bptr, int* __restrict__ prod, int* __restrict__ maxprod) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int p = 0;
    if (i < n)
        for (int k = aptr[i]; k < aptr[i + 1]; ++k) p += bptr[acol[k] + 1] - bptr[acol[k]];
    if (i < n) prod[i] = p;
    int m = p;
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxprod, m);
}
// copy rows from their upper-bound slots (uptr) to their exact places (cptr).
// A warp takes 32 consecutive rows; their outputs are contiguous, so the
// lanes stride over the concatenated output entries (coalesced stores) and
// find each entry's row by a search over the 32 row starts.
template <class V>
__global__ void k_compact_rows(int n, const int* __restrict__ uptr, const int* __restrict__ cptr,
                               const int* __restrict__ tcol, const V* __restrict__ tval, int* __restrict__ ccol,
                               V* __restrict__ cval) {
    const int warp = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    const int r0 = warp * 32;
    if (r0 >= n) return;
    const int row = min(r0 + lane, n);
    const int start = cptr[row];                      // lane's row start (n: the end)
    const int src = (r0 + lane < n) ? uptr[r0 + lane] : 0;
    const int base = __shfl_sync(0xffffffffu, start, 0);
    const int end = cptr[min(r0 + 32, n)];
    for (int e0 = base; e0 < end; e0 += 32) {        // uniform trip count: shuffles below are warp-wide
        const int e = e0 + lane;
        int j = 0;                                    // last lane whose row starts at or before e
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int sj = __shfl_sync(0xffffffffu, start, j + step);
            if (sj <= e) j += step;
        }
        const int sr = __shfl_sync(0xffffffffu, src, j) + (e - __shfl_sync(0xffffffffu, start, j));
        if (e < end) {
            ccol[e] = tcol[sr];
            cval[e] = tval[sr];
        }
    }
}

// Thread-per-row SpGEMM for rows with few distinct columns (the finest
// level's A*P: 7-entry rows times 2-7-entry rows).  The row's columns are
// kept sorted in a small local array and products are consumed in row order,
// so every sum has a fixed order.  Rows with more than kSmallCap distinct
// columns are marked -1 and left to the warp kernel.
// The row is held in registers (every index below is a compile-time constant
// after unrolling): columns sorted ascending with INT_MAX padding, a new
// column is bubbled into place by compare-and-swap.
constexpr int kSmallCap = 16;
constexpr int kSmallMaxProducts = 64;
template <class V>
__global__ void __launch_bounds__(128) k_spgemm_small(int n, const int* __restrict__ aptr,
                                                      const int* __restrict__ acol, const V* __restrict__ aval,
                                                      const int* __restrict__ bptr, const int* __restrict__ bcol,
                                                      const V* __restrict__ bval, int pass, int* __restrict__ small,
                                                      const int* __restrict__ cptr, int* __restrict__ ccol,
                                                      V* __restrict__ cval) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    if (pass == 1 && small[row] < 0) return;
    const int ab = aptr[row], ae = aptr[row + 1];
    if (pass != 1) {
        int prod = 0;
        for (int ka = ab; ka < ae; ++ka) prod += bptr[acol[ka] + 1] - bptr[acol[ka]];
        if (prod > kSmallMaxProducts) { small[row] = -1; return; }
    }
    int cols[kSmallCap];
    V vals[kSmallCap];
#pragma unroll
    for (int t = 0; t < kSmallCap; ++t) { cols[t] = 0x7FFFFFFF; vals[t] = V(0); }
    int d = 0;
    bool over = false;
    for (int ka = ab; ka < ae && !over; ++ka) {
        const int a = acol[ka];
        const V av = aval[ka];
        for (int q = bptr[a]; q < bptr[a + 1]; ++q) {
            const int cq = bcol[q];
            const V pv = (pass != 0) ? av * bval[q] : V(0);
            bool found = false;
#pragma unroll
            for (int t = 0; t < kSmallCap; ++t)
                if (cols[t] == cq) { vals[t] += pv; found = true; }
            if (found) continue;
            if (d == kSmallCap) { over = true; break; }
            int cn = cq;
            V vn = pv;
#pragma unroll
            for (int t = 0; t < kSmallCap; ++t) {
                if (cn < cols[t]) {
                    const int tc = cols[t]; cols[t] = cn; cn = tc;
                    const V tv = vals[t]; vals[t] = vn; vn = tv;
                }
            }
            ++d;
        }
    }
    if (pass == 0) {
        small[row] = over ? -1 : d;
    } else {
        if (pass == 2) {
            small[row] = over ? -1 : d;
            if (over) return;
        }
        const int base = cptr[row];
#pragma unroll
        for (int t = 0; t < kSmallCap; ++t)
            if (t < d) { ccol[base + t] = cols[t]; cval[base + t] = vals[t]; }
    }
}

// Row-wise SpGEMM C = A * B, one warp per row, open-addressing hash table in
// shared memory.  Pass 0 counts distinct columns (flagging rows that fill
// more than 3/4 of the table); pass 1 fills.  Products are consumed in a fixed
// order (A entries in row order, B entries in chunks of 32) and summed as
// 64-bit fixed-point integers (integer addition is associative, so the sums
// do not depend on the order the shared-memory atomics land in): with
// S = sum_k |a_ik| sum_j |b_kj| >= the row's sum of |products|, each product
// is scaled by 2^s, S 2^s < 2^62, and rounded to an integer -- an error of at
// most 2^-63 S per product, below what FP64 accumulation of the same
// products incurs (2^-53 S per addition).  Occupied slots are compacted and
// ranked by column, so output rows are sorted.
constexpr int kGemmWarps = 4;

// babs[k] = sum_j |b_kj| (FP64)
template <class V>
__global__ void k_row_abs(int n, const int* __restrict__ ptr, const V* __restrict__ val, double* __restrict__ babs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += fabs((double)val[k]);
    babs[i] = s;
}

// round(a b 2^sc) to the nearest integer (ties to even) for finite floats,
// on the integer pipes: the 24-bit significands multiply exactly into 48
// bits, so this equals __double2ll_rn(((double)a * b) * 2^sc) (the FP64
// product of two floats is exact too) without touching the FP64 unit.
// Requires |a b| 2^sc < 2^62.
__device__ __forceinline__ long long fixed_product(float a, float b, int sc) {
    const uint32_t ua = __float_as_uint(a), ub = __float_as_uint(b);
    int ea = (int)((ua >> 23) & 0xff), eb = (int)((ub >> 23) & 0xff);
    const uint32_t ma = (ua & 0x7fffffu) | (ea ? 0x800000u : 0u);
    const uint32_t mb = (ub & 0x7fffffu) | (eb ? 0x800000u : 0u);
    ea = ea ? ea : 1;
    eb = eb ? eb : 1;
    const unsigned long long m = (unsigned long long)ma * (unsigned long long)mb;   // exact
    const int e = (ea - 150) + (eb - 150) + sc;                                     // |a b| 2^sc = m 2^e
    unsigned long long q;
    if (m == 0ull) {
        q = 0ull;
    } else if (e >= 0) {
        q = (e < 64) ? (m << e) : 0ull;   // e <= 61 whenever the scale bound holds
    } else if (e <= -64) {
        q = 0ull;   // below half a unit (m < 2^48)
    } else {
        const int sh = -e;
        q = m >> sh;
        const unsigned long long rem = m & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (q & 1ull))) ++q;
    }
    return ((ua ^ ub) >> 31) ? -(long long)q : (long long)q;
}

template <class V, int HT>
__global__ void __launch_bounds__(32 * kGemmWarps) k_spgemm(int n, const int* __restrict__ aptr,
                                                            const int* __restrict__ acol, const V* __restrict__ aval,
                                                            const int* __restrict__ bptr, const int* __restrict__ bcol,
                                                            const V* __restrict__ bval,
                                                            const double* __restrict__ babs, int pass,
                                                            int* __restrict__ cnt, const int* __restrict__ cptr,
                                                            int* __restrict__ ccol, V* __restrict__ cval,
                                                            int* __restrict__ overflow,
                                                            const int* __restrict__ small, int defer,
                                                            int* __restrict__ list, int* __restrict__ nlist) {
    extern __shared__ unsigned char smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // per warp: keys[HT] int, ckeys[HT] int, vals[HT] and cvals[HT] 64-bit fixed point
    int* keys = reinterpret_cast<int*>(smem) + wid * 2 * HT;
    int* ckeys = keys + HT;
    unsigned long long* vals =
        reinterpret_cast<unsigned long long*>(smem + sizeof(int) * 2 * HT * kGemmWarps) + wid * 2 * HT;
    unsigned long long* cvals = vals + HT;
    // rows: all of them, or (list given, defer 0) the ones a previous launch deferred
    const int nrows = (list && !defer) ? *nlist : n;
    for (int idx = blockIdx.x * kGemmWarps + wid; idx < nrows; idx += gridDim.x * kGemmWarps) {
        const int row = (list && !defer) ? list[idx] : idx;
        if (small && small[row] >= 0) {   // the row was done by the thread-per-row kernel
            if (pass == 0 && lane == 0) cnt[row] = small[row];
            continue;
        }
        __syncwarp();
        // table size for this row (power of two, 32..HT): from the product
        // count in the counting pass, from the known column count when filling
        int need;
        if (pass == 0) {
            int prod = 0;
            for (int ka = aptr[row] + lane; ka < aptr[row + 1]; ka += 32) prod += bptr[acol[ka] + 1] - bptr[acol[ka]];
            for (int o = 16; o > 0; o >>= 1) prod += __shfl_xor_sync(0xffffffffu, prod, o);
            need = 2 * prod;
        } else {
            need = (4 * (cptr[row + 1] - cptr[row])) / 3 + 2;
        }
        int ht = 32;
        while (ht < need && ht < HT) ht <<= 1;
        const int hmask = ht - 1;
        for (int t = lane; t < ht; t += 32) { keys[t] = -1; vals[t] = 0ull; }
        // the row's fixed-point scale 2^sc (a fixed reduction tree: deterministic)
        double up_scale = 1.0, down_scale = 1.0;
        int sc = 0;
        if (pass != 0) {
            double bound = 0.0;
            for (int ka = aptr[row] + lane; ka < aptr[row + 1]; ka += 32)
                bound += fabs((double)aval[ka]) * babs[acol[ka]];
            for (int o = 16; o > 0; o >>= 1) bound += __shfl_xor_sync(0xffffffffu, bound, o);
            // bound < 2^e with e from the biased exponent (subnormals: e = -1022)
            const int be = (int)((__double_as_longlong(bound) >> 52) & 0x7ff);
            const int e = be ? be - 1022 : -1022;
            sc = max(-960, min(1000, 62 - e));
            up_scale = __longlong_as_double((long long)(1023 + sc) << 52);     // 2^sc
            down_scale = __longlong_as_double((long long)(1023 - sc) << 52);   // 2^-sc
        }
        __syncwarp();
        int distinct = 0;
        bool full = false;
        // Products are taken in a fixed flattened order: up to 32 A entries at
        // a time, their B rows laid end to end, 32 products per step.
        const int ab = aptr[row], ae = aptr[row + 1];
        for (int k0 = ab; k0 < ae && !full; k0 += 32) {
            const int k = k0 + lane;
            const bool ka = k < ae;
            const int a = ka ? acol[k] : 0;
            const V avk = ka ? aval[k] : V(0);
            const int bb = ka ? bptr[a] : 0;
            const int blen = ka ? bptr[a + 1] - bb : 0;
            int incl = blen;   // inclusive scan of the B row lengths over the lanes
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            const int excl = incl - blen;
            for (int t0 = 0; t0 < total; t0 += 32) {
                const int t = t0 + lane;
                const bool act = t < total;
                // owner lane: the last lane whose B-row run starts at or before t
                int j = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const int e = __shfl_sync(0xffffffffu, excl, j + step);
                    if (e <= t) j += step;
                }
                const int q = __shfl_sync(0xffffffffu, bb, j) + (t - __shfl_sync(0xffffffffu, excl, j));
                const V av = __shfl_sync(0xffffffffu, avk, j);
                const int c = act ? bcol[q] : -1;
                int slot = -1;
                bool fresh = false;
                if (act) {
                    uint32_t h = hash_u32((uint32_t)c) & hmask;
                    for (int probe = 0; probe < ht; ++probe) {
                        const int prev = atomicCAS(keys + h, -1, c);
                        if (prev == -1) { slot = (int)h; fresh = true; break; }
                        if (prev == c) { slot = (int)h; break; }
                        h = (h + 1) & hmask;
                    }
                }
                distinct += __popc(__ballot_sync(0xffffffffu, fresh));
                const bool lost = __any_sync(0xffffffffu, act && slot < 0);
                if (pass != 0 && !lost && act) {
                    long long fx;
                    if constexpr (sizeof(V) == 4) fx = fixed_product(av, bval[q], sc);
                    else fx = __double2ll_rn((av * bval[q]) * up_scale);
                    atomicAdd(vals + slot, (unsigned long long)fx);   // two's complement: signed sum mod 2^64
                }
                __syncwarp();
                if (lost || distinct > (ht * 3) / 4) { full = true; break; }
            }
        }
        if (full && pass == 2 && defer) {
            // single pass: a row that fills this launch's table is left for
            // the next launch, made with a larger one (it has written nothing)
            if (lane == 0) list[atomicAdd(nlist, 1)] = row;   // list order does not affect any result
            __syncwarp();
            continue;
        }
        if (full) {
            if (lane == 0) atomicExch(overflow, 1);
            if (pass != 1 && lane == 0) cnt[row] = 0;
            __syncwarp();
            continue;
        }
        if (pass == 0) {
            if (lane == 0) cnt[row] = distinct;
        } else {
            // compact occupied slots (slot order), then rank by column
            int base_c = 0;
            for (int t0 = 0; t0 < ht; t0 += 32) {
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
            if (pass == 2 && lane == 0) cnt[row] = base_c;
            __syncwarp();
            const int out = cptr[row];
            for (int e = lane; e < base_c; e += 32) {
                const int ce = ckeys[e];
                int rank = 0;
                for (int u = 0; u < base_c; ++u) rank += (ckeys[u] < ce);
                ccol[out + rank] = ce;
                cval[out + rank] = (V)((double)(long long)cvals[e] * down_scale);
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
// lanes per row for the per-row setup kernels, from the average row length
inline int row_lanes(int64_t nnz, int n) {
    const double avg = n ? (double)nnz / n : 1.0;
    return avg <= 12.0 ? 1 : (avg <= 48.0 ? 8 : 32);
}
template <class F>
void with_row_lanes(int64_t nnz, int n, F&& f) {
    const int vs = row_lanes(nnz, n);
    if (vs == 1) f(std::integral_constant<int, 1>{});
    else if (vs == 8) f(std::integral_constant<int, 8>{});
    else f(std::integral_constant<int, 32>{});
}

template <class V>
int pick_vs(const DCsr<V>& A) {
    const double avg = A.n ? (double)A.nnz / A.n : 1.0;
    return avg <= 6 ? 4 : (avg <= 12 ? 8 : (avg <= 24 ? 16 : 32));
}

template <class V>
void spgemm_pass(cudaStream_t s, int ht, int pass, const DCsr<V>& A, const DCsr<V>& B, const double* babs,
                 DCsr<V>& C, int* cnt,
                 int* overflow, const int* small, const int* cptr, int* ccol, V* cval, int defer, int* list,
                 int* nlist) {
    const int n = A.n;
    const size_t shm = (size_t)kGemmWarps * ht * 2 * (sizeof(int) + sizeof(double));
    // grid-stride over the rows, 32 blocks a multiprocessor (the sums are exact
    // integers, so the grid does not change the result)
    int dev = 0;
    SEMO_CUDA(cudaGetDevice(&dev));
    const int grid = std::max(1, std::min(blocks(n, kGemmWarps), sm_count(dev) * 32));
#define SEMO_GEMM_CASE(H)                                                                                        \
    case H:                                                                                                      \
        if (shm > 48 * 1024)                                                                                     \
            SEMO_CUDA(cudaFuncSetAttribute(k_spgemm<V, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm)); \
        k_spgemm<V, H><<<grid, 32 * kGemmWarps, shm, s>>>(n, A.ptr, A.col, A.val, B.ptr, B.col, B.val, babs, pass, \
                                                           cnt,                                                  \
                                                           cptr, ccol, cval, overflow, small, defer, list, nlist); \
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

// C = A * B in one numeric pass: every row is computed into a slot sized by
// its product count (an upper bound on its distinct columns), then the rows
// are compacted to their exact lengths.  Rows with few products go to the
// thread-per-row kernel, the rest to the warp hash kernel.
template <class V>
void spgemm(cudaStream_t s, semo_ctx* c, const DCsr<V>& A, const DCsr<V>& B, DCsr<V>& C) {
    const int n = A.n;
    C.n = n;
    C.m = B.m;
    C.ptr.alloc(n + 1, s);
    DBuf<int> up, cnt, flags;
    up.alloc(n + 1, s);
    cnt.alloc(std::max(n, 1), s);
    flags.alloc(2, s);
    flags.zero();
    SEMO_CUDA(cudaMemsetAsync(up.p + n, 0, sizeof(int), s));
    k_row_products<<<blocks(n, 256), 256, 0, s>>>(n, A.ptr, A.col, B.ptr, up.p, flags.p + 1);
    SEMO_CHECK_LAUNCH();
    int* const hp = c->hpin_int;   // pinned: these copies land by the scan's sync
    SEMO_CUDA(cudaMemcpyAsync(hp + 2, flags.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    const int64_t total = scan_exclusive(s, up.p, n + 1, hp + 4);   // syncs
    const int maxprod = hp[2];
    DBuf<int> tcol;
    DBuf<V> tval;
    tcol.alloc(std::max<int64_t>(total, 1), s);
    tval.alloc(std::max<int64_t>(total, 1), s);
    k_spgemm_small<V><<<blocks(n, 128), 128, 0, s>>>(n, A.ptr, A.col, A.val, B.ptr, B.col, B.val, 2, cnt.p, up.p,
                                                     tcol.p, tval.p);
    SEMO_CHECK_LAUNCH();
    if (maxprod > kSmallMaxProducts) {
        // tables sized per row from its products (<= 3/4 load); most rows fit
        // a 128-slot table, which keeps shared memory per block small (12 KB:
        // full occupancy, and room for the kernels of the other stream when
        // the setup runs beside the momentum pass; 64 slots defer too many
        // rows, 256 measured 1 ms slower per overlapped outer iteration); the
        // rest go to one more launch sized for the densest row
        int ht = 64;
        while (ht < 2048 && ht * 3 / 4 < maxprod + 2) ht <<= 1;
        const int first = std::min(ht, 128);
        DBuf<int> list, nlist;
        if (ht > first) {
            list.alloc(std::max(n, 1), s);
            nlist.alloc(1, s);
            nlist.zero();
        }
        DBuf<double> babs;   // per B row sum of |b|: the fixed-point scales
        babs.alloc(std::max(B.n, 1), s);
        k_row_abs<V><<<blocks(B.n, 256), 256, 0, s>>>(B.n, B.ptr, B.val, babs);
        SEMO_CHECK_LAUNCH();
        spgemm_pass(s, first, 2, A, B, babs.p, C, cnt.p, flags.p, cnt.p, up.p, tcol.p, tval.p, ht > first ? 1 : 0,
                    list.p, nlist.p);
        if (ht > first)
            spgemm_pass(s, ht, 2, A, B, babs.p, C, cnt.p, flags.p, cnt.p, up.p, tcol.p, tval.p, 0, list.p, nlist.p);
    }
    SEMO_CUDA(cudaMemcpyAsync(C.ptr.p, cnt.p, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
    SEMO_CUDA(cudaMemsetAsync(C.ptr.p + n, 0, sizeof(int), s));
    SEMO_CUDA(cudaMemcpyAsync(hp + 3, flags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    const int nnz = scan_exclusive(s, C.ptr.p, n + 1, hp + 4);   // syncs
    if (hp[3]) throw Error(SEMO_ERR_CUDA, "SpGEMM row has more than 1536 distinct columns");
    C.nnz = nnz;
    C.col.alloc(std::max(nnz, 1), s);
    C.val.alloc(std::max(nnz, 1), s);
    k_compact_rows<V><<<blocks(n, 256), 256, 0, s>>>(n, up.p, C.ptr.p, tcol.p, tval.p, C.col.p,
                                                                   C.val.p);
    SEMO_CHECK_LAUNCH();
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
    scan_async(s, T.ptr.p, T.n + 1, nullptr);   // the total is A.nnz
    DBuf<int> fill;
    fill.alloc(T.n + 1, s);
    SEMO_CUDA(cudaMemcpyAsync(fill.p, T.ptr.p, sizeof(int) * (T.n + 1), cudaMemcpyDeviceToDevice, s));
    k_transpose_fill<V><<<blocks(A.n, 256), 256, 0, s>>>(A.n, A.ptr, A.col, A.val, fill, tcol, tval);
    SEMO_CHECK_LAUNCH();
    k_sort_rows<V><<<blocks((int64_t)T.n * 32, 256), 256, 0, s>>>(T.n, T.ptr, tcol, tval, T.col, T.val);
    SEMO_CHECK_LAUNCH();
}

// max of kRedBlocks partial maxima into *out (one block; max is exact in
// any order)
__global__ void k_max_final(const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[32];
    double m = 0.0;
    for (int b = threadIdx.x; b < kRedBlocks; b += blockDim.x) m = fmax(m, part[b]);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, sh[w]);
        *out = r;
    }
}

// diagonal, its reciprocal and the Gershgorin bound of D^-1 A into *lam_dev
// (read back with the setup's last host sync)
template <class V>
void level_prepare(semo_ctx* c, AmgLevel<V>& L, DBuf<V>& dia, double* lam_dev) {
    cudaStream_t s = setup_stream(c);
    const int n = L.A.n;
    L.dinv.alloc(n, s);
    dia.alloc(n, s);
    DBuf<double> ratio, part;
    ratio.alloc(n, s);
    part.alloc(kRedBlocks, s);
    k_diag<V><<<blocks(n, 256), 256, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, dia, L.dinv, ratio, c->sflag);
    SEMO_CHECK_LAUNCH();
    k_max<<<kRedBlocks, kRedThreads, 0, s>>>(n, ratio, part);
    SEMO_CHECK_LAUNCH();
    k_max_final<<<1, 256, 0, s>>>(part, lam_dev);
    SEMO_CHECK_LAUNCH();
    L.x.alloc(n, s); L.b.alloc(n, s); L.r.alloc(n, s); L.t.alloc(n, s);
}

template <class V>
void amg_setup(semo_ctx* c, Amg<V>& h, const int* ptr, const int* col, const double* val64, int n, int64_t nnz) {
    cudaStream_t s = setup_stream(c);
    c->sflag.alloc(16, s);
    SEMO_CUDA(cudaMemsetAsync(c->sflag.p, 0, 16 * sizeof(int), s));
    DBuf<double> lam_dev;   // per level Gershgorin bounds
    lam_dev.alloc(64, s);
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
        {
            StageScope sc(c, ST_SETUP_LEVEL);
            level_prepare(c, L, dia, lam_dev.p + l);
        }
        h.total_nnz += L.A.nnz;
        const int nl = L.A.n;
        if (nl <= c->prm.coarse_enough || l == c->prm.max_levels - 1) break;
        // strength + MIS(2) aggregation
        DBuf<unsigned char> strong;
        DBuf<int> state, agg, agg2, undec;
        DBuf<unsigned long long> m1;
        strong.alloc(std::max<int64_t>(L.A.nnz, 1), s);
        state.alloc(nl, s); agg.alloc(nl + 1, s); agg2.alloc(nl, s);
        m1.alloc(nl, s);
        const double eps2 = (double)(eps * eps);
        eps *= 0.5f;
        int nagg = 0;
        {
            StageScope sc(c, ST_SETUP_AGG);
            with_row_lanes(L.A.nnz, nl, [&](auto vs) {
                constexpr int VS = decltype(vs)::value;
                k_strength<V, VS><<<blocks((int64_t)nl * VS, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, L.A.val, dia,
                                                                                eps2, strong, state);
            });
            SEMO_CHECK_LAUNCH();
            // Rounds go out in chunks; the undecided count after each chunk is
            // copied to pinned memory and read by the host while the next chunk
            // runs.  Rounds after the last undecided row is gone change nothing.
            constexpr int kChunk = 4, kMaxRounds = 200;
            DBuf<unsigned char> need;
            need.alloc(nl, s);
            SEMO_CUDA(cudaMemsetAsync(need.p, 1, nl, s));
            undec.alloc(2, s);
            for (auto& e : c->sync_ev)
                if (!e) SEMO_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            int* const hcnt = c->hpin_int;
            int hu = 1, ch = 0;
            for (; ch * kChunk < kMaxRounds && hu; ++ch) {
                int* const u = undec.p + (ch & 1);
                for (int k = 0; k < kChunk; ++k) {
                    SEMO_CUDA(cudaMemsetAsync(u, 0, sizeof(int), s));
                    with_row_lanes(L.A.nnz, nl, [&](auto vs) {
                        constexpr int VS = decltype(vs)::value;
                        const int g = blocks((int64_t)nl * VS, 256);
                        k_mis_max1<VS><<<g, 256, 0, s>>>(nl, L.A.ptr, L.A.col, strong, state, need, m1);
                        SEMO_CHECK_LAUNCH();
                        k_mis_max2<VS><<<g, 256, 0, s>>>(nl, L.A.ptr, L.A.col, strong, m1, state, need, u);
                        SEMO_CHECK_LAUNCH();
                    });
                }
                SEMO_CUDA(cudaMemcpyAsync(hcnt + (ch & 1), u, sizeof(int), cudaMemcpyDeviceToHost, s));
                SEMO_CUDA(cudaEventRecord(c->sync_ev[ch & 1], s));
                if (ch > 0) {
                    SEMO_CUDA(cudaEventSynchronize(c->sync_ev[(ch - 1) & 1]));
                    hu = hcnt[(ch - 1) & 1];
                }
            }
            if (hu) {   // the last chunk was launched but not yet read
                SEMO_CUDA(cudaEventSynchronize(c->sync_ev[(ch - 1) & 1]));
                hu = hcnt[(ch - 1) & 1];
            }
            if (hu) throw Error(SEMO_ERR_CUDA, "MIS(2) aggregation did not terminate");
            k_root_flags<<<blocks(nl, 256), 256, 0, s>>>(nl, state, agg2);
            SEMO_CHECK_LAUNCH();
            nagg = scan_exclusive(s, agg2.p, nl, c->hpin_int + 4);
            if (nagg > 0 && nagg < nl) {
                k_root_ids<<<blocks(nl, 256), 256, 0, s>>>(nl, state, agg2, agg);
                SEMO_CHECK_LAUNCH();
                for (int pass = 0; pass < 2; ++pass) {
                    with_row_lanes(L.A.nnz, nl, [&](auto vs) {
                        constexpr int VS = decltype(vs)::value;
                        k_agg_join<VS><<<blocks((int64_t)nl * VS, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, strong,
                                                                                     state, agg, agg2);
                    });
                    SEMO_CHECK_LAUNCH();
                    std::swap(agg.p, agg2.p);
                }
            }
        }
        if (nagg == 0 || nagg >= nl) break;
        L.nagg = nagg;
        {
        StageScope sp(c, ST_SETUP_PROLONG);
        // smoothed prolongation
        L.P.n = nl; L.P.m = nagg;
        L.P.ptr.alloc(nl + 1, s);
        SEMO_CUDA(cudaMemsetAsync(L.P.ptr.p + nl, 0, sizeof(int), s));
        DBuf<unsigned char> first;
        // counting: one thread a row costs O(row length x aggregates in the
        // row), the lane version O(row length^2 / lanes): a thread a row for
        // the finest level's short rows, lanes for the coarse levels' long ones
        const int lanes = row_lanes(L.A.nnz, nl);
        if (lanes == 1) {
            k_prolong_count<V><<<blocks(nl, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, strong, agg, L.P.ptr);
        } else {
            first.alloc(std::max<int64_t>(L.A.nnz, 1), s);
            with_row_lanes(L.A.nnz, nl, [&](auto vs) {
                constexpr int VS = decltype(vs)::value;
                if constexpr (VS > 1)
                    k_prolong_count_vs<VS><<<blocks((int64_t)nl * VS, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col,
                                                                                         strong, agg, first, L.P.ptr);
            });
        }
        SEMO_CHECK_LAUNCH();
        L.P.nnz = scan_exclusive(s, L.P.ptr.p, nl + 1, c->hpin_int + 4);
        L.P.col.alloc(std::max<int64_t>(L.P.nnz, 1), s);
        L.P.val.alloc(std::max<int64_t>(L.P.nnz, 1), s);
        // filling: the lane version rescans the row per output entry, which
        // only pays for the longest rows; both give the same values and order
        if (lanes < 32) {
            k_prolong_fill<V><<<blocks(nl, 256), 256, 0, s>>>(nl, L.A.ptr, L.A.col, L.A.val, strong, agg, omega,
                                                              L.P.ptr, L.P.col, L.P.val);
        } else {
            with_row_lanes(L.A.nnz, nl, [&](auto vs) {
                constexpr int VS = decltype(vs)::value;
                if constexpr (VS > 1)
                    k_prolong_fill_vs<V, VS><<<blocks((int64_t)nl * VS, 256), 256, 0, s>>>(
                        nl, L.A.ptr, L.A.col, L.A.val, strong, agg, first, omega, L.P.ptr, L.P.col, L.P.val);
            });
        }
        SEMO_CHECK_LAUNCH();
        transpose(s, L.P, L.R);
        }
        StageScope sg(c, ST_SETUP_GALERKIN);
        DCsr<V> AP;
        spgemm(s, c, L.A, L.P, AP);
        h.lev.emplace_back();   // capacity reserved above: L stays valid
        AmgLevel<V>& Lc = h.lev.back();
        AmgLevel<V>& Lf = h.lev[h.lev.size() - 2];
        spgemm(s, c, Lf.R, AP, Lc.A);
        Lc.A.m = Lc.A.n;
    }
    StageScope scs(c, ST_SETUP_COARSE);
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
    k_gauss_jordan<<<1, 1024, 0, s>>>(m, dense, h.cinv, c->sflag);
    SEMO_CHECK_LAUNCH();
    int* const hf = c->hpin_int + 8;   // sflag[0..5)
    const int nlev = (int)h.lev.size();
    SEMO_CUDA(cudaMemcpyAsync(c->hpin_setup, lam_dev.p, sizeof(double) * nlev, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaMemcpyAsync(hf, c->sflag.p, 5 * sizeof(int), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    for (int l = 0; l < nlev; ++l) h.lev[l].lam_max = c->hpin_setup[l];
    if (hf[2]) throw Error(SEMO_ERR_ARGUMENT, "matrix has a zero diagonal entry");
    if (hf[3]) throw Error(SEMO_ERR_NAN, "non-finite matrix entry");
    if (hf[4]) throw Error(SEMO_ERR_BREAKDOWN, "coarsest AMG matrix is singular");
    h.ready = true;
}

}  // namespace

template <class V>
void build_hierarchy(semo_ctx* c, Amg<V>& h, const int* ptr, const int* col, const double* val, int n,
                     int64_t nnz) {
    amg_setup<V>(c, h, ptr, col, val, n, nnz);
}
template void build_hierarchy<float>(semo_ctx*, Amg<float>&, const int*, const int*, const double*, int, int64_t);
template void build_hierarchy<double>(semo_ctx*, Amg<double>&, const int*, const int*, const double*, int, int64_t);

int device_scan(cudaStream_t s, int* d, int n, int* hpin) { return scan_exclusive(s, d, n, hpin); }

}  // namespace semo
