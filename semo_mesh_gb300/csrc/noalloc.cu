// Allocation-free residual norm: ||b - A x|| / ||b|| for a CSR system that
// already lives in device memory.
//
// For callers that cannot allocate device memory: a solver step running
// inside a memory arena or pool the caller manages itself, code that runs
// while the caller has a strict device-memory budget, or a loop that must not
// call cudaMalloc/cudaFree because those calls synchronise the device.  The
// solver's own residual check (cycle.cu: k_res64 + k_dot) writes the residual
// vector and the per-block partial sums into buffers the context allocates;
// this variant fuses the two and keeps its only scratch -- one pair of
// partial sums per 32-row block -- in a fixed array in the library's
// static device memory.
//
// The array is file-scope `__device__` memory: every GPU that loads the
// library holds its 1 MiB until the process exits, and every call shares it,
// so calls whose kernels overlap on a GPU (two streams, two host threads)
// race on it.  Each call overwrites every slot it reads, so nothing needs
// clearing between calls.
//
// Its device address is looked up on every call made outside stream capture
// (the lookup does not synchronise), so a primary context that was torn down
// and created again (cudaDeviceReset) never sees a stale address.  Inside a
// capture the address found by the last uncaptured call on that device is
// used; a device with no uncaptured call yet gets SEMO_ERR_STATE, so make the
// first call on each device before any stream capture.
//
// Launch errors: an error already pending in the caller's thread (from the
// caller's own earlier work) is left in place and reported as SEMO_ERR_CUDA
// before anything is launched; after the launches cudaGetLastError reads and
// clears only the error of these two launches.
#include <cuda_runtime.h>

#include <mutex>

#include "semo_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kRowsPerBlock = 32;                                  // 8 lanes a row
constexpr int kMaxBlocks = SEMO_STATIC_MAX_ROWS / kRowsPerBlock;   // 65536 partial pairs = 1 MiB
static_assert(SEMO_STATIC_MAX_ROWS % kRowsPerBlock == 0, "row limit must be a whole number of blocks");

__device__ __align__(256) double g_residual_scratch[2 * kMaxBlocks];

// per device: address of g_residual_scratch found by the last call made
// outside stream capture
std::mutex g_lock;
double* g_addr[64] = {nullptr};

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

// r_i = b_i - sum_j a_ij x_j with 8 lanes per row, summed exactly as the
// solver's FP64 residual kernel sums a row (so r_i is bit-identical to it);
// per block sum r^2 and b^2
constexpr int kLanes = 8;
__global__ void __launch_bounds__(kThreads) k_res_parts(int n, const int* __restrict__ ptr,
                                                        const int* __restrict__ col,
                                                        const double* __restrict__ val,
                                                        const double* __restrict__ x,
                                                        const double* __restrict__ b,
                                                        double* __restrict__ part, int nparts) {
    __shared__ double sh[32];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = g / kLanes, lane = g % kLanes;
    double s = 0.0;
    if (row < n) {
        const int e = ptr[row + 1];
        for (int k = ptr[row] + lane; k < e; k += kLanes) s += val[k] * __ldg(x + col[k]);
    }
#pragma unroll
    for (int o = kLanes / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, kLanes);
    double rr = 0.0, bb = 0.0;
    if (row < n && lane == 0) {
        const double bi = b[row], ri = bi - s;
        rr = ri * ri;
        bb = bi * bi;
    }
    rr = block_sum(rr, sh);
    bb = block_sum(bb, sh);
    if (threadIdx.x == 0) { part[blockIdx.x] = rr; part[nparts + blockIdx.x] = bb; }
}

// fixed-order sum of the partials: out = {||r||/||b|| (||r|| if b == 0), ||r||, ||b||}
__global__ void k_res_finish(int nparts, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[32];
    double rr = 0.0, bb = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) { rr += part[i]; bb += part[nparts + i]; }
    rr = block_sum(rr, sh);
    bb = block_sum(bb, sh);
    if (threadIdx.x == 0) {
        const double rn = sqrt(rr), bn = sqrt(bb);
        out[0] = (bn > 0.0) ? rn / bn : rn;
        out[1] = rn;
        out[2] = bn;
    }
}

}  // namespace

extern "C" semo_status semo_residual_norm_static(const int32_t* ptr, const int32_t* col, const double* val, int n,
                                                 const double* x, const double* b, double* out3, void* stream) {
    if (!ptr || !col || !val || !x || !b || !out3 || n <= 0) return SEMO_ERR_ARGUMENT;
    if (n > SEMO_STATIC_MAX_ROWS) return SEMO_ERR_ARGUMENT;   // the static scratch holds 65536 blocks of 32 rows
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SEMO_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // an error left by the caller's own work stays the caller's: do not launch, do not clear it
    if (cudaPeekAtLastError() != cudaSuccess) return SEMO_ERR_CUDA;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return SEMO_ERR_CUDA;
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> g(g_lock);
        if (cap == cudaStreamCaptureStatusNone) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_residual_scratch) != cudaSuccess || !p) return SEMO_ERR_CUDA;
            g_addr[dev] = static_cast<double*>(p);
        } else if (!g_addr[dev]) {
            return SEMO_ERR_STATE;   // no uncaptured call on this device yet: the address is unknown
        }
        scratch = g_addr[dev];
    }
    const int nparts = (n + kRowsPerBlock - 1) / kRowsPerBlock;
    k_res_parts<<<nparts, kThreads, 0, s>>>(n, ptr, col, val, x, b, scratch, nparts);
    if (cudaGetLastError() != cudaSuccess) return SEMO_ERR_CUDA;
    k_res_finish<<<1, 256, 0, s>>>(nparts, scratch, out3);
    if (cudaGetLastError() != cudaSuccess) return SEMO_ERR_CUDA;
    __atomic_add_fetch(&semo::g_kernel_launches, 2, __ATOMIC_RELAXED);
    return SEMO_OK;
}
