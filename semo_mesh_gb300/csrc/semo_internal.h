// Internal declarations shared by the host C-ABI layer and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/semo_gb300.h"

namespace semo {

struct Error : std::runtime_error {
    semo_status status;
    Error(semo_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define SEMO_CUDA(call)                                                                      \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            throw ::semo::Error(e_ == cudaErrorMemoryAllocation ? SEMO_ERR_OUT_OF_MEMORY     \
                                                                : SEMO_ERR_CUDA,             \
                                std::string(#call) + ": " + cudaGetErrorString(e_));         \
    } while (0)

// Every kernel launch is followed by this check, which also counts launches.
extern long long g_kernel_launches;
#define SEMO_CHECK_LAUNCH()                         \
    do {                                            \
        __atomic_add_fetch(&::semo::g_kernel_launches, 1, __ATOMIC_RELAXED); \
        SEMO_CUDA(cudaGetLastError());              \
    } while (0)

// Named stages timed with CUDA events on the context's stream when profiling is on.
enum Stage { ST_FACE_VALUES, ST_GRAVITY, ST_STENCIL, ST_PFACE, ST_PBFACE, ST_PCELL, ST_AMG_SETUP, ST_PCG,
             ST_GG, ST_UPDATE, ST_VCYCLE, ST_SETUP_AGG, ST_SETUP_PROLONG, ST_SETUP_GALERKIN, ST_SETUP_LEVEL,
             ST_SETUP_COARSE, ST_MFACE, ST_MCELL, ST_MSOLVE, ST_MUPDATE, ST_MSTACS, ST_VFACE, ST_VSOLVE, ST_VUPDATE,
             ST_STENCIL_UVW, ST_MBFACE, ST_CGRAD, ST_CFACE, ST_CCELL, ST_CSOLVE, ST_CUPDATE, ST_SFT, ST_SETUP_CYCLE, ST_COUNT };
static const char* const kStageNames[ST_COUNT] = {"face_values", "gravity", "stencil", "pface", "pbface", "pcell",
                                                  "amg_setup", "pcg", "gauss_green", "update", "vcycle",
                                                  "setup_aggregate", "setup_prolong", "setup_galerkin",
                                                  "setup_level", "setup_coarse", "mface", "mcell", "msolve",
                                                  "mupdate", "mstacs", "vface", "vsolve", "vupdate", "stencil_uvw", "mbface",
                                                  "cgrad", "cface", "ccell", "csolve", "cupdate", "surface_tension",
                                                  "setup_cycle"};

// Device buffer, stream-ordered allocation (memory pool keeps freed blocks).
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept { *this = std::move(o); }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; s = o.s; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DBuf() { release(); }
    void alloc(size_t count, cudaStream_t st) {
        if (count == n && p) return;
        release();
        s = st;
        n = count;
        if (count) SEMO_CUDA(cudaMallocAsync((void**)&p, sizeof(T) * count, st));
    }
    void zero() { if (n) SEMO_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * n, s)); }
    void upload(const T* h, size_t count, cudaStream_t st) {
        alloc(count, st);
        if (count) SEMO_CUDA(cudaMemcpyAsync(p, h, sizeof(T) * count, cudaMemcpyHostToDevice, st));
    }
    void release() {
        if (p) { cudaFreeAsync(p, s); p = nullptr; }
        n = 0;
    }
    operator T*() const { return p; }
};

// Scalar CSR matrix on the device.
template <class V>
struct DCsr {
    int n = 0, m = 0;      // rows, cols
    int64_t nnz = 0;
    DBuf<int> ptr, col;
    DBuf<V> val;
};

// One level of the smoothed-aggregation hierarchy, value type V.
template <class V>
struct AmgLevel {
    DCsr<V> A, P, R;
    DBuf<V> dinv;          // 1 / a_ii
    double lam_max = 0.0;  // Gershgorin bound on rho(D^-1 A)
    DBuf<V> x, b, r, t;    // work vectors
    int nagg = 0;
};

template <class V>
struct Amg {
    std::vector<AmgLevel<V>> lev;
    int coarse_n = 0;
    DBuf<double> cinv;     // explicit FP64 inverse of the coarsest matrix (row-major)
    int64_t total_nnz = 0;
    bool ready = false;
    void clear() { lev.clear(); cinv.release(); coarse_n = 0; total_nnz = 0; ready = false; }
};

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
};

constexpr int kHostScalars = 128;   // doubles in semo_ctx::hpin and ::hpin_setup
constexpr int kHostInts = 16;       // ints in semo_ctx::hpin_scan and ::hpin_int

}  // namespace semo

struct semo_ctx {
    semo_params prm{};
    semo_physics phys{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    // mesh sizes
    int np = 0, nf = 0, ni = 0, nc = 0, nb = 0, npatch = 0;
    int64_t nnz = 0, st_nnz = 0, cf_nnz = 0;
    std::vector<int> perm, iperm;                 // RCM
    std::vector<int> fperm, fiperm;               // stored face order: fperm[stored] = caller's face
    std::vector<int> patch_start, patch_size;
    std::vector<int> h_bc_type;                   // npatch*3
    std::vector<double> h_bc_value;               // npatch*5

    // ---- device mesh (cells in RCM numbering, faces in caller order) ----
    semo::DBuf<int> own, nei;                     // face -> cell (RCM numbering)
    semo::DBuf<int> cf_ptr, cf_idx;               // cell -> faces, ascending face, bit 30 = neighbour side
    semo::DBuf<int> st_ptr, st_idx;               // vertex stencil (reference order)
    semo::DBuf<int> bpatch;                       // boundary face -> patch
    semo::DBuf<int> bc_type;                      // npatch*3
    semo::DBuf<double> bc_value;                  // npatch*5
    // geometry (SoA, 3-vectors stored as 3 planes of length nf or nc)
    semo::DBuf<double> fn, fa, fc, wc, mpn, alf, epn, skew, pf, nfv;
    semo::DBuf<double> vol, cc, minv;             // cc: 3 planes; minv: 6 planes
    semo::DBuf<double> stw;                       // 3 planes of st_nnz: w_k * d_k (LSQ weight vectors)
    semo::DBuf<double> bfw;                       // 3 planes of nb: boundary-face LSQ weight vectors
    semo::DBuf<double> stws;                      // 3 planes of nc: per-cell sum of the stencil and boundary weights
    semo::DBuf<int> st_tpos;                      // per stencil entry (j, i): the entry's position in i's row (adjoint)
    int st_tpos_gen = -1;                         // mesh generation st_tpos was built for
    // derived per-face constants for the hot face kernel
    semo::DBuf<double> fk;                        // 4 planes of ni: kA = alpha*area/magPN, kP = alpha/magPN, area, wC

    // ---- CSR pattern (RCM order) ----
    semo::DBuf<int> A_ptr, A_col, A_dig, A_lr, A_rl;
    semo::DBuf<double> A_val, b;

    // ---- fields (RCM order) ----
    semo::DBuf<double> P, U, V, W, VF, rho, irho;
    semo::DBuf<double> grad;                      // 15 planes: P,U,V,W,VF x (x,y,z)
    semo::DBuf<double> mm;                        // 10 planes: maxU,minU,maxV,minV,maxW,minW,maxVF,minVF,maxP,minP
    semo::DBuf<double> sg;                        // 4 planes gravity source
    semo::DBuf<double> bface;                     // boundary face values: 10 planes of nb
    semo::DBuf<double> fscr;                      // face scratch: 3 planes of nf
    semo::DBuf<double> unf;                       // UnF per face
    semo::DBuf<double> x, gx;                     // solution and its Gauss-Green gradient (3 planes)
    semo::DBuf<double> src;                       // optional per-cell source s (b_i += s_i V_i)
    semo::DBuf<double> stage;                     // caller-order staging for field copies (5 planes)
    semo::DBuf<int> dperm;                        // RCM permutation on the device: dperm[r] = caller's cell
    bool has_src = false;

    // ---- momentum equation (RCM order; matrix on the A_ptr/A_col pattern) ----
    semo::DBuf<double> mu;                        // 2 planes: cell viscosity, its reciprocal
    semo::DBuf<double> old;                       // 6 planes: oldU, oldV, oldW, old2U, old2V, old2W
    bool has_old = false;
    semo::DBuf<double> Am_val;                    // values; dropped off-diagonals hold 0
    semo::DBuf<double> bm, xm;                    // 3 planes each (x, y, z)
    semo::DBuf<double> msc;                       // face scratch: 8 planes of nf
    bool mom_assembled = false;
    // grad P, grad VF, their stencil limits and the gravity source match the
    // current P and VF (set by the momentum assembly, cleared when P, VF or the
    // physics change); the pressure assembly then recomputes only the U,V,W parts
    bool pvf_current = false;
    // the gravity source was computed since the last change of fields or physics
    // (the VOF sub-iterations keep it, as SEMO keeps its per-time-step source)
    bool sg_current = false;
    // curvature and surface-tension source (phys.sigma != 0): planes of nc
    // 0 kappa, 1 ls, 2-5 src (x, y, z, .U), 6-11 scratch; computed with the
    // gravity source and kept with it
    semo::DBuf<double> sft;
    semo::DBuf<int> sft_iface;
    bool sft_current = false;

    // ---- volume fraction (RCM order; matrix on the A_ptr/A_col pattern) ----
    semo::DBuf<double> oldvf;                     // 2 planes: oldVF, old2VF
    bool has_oldvf = false;
    semo::DBuf<double> Av_val, bvf, xvf;          // VOF matrix values, RHS, solution
    semo::DBuf<double> vsc;                       // face scratch: 3 planes of nf
    semo::DBuf<double> fvf;                       // MSTACS face values: 2 planes of nf (left, right)
    semo::DBuf<double> co;                        // cell Courant number
    bool vof_assembled = false;

    // ---- compressible coupled system (RCM order; 5x5 blocks on A_ptr/A_col) ----
    semo_coupled_physics cphys{};
    bool cpl_phys = false, cpl_fields = false, cpl_assembled = false;
    semo::DBuf<int> cpl_bct;                      // npatch*3: type of p, u, T
    semo::DBuf<double> cpl_bcv;                   // npatch*5: p, u, v, w, T
    semo::DBuf<double> cpl_f;                     // 15 planes: P,U,V,W,T; at n-1; at n-2
    semo::DBuf<double> cpl_eos;                   // 7 planes: rho, C, Ht, drho/dp, drho/dT, dHt/dp, dHt/dT
    semo::DBuf<double> cpl_bR;                    // 12 planes of nb: boundary right primitives + EOS
    semo::DBuf<double> cpl_grad, cpl_mm;          // 15 planes of gradients; 10 planes of stencil limits
    semo::DBuf<double> cpl_val;                   // 25 per slot of the scalar pattern
    semo::DBuf<double> cpl_b, cpl_x;              // 5 planes each (field-split)
    semo::DBuf<double> cpl_scr;                   // 5 planes of nf face fluxes + 27 planes of nb
    semo::DBuf<double> cpl_lim;                   // 10 update clamps
    std::shared_ptr<void> cpl_solver;             // solver state (coupled.cu)
    std::shared_ptr<void> cpr;                    // AMG on the coupled pressure equation (cycle.cu)
    std::shared_ptr<void> mom_apply;              // momentum Krylov state (cycle.cu)
    semo::DBuf<double> red;                       // reduction partials
    semo::DBuf<int> flag;                         // device error flags

    // ---- pressure hierarchy built beside the momentum pass ----
    // The pressure matrix depends only on geometry, dt and the densities, so
    // semo_outer_iteration assembles it and builds its AMG hierarchy on a
    // second stream (from a second host thread) while the momentum pass runs.
    // The setup functions launch on setup_s (the context's stream otherwise)
    // and report through sflag; the pressure pass then leaves A_val alone.
    cudaStream_t aux_stream = nullptr;
    cudaStream_t setup_s = nullptr;
    semo::DBuf<int> sflag;                        // setup error flags (16)
    semo::DBuf<double> pm_coef;                   // face coefficients of the early matrix (nf)
    bool matrix_prebuilt = false;
    double side_setup_ms = 0.0;                   // host time of the setup on its thread
    std::function<void()> before_solve;           // with matrix_prebuilt: join the setup, wait for it
    // face values done (main) / hierarchy done (aux) / early matrix done (aux)
    cudaEvent_t ov_ev[3] = {nullptr, nullptr, nullptr};
    std::mutex prof_mu;                           // stage timers are recorded from both threads

    // solver state
    semo::Amg<double> amg64;
    semo::Amg<float> amg32;
    semo::DBuf<double> kr, kz, kp, kq;            // Krylov vectors (FP64)
    semo::DBuf<float> kz32, kr32;
    // Pinned host scalars, one set per host thread that reads results back:
    // a device-to-host copy into pageable memory waits inside the CUDA runtime for
    // its stream, and while it waits the other thread's CUDA calls queue
    // behind it (the hierarchy built beside the momentum pass stalled for the
    // momentum assembly's duration on such a read).  Allocated with the context.
    double* hpin = nullptr;                       // context's stream: convergence checks, norms (kHostScalars)
    int* hpin_scan = nullptr;                     // context's stream: scan totals and flags (kHostInts)
    int* hpin_int = nullptr;                      // setup: counters and scan totals (kHostInts)
    double* hpin_setup = nullptr;                 // setup: per-level scalars (kHostScalars)
    cudaEvent_t sync_ev[2] = {nullptr, nullptr};  // completion of those counter copies
    std::shared_ptr<void> apply;                  // V-cycle/Krylov apply state (cycle.cu)
    std::shared_ptr<void> setup_worker;           // host thread of the overlapped pressure setup (capi.cpp)

    bool mesh_ready = false, phys_ready = false, fields_ready = false, assembled = false;
    int mesh_gen = 0;                             // bumped by every mesh upload (cached layouts check it)
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // the pressure setup's own timing pair: the setup may run on the second
    // host thread while the momentum solve records ev[] on the main one
    cudaEvent_t setup_ev[2] = {nullptr, nullptr};

    // profiling: per-stage device time from event pairs, resolved after each call
    bool profiling = false;
    double stage_ms[semo::ST_COUNT] = {0};
    long long stage_calls[semo::ST_COUNT] = {0};
    std::vector<cudaEvent_t> ev_pool;
    struct Pending { int stage; cudaEvent_t a, b; };
    std::vector<Pending> pending;
};

namespace semo {

inline cudaEvent_t take_event(semo_ctx* c) {
    if (!c->ev_pool.empty()) { cudaEvent_t e = c->ev_pool.back(); c->ev_pool.pop_back(); return e; }
    cudaEvent_t e;
    SEMO_CUDA(cudaEventCreate(&e));
    return e;
}

// the stream the AMG setup launches on
inline cudaStream_t setup_stream(const semo_ctx* c) { return c->setup_s ? c->setup_s : c->stream; }

// the AMG setup stages run on setup_s
inline bool is_setup_stage(int st) {
    return st == ST_AMG_SETUP || st == ST_SETUP_AGG || st == ST_SETUP_PROLONG || st == ST_SETUP_GALERKIN ||
           st == ST_SETUP_LEVEL || st == ST_SETUP_COARSE || st == ST_SETUP_CYCLE;
}

// RAII: times the enclosed launches of one stage when profiling is enabled.
struct StageScope {
    semo_ctx* c;
    int stage;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    StageScope(semo_ctx* ctx, int st) : c(ctx), stage(st) {
        s = is_setup_stage(st) ? setup_stream(c) : c->stream;
        if (c->profiling) {
            std::lock_guard<std::mutex> lk(c->prof_mu);
            a = take_event(c);
            cudaEventRecord(a, s);
        }
    }
    ~StageScope() {
        if (a) {
            std::lock_guard<std::mutex> lk(c->prof_mu);
            cudaEvent_t b = take_event(c);
            cudaEventRecord(b, s);
            c->pending.push_back({stage, a, b});
        }
    }
};

// Accumulate finished stage timings (call after the stream is synchronized).
inline void resolve_stage_timers(semo_ctx* c) {
    std::lock_guard<std::mutex> lk(c->prof_mu);
    for (auto& p : c->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            c->stage_ms[p.stage] += ms;
            c->stage_calls[p.stage] += 1;
        }
        c->ev_pool.push_back(p.a);
        c->ev_pool.push_back(p.b);
    }
    c->pending.clear();
}

}  // namespace semo

namespace semo {

// host-side mesh preprocessing (topology.cpp, rcm.cpp)
void genrcm_perm(int n, const std::vector<int>& xadj, const std::vector<int>& adj, std::vector<int>& perm);

// geometry.cu
void geometry_build(semo_ctx* c, const double* d_points, const int* d_fptr, const int* d_fpts,
                    const std::vector<int>& h_own_rcm);

// assemble.cu
void assemble_pressure(semo_ctx* c);
double pressure_update(semo_ctx* c);
// EOS + boundary face values (+ cell viscosity when with_mu)
void assemble_face_values(semo_ctx* c, bool with_mu);
// gravity source + one stencil pass (gradients of P,U,V,W,VF; min/max of U,V,W,VF,P)
void assemble_gravity_stencil(semo_ctx* c);
void assemble_gravity(semo_ctx* c);
// full: all five fields; else U, V, W only (P and VF planes left as they are)
void stencil_pass(semo_ctx* c, bool full);
// surftens.cu: curvature and surface-tension source (no-op when sigma == 0);
// after assemble_face_values and a full stencil_pass
void assemble_surface_tension(semo_ctx* c);
// dst[q][r] = src[q*n + perm[r]] for q < planes; false if any value is not finite (syncs)
bool fields_from_caller_order(semo_ctx* c, const double* src, double* const* dst, int planes);
// dst[q*n + perm[r]] = src[q][r] for q < planes (async)
void fields_to_caller_order(semo_ctx* c, const double* const* src, double* dst, int planes);
// out[i] = a[i] * b[i] over the cells (async)
void cellwise_product(semo_ctx* c, const double* a, const double* b, double* out);

// LSQ gradients (15 planes) and stencil limits (10 planes) of five cell
// fields f0..f4 with boundary-face values bf (5 planes of nb)
void lsq_gradients5(semo_ctx* c, const double* f0, const double* f1, const double* f2, const double* f3,
                    const double* f4, const double* bf, double* grad, double* mm);

// cycle.cu: AMG on the pressure equation of the coupled system (value type float or double)
template <class V>
void cpr_setup(semo_ctx* c, const int* ptr, const int* col, const double* val, int n, int64_t nnz);
// x = one V-cycle on b (device arrays of n)
template <class V>
void cpr_vcycle(semo_ctx* c, const V* b, V* x);

// coupled.cu: compressible coupled 5x5 system
void coupled_assemble(semo_ctx* c);
semo_status coupled_solve(semo_ctx* c, semo_solve_info* info);   // c->cpl_b -> c->cpl_x
double coupled_update(semo_ctx* c);

// amg_setup.cu: smoothed-aggregation hierarchy (value type float or double)
template <class V>
void build_hierarchy(semo_ctx* c, Amg<V>& h, const int* ptr, const int* col, const double* val, int n,
                     int64_t nnz);
// exclusive scan of d[0..n) in place on the context's stream; returns the total
// exclusive scan of d[0..n) on the stream; returns the total, read through
// the pinned int *hpin (one host sync)
int device_scan(cudaStream_t s, int* d, int n, int* hpin);

// pressure matrix values only (A_val: off-diagonals and diagonal, the values
// assemble_pressure writes) on stream s, after assemble_face_values
void pressure_matrix(semo_ctx* c, cudaStream_t s);

// cycle.cu
// AMG hierarchy (and the FP64 outer operator) of the matrix, on c->setup_s;
// may_reuse: the matrix is the context's own pressure system, so a hierarchy
// built from bit-identical values may be kept (semo_params.reuse_hierarchy).
// Records the setup time in info->setup_ms.
void pressure_setup(semo_ctx* c, const int* d_ptr, const int* d_col, const double* d_val, int n, int64_t nnz,
                    bool may_reuse, semo_solve_info* info);
// setup (unless c->matrix_prebuilt: the hierarchy is already there) and solve
void solve_system(semo_ctx* c, const int* d_ptr, const int* d_col, const double* d_val, int n, int64_t nnz,
                  const double* d_b, double* d_x, semo_solve_info* info, bool zero_guess, bool may_reuse = false);

void solve_transpose_reuse(semo_ctx* c, const double* d_g, double* d_lam, semo_solve_info* info);
// measurement: ms per launch of y = A x on the last pressure hierarchy's finest
// operator in the V-cycle's layout (which 0) or the FP64 outer operator (which 1)
double time_pressure_spmv(semo_ctx* c, int which, int reps);
// per level of the last pressure hierarchy, 6 values: rows, nnz(A), nnz(P),
// nnz(R), layout of A in the V-cycle (2 SELL-32 16-bit offsets, 1 SELL-32,
// 0 CSR, -1 coarsest: direct solve), value bytes; returns the level count
int pressure_levels(semo_ctx* c, int64_t* out, int max_levels);
// three right-hand sides of the momentum system (c->Am_val, c->bm) -> c->xm; info[3]; returns the
// worst status (SEMO_OK, SEMO_ERR_NOT_CONVERGED or SEMO_ERR_BREAKDOWN)
semo_status solve_momentum(semo_ctx* c, semo_solve_info* info);
// the volume-fraction system (c->Av_val, c->bvf) -> c->xvf; info[1]
semo_status solve_vof(semo_ctx* c, semo_solve_info* info);
// nrhs (1..3) right-hand sides (planes of n) of a caller's CSR matrix (device
// arrays; dig = position of each row's diagonal) by the momentum solver
// (Jacobi BiCGStab, batched for three); x in/out (the initial guess is used
// when guess); info[nrhs]; returns the worst status as solve_momentum does
semo_status solve_csr_multi(semo_ctx* c, int n, const int* ptr, const int* col, const int* dig, const double* val,
                            int nrhs, const double* b, double* x, bool guess, semo_solve_info* info);

// momentum.cu (face_values_done: assemble_face_values(c, true) already ran)
void assemble_momentum(semo_ctx* c, bool face_values_done = false);
double momentum_update(semo_ctx* c);

// adjoint.cu: lambda^T db/d(U, V, W, P) of the pressure equation's right-hand
// side at the current fields (lambda device, RCM order) -> out, 4 planes
// (dJ/dU, dJ/dV, dJ/dW, dJ/dP), RCM order
void vjp_fields(semo_ctx* c, const double* lam, double* out);

// vof.cu
void assemble_vof(semo_ctx* c);
double vof_update(semo_ctx* c);

int sm_count(int device);

}  // namespace semo
