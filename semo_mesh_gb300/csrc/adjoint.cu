// Discrete adjoint of the pressure-correction right-hand side: the
// vector-Jacobian product lambda^T db/d(U, V, W, P) of calcPressureEq's face
// flux residual (src/solvers/eqPressure.cpp:246-673 with the face velocity of
// src/solvers/surfaceNormalVelocity.cpp:100-187).
//
// b_i = sum over the faces of cell i of -/+ UnF_f A_f (owner -, neighbour +),
// with UnF the skew-corrected, stencil-limited, wC-weighted face velocity
// plus the Rhie-Chow pressure terms.  The matrix depends only on geometry,
// dt and the densities, so dJ/dphi = (db/dphi)^T lambda with lambda = A^-T
// dJ/dx.  b is piecewise linear in the fields; the derivative taken is the
// one of the active piece: a reconstruction clamped to its cell's stencil
// maximum (minimum) passes its adjoint to the stencil cell that holds that
// maximum (minimum), the first one in the stencil's order as the forward
// min/max keeps it.
//
// Nothing is stored by the forward pass for this: the LSQ gradients, stencil
// limits and their arg-extrema are recomputed from the cell fields (the
// checkpoint) into scratch, then three gathers run, each cell summing what
// reaches it in a fixed order (no atomics):
//   k_adj_cell    over the cell's faces: the face adjoint mu_f = A_f
//                 (lambda_q - lambda_o), the direct field terms, the
//                 adjoints of the cell's own gradients (mapped through the
//                 symmetric M^-1 of its LSQ fit) and of its clamped limits;
//   k_adj_gather  over the cell's vertex stencil (symmetric, so the cells
//                 whose gradients read cell j are j's own stencil; the weight
//                 w_ij is read at its position in i's row, st_tpos), its
//                 boundary faces (through the boundary-value rules) and the
//                 limit adjoints of the stencil cells whose extremum it holds.
#include <cuda_runtime.h>

#include "face_common.cuh"
#include "semo_internal.h"

namespace {

using namespace semo::face;

// position of j in i's stencil row for every entry (j, i) of j's row; -1 (and
// flag) when the stencil is not symmetric
__global__ void k_stencil_tpos(int nc, const int* __restrict__ stp, const int* __restrict__ sti,
                               int* __restrict__ tpos, int* __restrict__ flag) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nc) return;
    for (int k = stp[j]; k < stp[j + 1]; ++k) {
        const int i = sti[k];
        int t = -1;
        for (int kk = stp[i]; kk < stp[i + 1]; ++kk)
            if (sti[kk] == j) { t = kk; break; }
        tpos[k] = t;
        if (t < 0) atomicExch(flag, 1);
    }
}

// index of the stencil maximum and minimum of U, V, W (self first, then the
// stencil in order, keeping the first extreme value as k_stencil does):
// planes 0-2 argmax U, V, W; 3-5 argmin
__global__ void k_adj_argext(int nc, const int* __restrict__ stp, const int* __restrict__ sti,
                             const double* __restrict__ U, const double* __restrict__ V,
                             const double* __restrict__ W, int* __restrict__ arg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double* F[3] = {U, V, W};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        long long kmax = okey(F[c][i]), kmin = kmax;
        int imax = i, imin = i;
        for (int k = stp[i]; k < stp[i + 1]; ++k) {
            const int j = __ldg(sti + k);
            const long long t = okey(__ldg(F[c] + j));
            if (kmax < t) { kmax = t; imax = j; }
            if (t < kmin) { kmin = t; imin = j; }
        }
        arg[(size_t)c * nc + i] = imax;
        arg[(size_t)(3 + c) * nc + i] = imin;
    }
}

struct AdjCellArgs {
    int nc, ni, nf, nb;
    const int *cfp, *cfi, *own, *nei, *bpatch, *bct;
    const double *fn, *skew, *alf, *epn, *fk, *fa, *mpn, *bf, *irho;
    const double *U, *V, *W, *grad, *mm, *minv, *lam;
    double dt;
    double *gdir, *gm, *lim;   // 4 planes; 12 planes (U, V, W, P x xyz); 6 planes (max U,V,W; min U,V,W)
};

__global__ void __launch_bounds__(128) k_adj_cell(AdjCellArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nc) return;
    const size_t N = a.nc;
    const int nf = a.nf, ni = a.ni, nb = a.nb;
    const double li = a.lam[i], iri = a.irho[i];
    const double phi[3] = {a.U[i], a.V[i], a.W[i]};
    double G[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) G[c][d] = a.grad[(3 * (c + 1) + d) * N + i];
    long long khi[3], klo[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        khi[c] = okey(a.mm[(2 * c) * N + i]);
        klo[c] = okey(a.mm[(2 * c + 1) * N + i]);
    }
    double gd[4] = {0.0, 0.0, 0.0, 0.0};
    double gg[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double lmax[3] = {0, 0, 0}, lmin[3] = {0, 0, 0};
    for (int k = a.cfp[i]; k < a.cfp[i + 1]; ++k) {
        const int e = a.cfi[k], f = e & kFaceMask;
        const double n[3] = {a.fn[f], a.fn[nf + f], a.fn[2 * nf + f]};
        if (f < ni) {
            const bool own_side = (e >> 30) == 0;
            const int other = own_side ? a.nei[f] : a.own[f];
            const double lo = __ldg(a.lam + other), iro = __ldg(a.irho + other);
            const double area = a.fk[2 * ni + f], wL = a.fk[3 * ni + f], wR = 1.0 - wL, kP = a.fk[ni + f];
            const double mu = own_side ? area * (lo - li) : area * (li - lo);
            const double w = own_side ? wL : wR;
            const double s0 = a.skew[f], s1 = a.skew[nf + f], s2 = a.skew[2 * nf + f];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                // the reconstruction of face_unf, and its clamp's active piece
                const double r = phi[c] + G[c][0] * s0 + G[c][1] * s1 + G[c][2] * s2;
                const long long kr = okey(r);
                const double ad = mu * w * n[c];
                if (kr > khi[c]) lmax[c] += ad;
                else if (kr < klo[c]) lmin[c] += ad;
                else { gd[c] += ad; gg[c][0] += ad * s0; gg[c][1] += ad * s1; gg[c][2] += ad * s2; }
            }
            // -tt kP (P_q - P_o) and the (dt w / rho) grad P . alpha e terms
            const double iRL = own_side ? iri : iro, iRR = own_side ? iro : iri;
            const double tt = a.dt * (wL * iRL + wR * iRR);
            gd[3] += own_side ? mu * tt * kP : -(mu * tt * kP);
            const double as = own_side ? a.dt * wL * iRL : a.dt * wR * iRR;
            const double al = a.alf[f];
#pragma unroll
            for (int d = 0; d < 3; ++d) gg[3][d] += mu * as * (al * a.epn[(size_t)d * nf + f]);
        } else {
            const int b = f - ni, p = a.bpatch[b];
            const double mu = -(a.fa[f] * li);
            const int tp = a.bct[3 * p], tu = a.bct[3 * p + 1];
            if (tu == SEMO_BC_SLIP) {
                const double nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
#pragma unroll
                for (int c = 0; c < 3; ++c) gd[c] += mu * (n[c] - n[c] * nn);
            } else if (tu != SEMO_BC_FIXED_VALUE && tu != SEMO_BC_NO_SLIP) {
#pragma unroll
                for (int c = 0; c < 3; ++c) gd[c] += mu * n[c];
            }
            if (tp == SEMO_BC_FIXED_VALUE) {
                const double tmp1 = 1.0 / a.bf[5 * nb + b] * a.dt, dPN = 0.5 * a.mpn[f], al = a.alf[f];
                gd[3] += mu * al * tmp1 / dPN;
#pragma unroll
                for (int d = 0; d < 3; ++d) gg[3][d] += mu * al * tmp1 * a.epn[(size_t)d * nf + f];
            }
        }
    }
    const double m0 = a.minv[i], m1 = a.minv[N + i], m2 = a.minv[2 * N + i];
    const double m3 = a.minv[3 * N + i], m4 = a.minv[4 * N + i], m5 = a.minv[5 * N + i];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        a.gdir[q * N + i] = gd[q];
        a.gm[(3 * q + 0) * N + i] = m0 * gg[q][0] + m1 * gg[q][1] + m2 * gg[q][2];
        a.gm[(3 * q + 1) * N + i] = m1 * gg[q][0] + m3 * gg[q][1] + m4 * gg[q][2];
        a.gm[(3 * q + 2) * N + i] = m2 * gg[q][0] + m4 * gg[q][1] + m5 * gg[q][2];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        a.lim[c * N + i] = lmax[c];
        a.lim[(3 + c) * N + i] = lmin[c];
    }
}

struct AdjGatherArgs {
    int nc, ni, nf, nb;
    int64_t stn;
    const int *stp, *sti, *tpos, *cfp, *cfi, *bpatch, *bct, *arg;
    const double *stw, *stws, *bfw, *fn, *gdir, *gm, *lim;
    double* out;   // 4 planes: dJ/dU, dJ/dV, dJ/dW, dJ/dP
};

__global__ void __launch_bounds__(128) k_adj_gather(AdjGatherArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.nc) return;
    const size_t N = a.nc;
    const int nf = a.nf, ni = a.ni, nb = a.nb;
    const double S[3] = {a.stws[j], a.stws[N + j], a.stws[2 * N + j]};
    double mj[4][3];
    double acc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int d = 0; d < 3; ++d) mj[q][d] = a.gm[(3 * q + d) * N + j];
        acc[q] = a.gdir[q * N + j] - (S[0] * mj[q][0] + S[1] * mj[q][1] + S[2] * mj[q][2]);
    }
    // limits held by j itself
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (a.arg[c * N + j] == j) acc[c] += a.lim[c * N + j];
        if (a.arg[(3 + c) * N + j] == j) acc[c] += a.lim[(3 + c) * N + j];
    }
    for (int k = a.stp[j]; k < a.stp[j + 1]; ++k) {
        const int i = __ldg(a.sti + k);
        const int t = __ldg(a.tpos + k);
        const double wx = __ldg(a.stw + t), wy = __ldg(a.stw + a.stn + t), wz = __ldg(a.stw + 2 * a.stn + t);
#pragma unroll
        for (int q = 0; q < 4; ++q)
            acc[q] += wx * __ldg(a.gm + (3 * q) * N + i) + wy * __ldg(a.gm + (3 * q + 1) * N + i) +
                      wz * __ldg(a.gm + (3 * q + 2) * N + i);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (__ldg(a.arg + c * N + i) == j) acc[c] += __ldg(a.lim + c * N + i);
            if (__ldg(a.arg + (3 + c) * N + i) == j) acc[c] += __ldg(a.lim + (3 + c) * N + i);
        }
    }
    // boundary faces: the LSQ fit's boundary values as functions of the cell's fields
    for (int k = a.cfp[j]; k < a.cfp[j + 1]; ++k) {
        const int f = a.cfi[k] & kFaceMask;
        if (f < ni) continue;
        const int b = f - ni, p = a.bpatch[b];
        const double w[3] = {a.bfw[b], a.bfw[nb + b], a.bfw[2 * nb + b]};
        if (a.bct[3 * p] != SEMO_BC_FIXED_VALUE) acc[3] += w[0] * mj[3][0] + w[1] * mj[3][1] + w[2] * mj[3][2];
        const int tu = a.bct[3 * p + 1];
        double v[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = w[0] * mj[c][0] + w[1] * mj[c][1] + w[2] * mj[c][2];
        if (tu == SEMO_BC_SLIP) {   // u_b = u - (u . n) n
            const double n[3] = {a.fn[f], a.fn[nf + f], a.fn[2 * nf + f]};
            const double nv = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] += v[c] - n[c] * nv;
        } else if (tu != SEMO_BC_FIXED_VALUE && tu != SEMO_BC_NO_SLIP) {   // u_b = u
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] += v[c];
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) a.out[q * N + j] = acc[q];
}

inline int nblocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

namespace semo {

void vjp_fields(semo_ctx* c, const double* lam, double* out) {
    const int nc = c->nc, nf = c->nf, ni = c->ni, nb = c->nb;
    const size_t N = nc;
    cudaStream_t s = c->stream;
    // the stencil's transpose positions, once per mesh
    if (c->st_tpos_gen != c->mesh_gen) {
        c->st_tpos.alloc((size_t)std::max<int64_t>(c->st_nnz, 1), s);
        SEMO_CUDA(cudaMemsetAsync(c->flag.p + 13, 0, sizeof(int), s));
        k_stencil_tpos<<<nblocks(nc, 128), 128, 0, s>>>(nc, c->st_ptr, c->st_idx, c->st_tpos, c->flag.p + 13);
        SEMO_CHECK_LAUNCH();
        int* const bad = c->hpin_scan + 2;
        SEMO_CUDA(cudaMemcpyAsync(bad, c->flag.p + 13, sizeof(int), cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
        if (*bad) throw Error(SEMO_ERR_MESH, "vertex stencil is not symmetric");
        c->st_tpos_gen = c->mesh_gen;
    }
    // checkpointed recomputation: face values, gradients, limits and their
    // arg-extrema from the current cell fields
    DBuf<double> grad, mm, gdir, gm, lim;
    DBuf<int> arg;
    grad.alloc(15 * N, s);
    mm.alloc(10 * N, s);
    gdir.alloc(4 * N, s);
    gm.alloc(12 * N, s);
    lim.alloc(6 * N, s);
    arg.alloc(6 * N, s);
    assemble_face_values(c, false);
    lsq_gradients5(c, c->P, c->U, c->V, c->W, c->VF, c->bface, grad.p, mm.p);
    k_adj_argext<<<nblocks(nc, 128), 128, 0, s>>>(nc, c->st_ptr, c->st_idx, c->U, c->V, c->W, arg.p);
    SEMO_CHECK_LAUNCH();
    AdjCellArgs a{};
    a.nc = nc; a.ni = ni; a.nf = nf; a.nb = nb;
    a.cfp = c->cf_ptr; a.cfi = c->cf_idx; a.own = c->own; a.nei = c->nei; a.bpatch = c->bpatch; a.bct = c->bc_type;
    a.fn = c->fn; a.skew = c->skew; a.alf = c->alf; a.epn = c->epn; a.fk = c->fk; a.fa = c->fa; a.mpn = c->mpn;
    a.bf = c->bface; a.irho = c->irho;
    a.U = c->U; a.V = c->V; a.W = c->W; a.grad = grad.p; a.mm = mm.p; a.minv = c->minv; a.lam = lam;
    a.dt = c->phys.dt;
    a.gdir = gdir.p; a.gm = gm.p; a.lim = lim.p;
    k_adj_cell<<<nblocks(nc, 128), 128, 0, s>>>(a);
    SEMO_CHECK_LAUNCH();
    AdjGatherArgs g{};
    g.nc = nc; g.ni = ni; g.nf = nf; g.nb = nb; g.stn = c->st_nnz;
    g.stp = c->st_ptr; g.sti = c->st_idx; g.tpos = c->st_tpos; g.cfp = c->cf_ptr; g.cfi = c->cf_idx;
    g.bpatch = c->bpatch; g.bct = c->bc_type; g.arg = arg.p;
    g.stw = c->stw; g.stws = c->stws; g.bfw = c->bfw; g.fn = c->fn; g.gdir = gdir.p; g.gm = gm.p; g.lim = lim.p;
    g.out = out;
    k_adj_gather<<<nblocks(nc, 128), 128, 0, s>>>(g);
    SEMO_CHECK_LAUNCH();
}

}  // namespace semo
