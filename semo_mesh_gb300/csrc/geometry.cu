// Mesh geometry on the GPU, once per mesh.
//
// Restates SEMO_Mesh_Geometric (src/mesh/geometric.cpp): the five-pass
// triangle-fan polygon normal/area/centroid (:16-~370), cell volumes and
// centroids (:814-880), distCells (:1206-1227), face weights and
// non-orthogonality vectors (:1297-1500), and the first-order block of
// SEMO_Utility_Math::initLeastSquare for the vertex stencil
// (src/math/gradient.cpp:246-453).  This translation unit is compiled with
// --fmad=false and keeps SEMO's operation order so every value is
// bit-identical to the reference: wC is rounded to 7 decimals through a
// float, so a one-ulp difference upstream could move it by 1e-7.
//
// Layout: face quantities are structure-of-arrays planes of length nf
// (3-vectors as 3 planes); cell quantities are planes of length nc in RCM
// order.  Cell accumulations are gathers over the cell->face list in
// ascending face order, which is the order SEMO's face loop adds them in.
#include <cuda_runtime.h>

#include "semo_internal.h"

namespace {

constexpr int kFaceMask = 0x3FFFFFFF;

// sqrt as the reference computes it: SEMO calls sqrtl on a double argument
// (geometric.cpp, calcUnitNormals_Area3dPolygon), i.e. the root rounded to
// the x87 64-bit significand and then to double.  That double rounding
// differs from IEEE sqrt only when the root lies within 2^-12 ulp of a
// midpoint between doubles; the exact residual x - y*y (representable for
// y = RN(sqrt x)) tells which side and how close.
__device__ __forceinline__ double sqrt_ext_rounded(double x) {
    double y = sqrt(x);
    if (!(y > 0.0) || !isfinite(y)) return y;
    const long long yb = __double_as_longlong(y);
    if (!(yb & 1)) return y;                      // ties at 53 bits resolve to y itself
    const double t = fma(-y, y, x);               // exact residual
    const double up = __longlong_as_double(yb + 1), dn = __longlong_as_double(yb - 1);
    const double half = 0.5 * (up - y);
    const double z = t / (2.0 * y);               // sqrt(x) - y, to ~2^-53 relative
    const double edge = half - half * (1.0 / 2048.0);
    if (z > edge) return up;
    if (z < -edge) return dn;
    return y;
}

__global__ void k_face_polygon(int nf, const double* __restrict__ pts, const int* __restrict__ fptr,
                               const int* __restrict__ fpts, double* __restrict__ fn, double* __restrict__ fa,
                               double* __restrict__ fc, double* __restrict__ vsn3, double* __restrict__ cen) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int b0 = fptr[f], n = fptr[f + 1] - b0;
    double xa = 0.0, ya = 0.0, za = 0.0;
    for (int i = 0; i < n; ++i) {
        const int p = fpts[b0 + i];
        xa += pts[3 * p]; ya += pts[3 * p + 1]; za += pts[3 * p + 2];
    }
    xa /= (double)n; ya /= (double)n; za /= (double)n;
    double xt = 0, yt = 0, zt = 0, x0o = 0, y0o = 0, z0o = 0;
    double u0 = 0, u1 = 0, u2 = 0, c0 = 0, c1 = 0, c2 = 0, area = 0, vs = 0;
    for (int pass = 0; pass < 5; ++pass) {
        u0 = u1 = u2 = 0.0; c0 = c1 = c2 = 0.0; vs = 0.0;
        double X0, Y0, Z0;
        if (pass == 0) { X0 = xa; Y0 = ya; Z0 = za; }
        else { X0 = x0o + 1.0 * (xt - x0o); Y0 = y0o + 1.0 * (yt - y0o); Z0 = z0o + 1.0 * (zt - z0o); }
        x0o = X0; y0o = Y0; z0o = Z0;
        xt = yt = zt = 0.0;
        double tot = 0.0;
        for (int i = 0; i < n; ++i) {
            const int pb = fpts[b0 + i], pc = fpts[b0 + ((i == n - 1) ? 0 : i + 1)];
            const double bx = pts[3 * pb], by = pts[3 * pb + 1], bz = pts[3 * pb + 2];
            const double qx = pts[3 * pc], qy = pts[3 * pc + 1], qz = pts[3 * pc + 2];
            const double A0 = bx - X0, A1 = by - Y0, A2 = bz - Z0;
            const double B0 = qx - X0, B1 = qy - Y0, B2 = qz - Z0;
            const double Nx = 0.5 * (A1 * B2 - A2 * B1);
            const double Ny = 0.5 * (A2 * B0 - A0 * B2);
            const double Nz = 0.5 * (A0 * B1 - A1 * B0);
            u0 += Nx; u1 += Ny; u2 += Nz;
            const double ta = sqrt_ext_rounded(Nx * Nx + Ny * Ny + Nz * Nz);
            const double rx = (X0 + bx + qx) / 3.0, ry = (Y0 + by + qy) / 3.0, rz = (Z0 + bz + qz) / 3.0;
            xt += rx * ta; yt += ry * ta; zt += rz * ta;
            tot += ta;
            vs += X0 * Nx; vs += Y0 * Ny; vs += Z0 * Nz;
            c0 += 2.0 * Nx * ((X0 + bx) * (X0 + bx) + (bx + qx) * (bx + qx) + (qx + X0) * (qx + X0));
            c1 += 2.0 * Ny * ((Y0 + by) * (Y0 + by) + (by + qy) * (by + qy) + (qy + Y0) * (qy + Y0));
            c2 += 2.0 * Nz * ((Z0 + bz) * (Z0 + bz) + (bz + qz) * (bz + qz) + (qz + Z0) * (qz + Z0));
        }
        const double mag = sqrt_ext_rounded(u0 * u0 + u1 * u1 + u2 * u2);
        u0 /= mag; u1 /= mag; u2 /= mag;
        area = mag;
        xt /= tot; yt /= tot; zt /= tot;
    }
    fn[f] = u0; fn[nf + f] = u1; fn[2 * nf + f] = u2;
    fa[f] = area;
    fc[f] = xt; fc[nf + f] = yt; fc[2 * nf + f] = zt;
    vsn3[f] = vs / 3.0;
    cen[f] = c0; cen[nf + f] = c1; cen[2 * nf + f] = c2;
}

__global__ void k_cell_volume(int nc, int nf, const int* __restrict__ cfp, const int* __restrict__ cfi,
                              const double* __restrict__ vsn3, const double* __restrict__ cen,
                              double* __restrict__ vol, double* __restrict__ cc, int* __restrict__ flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double v = 0.0, x = 0.0, y = 0.0, z = 0.0;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int e = cfi[k], f = e & kFaceMask;
        if (e >> 30) { v -= vsn3[f]; x -= cen[f]; y -= cen[nf + f]; z -= cen[2 * nf + f]; }
        else { v += vsn3[f]; x += cen[f]; y += cen[nf + f]; z += cen[2 * nf + f]; }
    }
    const double s = 1.0 / (24.0 * 2.0 * v);
    vol[i] = v;
    cc[i] = x * s; cc[nc + i] = y * s; cc[2 * nc + i] = z * s;
    if (!(v >= 2.2250738585072014e-308)) atomicExch(flag + 0, 1);   // non-positive volume
}

__global__ void k_face_weights(int nf, int ni, int nc, const int* __restrict__ own, const int* __restrict__ nei,
                               const double* __restrict__ cc, const double* __restrict__ fn,
                               const double* __restrict__ fc, double* __restrict__ wc, double* __restrict__ mpn,
                               double* __restrict__ alf, double* __restrict__ epn, double* __restrict__ skew,
                               double* __restrict__ pf, double* __restrict__ nfv) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int o = own[f];
    const double n0 = fn[f], n1 = fn[nf + f], n2 = fn[2 * nf + f];
    const double ox = cc[o], oy = cc[nc + o], oz = cc[2 * nc + o];
    const double fx = fc[f], fy = fc[nf + f], fz = fc[2 * nf + f];
    const double dxFP = fx - ox, dyFP = fy - oy, dzFP = fz - oz;
    if (f < ni) {
        const int q = nei[f];
        const double nx = cc[q], ny = cc[nc + q], nz = cc[2 * nc + q];
        const double dxFN = fx - nx, dyFN = fy - ny, dzFN = fz - nz;
        const double dxPN = nx - ox, dyPN = ny - oy, dzPN = nz - oz;
        const double dPN = sqrt(dxPN * dxPN + dyPN * dyPN + dzPN * dzPN);
        pf[f] = dxFP; pf[nf + f] = dyFP; pf[2 * nf + f] = dzFP;
        nfv[f] = dxFN; nfv[nf + f] = dyFN; nfv[2 * nf + f] = dzFN;
        const double dFPo = fabs(dxFP * n0 + dyFP * n1 + dzFP * n2);
        const double dFNo = fabs(dxFN * n0 + dyFN * n1 + dzFN * n2);
        const double w = dFNo / (dFPo + dFNo);
        wc[f] = (double)(float)(round(w * 10000000) / 10000000);
        mpn[f] = dPN;
        const double e0 = dxPN / dPN, e1 = dyPN / dPN, e2 = dzPN / dPN;
        epn[f] = e0; epn[nf + f] = e1; epn[2 * nf + f] = e2;
        double a = 0.0;
        a += n0 * e0; a += n1 * e1; a += n2 * e2;
        alf[f] = 1.0 / fabs(a);
        const double Dp = -(n0 * fx + n1 * fy + n2 * fz);
        const double u = (n0 * ox + n1 * oy + n2 * oz + Dp) / (n0 * (ox - nx) + n1 * (oy - ny) + n2 * (oz - nz));
        const double s0 = ox - u * (ox - nx), s1 = oy - u * (oy - ny), s2 = oz - u * (oz - nz);
        skew[f] = fx - s0; skew[nf + f] = fy - s1; skew[2 * nf + f] = fz - s2;
    } else {
        wc[f] = (double)(float)(round(0.5 * 10000000) / 10000000);
        const double dFP = sqrt(dxFP * dxFP + dyFP * dyFP + dzFP * dzFP);
        pf[f] = dxFP; pf[nf + f] = dyFP; pf[2 * nf + f] = dzFP;
        nfv[f] = dxFP; nfv[nf + f] = dyFP; nfv[2 * nf + f] = dzFP;
        const double dFPo = fabs(dxFP * n0 + dyFP * n1 + dzFP * n2);
        mpn[f] = 2.0 * dFPo;
        const double e0 = dxFP / dFP, e1 = dyFP / dFP, e2 = dzFP / dFP;
        epn[f] = e0; epn[nf + f] = e1; epn[2 * nf + f] = e2;
        double a = 0.0;
        a += n0 * e0; a += n1 * e1; a += n2 * e2;
        alf[f] = 1.0 / fabs(a);
        skew[f] = 0.0; skew[nf + f] = 0.0; skew[2 * nf + f] = 0.0;
    }
}

// LSQ normal matrix over the vertex stencil then the cell's boundary faces,
// its cofactor inverse, the per-entry weight vectors w_k * d_k reused by
// every gradient evaluation (w_k = 1/|d_k|^2), and their per-cell sum over the
// stencil and the boundary faces (3 planes of nc), with which a gradient sums
// w_k phi_k and subtracts phi_i sum_k w_k once instead of forming every
// difference phi_k - phi_i.
__global__ void k_lsq_setup(int nc, int nf, int ni, const int* __restrict__ stp, const int* __restrict__ sti,
                            const int* __restrict__ cfp, const int* __restrict__ cfi, const double* __restrict__ cc,
                            const double* __restrict__ fc, int64_t stn, double* __restrict__ stw,
                            double* __restrict__ bfw, double* __restrict__ minv, double* __restrict__ stws,
                            int* __restrict__ flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double xi = cc[i], yi = cc[nc + i], zi = cc[2 * nc + i];
    double v0 = 0, v1 = 0, v2 = 0, v9 = 0, v10 = 0, v17 = 0;
    double sx = 0, sy = 0, sz = 0;
    for (int k = stp[i]; k < stp[i + 1]; ++k) {
        const int j = sti[k];
        const double dx = cc[j] - xi, dy = cc[nc + j] - yi, dz = cc[2 * nc + j] - zi;
        const double wk = 1.0 / (dx * dx + dy * dy + dz * dz);
        const double wx = wk * dx, wy = wk * dy, wz = wk * dz;
        v0 += wx * dx; v1 += wx * dy; v2 += wx * dz;
        v9 += wy * dy; v10 += wy * dz; v17 += wz * dz;
        stw[k] = wx; stw[stn + k] = wy; stw[2 * stn + k] = wz;
        sx += wx; sy += wy; sz += wz;
    }
    const int nb = nf - ni;
    for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
        const int f = cfi[k] & kFaceMask;
        if (f < ni) continue;
        const double dx = fc[f] - xi, dy = fc[nf + f] - yi, dz = fc[2 * nf + f] - zi;
        const double wk = 1.0 / (dx * dx + dy * dy + dz * dz);
        const double wx = wk * dx, wy = wk * dy, wz = wk * dz;
        v0 += wx * dx; v1 += wx * dy; v2 += wx * dz;
        v9 += wy * dy; v10 += wy * dz; v17 += wz * dz;
        const int b = f - ni;
        bfw[b] = wx; bfw[nb + b] = wy; bfw[2 * nb + b] = wz;
        sx += wx; sy += wy; sz += wz;
    }
    stws[i] = sx; stws[nc + i] = sy; stws[2 * nc + i] = sz;
    const double det = v0 * v9 * v17 + v1 * v10 * v2 + v2 * v1 * v10 - v0 * v10 * v10 - v2 * v9 * v2 - v1 * v1 * v17;
    if (det == 0.0) atomicExch(flag + 1, 1);
    minv[i] = (v9 * v17 - v10 * v10) / det;
    minv[nc + i] = (v2 * v10 - v1 * v17) / det;
    minv[2 * nc + i] = (v1 * v10 - v2 * v9) / det;
    minv[3 * nc + i] = (v0 * v17 - v2 * v2) / det;
    minv[4 * nc + i] = (v2 * v1 - v0 * v10) / det;
    minv[5 * nc + i] = (v0 * v9 - v1 * v1) / det;
}

// Per-internal-face constants of the pressure face kernel:
// kA = alpha*area/magPN (coefficient factor), kP = alpha/magPN (pressure jump).
__global__ void k_face_consts(int ni, int nf, const double* __restrict__ fa, const double* __restrict__ mpn,
                              const double* __restrict__ alf, const double* __restrict__ wc, double* __restrict__ fk) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= ni) return;
    fk[f] = alf[f] * fa[f] / mpn[f];
    fk[ni + f] = alf[f] / mpn[f];
    fk[2 * ni + f] = fa[f];
    fk[3 * ni + f] = wc[f];
}

inline int blocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

namespace semo {

void geometry_build(semo_ctx* c, const double* d_points, const int* d_fptr, const int* d_fpts,
                    const std::vector<int>&) {
    const int nf = c->nf, nc = c->nc, ni = c->ni, nb = c->nb;
    cudaStream_t s = c->stream;
    c->fn.alloc(3 * (size_t)nf, s); c->fa.alloc(nf, s); c->fc.alloc(3 * (size_t)nf, s);
    c->wc.alloc(nf, s); c->mpn.alloc(nf, s); c->alf.alloc(nf, s); c->epn.alloc(3 * (size_t)nf, s);
    c->skew.alloc(3 * (size_t)nf, s); c->pf.alloc(3 * (size_t)nf, s); c->nfv.alloc(3 * (size_t)nf, s);
    c->vol.alloc(nc, s); c->cc.alloc(3 * (size_t)nc, s); c->minv.alloc(6 * (size_t)nc, s);
    c->stw.alloc(3 * (size_t)std::max<int64_t>(c->st_nnz, 1), s);
    c->bfw.alloc(3 * (size_t)std::max(nb, 1), s);
    c->stws.alloc(3 * (size_t)nc, s);
    c->fk.alloc(4 * (size_t)std::max(ni, 1), s);
    DBuf<double> vsn3, cen;
    vsn3.alloc(nf, s);
    cen.alloc(3 * (size_t)nf, s);
    c->flag.zero();
    const int T = 128;
    k_face_polygon<<<blocks(nf, T), T, 0, s>>>(nf, d_points, d_fptr, d_fpts, c->fn, c->fa, c->fc, vsn3, cen);
    SEMO_CHECK_LAUNCH();
    k_cell_volume<<<blocks(nc, T), T, 0, s>>>(nc, nf, c->cf_ptr, c->cf_idx, vsn3, cen, c->vol, c->cc, c->flag);
    SEMO_CHECK_LAUNCH();
    k_face_weights<<<blocks(nf, T), T, 0, s>>>(nf, ni, nc, c->own, c->nei, c->cc, c->fn, c->fc, c->wc, c->mpn,
                                                c->alf, c->epn, c->skew, c->pf, c->nfv);
    SEMO_CHECK_LAUNCH();
    k_lsq_setup<<<blocks(nc, T), T, 0, s>>>(nc, nf, ni, c->st_ptr, c->st_idx, c->cf_ptr, c->cf_idx, c->cc, c->fc,
                                             c->st_nnz, c->stw, c->bfw, c->minv, c->stws, c->flag);
    SEMO_CHECK_LAUNCH();
    if (ni > 0) {
        k_face_consts<<<blocks(ni, T), T, 0, s>>>(ni, nf, c->fa, c->mpn, c->alf, c->wc, c->fk);
        SEMO_CHECK_LAUNCH();
    }
    int hflag[2] = {0, 0};
    SEMO_CUDA(cudaMemcpyAsync(hflag, c->flag.p, sizeof(hflag), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    if (hflag[0]) throw Error(SEMO_ERR_MESH, "non-positive cell volume (check face orientation)");
    if (hflag[1]) throw Error(SEMO_ERR_MESH, "singular least-squares normal matrix (detA == 0)");
}

int sm_count(int device) {
    static int cached[64] = {0};
    if (device >= 0 && device < 64 && cached[device]) return cached[device];
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    if (device >= 0 && device < 64) cached[device] = v;
    return v;
}

}  // namespace semo
