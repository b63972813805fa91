/*
 * semo_oracle.c -- CPU restatement of SEMO's pressure-correction pass.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU path is compared
 * against (tests/, __graft_entry__.smoke) and the CPU baseline bench.py
 * times.  Nothing in the shipped library links or calls it.
 *
 * Each stage restates the reference function cited beside it, with the same
 * floating-point operation order, so that on the same inputs the results
 * agree with the reference to the last bit (x86, no FMA contraction; it is
 * built with -ffp-contract=off so it also stays FMA-free on other hosts).
 * Parity of this restatement is pinned against the reference's own code,
 * compiled from its sources into oracle/_ref (see tests/golden/).
 *
 * The linear solve is not AMGCL's IDR(s)/ILU0: it restates the GPU solver's
 * algorithm (smoothed aggregation with MIS(2) aggregation, Chebyshev
 * smoothing, dense Cholesky on the coarsest level, preconditioned CG), so the
 * GPU hierarchy can be compared entry by entry.  Solutions are compared with
 * the reference's AMGCL solution through the solution vector.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_ARR 192

typedef struct {
    char name[32];
    int type;            /* 0 = double, 1 = int */
    long long n;
    void* p;
} orc_arr;

typedef struct {
    /* mesh */
    int np, nf, ni, nc, npatch;
    double* pts; int *fptr, *fpts, *own, *nei, *pstart, *psize;
    /* bc per patch: type p/u/vf and values p,u,v,w,vf */
    int* bct; double* bcv;
    /* parameters */
    double dt, rho0, rho1, mu0, mu1, urf_p, urf_u, urf_mom, urf_vof, g[3], sigma;
    int use_gravity;
    double minP, maxP, minU, maxU, minV, maxV, minW, maxW;
    /* registry of named arrays (owned) */
    int narr;
    orc_arr arr[ORC_MAX_ARR];
} orc_ctx;

static double* dget(orc_ctx* c, const char* name);
static int* iget(orc_ctx* c, const char* name);

static void* reg(orc_ctx* c, const char* name, int type, long long n) {
    for (int i = 0; i < c->narr; ++i)
        if (!strcmp(c->arr[i].name, name)) {
            free(c->arr[i].p);
            c->arr[i].p = calloc(n > 0 ? (size_t)n : 1, type ? sizeof(int) : sizeof(double));
            c->arr[i].n = n; c->arr[i].type = type;
            return c->arr[i].p;
        }
    if (c->narr >= ORC_MAX_ARR) { fprintf(stderr, "oracle: registry full\n"); abort(); }
    orc_arr* a = &c->arr[c->narr++];
    snprintf(a->name, sizeof a->name, "%s", name);
    a->type = type; a->n = n;
    a->p = calloc(n > 0 ? (size_t)n : 1, type ? sizeof(int) : sizeof(double));
    return a->p;
}
static double* dreg(orc_ctx* c, const char* n, long long k) { return (double*)reg(c, n, 0, k); }
static int* ireg(orc_ctx* c, const char* n, long long k) { return (int*)reg(c, n, 1, k); }
static orc_arr* find(orc_ctx* c, const char* name) {
    for (int i = 0; i < c->narr; ++i) if (!strcmp(c->arr[i].name, name)) return &c->arr[i];
    return NULL;
}
static double* dget(orc_ctx* c, const char* name) { orc_arr* a = find(c, name); return a ? (double*)a->p : NULL; }
static int* iget(orc_ctx* c, const char* name) { orc_arr* a = find(c, name); return a ? (int*)a->p : NULL; }

long long orc_len(orc_ctx* c, const char* name) { orc_arr* a = find(c, name); return a ? a->n : -1; }
int orc_type(orc_ctx* c, const char* name) { orc_arr* a = find(c, name); return a ? a->type : -1; }
int orc_get(orc_ctx* c, const char* name, void* dst) {
    orc_arr* a = find(c, name);
    if (!a) return -1;
    memcpy(dst, a->p, (size_t)a->n * (a->type ? sizeof(int) : sizeof(double)));
    return 0;
}
int orc_set(orc_ctx* c, const char* name, int type, long long n, const void* src) {
    void* p = reg(c, name, type, n);
    memcpy(p, src, (size_t)n * (type ? sizeof(int) : sizeof(double)));
    return 0;
}

/* ------------------------------------------------------------------------ */
/* geometry: src/mesh/geometric.cpp:16-~370 (calcUnitNormals_Area3dPolygon), */
/* :792-880 (volumes/centroids), :1206-1227 (distCells), :1297-1500 (weights) */
/* ------------------------------------------------------------------------ */
/* The reference takes sqrtl of a double (x87: root rounded to a 64-bit
   significand, then to double).  Restated portably so the oracle gives the
   same bits on hosts whose long double is not x87: IEEE sqrt, corrected when
   the root lies within 2^-12 ulp of a midpoint (exact residual via fma). */
static double sqrt_ext_rounded(double x) {
    double y = sqrt(x);
    if (!(y > 0.0) || !isfinite(y)) return y;
    uint64_t yb; memcpy(&yb, &y, 8);
    if (!(yb & 1)) return y;
    double t = fma(-y, y, x);
    uint64_t ub = yb + 1, db = yb - 1;
    double up, dn; memcpy(&up, &ub, 8); memcpy(&dn, &db, 8);
    double half = 0.5 * (up - y);
    double z = t / (2.0 * y);
    double edge = half - half * (1.0 / 2048.0);
    if (z > edge) return up;
    if (z < -edge) return dn;
    return y;
}

static void face_polygon(const double* pts, const int* idx, int n, double* nrm, double* area,
                         double* cx, double* cy, double* cz, double* vsn, double* cen) {
    double xa = 0.0, ya = 0.0, za = 0.0;
    for (int i = 0; i < n; ++i) { xa += pts[3 * idx[i]]; ya += pts[3 * idx[i] + 1]; za += pts[3 * idx[i] + 2]; }
    xa /= (double)n; ya /= (double)n; za /= (double)n;
    double xt = 0, yt = 0, zt = 0, x0o = 0, y0o = 0, z0o = 0;
    double un[3] = {0, 0, 0}, cc[3] = {0, 0, 0}, ar = 0, vs = 0;
    for (int pass = 0; pass < 5; ++pass) {
        un[0] = un[1] = un[2] = 0.0; cc[0] = cc[1] = cc[2] = 0.0; vs = 0.0;
        double X0, Y0, Z0;
        if (pass == 0) { X0 = xa; Y0 = ya; Z0 = za; }
        else { X0 = x0o + 1.0 * (xt - x0o); Y0 = y0o + 1.0 * (yt - y0o); Z0 = z0o + 1.0 * (zt - z0o); }
        x0o = X0; y0o = Y0; z0o = Z0;
        xt = yt = zt = 0.0;
        double tot = 0.0;
        for (int i = 0; i < n; ++i) {
            int b = idx[i], c = idx[(i == n - 1) ? 0 : i + 1];
            double bx = pts[3 * b], by = pts[3 * b + 1], bz = pts[3 * b + 2];
            double qx = pts[3 * c], qy = pts[3 * c + 1], qz = pts[3 * c + 2];
            double A0 = bx - X0, A1 = by - Y0, A2 = bz - Z0;
            double B0 = qx - X0, B1 = qy - Y0, B2 = qz - Z0;
            double Nx = 0.5 * (A1 * B2 - A2 * B1);
            double Ny = 0.5 * (A2 * B0 - A0 * B2);
            double Nz = 0.5 * (A0 * B1 - A1 * B0);
            un[0] += Nx; un[1] += Ny; un[2] += Nz;
            double ta = sqrt_ext_rounded(Nx * Nx + Ny * Ny + Nz * Nz);
            double rx = (X0 + bx + qx) / 3.0, ry = (Y0 + by + qy) / 3.0, rz = (Z0 + bz + qz) / 3.0;
            xt += rx * ta; yt += ry * ta; zt += rz * ta;
            tot += ta;
            vs += X0 * Nx; vs += Y0 * Ny; vs += Z0 * Nz;
            cc[0] += 2.0 * Nx * ((X0 + bx) * (X0 + bx) + (bx + qx) * (bx + qx) + (qx + X0) * (qx + X0));
            cc[1] += 2.0 * Ny * ((Y0 + by) * (Y0 + by) + (by + qy) * (by + qy) + (qy + Y0) * (qy + Y0));
            cc[2] += 2.0 * Nz * ((Z0 + bz) * (Z0 + bz) + (bz + qz) * (bz + qz) + (qz + Z0) * (qz + Z0));
        }
        double mag = sqrt_ext_rounded(un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
        un[0] /= mag; un[1] /= mag; un[2] /= mag;
        ar = mag;
        xt /= tot; yt /= tot; zt /= tot;
    }
    nrm[0] = un[0]; nrm[1] = un[1]; nrm[2] = un[2];
    *area = ar; *cx = xt; *cy = yt; *cz = zt; *vsn = vs;
    cen[0] = cc[0]; cen[1] = cc[1]; cen[2] = cc[2];
}

static void build_geometry(orc_ctx* c) {
    int nf = c->nf, nc = c->nc, ni = c->ni;
    double* fa = dreg(c, "face_area", nf); double* fn = dreg(c, "face_n", 3LL * nf);
    double* fc = dreg(c, "face_c", 3LL * nf); double* wc = dreg(c, "face_wC", nf);
    double* mpn = dreg(c, "face_magPN", nf); double* al = dreg(c, "face_alphaF", nf);
    double* epn = dreg(c, "face_ePN", 3LL * nf); double* sk = dreg(c, "face_skew", 3LL * nf);
    double* pf = dreg(c, "face_vecPF", 3LL * nf); double* nfv = dreg(c, "face_vecNF", 3LL * nf);
    double* dist = dreg(c, "face_dist", 3LL * nf);
    double* vol = dreg(c, "cell_vol", nc); double* cc = dreg(c, "cell_c", 3LL * nc);
    for (int f = 0; f < nf; ++f) {
        double vsn, cen[3];
        face_polygon(c->pts, c->fpts + c->fptr[f], c->fptr[f + 1] - c->fptr[f], fn + 3 * f, fa + f,
                     fc + 3 * f, fc + 3 * f + 1, fc + 3 * f + 2, &vsn, cen);
        int o = c->own[f];
        vol[o] += vsn / 3.0; cc[3 * o] += cen[0]; cc[3 * o + 1] += cen[1]; cc[3 * o + 2] += cen[2];
        if (f < ni) {
            int q = c->nei[f];
            vol[q] -= vsn / 3.0; cc[3 * q] -= cen[0]; cc[3 * q + 1] -= cen[1]; cc[3 * q + 2] -= cen[2];
        }
    }
    for (int i = 0; i < nc; ++i) {
        double s = 1.0 / (24.0 * 2.0 * vol[i]);
        cc[3 * i] *= s; cc[3 * i + 1] *= s; cc[3 * i + 2] *= s;
    }
    for (int f = 0; f < nf; ++f) {
        int o = c->own[f];
        const double* n = fn + 3 * f;
        double ox = cc[3 * o], oy = cc[3 * o + 1], oz = cc[3 * o + 2];
        double fx = fc[3 * f], fy = fc[3 * f + 1], fz = fc[3 * f + 2];
        if (f < ni) {
            int q = c->nei[f];
            double nx = cc[3 * q], ny = cc[3 * q + 1], nz = cc[3 * q + 2];
            dist[3 * f] = nx - ox; dist[3 * f + 1] = ny - oy; dist[3 * f + 2] = nz - oz;
            double dxFP = fx - ox, dyFP = fy - oy, dzFP = fz - oz;
            double dxFN = fx - nx, dyFN = fy - ny, dzFN = fz - nz;
            double dxPN = nx - ox, dyPN = ny - oy, dzPN = nz - oz;
            double dPN = sqrt(dxPN * dxPN + dyPN * dyPN + dzPN * dzPN);
            pf[3 * f] = dxFP; pf[3 * f + 1] = dyFP; pf[3 * f + 2] = dzFP;
            nfv[3 * f] = dxFN; nfv[3 * f + 1] = dyFN; nfv[3 * f + 2] = dzFN;
            double dFPo = fabs(dxFP * n[0] + dyFP * n[1] + dzFP * n[2]);
            double dFNo = fabs(dxFN * n[0] + dyFN * n[1] + dzFN * n[2]);
            double w = dFNo / (dFPo + dFNo);
            wc[f] = (double)(float)(round(w * 10000000) / 10000000);
            mpn[f] = dPN;
            epn[3 * f] = dxPN / dPN; epn[3 * f + 1] = dyPN / dPN; epn[3 * f + 2] = dzPN / dPN;
            double a = 0.0;
            a += n[0] * epn[3 * f]; a += n[1] * epn[3 * f + 1]; a += n[2] * epn[3 * f + 2];
            al[f] = 1.0 / fabs(a);
            double Dp = -(n[0] * fx + n[1] * fy + n[2] * fz);
            double u = (n[0] * ox + n[1] * oy + n[2] * oz + Dp) /
                       (n[0] * (ox - nx) + n[1] * (oy - ny) + n[2] * (oz - nz));
            double s0 = ox - u * (ox - nx), s1 = oy - u * (oy - ny), s2 = oz - u * (oz - nz);
            sk[3 * f] = fx - s0; sk[3 * f + 1] = fy - s1; sk[3 * f + 2] = fz - s2;
        } else {
            dist[3 * f] = fx - ox; dist[3 * f + 1] = fy - oy; dist[3 * f + 2] = fz - oz;
            wc[f] = (double)(float)(round(0.5 * 10000000) / 10000000);
            double dxFP = fx - ox, dyFP = fy - oy, dzFP = fz - oz;
            double dFP = sqrt(dxFP * dxFP + dyFP * dyFP + dzFP * dzFP);
            pf[3 * f] = dxFP; pf[3 * f + 1] = dyFP; pf[3 * f + 2] = dzFP;
            nfv[3 * f] = dxFP; nfv[3 * f + 1] = dyFP; nfv[3 * f + 2] = dzFP;
            double dFPo = fabs(dxFP * n[0] + dyFP * n[1] + dzFP * n[2]);
            mpn[f] = 2.0 * dFPo;
            epn[3 * f] = dxFP / dFP; epn[3 * f + 1] = dyFP / dFP; epn[3 * f + 2] = dzFP / dFP;
            double a = 0.0;
            a += n[0] * epn[3 * f]; a += n[1] * epn[3 * f + 1]; a += n[2] * epn[3 * f + 2];
            al[f] = 1.0 / fabs(a);
            sk[3 * f] = sk[3 * f + 1] = sk[3 * f + 2] = 0.0;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* topology: src/mesh/build.cpp:587-608 (connectCelltoFaces), :613-690      */
/* (connectCelltoPoints), src/mesh/geometric.cpp:1781-1845 (setStencil),     */
/* src/mesh/build.cpp:1319-1424 (cellsGlobal CSR + face->slot maps)          */
/* ------------------------------------------------------------------------ */
typedef struct { int* p; int n, cap; } ivec;
static void ivec_push(ivec* v, int x) {
    if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 8; v->p = (int*)realloc(v->p, sizeof(int) * v->cap); }
    v->p[v->n++] = x;
}
static int ivec_has(const ivec* v, int x) { for (int i = 0; i < v->n; ++i) if (v->p[i] == x) return 1; return 0; }

static void flatten(orc_ctx* c, const char* pn, const char* in, ivec* v, int n) {
    int* ptr = ireg(c, pn, n + 1);
    for (int i = 0; i < n; ++i) ptr[i + 1] = ptr[i] + v[i].n;
    int* idx = ireg(c, in, ptr[n]);
    for (int i = 0; i < n; ++i) { memcpy(idx + ptr[i], v[i].p, sizeof(int) * v[i].n); free(v[i].p); }
    free(v);
}

static void build_topology(orc_ctx* c) {
    int nf = c->nf, nc = c->nc, ni = c->ni;
    ivec* cf = (ivec*)calloc(nc, sizeof(ivec));
    for (int f = 0; f < nf; ++f) { ivec_push(&cf[c->own[f]], f); if (f < ni) ivec_push(&cf[c->nei[f]], f); }
    flatten(c, "cf_ptr", "cf_idx", cf, nc);
    ivec* cp = (ivec*)calloc(nc, sizeof(ivec));
    for (int f = 0; f < nf; ++f)
        for (int k = c->fptr[f]; k < c->fptr[f + 1]; ++k) {
            int p = c->fpts[k];
            if (!ivec_has(&cp[c->own[f]], p)) ivec_push(&cp[c->own[f]], p);
            if (f < ni && !ivec_has(&cp[c->nei[f]], p)) ivec_push(&cp[c->nei[f]], p);
        }
    flatten(c, "cp_ptr", "cp_idx", cp, nc);
    int* cpp = iget(c, "cp_ptr"); int* cpi = iget(c, "cp_idx");
    ivec* pc = (ivec*)calloc(c->np, sizeof(ivec));
    for (int i = 0; i < nc; ++i) for (int k = cpp[i]; k < cpp[i + 1]; ++k) ivec_push(&pc[cpi[k]], i);
    ivec* st = (ivec*)calloc(nc, sizeof(ivec));
    for (int i = 0; i < nc; ++i)
        for (int k = cpp[i]; k < cpp[i + 1]; ++k) {
            ivec* pl = &pc[cpi[k]];
            for (int q = 0; q < pl->n; ++q) {
                int j = pl->p[q];
                if (j == i) continue;
                if (!ivec_has(&st[i], j)) ivec_push(&st[i], j);
            }
        }
    for (int p = 0; p < c->np; ++p) free(pc[p].p);
    free(pc);
    flatten(c, "stencil_ptr", "stencil_idx", st, nc);
    /* CSR pattern: COO = N diagonals, then per internal face (LR, RL) */
    int nnz = nc + 2 * ni;
    int* ptr = ireg(c, "CRS_ptr", nc + 1);
    int* col = ireg(c, "CRS_col", nnz);
    int* dig = ireg(c, "CRS_dig", nc);
    int* lr = ireg(c, "CRS_LR", nf); int* rl = ireg(c, "CRS_RL", nf);
    for (int f = 0; f < nf; ++f) { lr[f] = -1; rl[f] = -1; }
    int* cnt = (int*)calloc(nc + 1, sizeof(int));
    for (int i = 0; i < nc; ++i) cnt[i]++;
    for (int f = 0; f < ni; ++f) { cnt[c->own[f]]++; cnt[c->nei[f]]++; }
    for (int i = 0, s = 0; i < nc; ++i) { ptr[i] = s; s += cnt[i]; }
    ptr[nc] = nnz;
    int* fill = (int*)malloc(sizeof(int) * nc);
    for (int i = 0; i < nc; ++i) fill[i] = ptr[i];
    for (int i = 0; i < nc; ++i) { int d = fill[i]++; col[d] = i; dig[i] = d; }
    for (int f = 0; f < ni; ++f) {
        int o = c->own[f], q = c->nei[f];
        int d = fill[o]++; col[d] = q; lr[f] = d;
        d = fill[q]++; col[d] = o; rl[f] = d;
    }
    free(cnt); free(fill);
}

/* ------------------------------------------------------------------------ */
/* LSQ setup: src/math/gradient.cpp:246-453 (initLeastSquare, cellVertex,    */
/* first-order block of the normal matrix, cofactor inverse)                 */
/* ------------------------------------------------------------------------ */
static void build_lsq(orc_ctx* c) {
    int nc = c->nc;
    double* cc = dget(c, "cell_c"); double* fc = dget(c, "face_c");
    int* sp = iget(c, "stencil_ptr"); int* si = iget(c, "stencil_idx");
    double* minv = dreg(c, "lsq_minv", 6LL * nc);
    double* vs = (double*)calloc(6 * (size_t)nc, sizeof(double)); /* v0 v1 v2 v9 v10 v17 */
    for (int i = 0; i < nc; ++i)
        for (int k = sp[i]; k < sp[i + 1]; ++k) {
            int j = si[k];
            double dx = cc[3 * j] - cc[3 * i], dy = cc[3 * j + 1] - cc[3 * i + 1], dz = cc[3 * j + 2] - cc[3 * i + 2];
            double wk = 1.0 / (dx * dx + dy * dy + dz * dz);
            double* v = vs + 6 * i;
            v[0] += wk * dx * dx; v[1] += wk * dx * dy; v[2] += wk * dx * dz;
            v[3] += wk * dy * dy; v[4] += wk * dy * dz; v[5] += wk * dz * dz;
        }
    for (int f = c->ni; f < c->nf; ++f) {
        int i = c->own[f];
        double dx = fc[3 * f] - cc[3 * i], dy = fc[3 * f + 1] - cc[3 * i + 1], dz = fc[3 * f + 2] - cc[3 * i + 2];
        double wk = 1.0 / (dx * dx + dy * dy + dz * dz);
        double* v = vs + 6 * i;
        v[0] += wk * dx * dx; v[1] += wk * dx * dy; v[2] += wk * dx * dz;
        v[3] += wk * dy * dy; v[4] += wk * dy * dz; v[5] += wk * dz * dz;
    }
    for (int i = 0; i < nc; ++i) {
        double a0 = vs[6 * i], a1 = vs[6 * i + 1], a2 = vs[6 * i + 2], a9 = vs[6 * i + 3], a10 = vs[6 * i + 4], a17 = vs[6 * i + 5];
        double det = a0 * a9 * a17 + a1 * a10 * a2 + a2 * a1 * a10 - a0 * a10 * a10 - a2 * a9 * a2 - a1 * a1 * a17;
        double* m = minv + 6 * i;
        m[0] = (a9 * a17 - a10 * a10) / det;
        m[1] = (a2 * a10 - a1 * a17) / det;
        m[2] = (a1 * a10 - a2 * a9) / det;
        m[3] = (a0 * a17 - a2 * a2) / det;
        m[4] = (a2 * a1 - a0 * a10) / det;
        m[5] = (a0 * a9 - a1 * a1) / det;
    }
    free(vs);
}

/* ------------------------------------------------------------------------ */
/* RCM: src/math/RCM.cpp:34-218 (lib_RCM) over SPARSEPAK genrcm / rcm /      */
/* root_find / level_set / degree (George & Liu), 1-based adjacency built    */
/* from each cell's internal faces in cell.faces order                       */
/* ------------------------------------------------------------------------ */
static void rcm_degree(int root, int* xadj, const int* adj, const int* mask, int* deg, int* ccsize, int* ls) {
    ls[0] = root; xadj[root - 1] = -xadj[root - 1];
    int lvlend = 0; *ccsize = 1;
    for (;;) {
        int lbegin = lvlend + 1; lvlend = *ccsize;
        for (int i = lbegin; i <= lvlend; ++i) {
            int node = ls[i - 1];
            int jstrt = -xadj[node - 1], jstop = abs(xadj[node]) - 1, ideg = 0;
            for (int j = jstrt; j <= jstop; ++j) {
                int nbr = adj[j - 1];
                if (mask[nbr - 1] != 0) {
                    ideg++;
                    if (xadj[nbr - 1] >= 0) { xadj[nbr - 1] = -xadj[nbr - 1]; (*ccsize)++; ls[*ccsize - 1] = nbr; }
                }
            }
            deg[node - 1] = ideg;
        }
        if (*ccsize - lvlend == 0) break;
    }
    for (int i = 0; i < *ccsize; ++i) { int node = ls[i] - 1; xadj[node] = -xadj[node]; }
}
static void rcm_level_set(int root, const int* xadj, const int* adj, int* mask, int* nlvl, int* xls, int* ls) {
    mask[root - 1] = 0; ls[0] = root; *nlvl = 0;
    int lvlend = 0, ccsize = 1;
    for (;;) {
        int lbegin = lvlend + 1; lvlend = ccsize; (*nlvl)++;
        xls[*nlvl - 1] = lbegin;
        for (int i = lbegin; i <= lvlend; ++i) {
            int node = ls[i - 1];
            for (int j = xadj[node - 1]; j <= xadj[node] - 1; ++j) {
                int nbr = adj[j - 1];
                if (mask[nbr - 1] != 0) { ccsize++; ls[ccsize - 1] = nbr; mask[nbr - 1] = 0; }
            }
        }
        if (ccsize - lvlend <= 0) break;
    }
    xls[*nlvl] = lvlend + 1;
    for (int i = 0; i < ccsize; ++i) mask[ls[i] - 1] = 1;
}
static void rcm_root_find(int* root, const int* xadj, const int* adj, int* mask, int* nlvl, int* xls, int* ls) {
    rcm_level_set(*root, xadj, adj, mask, nlvl, xls, ls);
    int ccsize = xls[*nlvl] - 1;
    if (*nlvl == 1 || *nlvl == ccsize) return;
    for (;;) {
        int mindeg = ccsize, jstrt = xls[*nlvl - 1];
        *root = ls[jstrt - 1];
        if (jstrt < ccsize)
            for (int j = jstrt; j <= ccsize; ++j) {
                int node = ls[j - 1], ndeg = 0;
                for (int k = xadj[node - 1]; k <= xadj[node] - 1; ++k) if (mask[adj[k - 1] - 1] > 0) ndeg++;
                if (ndeg < mindeg) { *root = node; mindeg = ndeg; }
            }
        int nlvl2;
        rcm_level_set(*root, xadj, adj, mask, &nlvl2, xls, ls);
        if (nlvl2 <= *nlvl) break;
        *nlvl = nlvl2;
        if (ccsize <= *nlvl) break;
    }
}
static void rcm_one(int root, int* xadj, const int* adj, int* mask, int* perm, int* ccsize, int n) {
    int* deg = (int*)malloc(sizeof(int) * n);
    rcm_degree(root, xadj, adj, mask, deg, ccsize, perm);
    mask[root - 1] = 0;
    if (*ccsize == 1) { free(deg); return; }
    int lvlend = 0, lnbr = 1;
    while (lvlend < lnbr) {
        int lbegin = lvlend + 1; lvlend = lnbr;
        for (int i = lbegin; i <= lvlend; ++i) {
            int node = perm[i - 1];
            int fnbr = lnbr + 1;
            for (int j = xadj[node - 1]; j <= xadj[node] - 1; ++j) {
                int nbr = adj[j - 1];
                if (mask[nbr - 1] != 0) { lnbr++; mask[nbr - 1] = 0; perm[lnbr - 1] = nbr; }
            }
            if (lnbr <= fnbr) continue;
            int k = fnbr;
            while (k < lnbr) {
                int l = k; k++;
                int nbr = perm[k - 1];
                while (fnbr < l) {
                    int lperm = perm[l - 1];
                    if (deg[lperm - 1] <= deg[nbr - 1]) break;
                    perm[l] = lperm; l--;
                }
                perm[l] = nbr;
            }
        }
    }
    for (int i = 0, j = *ccsize - 1; i < j; ++i, --j) { int t = perm[i]; perm[i] = perm[j]; perm[j] = t; }
    free(deg);
}
static void build_rcm(orc_ctx* c) {
    int n = c->nc;
    int* cfp = iget(c, "cf_ptr"); int* cfi = iget(c, "cf_idx");
    int* xadj = (int*)malloc(sizeof(int) * (n + 1));
    int* adj = (int*)malloc(sizeof(int) * (2 * (size_t)c->ni + 1));
    int m = 0; xadj[0] = 1;
    for (int i = 0; i < n; ++i) {
        for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
            int f = cfi[k];
            if (f >= c->ni) continue;
            adj[m++] = (c->own[f] == i ? c->nei[f] : c->own[f]) + 1;
        }
        xadj[i + 1] = m + 1;
    }
    int* perm1 = (int*)malloc(sizeof(int) * n);
    int* mask = (int*)malloc(sizeof(int) * n);
    int* xls = (int*)malloc(sizeof(int) * (n + 1));
    for (int i = 0; i < n; ++i) mask[i] = 1;
    int num = 1;
    for (int i = 0; i < n; ++i) {
        if (mask[i] == 0) continue;
        int root = i + 1, nlvl, cs;
        rcm_root_find(&root, xadj, adj, mask, &nlvl, xls, perm1 + num - 1);
        rcm_one(root, xadj, adj, mask, perm1 + num - 1, &cs, n);
        num += cs;
        if (num > n) break;
    }
    int* perm = ireg(c, "rcm_perm", n); int* iperm = ireg(c, "rcm_iperm", n);
    for (int i = 0; i < n; ++i) perm[i] = perm1[i] - 1;
    for (int i = 0; i < n; ++i) iperm[perm[i]] = i;
    free(xadj); free(adj); free(perm1); free(mask); free(xls);
}

/* ------------------------------------------------------------------------ */
/* public: mesh                                                             */
/* ------------------------------------------------------------------------ */
orc_ctx* orc_create(int np, const double* pts, int nf, int ni, int nc, const int* fptr, const int* fpts,
                    const int* own, const int* nei, int npatch, const int* pstart, const int* psize) {
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    c->np = np; c->nf = nf; c->ni = ni; c->nc = nc; c->npatch = npatch;
    c->pts = dreg(c, "points", 3LL * np); memcpy(c->pts, pts, sizeof(double) * 3 * (size_t)np);
    c->fptr = ireg(c, "face_ptr", nf + 1); memcpy(c->fptr, fptr, sizeof(int) * (nf + 1));
    c->fpts = ireg(c, "face_pts", fptr[nf]); memcpy(c->fpts, fpts, sizeof(int) * fptr[nf]);
    c->own = ireg(c, "owner", nf); memcpy(c->own, own, sizeof(int) * nf);
    c->nei = ireg(c, "neighbour", ni > 0 ? ni : 1); if (ni) memcpy(c->nei, nei, sizeof(int) * ni);
    c->pstart = ireg(c, "patch_start", npatch); memcpy(c->pstart, pstart, sizeof(int) * npatch);
    c->psize = ireg(c, "patch_size", npatch); memcpy(c->psize, psize, sizeof(int) * npatch);
    c->bct = ireg(c, "bc_type", 3LL * npatch);
    c->bcv = dreg(c, "bc_value", 5LL * npatch);
    c->minP = c->minU = c->minV = c->minW = -1e300;
    c->maxP = c->maxU = c->maxV = c->maxW = 1e300;
    build_geometry(c);
    build_topology(c);
    build_lsq(c);
    build_rcm(c);
    return c;
}

void orc_destroy(orc_ctx* c) {
    if (!c) return;
    for (int i = 0; i < c->narr; ++i) free(c->arr[i].p);
    free(c);
}

void orc_set_case(orc_ctx* c, const int* bct, const double* bcv, const double* prm) {
    memcpy(c->bct, bct, sizeof(int) * 3 * c->npatch);
    memcpy(c->bcv, bcv, sizeof(double) * 5 * c->npatch);
    c->dt = prm[0]; c->rho0 = prm[1]; c->rho1 = prm[2]; c->mu0 = prm[3]; c->mu1 = prm[4]; c->sigma = prm[5];
    c->urf_mom = prm[12]; c->urf_vof = prm[13];
    c->g[0] = prm[6]; c->g[1] = prm[7]; c->g[2] = prm[8];
    c->urf_p = prm[9]; c->urf_u = prm[10]; c->use_gravity = prm[11] != 0.0;
}

/* ------------------------------------------------------------------------ */
/* face values + EOS: src/solvers/eos.cpp:10-151 (calcIncomCellEOSVF),       */
/* :439-520 (getValuesFromEOSVF), src/solvers/reconIncom.cpp:501-1035        */
/* (reconIncomZeroOrder), :440-496 (calcOtherDataIncomFromEOS)               */
/* ------------------------------------------------------------------------ */
/* std::max / std::min semantics: max(a,b) = (a<b)?b:a, min(a,b) = (b<a)?b:a */
static double smax(double a, double b) { return (a < b) ? b : a; }
static double smin(double a, double b) { return (b < a) ? b : a; }
static double clamp01(double x) { return smax(0.0, smin(1.0, x)); }
static double eos_face(double vf, double r0, double r1) {
    double v0 = clamp01(vf), v1 = clamp01(1.0 - vf);
    double rho = 0.0; rho += v0 * r0; rho += v1 * r1;
    return rho;
}
static int patch_of(orc_ctx* c, int f) {
    for (int p = 0; p < c->npatch; ++p) if (f >= c->pstart[p] && f < c->pstart[p] + c->psize[p]) return p;
    return -1;
}
static void face_values(orc_ctx* c) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    double *P = dget(c, "P"), *U = dget(c, "U"), *V = dget(c, "V"), *W = dget(c, "W"), *VF = dget(c, "VF");
    double* rho = dreg(c, "rho", nc);
    for (int i = 0; i < nc; ++i) {
        double mf = clamp01(VF[i]);
        double v0 = clamp01(mf);
        double v1 = clamp01(1.0 - mf);
        double r = 0.0; r += v0 * c->rho0; r += v1 * c->rho1;
        rho[i] = r; VF[i] = v0;
    }
    double* fn = dget(c, "face_n");
    double *pl = dreg(c, "face_pL", nf), *pr = dreg(c, "face_pR", nf);
    double *ul = dreg(c, "face_uL", 3LL * nf), *ur = dreg(c, "face_uR", 3LL * nf);
    double *vl = dreg(c, "face_vfL", nf), *vr = dreg(c, "face_vfR", nf);
    double *rl = dreg(c, "face_rhoL", nf), *rr = dreg(c, "face_rhoR", nf);
    for (int f = 0; f < nf; ++f) {
        int o = c->own[f];
        if (f < ni) {
            int q = c->nei[f];
            pl[f] = P[o]; ul[3 * f] = U[o]; ul[3 * f + 1] = V[o]; ul[3 * f + 2] = W[o]; vl[f] = VF[o];
            pr[f] = P[q]; ur[3 * f] = U[q]; ur[3 * f + 1] = V[q]; ur[3 * f + 2] = W[q]; vr[f] = VF[q];
        } else {
            int p = patch_of(c, f);
            const int* t = c->bct + 3 * p; const double* bv = c->bcv + 5 * p;
            pl[f] = (t[0] == 1) ? bv[0] : P[o]; pr[f] = pl[f];
            const double* n = fn + 3 * f;
            if (t[1] == 1) { ul[3 * f] = bv[1]; ul[3 * f + 1] = bv[2]; ul[3 * f + 2] = bv[3]; }
            else if (t[1] == 2) { ul[3 * f] = 0.0; ul[3 * f + 1] = 0.0; ul[3 * f + 2] = 0.0; }
            else if (t[1] == 3) {
                double un = U[o] * n[0] + V[o] * n[1] + W[o] * n[2];
                ul[3 * f] = U[o] - un * n[0]; ul[3 * f + 1] = V[o] - un * n[1]; ul[3 * f + 2] = W[o] - un * n[2];
            } else { ul[3 * f] = U[o]; ul[3 * f + 1] = V[o]; ul[3 * f + 2] = W[o]; }
            /* fixedValue velocity keeps the boundary value on the right only; the
               left carries it too except for the reference's orifice special case */
            ur[3 * f] = ul[3 * f]; ur[3 * f + 1] = ul[3 * f + 1]; ur[3 * f + 2] = ul[3 * f + 2];
            vl[f] = (t[2] == 1) ? bv[4] : VF[o]; vr[f] = vl[f];
        }
        rl[f] = eos_face(vl[f], c->rho0, c->rho1);
        rr[f] = eos_face(vr[f], c->rho0, c->rho1);
    }
}

/* gravity source: src/solvers/source/gravity.cpp:7-75 (calcSourceGravity) */
static void gravity_source(orc_ctx* c) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    double* sg = dreg(c, "src_grav", 4LL * nc);
    if (!c->use_gravity) return;
    double *fn = dget(c, "face_n"), *fa = dget(c, "face_area"), *wc = dget(c, "face_wC");
    double *pf = dget(c, "face_vecPF"), *nfv = dget(c, "face_vecNF"), *vol = dget(c, "cell_vol");
    double *ul = dget(c, "face_uL"), *ur = dget(c, "face_uR"), *rl = dget(c, "face_rhoL"), *rr = dget(c, "face_rhoR");
    for (int f = 0; f < nf; ++f) {
        double wL = wc[f], wR = 1.0 - wL;
        const double* n = fn + 3 * f;
        double UnL = ul[3 * f] * n[0] + ul[3 * f + 1] * n[1] + ul[3 * f + 2] * n[2];
        double UnR = ur[3 * f] * n[0] + ur[3 * f + 1] * n[1] + ur[3 * f + 2] * n[2];
        double UnF = wL * UnL + wR * UnR;
        double RhoF = 1.0 / (wL / rl[f] + wR / rr[f]);
        double gL = 0.0, gR = 0.0;
        for (int k = 0; k < 3; ++k) { gL += c->g[k] * pf[3 * f + k]; gR += c->g[k] * nfv[3 * f + k]; }
        int o = c->own[f];
        for (int k = 0; k < 3; ++k) sg[4 * o + k] += ((RhoF * gL * n[k]) * fa[f] / vol[o]);
        sg[4 * o + 3] += ((RhoF * gL * UnF) * fa[f] / vol[o]);
        if (f < ni) {
            int q = c->nei[f];
            for (int k = 0; k < 3; ++k) sg[4 * q + k] -= ((RhoF * gR * n[k]) * fa[f] / vol[q]);
            sg[4 * q + 3] -= ((RhoF * gR * UnF) * fa[f] / vol[q]);
        }
    }
}

/* stencil min/max: src/solvers/cellVarMinMax.cpp:8-23 (setCellVarMinMax) */
static void minmax(orc_ctx* c, const double* phi, double* mx, double* mn) {
    int* sp = iget(c, "stencil_ptr"); int* si = iget(c, "stencil_idx");
    for (int i = 0; i < c->nc; ++i) {
        double a = phi[i], b = phi[i];
        for (int k = sp[i]; k < sp[i + 1]; ++k) {
            double v = phi[si[k]];
            a = (a < v) ? v : a;       /* std::max(a, v) */
            b = (v < b) ? v : b;       /* std::min(b, v) */
        }
        mx[i] = a; mn[i] = b;
    }
}

/* LSQ gradient: src/math/gradient.cpp:761-816 (cellVertex stencil), :997-1050
   (boundary faces, phi_f = face varR), :1136-1159 (M^-1 apply) */
static void lsq_grad(orc_ctx* c, const double* phi, const double* phiR, double* grad) {
    int* sp = iget(c, "stencil_ptr"); int* si = iget(c, "stencil_idx");
    double *cc = dget(c, "cell_c"), *fc = dget(c, "face_c"), *minv = dget(c, "lsq_minv");
    int nc = c->nc;
    double* gt = (double*)calloc(3 * (size_t)nc, sizeof(double));
    for (int i = 0; i < nc; ++i)
        for (int k = sp[i]; k < sp[i + 1]; ++k) {
            int j = si[k];
            double dx = cc[3 * j] - cc[3 * i], dy = cc[3 * j + 1] - cc[3 * i + 1], dz = cc[3 * j + 2] - cc[3 * i + 2];
            double wk = 1.0 / (dx * dx + dy * dy + dz * dz);
            double dv = phi[j] - phi[i];
            gt[3 * i] += wk * dx * dv; gt[3 * i + 1] += wk * dy * dv; gt[3 * i + 2] += wk * dz * dv;
        }
    for (int f = c->ni; f < c->nf; ++f) {
        int i = c->own[f];
        double dv = phiR[f] - phi[i];
        double dx = fc[3 * f] - cc[3 * i], dy = fc[3 * f + 1] - cc[3 * i + 1], dz = fc[3 * f + 2] - cc[3 * i + 2];
        double wk = 1.0 / (dx * dx + dy * dy + dz * dz);
        gt[3 * i] += wk * dx * dv; gt[3 * i + 1] += wk * dy * dv; gt[3 * i + 2] += wk * dz * dv;
    }
    for (int i = 0; i < nc; ++i) {
        const double* m = minv + 6 * i; const double* g = gt + 3 * i;
        double t0 = 0.0; t0 += m[0] * g[0]; t0 += m[1] * g[1]; t0 += m[2] * g[2];
        double t1 = 0.0; t1 += m[1] * g[0]; t1 += m[3] * g[1]; t1 += m[4] * g[2];
        double t2 = 0.0; t2 += m[2] * g[0]; t2 += m[4] * g[1]; t2 += m[5] * g[2];
        grad[3 * i] = t0; grad[3 * i + 1] = t1; grad[3 * i + 2] = t2;
    }
    free(gt);
}

/* ------------------------------------------------------------------------ */
/* pressure equation assembly: src/solvers/eqPressure.cpp:40-105 (min/max,   */
/* gradients), :217-564 (diagonal COO + internal face loop, with             */
/* src/solvers/surfaceNormalVelocity.cpp:125-221 Rhie-Chow terms), :570-673  */
/* (boundary loop).  COO order: N diagonals, then (LR, RL) per internal face */
/* ------------------------------------------------------------------------ */
/* surfaceNormalVelocity.cpp:190-221 (calcInterpolVelSurfTens), with kappa
   and src_sft from orc_surface_tension and the cell volume fractions; all
   its terms carry sigma, so with sigma = 0 (or no curvature computed) UnF is
   left as it is */
static double sft_unf(orc_ctx* c, double UnF, int o, int q, double RhoL, double RhoR, double wCL, double wCR,
                      double alpha, double dPN, const double* n, const double* e) {
    double* kap = dget(c, "kappa"); double* ss = dget(c, "src_sft");
    if (c->sigma == 0.0 || !kap || !ss) return UnF;
    double* VF = dget(c, "VF");
    double rs = 1.0 / (wCL / RhoL + wCR / RhoR);
    double tt = c->dt / rs;
    UnF += alpha * tt * c->sigma * (wCL * kap[o] + wCR * kap[q]) * (VF[q] - VF[o]) / dPN;
    for (int k = 0; k < 3; ++k) {
        UnF += tt * rs * wCL / RhoL * ss[4 * o + k] * (n[k] - alpha * e[k]);
        UnF += tt * rs * wCR / RhoR * ss[4 * q + k] * (n[k] - alpha * e[k]);
    }
    for (int k = 0; k < 3; ++k) {
        UnF -= alpha * tt * rs * wCL / RhoL * ss[4 * o + k] * n[k];
        UnF -= alpha * tt * rs * wCR / RhoR * ss[4 * q + k] * n[k];
    }
    return UnF;
}

void orc_assemble_pressure(orc_ctx* c) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    face_values(c);
    double* mxvf = dreg(c, "max_vf", nc); double* mnvf = dreg(c, "min_vf", nc);
    minmax(c, dget(c, "VF"), mxvf, mnvf);
    gravity_source(c);
    double *P = dget(c, "P"), *U = dget(c, "U"), *V = dget(c, "V"), *W = dget(c, "W"), *VF = dget(c, "VF");
    double *rho = dget(c, "rho"), *sg = dget(c, "src_grav");
    double* mm = dreg(c, "minmax_uvw", 6LL * nc);
    double *t1 = (double*)malloc(sizeof(double) * nc), *t2 = (double*)malloc(sizeof(double) * nc);
    minmax(c, U, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i] = t1[i]; mm[6 * i + 1] = t2[i]; }
    minmax(c, V, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i + 2] = t1[i]; mm[6 * i + 3] = t2[i]; }
    minmax(c, W, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i + 4] = t1[i]; mm[6 * i + 5] = t2[i]; }
    free(t1); free(t2);
    double *pr = dget(c, "face_pR"), *ur = dget(c, "face_uR"), *vr = dget(c, "face_vfR");
    double* tmp = (double*)malloc(sizeof(double) * nf);
    double* gP = dreg(c, "grad_P", 3LL * nc); lsq_grad(c, P, pr, gP);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f];
    double* gU = dreg(c, "grad_U", 3LL * nc); lsq_grad(c, U, tmp, gU);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f + 1];
    double* gV = dreg(c, "grad_V", 3LL * nc); lsq_grad(c, V, tmp, gV);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f + 2];
    double* gW = dreg(c, "grad_W", 3LL * nc); lsq_grad(c, W, tmp, gW);
    double* gVF = dreg(c, "grad_VF", 3LL * nc); lsq_grad(c, VF, vr, gVF);
    free(tmp);

    double *fn = dget(c, "face_n"), *fa = dget(c, "face_area"), *wc = dget(c, "face_wC");
    double *mpn = dget(c, "face_magPN"), *al = dget(c, "face_alphaF"), *epn = dget(c, "face_ePN");
    double *sk = dget(c, "face_skew"), *ul = dget(c, "face_uL"), *rl = dget(c, "face_rhoL");
    int nnz = nc + 2 * ni;
    int* ar = ireg(c, "A_rows", nnz); int* acl = ireg(c, "A_cols", nnz);
    double* av = dreg(c, "A_vals", nnz); double* B = dreg(c, "B", nc);
    double* unf = dreg(c, "face_UnF", nf);
    for (int i = 0; i < nc; ++i) { ar[i] = i; acl[i] = i; }
    const double dt = c->dt;
    for (int f = 0; f < ni; ++f) {
        int o = c->own[f], q = c->nei[f];
        const double* n = fn + 3 * f; const double* e = epn + 3 * f; const double* s = sk + 3 * f;
        double area = fa[f], wCL = wc[f], wCR = 1.0 - wCL;
        double RhoL = rho[o], RhoR = rho[q], PL = P[o], PR = P[q];
        double Rho_star = 1.0 / (wCR / RhoL + wCR / RhoR);    /* eqPressure.cpp:396 (wCR twice) */
        double tmp1 = dt / Rho_star;
        double dPN = mpn[f], alpha = al[f];
        double ULs = U[o], VLs = V[o], WLs = W[o], URs = U[q], VRs = V[q], WRs = W[q];
        for (int k = 0; k < 3; ++k) {
            ULs += gU[3 * o + k] * s[k]; URs += gU[3 * q + k] * s[k];
            VLs += gV[3 * o + k] * s[k]; VRs += gV[3 * q + k] * s[k];
            WLs += gW[3 * o + k] * s[k]; WRs += gW[3 * q + k] * s[k];
        }
        ULs = smax(mm[6 * o + 1], smin(mm[6 * o + 0], ULs)); URs = smax(mm[6 * q + 1], smin(mm[6 * q + 0], URs));
        VLs = smax(mm[6 * o + 3], smin(mm[6 * o + 2], VLs)); VRs = smax(mm[6 * q + 3], smin(mm[6 * q + 2], VRs));
        WLs = smax(mm[6 * o + 5], smin(mm[6 * o + 4], WLs)); WRs = smax(mm[6 * q + 5], smin(mm[6 * q + 4], WRs));
        double UnL = ULs * n[0] + VLs * n[1] + WLs * n[2];
        double UnR = URs * n[0] + VRs * n[1] + WRs * n[2];
        double UnF = wCL * UnL + wCR * UnR;
        /* surfaceNormalVelocity.cpp:125-155 (pressure) */
        double rs = 1.0 / (wCL / RhoL + wCR / RhoR);
        double tt = dt / rs;
        UnF -= alpha * tt * (PR - PL) / dPN;
        for (int k = 0; k < 3; ++k) {
            UnF -= tt * rs * wCL / RhoL * gP[3 * o + k] * (n[k] - alpha * e[k]);
            UnF -= tt * rs * wCR / RhoR * gP[3 * q + k] * (n[k] - alpha * e[k]);
        }
        for (int k = 0; k < 3; ++k) {
            UnF += tt * rs * wCL / RhoL * gP[3 * o + k] * n[k];
            UnF += tt * rs * wCR / RhoR * gP[3 * q + k] * n[k];
        }
        /* surfaceNormalVelocity.cpp:156-187 (gravity) */
        for (int k = 0; k < 3; ++k) UnF += alpha * tt * rs * c->g[k] * alpha * e[k];
        for (int k = 0; k < 3; ++k) {
            UnF += tt * rs * wCL / RhoL * sg[4 * o + k] * (n[k] - alpha * e[k]);
            UnF += tt * rs * wCR / RhoR * sg[4 * q + k] * (n[k] - alpha * e[k]);
        }
        for (int k = 0; k < 3; ++k) {
            UnF -= alpha * tt * rs * wCL / RhoL * sg[4 * o + k] * n[k];
            UnF -= alpha * tt * rs * wCR / RhoR * sg[4 * q + k] * n[k];
        }
        UnF = sft_unf(c, UnF, o, q, RhoL, RhoR, wCL, wCR, alpha, dPN, n, e);
        unf[f] = UnF;
        double coef = alpha * tmp1 / dPN * area;
        av[o] += (+coef);
        ar[nc + 2 * f] = o; acl[nc + 2 * f] = q; av[nc + 2 * f] = (-coef);
        av[q] -= (-coef);
        ar[nc + 2 * f + 1] = q; acl[nc + 2 * f + 1] = o; av[nc + 2 * f + 1] = -(+coef);
        B[o] -= (UnF * area);
        B[q] += (UnF * area);
    }
    double* pRf = dget(c, "face_pR");
    for (int f = ni; f < nf; ++f) {
        int p = patch_of(c, f), o = c->own[f];
        const double* n = fn + 3 * f; const double* e = epn + 3 * f;
        double area = fa[f];
        double UnL = ul[3 * f] * n[0] + ul[3 * f + 1] * n[1] + ul[3 * f + 2] * n[2];
        double UnR = ur[3 * f] * n[0] + ur[3 * f + 1] * n[1] + ur[3 * f + 2] * n[2];
        double UnF = 0.5 * UnL + 0.5 * UnR;
        double RhoL = rl[f];
        double tmp1 = 1.0 / RhoL * dt;
        double diff = (c->bct[3 * p] == 1) ? 1.0 : 0.0;
        double dPN = 0.5 * mpn[f], alpha = al[f];
        double PL = P[o], PR = pRf[f];
        if (c->bct[3 * p] == 1) {
            UnF -= alpha * tmp1 * (PR - PL) / dPN;
            for (int k = 0; k < 3; ++k) UnF += alpha * tmp1 * gP[3 * o + k] * e[k];
        }
        unf[f] = UnF;
        av[o] += diff * (alpha * tmp1 / dPN * area);
        B[o] -= (UnF * area);
    }
}

/* COO -> CSR, src/solvers/solveAMGCL.cpp:206-251 (in-row order = COO order) */
void orc_coo_to_csr(orc_ctx* c) {
    int n = c->nc, nnz = c->nc + 2 * c->ni;
    int *r = iget(c, "A_rows"), *cl = iget(c, "A_cols"); double* v = dget(c, "A_vals");
    int* ptr = ireg(c, "csr_ptr", n + 1); int* col = ireg(c, "csr_col", nnz); double* val = dreg(c, "csr_val", nnz);
    for (int k = 0; k < nnz; ++k) ptr[r[k]]++;
    for (int i = 0, s = 0; i < n; ++i) { int t = ptr[i]; ptr[i] = s; s += t; }
    ptr[n] = nnz;
    for (int k = 0; k < nnz; ++k) { int d = ptr[r[k]]++; col[d] = cl[k]; val[d] = v[k]; }
    for (int i = 0, last = 0; i <= n; ++i) { int t = ptr[i]; ptr[i] = last; last = t; }
}

/* Symmetric RCM permutation of the CSR system (rows in RCM order, in-row
   order kept, column indices renumbered through the inverse permutation). */
void orc_permute_csr(orc_ctx* c) {
    int n = c->nc;
    int *ptr = iget(c, "csr_ptr"), *col = iget(c, "csr_col"); double* val = dget(c, "csr_val");
    int *perm = iget(c, "rcm_perm"), *iperm = iget(c, "rcm_iperm");
    double* B = dget(c, "B");
    int nnz = ptr[n];
    int* pp = ireg(c, "rcm_csr_ptr", n + 1); int* pc = ireg(c, "rcm_csr_col", nnz);
    double* pv = dreg(c, "rcm_csr_val", nnz); double* pb = dreg(c, "rcm_B", n);
    for (int r = 0; r < n; ++r) {
        int o = perm[r];
        pp[r + 1] = pp[r] + (ptr[o + 1] - ptr[o]);
        for (int k = ptr[o], d = pp[r]; k < ptr[o + 1]; ++k, ++d) { pc[d] = iperm[col[k]]; pv[d] = val[k]; }
        pb[r] = B[o];
    }
}

/* ------------------------------------------------------------------------ */
/* Solver: smoothed-aggregation AMG (AMGCL coarsening/smoothed_aggregation   */
/* .hpp:130-215 semantics: strength eps^2 d_i d_j < a_ij^2 (eps 0.03 here)    */
/* halved per level, filtered diagonal, omega 2/3) with MIS(2) aggregation,  */
/* Chebyshev smoothing, dense Cholesky on the coarsest level, inside CG.     */
/* ------------------------------------------------------------------------ */
typedef struct { int n, nnz; int *ptr, *col; double* val; } csr_t;
typedef struct {
    csr_t A, P, R;
    double *dinv, lam_max;
    double *r, *x, *b, *t1, *t2;   /* work vectors */
    int nagg;
    int ncolors; int *cptr, *crow;  /* Gauss-Seidel: rows grouped by colour */
} level_t;
typedef struct {
    int nlev;
    level_t lev[32];
    int nc; double* chol;  /* coarsest dense Cholesky factor (lower, row-major) */
    int cheb_degree;
    int smoother;          /* 0 Chebyshev, 1 multicolour Gauss-Seidel */
    long long total_nnz;
} amg_t;

/* Smoother of the oracle's AMG (orc_set_smoother): 0 Chebyshev, 1 multicolour
   Gauss-Seidel, restating the GPU's (its colouring and its sweep order). */
static int g_smoother = 0;
void orc_set_smoother(int s) { g_smoother = s; }

static void csr_free(csr_t* a) { free(a->ptr); free(a->col); free(a->val); memset(a, 0, sizeof *a); }

static uint32_t hash_u32(uint32_t x) {
    /* integer avalanche mixer (public-domain "lowbias32" constants) */
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

/* MIS(2) aggregation over the strong graph, as the GPU does it: synchronous
   rounds of two max-propagations of the tuple (state, hash, index). */
static int aggregate(const csr_t* A, const char* strong, int* agg) {
    int n = A->n;
    /* state: 2 root, 1 undecided, 0 out; tuple key packed into 64 bits */
    uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * n);
    uint64_t* m1 = (uint64_t*)malloc(sizeof(uint64_t) * n);
    uint64_t* m2 = (uint64_t*)malloc(sizeof(uint64_t) * n);
    int* st = (int*)malloc(sizeof(int) * n);
    for (int i = 0; i < n; ++i) {
        int has = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) if (strong[k]) { has = 1; break; }
        st[i] = has ? 1 : -1;    /* -1: isolated, never aggregated */
    }
#define MKKEY(s, i) ((((uint64_t)(s)) << 62) | (((uint64_t)hash_u32((uint32_t)(i))) << 30) | (uint64_t)(i))
    for (int round = 0; round < 1000; ++round) {
        int und = 0;
        for (int i = 0; i < n; ++i) { int s = st[i] < 0 ? 0 : st[i]; key[i] = MKKEY(s, i); if (st[i] == 1) und++; }
        if (!und) break;
        for (int i = 0; i < n; ++i) {
            uint64_t m = key[i];
            for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) if (strong[k] && key[A->col[k]] > m) m = key[A->col[k]];
            m1[i] = m;
        }
        for (int i = 0; i < n; ++i) {
            uint64_t m = m1[i];
            for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) if (strong[k] && m1[A->col[k]] > m) m = m1[A->col[k]];
            m2[i] = m;
        }
        for (int i = 0; i < n; ++i) {
            if (st[i] != 1) continue;
            if (m2[i] == key[i]) st[i] = 2;
            else if ((m2[i] >> 62) == 2) st[i] = 0;
        }
    }
#undef MKKEY
    int nagg = 0;
    for (int i = 0; i < n; ++i) agg[i] = (st[i] == 2) ? nagg++ : -1;
    /* pass 1: join the strongest-keyed root neighbour; pass 2: join through
       a neighbour assigned in pass 1 (synchronous, so order-independent) */
    int* a1 = (int*)malloc(sizeof(int) * n);
    for (int pass = 0; pass < 2; ++pass) {
        for (int i = 0; i < n; ++i) {
            a1[i] = agg[i];
            if (agg[i] >= 0 || st[i] < 0) continue;
            uint64_t best = 0; int ba = -1;
            for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
                int j = A->col[k];
                if (!strong[k] || agg[j] < 0) continue;
                uint64_t kj = (((uint64_t)hash_u32((uint32_t)j)) << 32) | (uint64_t)j;
                if (ba < 0 || kj > best) { best = kj; ba = agg[j]; }
            }
            a1[i] = ba;
        }
        memcpy(agg, a1, sizeof(int) * n);
    }
    free(a1); free(key); free(m1); free(m2); free(st);
    return nagg;
}

/* C = A * B, rows of C sorted by column; accumulation in product order */
static void spgemm(const csr_t* A, const csr_t* B, int ncolB, csr_t* C) {
    int n = A->n;
    C->n = n; C->ptr = (int*)calloc(n + 1, sizeof(int));
    int* mark = (int*)malloc(sizeof(int) * ncolB);
    for (int j = 0; j < ncolB; ++j) mark[j] = -1;
    for (int i = 0; i < n; ++i) {
        int cnt = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
            int a = A->col[k];
            for (int q = B->ptr[a]; q < B->ptr[a + 1]; ++q) if (mark[B->col[q]] != i) { mark[B->col[q]] = i; cnt++; }
        }
        C->ptr[i + 1] = C->ptr[i] + cnt;
    }
    C->nnz = C->ptr[n];
    C->col = (int*)malloc(sizeof(int) * (C->nnz + 1)); C->val = (double*)malloc(sizeof(double) * (C->nnz + 1));
    double* acc = (double*)calloc(ncolB, sizeof(double));
    for (int j = 0; j < ncolB; ++j) mark[j] = -1;
    int* tmp = (int*)malloc(sizeof(int) * (ncolB + 1));
    for (int i = 0; i < n; ++i) {
        int cnt = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
            int a = A->col[k]; double va = A->val[k];
            for (int q = B->ptr[a]; q < B->ptr[a + 1]; ++q) {
                int j = B->col[q];
                if (mark[j] != i) { mark[j] = i; acc[j] = 0.0; tmp[cnt++] = j; }
                acc[j] += va * B->val[q];
            }
        }
        /* insertion sort of the (short) column list */
        for (int s = 1; s < cnt; ++s) { int v = tmp[s], t = s - 1; while (t >= 0 && tmp[t] > v) { tmp[t + 1] = tmp[t]; --t; } tmp[t + 1] = v; }
        for (int s = 0; s < cnt; ++s) { C->col[C->ptr[i] + s] = tmp[s]; C->val[C->ptr[i] + s] = acc[tmp[s]]; }
    }
    free(mark); free(acc); free(tmp);
}

static void transpose(const csr_t* A, int ncol, csr_t* T) {
    T->n = ncol; T->nnz = A->nnz;
    T->ptr = (int*)calloc(ncol + 1, sizeof(int));
    T->col = (int*)malloc(sizeof(int) * (A->nnz + 1)); T->val = (double*)malloc(sizeof(double) * (A->nnz + 1));
    for (int k = 0; k < A->nnz; ++k) T->ptr[A->col[k] + 1]++;
    for (int j = 0; j < ncol; ++j) T->ptr[j + 1] += T->ptr[j];
    int* fill = (int*)malloc(sizeof(int) * (ncol + 1));
    memcpy(fill, T->ptr, sizeof(int) * (ncol + 1));
    for (int i = 0; i < A->n; ++i)
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) { int d = fill[A->col[k]]++; T->col[d] = i; T->val[d] = A->val[k]; }
    free(fill);
}

static void spmv(const csr_t* A, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < A->n; ++i) {
        double s = 0.0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) s += A->val[k] * x[A->col[k]];
        y[i] = s;
    }
}

typedef struct { double eps_strong; int coarse_enough; int max_levels; int cheb_degree; } amg_prm;

/* Jones-Plassmann colouring in synchronous rounds (the GPU's k_color_round):
   an uncoloured row whose (hash, index) key exceeds every uncoloured
   neighbour's takes the smallest colour that no neighbour coloured in an
   earlier round holds.  Fills L->cptr / L->crow (rows grouped by colour,
   ascending row order inside a colour); returns -1 beyond 128 colours. */
static int color_level(level_t* L) {
    const csr_t* A = &L->A;
    int n = A->n;
    int* cold = (int*)malloc(sizeof(int) * n);
    int* cnew = (int*)malloc(sizeof(int) * n);
    for (int i = 0; i < n; ++i) cold[i] = -1;
    int left = n, bad = 0;
    while (left > 0 && !bad) {
        memcpy(cnew, cold, sizeof(int) * n);
        left = 0;
        for (int i = 0; i < n; ++i) {
            if (cold[i] >= 0) continue;
            uint64_t ki = (((uint64_t)hash_u32((uint32_t)i)) << 32) | (uint64_t)(uint32_t)i;
            uint64_t used0 = 0, used1 = 0;
            int top = 1;
            for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
                int j = A->col[k];
                if (j == i) continue;
                int cj = cold[j];
                if (cj < 0) {
                    uint64_t kj = (((uint64_t)hash_u32((uint32_t)j)) << 32) | (uint64_t)(uint32_t)j;
                    if (kj > ki) { top = 0; break; }
                } else if (cj < 64) used0 |= 1ull << cj;
                else if (cj < 128) used1 |= 1ull << (cj - 64);
            }
            if (!top) { left++; continue; }
            int c = -1;
            for (int b = 0; b < 64 && c < 0; ++b) if (!(used0 >> b & 1)) c = b;
            for (int b = 0; b < 64 && c < 0; ++b) if (!(used1 >> b & 1)) c = 64 + b;
            if (c < 0) { bad = 1; break; }
            cnew[i] = c;
        }
        int* t = cold; cold = cnew; cnew = t;
    }
    int nc = 0;
    for (int i = 0; i < n && !bad; ++i) if (cold[i] + 1 > nc) nc = cold[i] + 1;
    if (!bad) {
        L->ncolors = nc;
        L->cptr = (int*)calloc(nc + 1, sizeof(int));
        L->crow = (int*)malloc(sizeof(int) * (n + 1));
        for (int i = 0; i < n; ++i) L->cptr[cold[i] + 1]++;
        for (int k = 0; k < nc; ++k) L->cptr[k + 1] += L->cptr[k];
        int* fill = (int*)malloc(sizeof(int) * (nc + 1));
        memcpy(fill, L->cptr, sizeof(int) * (nc + 1));
        for (int i = 0; i < n; ++i) L->crow[fill[cold[i]]++] = i;
        free(fill);
    }
    free(cold); free(cnew);
    return bad ? -1 : nc;
}

/* one Gauss-Seidel sweep, colours ascending (forward) or descending */
static void gs_sweep(const level_t* L, const double* b, double* x, int backward) {
    const csr_t* A = &L->A;
    for (int q = 0; q < L->ncolors; ++q) {
        int k = backward ? L->ncolors - 1 - q : q;
#pragma omp parallel for schedule(static)
        for (int t = L->cptr[k]; t < L->cptr[k + 1]; ++t) {
            int i = L->crow[t];
            double s = 0.0;
            for (int e = A->ptr[i]; e < A->ptr[i + 1]; ++e) s += A->val[e] * x[A->col[e]];
            x[i] += L->dinv[i] * (b[i] - s);
        }
    }
}

static void amg_free(amg_t* h) {
    for (int l = 0; l < h->nlev; ++l) {
        level_t* L = &h->lev[l];
        if (l > 0) csr_free(&L->A);
        csr_free(&L->P); csr_free(&L->R);
        free(L->dinv); free(L->r); free(L->x); free(L->b); free(L->t1); free(L->t2);
        free(L->cptr); free(L->crow);
    }
    free(h->chol);
    memset(h, 0, sizeof *h);
}

static int dense_cholesky(int n, double* a) {
    for (int j = 0; j < n; ++j) {
        double d = a[j * n + j];
        for (int k = 0; k < j; ++k) d -= a[j * n + k] * a[j * n + k];
        if (!(d > 0.0)) return -1;
        d = sqrt(d); a[j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double s = a[i * n + j];
            for (int k = 0; k < j; ++k) s -= a[i * n + k] * a[j * n + k];
            a[i * n + j] = s / d;
        }
        for (int i = 0; i < j; ++i) a[i * n + j] = 0.0;
    }
    return 0;
}

static int amg_setup(amg_t* h, const csr_t* A0, const amg_prm* prm) {
    memset(h, 0, sizeof *h);
    h->cheb_degree = prm->cheb_degree;
    h->smoother = g_smoother;
    float eps = (float)prm->eps_strong;
    h->lev[0].A = *A0;
    int l = 0;
    for (;;) {
        level_t* L = &h->lev[l];
        csr_t* A = &L->A;
        int n = A->n;
        h->total_nnz += A->nnz;
        L->dinv = (double*)malloc(sizeof(double) * n);
        double lam = 0.0;
        for (int i = 0; i < n; ++i) {
            double d = 0.0, rs = 0.0;
            for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) { if (A->col[k] == i) d = A->val[k]; rs += fabs(A->val[k]); }
            L->dinv[i] = 1.0 / d;
            double r = rs / fabs(d);
            if (r > lam) lam = r;
        }
        L->lam_max = lam;   /* Gershgorin bound on rho(D^-1 A) */
        L->r = (double*)calloc(n, sizeof(double)); L->x = (double*)calloc(n, sizeof(double));
        L->b = (double*)calloc(n, sizeof(double)); L->t1 = (double*)calloc(n, sizeof(double));
        L->t2 = (double*)calloc(n, sizeof(double));
        if (n <= prm->coarse_enough || l == prm->max_levels - 1) break;
        /* strength */
        double eps2 = (double)(eps * eps);
        char* strong = (char*)malloc(A->nnz + 1);
        double* dia = (double*)malloc(sizeof(double) * n);
        for (int i = 0; i < n; ++i) { dia[i] = 0.0; for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) if (A->col[k] == i) dia[i] = A->val[k]; }
        for (int i = 0; i < n; ++i) {
            double ed = eps2 * dia[i];
            for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
                int j = A->col[k]; double v = A->val[k];
                strong[k] = (j != i) && (ed * dia[j] < v * v);
            }
        }
        eps *= 0.5f;
        int* agg = (int*)malloc(sizeof(int) * n);
        int nagg = aggregate(A, strong, agg);
        if (nagg == 0 || nagg >= n) { free(strong); free(dia); free(agg); break; }
        L->nagg = nagg;
        /* smoothed prolongation: row i = (1-w) e_agg(i) + sum_strong (-w/df_i) a_ij e_agg(j) */
        const double omega = 2.0 / 3.0;
        csr_t* P = &L->P;
        P->n = n; P->ptr = (int*)calloc(n + 1, sizeof(int));
        int cap = A->nnz + 1;
        P->col = (int*)malloc(sizeof(int) * cap); P->val = (double*)malloc(sizeof(double) * cap);
        int* mark = (int*)malloc(sizeof(int) * nagg); for (int j = 0; j < nagg; ++j) mark[j] = -1;
        int m = 0;
        for (int i = 0; i < n; ++i) {
            double df = 0.0;
            for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) if (A->col[k] == i || !strong[k]) df += A->val[k];
            df = -omega * (1.0 / df);
            int rb = m;
            for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
                int j = A->col[k];
                if (j != i && !strong[k]) continue;
                int g = agg[j];
                if (g < 0) continue;
                double v = (j == i) ? (1.0 - omega) : df * A->val[k];
                if (mark[g] >= rb) P->val[mark[g]] += v;
                else { mark[g] = m; P->col[m] = g; P->val[m] = v; m++; }
            }
            /* sort row by column */
            for (int s = rb + 1; s < m; ++s) {
                int cv = P->col[s]; double vv = P->val[s]; int t = s - 1;
                while (t >= rb && P->col[t] > cv) { P->col[t + 1] = P->col[t]; P->val[t + 1] = P->val[t]; --t; }
                P->col[t + 1] = cv; P->val[t + 1] = vv;
            }
            for (int s = rb; s < m; ++s) mark[P->col[s]] = -1;
            P->ptr[i + 1] = m;
        }
        P->nnz = m;
        free(mark); free(strong); free(dia); free(agg);
        transpose(P, nagg, &L->R);
        csr_t AP, Ac;
        spgemm(A, P, nagg, &AP);
        spgemm(&L->R, &AP, nagg, &Ac);
        csr_free(&AP);
        l++;
        h->lev[l].A = Ac;
    }
    h->nlev = l + 1;
    /* the finest level above 16384 rows (the GPU keeps Chebyshev elsewhere) */
    if (h->smoother == 1 && h->nlev > 1 && h->lev[0].A.n > 16384 && color_level(&h->lev[0]) < 0) return -3;
    /* coarsest: dense Cholesky */
    csr_t* Ac = &h->lev[l].A;
    h->nc = Ac->n;
    h->chol = (double*)calloc((size_t)h->nc * h->nc, sizeof(double));
    for (int i = 0; i < Ac->n; ++i) for (int k = Ac->ptr[i]; k < Ac->ptr[i + 1]; ++k) h->chol[(size_t)i * h->nc + Ac->col[k]] = Ac->val[k];
    return dense_cholesky(h->nc, h->chol);
}

/* Chebyshev smoother on D^-1 A over [lam/30, lam]; x updated in place */
static void cheb_smooth(const level_t* L, const double* b, double* x, int degree) {
    int n = L->A.n;
    double hi = L->lam_max, lo = hi / 30.0;
    double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
    double sigma = theta / delta, rho = 1.0 / sigma;
    double* r = L->t1; double* d = L->t2;
    spmv(&L->A, x, r);
    for (int i = 0; i < n; ++i) { r[i] = L->dinv[i] * (b[i] - r[i]); d[i] = r[i] / theta; }
    for (int k = 0; k < degree; ++k) {
        for (int i = 0; i < n; ++i) x[i] += d[i];
        if (k == degree - 1) break;
        spmv(&L->A, x, r);
        double rho_new = 1.0 / (2.0 * sigma - rho);
        for (int i = 0; i < n; ++i) {
            double z = L->dinv[i] * (b[i] - r[i]);
            d[i] = rho_new * rho * d[i] + 2.0 * rho_new / delta * z;
        }
        rho = rho_new;
    }
}

static void vcycle(amg_t* h, int l, const double* b, double* x) {
    level_t* L = &h->lev[l];
    int n = L->A.n;
    if (l == h->nlev - 1) {
        int m = h->nc; const double* c = h->chol;
        double* y = L->t1;
        for (int i = 0; i < m; ++i) { double s = b[i]; for (int k = 0; k < i; ++k) s -= c[(size_t)i * m + k] * y[k]; y[i] = s / c[(size_t)i * m + i]; }
        for (int i = m - 1; i >= 0; --i) { double s = y[i]; for (int k = i + 1; k < m; ++k) s -= c[(size_t)k * m + i] * x[k]; x[i] = s / c[(size_t)i * m + i]; }
        return;
    }
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    if (L->ncolors > 0) gs_sweep(L, b, x, 0);
    else cheb_smooth(L, b, x, h->cheb_degree);
    spmv(&L->A, x, L->r);
    for (int i = 0; i < n; ++i) L->r[i] = b[i] - L->r[i];
    level_t* C = &h->lev[l + 1];
    spmv(&L->R, L->r, C->b);
    vcycle(h, l + 1, C->b, C->x);
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = L->P.ptr[i]; k < L->P.ptr[i + 1]; ++k) s += L->P.val[k] * C->x[L->P.col[k]];
        x[i] += s;
    }
    if (L->ncolors > 0) gs_sweep(L, b, x, 1);
    else cheb_smooth(L, b, x, h->cheb_degree);
}

static double dot(const double* a, const double* b, int n) {
    double s = 0.0;
#pragma omp parallel for reduction(+:s) schedule(static)
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* preconditioned CG on the system in csr_ptr/col/val (or its RCM form) */
int orc_solve(orc_ctx* c, int use_rcm, double tol, int maxiter, double* out_info) {
    csr_t A;
    A.n = c->nc;
    A.ptr = iget(c, use_rcm ? "rcm_csr_ptr" : "csr_ptr");
    A.col = iget(c, use_rcm ? "rcm_csr_col" : "csr_col");
    A.val = dget(c, use_rcm ? "rcm_csr_val" : "csr_val");
    A.nnz = A.ptr[A.n];
    double* b = dget(c, use_rcm ? "rcm_B" : "B");
    int n = A.n;
    amg_t h; amg_prm prm = {0.03, 64, 24, 2};
    if (amg_setup(&h, &A, &prm) != 0) { amg_free(&h); return -2; }
    double* x = dreg(c, use_rcm ? "rcm_x_orc" : "x_orc", n);
    double *r = (double*)malloc(sizeof(double) * n), *z = (double*)malloc(sizeof(double) * n);
    double *p = (double*)malloc(sizeof(double) * n), *q = (double*)malloc(sizeof(double) * n);
    memcpy(r, b, sizeof(double) * n);
    double bn = sqrt(dot(b, b, n));
    double rn = bn;
    int it = 0;
    double rz = 0.0;
    if (bn == 0.0) { bn = 1.0; rn = 0.0; }
    while (it < maxiter && rn > tol * bn) {
        vcycle(&h, 0, r, z);
        double rz_new = dot(r, z, n);
        if (it == 0) memcpy(p, z, sizeof(double) * n);
        else { double beta = rz_new / rz; for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i]; }
        rz = rz_new;
        spmv(&A, p, q);
        double alpha = rz / dot(p, q, n);
        for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
        rn = sqrt(dot(r, r, n));
        it++;
    }
    /* true residual */
    spmv(&A, x, q);
    double tr = 0.0;
    for (int i = 0; i < n; ++i) { double d = b[i] - q[i]; tr += d * d; }
    if (out_info) {
        out_info[0] = it; out_info[1] = sqrt(tr) / bn; out_info[2] = h.nlev;
        out_info[3] = (double)h.total_nnz / (double)A.nnz;
        out_info[4] = h.nc;
        for (int l = 0; l < h.nlev && l < 10; ++l) out_info[5 + l] = h.lev[l].A.n;
    }
    /* the finest level's A is borrowed */
    memset(&h.lev[0].A, 0, sizeof(csr_t));
    amg_free(&h);
    free(r); free(z); free(p); free(q);
    return it;
}

/* ------------------------------------------------------------------------ */
/* post-solve: src/solvers/eqPressure.cpp:686-809 (Gauss-Green grad p', two */
/* sweeps with skewness correction), :823-883 (update + norms)               */
/* ------------------------------------------------------------------------ */
double orc_update(orc_ctx* c, const double* x) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    double *fn = dget(c, "face_n"), *fa = dget(c, "face_area"), *wc = dget(c, "face_wC");
    double *sk = dget(c, "face_skew"), *vol = dget(c, "cell_vol");
    double *P = dget(c, "P"), *U = dget(c, "U"), *V = dget(c, "V"), *W = dget(c, "W"), *rho = dget(c, "rho");
    double* g = dreg(c, "grad_x", 3LL * nc);
    double* gt = (double*)malloc(sizeof(double) * 3 * nc);
    for (int it = 0; it < 2; ++it) {
        memset(gt, 0, sizeof(double) * 3 * nc);
        for (int f = 0; f < ni; ++f) {
            int o = c->own[f], q = c->nei[f];
            double wL = wc[f], wR = 1.0 - wL;
            double vF = wL * x[o] + wR * x[q];
            for (int k = 0; k < 3; ++k) { vF += wL * g[3 * o + k] * sk[3 * f + k]; vF += wR * g[3 * q + k] * sk[3 * f + k]; }
            for (int k = 0; k < 3; ++k) gt[3 * o + k] += vF * fn[3 * f + k] * fa[f] / vol[o];
            for (int k = 0; k < 3; ++k) gt[3 * q + k] -= vF * fn[3 * f + k] * fa[f] / vol[q];
        }
        /* the reference tests the type of variable 0 (pressure) per patch */
        for (int f = ni; f < nf; ++f) {
            int o = c->own[f], p = patch_of(c, f);
            double vF = x[o];
            if (c->bct[3 * p] == 1) vF = 0.0;
            for (int k = 0; k < 3; ++k) gt[3 * o + k] += vF * fn[3 * f + k] * fa[f] / vol[o];
        }
        memcpy(g, gt, sizeof(double) * 3 * nc);
    }
    free(gt);
    double nd = 0.0, npn = 0.0;
    for (int i = 0; i < nc; ++i) {
        P[i] += c->urf_p * x[i];
        double t = c->dt / rho[i];
        double ru = c->urf_u * t * g[3 * i], rv = c->urf_u * t * g[3 * i + 1], rw = c->urf_u * t * g[3 * i + 2];
        U[i] -= ru; V[i] -= rv; W[i] -= rw;
        if (P[i] <= c->minP) P[i] = c->minP;
        if (P[i] >= c->maxP) P[i] = c->maxP;
        if (U[i] <= c->minU) U[i] = c->minU;
        if (U[i] >= c->maxU) U[i] = c->maxU;
        if (V[i] <= c->minV) V[i] = c->minV;
        if (V[i] >= c->maxV) V[i] = c->maxV;
        if (W[i] <= c->minW) W[i] = c->minW;
        if (W[i] >= c->maxW) W[i] = c->maxW;
        nd += x[i] * x[i]; nd += ru * ru; nd += rv * rv; nd += rw * rw;
        npn += P[i] * P[i]; npn += U[i] * U[i]; npn += V[i] * V[i]; npn += W[i] * W[i];
    }
    return sqrt(nd) / sqrt(npn);
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* momentum equation: src/solvers/transport.cpp:9-98 (calcCellTransport,      */
/* laminar), src/solvers/reconIncom.cpp:501-545, :1015-1030 (face viscosity),  */
/* src/solvers/eqMomentum.cpp:9-1122 (calcMomentumEqs, 3-argument overload):   */
/* BDF2 diagonal and RHS :223-326, internal faces :331-787, boundary faces     */
/* :795-1008, update + norm :1029-1119.  COO order: N diagonals, then per      */
/* internal face (LR, RL), each left out when |a| < DBL_MIN (:699-711).        */
/* Old (n-1) and second-old (n-2) velocities come from arrays oldU/V/W and     */
/* old2U/V/W; absent, they default to the current velocity.                    */
/* ------------------------------------------------------------------------ */
static double* hist(orc_ctx* c, const char* name, const double* cur) {
    double* p = dget(c, name);
    return p ? p : (double*)cur;
}

void orc_assemble_momentum(orc_ctx* c) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    face_values(c);
    gravity_source(c);
    double *P = dget(c, "P"), *U = dget(c, "U"), *V = dget(c, "V"), *W = dget(c, "W"), *VF = dget(c, "VF");
    double *rho = dget(c, "rho"), *sg = dget(c, "src_grav"), *vol = dget(c, "cell_vol");
    /* calcCellTransport: mu = VF mu0 + (1 - VF) mu1 on the clamped VF */
    double* mu = dreg(c, "mu", nc);
    for (int i = 0; i < nc; ++i) {
        double t = 0.0; t += VF[i];
        double v1 = 1.0 - t;
        double m = 0.0; m += VF[i] * c->mu0; m += v1 * c->mu1;
        m += 0.0;                                   /* muT, laminar */
        mu[i] = m;
    }
    /* stencil min/max of P, U, V, W (eqMomentum.cpp:40-43) */
    double* mmp = dreg(c, "mom_minmax_p", 2LL * nc);
    double* mm = dreg(c, "mom_minmax_uvw", 6LL * nc);
    double *t1 = (double*)malloc(sizeof(double) * nc), *t2 = (double*)malloc(sizeof(double) * nc);
    minmax(c, P, t1, t2); for (int i = 0; i < nc; ++i) { mmp[2 * i] = t1[i]; mmp[2 * i + 1] = t2[i]; }
    minmax(c, U, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i] = t1[i]; mm[6 * i + 1] = t2[i]; }
    minmax(c, V, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i + 2] = t1[i]; mm[6 * i + 3] = t2[i]; }
    minmax(c, W, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i + 4] = t1[i]; mm[6 * i + 5] = t2[i]; }
    free(t1); free(t2);
    /* gradients (eqMomentum.cpp:94-105) */
    double *pr = dget(c, "face_pR"), *ur = dget(c, "face_uR"), *vr = dget(c, "face_vfR");
    double* tmp = (double*)malloc(sizeof(double) * nf);
    double* gP = dreg(c, "mom_grad_P", 3LL * nc); lsq_grad(c, P, pr, gP);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f];
    double* gU = dreg(c, "mom_grad_U", 3LL * nc); lsq_grad(c, U, tmp, gU);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f + 1];
    double* gV = dreg(c, "mom_grad_V", 3LL * nc); lsq_grad(c, V, tmp, gV);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f + 2];
    double* gW = dreg(c, "mom_grad_W", 3LL * nc); lsq_grad(c, W, tmp, gW);
    double* gVF = dreg(c, "mom_grad_VF", 3LL * nc); lsq_grad(c, VF, vr, gVF);
    free(tmp);

    double *oU = hist(c, "oldU", U), *oV = hist(c, "oldV", V), *oW = hist(c, "oldW", W);
    double *o2U = hist(c, "old2U", U), *o2V = hist(c, "old2V", V), *o2W = hist(c, "old2W", W);
    const double dt = c->dt;
    int cap = nc + 2 * ni;
    int* ar = ireg(c, "mom_A_rows", cap); int* acl = ireg(c, "mom_A_cols", cap);
    double* av = dreg(c, "mom_A_vals", cap);
    double* B = dreg(c, "mom_B", 3LL * nc);          /* 3 planes: B0 | B1 | B2 */
    double *B0 = B, *B1 = B + nc, *B2 = B + 2 * (size_t)nc;
    for (int i = 0; i < nc; ++i) {
        double Rho = rho[i], volume = vol[i];
        ar[i] = i; acl[i] = i;
        av[i] = Rho * 1.5 * volume / dt;
        B0[i] = -Rho * (1.5 * U[i] - 2.0 * oU[i] + 0.5 * o2U[i]) * volume / dt;
        B1[i] = -Rho * (1.5 * V[i] - 2.0 * oV[i] + 0.5 * o2V[i]) * volume / dt;
        B2[i] = -Rho * (1.5 * W[i] - 2.0 * oW[i] + 0.5 * o2W[i]) * volume / dt;
        B0[i] += volume * sg[4 * i]; B1[i] += volume * sg[4 * i + 1]; B2[i] += volume * sg[4 * i + 2];
        {   /* surface-tension source (eqMomentum.cpp:320-322) */
            double* ss = dget(c, "src_sft");
            double s0 = 0.0, s1 = 0.0, s2 = 0.0;
            if (ss && c->sigma != 0.0) { s0 = ss[4 * i]; s1 = ss[4 * i + 1]; s2 = ss[4 * i + 2]; }
            B0[i] += volume * s0; B1[i] += volume * s1; B2[i] += volume * s2;
        }
    }
    double *fn = dget(c, "face_n"), *fa = dget(c, "face_area"), *wc = dget(c, "face_wC");
    double *mpn = dget(c, "face_magPN"), *al = dget(c, "face_alphaF"), *epn = dget(c, "face_ePN");
    double *sk = dget(c, "face_skew"), *ul = dget(c, "face_uL"), *pl = dget(c, "face_pL"), *rl = dget(c, "face_rhoL");
    double* unf = dreg(c, "mom_face_UnF", nf);
    int nnz = nc;
    for (int f = 0; f < ni; ++f) {
        int o = c->own[f], q = c->nei[f];
        const double* n = fn + 3 * f; const double* e = epn + 3 * f; const double* s = sk + 3 * f;
        double area = fa[f], wCL = wc[f], wCR = 1.0 - wCL;
        double UL_HO = U[o], VL_HO = V[o], WL_HO = W[o], UR_HO = U[q], VR_HO = V[q], WR_HO = W[q];
        double muF = 1.0 / (wCL / mu[o] + wCR / mu[q]);
        double RhoL = rho[o], RhoR = rho[q], PL = P[o], PR = P[q];
        double UL = U[o], VL = V[o], WL = W[o], UR = U[q], VR = V[q], WR = W[q];
        double dPN = mpn[f], alpha = al[f];
        double ULs = UL, VLs = VL, WLs = WL, URs = UR, VRs = VR, WRs = WR;
        for (int k = 0; k < 3; ++k) {
            ULs += gU[3 * o + k] * s[k]; URs += gU[3 * q + k] * s[k];
            VLs += gV[3 * o + k] * s[k]; VRs += gV[3 * q + k] * s[k];
            WLs += gW[3 * o + k] * s[k]; WRs += gW[3 * q + k] * s[k];
        }
        ULs = smax(mm[6 * o + 1], smin(mm[6 * o + 0], ULs)); URs = smax(mm[6 * q + 1], smin(mm[6 * q + 0], URs));
        VLs = smax(mm[6 * o + 3], smin(mm[6 * o + 2], VLs)); VRs = smax(mm[6 * q + 3], smin(mm[6 * q + 2], VRs));
        WLs = smax(mm[6 * o + 5], smin(mm[6 * o + 4], WLs)); WRs = smax(mm[6 * q + 5], smin(mm[6 * q + 4], WRs));
        double UnL = ULs * n[0] + VLs * n[1] + WLs * n[2];
        double UnR = URs * n[0] + VRs * n[1] + WRs * n[2];
        double UnF = wCL * UnL + wCR * UnR;
        /* surfaceNormalVelocity.cpp:125-155 (pressure) */
        double rs = 1.0 / (wCL / RhoL + wCR / RhoR);
        double tt = dt / rs;
        UnF -= alpha * tt * (PR - PL) / dPN;
        for (int k = 0; k < 3; ++k) {
            UnF -= tt * rs * wCL / RhoL * gP[3 * o + k] * (n[k] - alpha * e[k]);
            UnF -= tt * rs * wCR / RhoR * gP[3 * q + k] * (n[k] - alpha * e[k]);
        }
        for (int k = 0; k < 3; ++k) {
            UnF += tt * rs * wCL / RhoL * gP[3 * o + k] * n[k];
            UnF += tt * rs * wCR / RhoR * gP[3 * q + k] * n[k];
        }
        /* surfaceNormalVelocity.cpp:156-187 (gravity), then :190-221 (surface tension) */
        for (int k = 0; k < 3; ++k) UnF += alpha * tt * rs * c->g[k] * alpha * e[k];
        for (int k = 0; k < 3; ++k) {
            UnF += tt * rs * wCL / RhoL * sg[4 * o + k] * (n[k] - alpha * e[k]);
            UnF += tt * rs * wCR / RhoR * sg[4 * q + k] * (n[k] - alpha * e[k]);
        }
        for (int k = 0; k < 3; ++k) {
            UnF -= alpha * tt * rs * wCL / RhoL * sg[4 * o + k] * n[k];
            UnF -= alpha * tt * rs * wCR / RhoR * sg[4 * q + k] * n[k];
        }
        UnF = sft_unf(c, UnF, o, q, RhoL, RhoR, wCL, wCR, alpha, dPN, n, e);
        unf[f] = UnF;
        double weightL = (UnF > 0.0) ? 1.0 : 0.0;
        double weightR = 1.0 - weightL;
        double PF = wCL * PL + wCR * PR;
        double UF_HO = weightL * UL_HO + weightR * UR_HO;
        double VF_HO = weightL * VL_HO + weightR * VR_HO;
        double WF_HO = weightL * WL_HO + weightR * WR_HO;
        PF = wCL * PL + wCR * PR;
        for (int k = 0; k < 3; ++k) {
            PF += wCL * gP[3 * o + k] * s[k];
            PF += wCR * gP[3 * q + k] * s[k];
        }
        PF = smax(mmp[2 * o + 1], smin(mmp[2 * o], PF));
        PF = smax(mmp[2 * q + 1], smin(mmp[2 * q], PF));
        /* coefficients (eqMomentum.cpp:694-712) */
        av[o] += (weightL * RhoL * UnF * area + alpha * muF / dPN * area);
        {
            double a = (weightR * RhoL * UnF * area - alpha * muF / dPN * area);
            if (!(fabs(a) < 2.2250738585072014e-308)) { ar[nnz] = o; acl[nnz] = q; av[nnz] = a; ++nnz; }
        }
        av[q] -= (weightR * RhoR * UnF * area - alpha * muF / dPN * area);
        {
            double a = -(weightL * RhoR * UnF * area + alpha * muF / dPN * area);
            if (!(fabs(a) < 2.2250738585072014e-308)) { ar[nnz] = q; acl[nnz] = o; av[nnz] = a; ++nnz; }
        }
        /* fluxes (eqMomentum.cpp:740-779) */
        double cL[3], cR[3], d[3], dL[3], dR[3];
        cL[0] = (RhoL * UF_HO * UnF + PF * n[0]) * area;
        cL[1] = (RhoL * VF_HO * UnF + PF * n[1]) * area;
        cL[2] = (RhoL * WF_HO * UnF + PF * n[2]) * area;
        cR[0] = (RhoR * UF_HO * UnF + PF * n[0]) * area;
        cR[1] = (RhoR * VF_HO * UnF + PF * n[1]) * area;
        cR[2] = (RhoR * WF_HO * UnF + PF * n[2]) * area;
        d[0] = alpha * muF * (UR - UL) / dPN * area;
        d[1] = alpha * muF * (VR - VL) / dPN * area;
        d[2] = alpha * muF * (WR - WL) / dPN * area;
        for (int k = 0; k < 3; ++k) {
            d[0] += (muF * (wCL * gU[3 * o + k] + wCR * gU[3 * q + k]) * (n[k] - alpha * e[k]) * area);
            d[1] += (muF * (wCL * gV[3 * o + k] + wCR * gV[3 * q + k]) * (n[k] - alpha * e[k]) * area);
            d[2] += (muF * (wCL * gW[3 * o + k] + wCR * gW[3 * q + k]) * (n[k] - alpha * e[k]) * area);
        }
        dL[0] = ((gU[3 * o] * n[0] + gU[3 * o + 1] * n[1] + gU[3 * o + 2] * n[2]) * muF * area);
        dL[1] = ((gV[3 * o] * n[0] + gV[3 * o + 1] * n[1] + gV[3 * o + 2] * n[2]) * muF * area);
        dL[2] = ((gW[3 * o] * n[0] + gW[3 * o + 1] * n[1] + gW[3 * o + 2] * n[2]) * muF * area);
        dR[0] = ((gU[3 * q] * n[0] + gU[3 * q + 1] * n[1] + gU[3 * q + 2] * n[2]) * muF * area);
        dR[1] = ((gV[3 * q] * n[0] + gV[3 * q + 1] * n[1] + gV[3 * q + 2] * n[2]) * muF * area);
        dR[2] = ((gW[3 * q] * n[0] + gW[3 * q + 1] * n[1] + gW[3 * q + 2] * n[2]) * muF * area);
        B0[o] -= (cL[0] - d[0] - dL[0]); B1[o] -= (cL[1] - d[1] - dL[1]); B2[o] -= (cL[2] - d[2] - dL[2]);
        B0[q] += (cR[0] - d[0] - dR[0]); B1[q] += (cR[1] - d[1] - dR[1]); B2[q] += (cR[2] - d[2] - dR[2]);
    }
    /* boundary faces, patch by patch (eqMomentum.cpp:795-1008) */
    for (int f = ni; f < nf; ++f) {
        int p = patch_of(c, f), o = c->own[f];
        const double* n = fn + 3 * f; const double* e = epn + 3 * f;
        const double* uL = ul + 3 * f; const double* uR = ur + 3 * f;
        double area = fa[f];
        double UnL = uL[0] * n[0] + uL[1] * n[1] + uL[2] * n[2];
        double UnR = uR[0] * n[0] + uR[1] * n[1] + uR[2] * n[2];
        double UnF = 0.5 * UnL + 0.5 * UnR;
        double RhoL = rl[f];
        double tmp1 = 1.0 / RhoL * dt;
        double UF = 0.5 * uL[0] + 0.5 * uR[0], VF_ = 0.5 * uL[1] + 0.5 * uR[1], WF = 0.5 * uL[2] + 0.5 * uR[2];
        double PF = 0.5 * pl[f] + 0.5 * pr[f];
        int tu = c->bct[3 * p + 1];
        double cU = 0.0, cUd = 0.0;
        if (tu == 1) { cU = 0.0; cUd = 1.0; }        /* fixedValue */
        else if (tu == 0) { cU = 1.0; cUd = 0.0; }   /* zeroGradient */
        else if (tu == 3) { cU = 0.0; cUd = 0.0; }   /* slip */
        else { cU = 0.0; cUd = 1.0; }                /* noSlip */
        double muF = 0.5 * mu[o] + 0.5 * mu[o];
        double orgUL = U[o], orgUR = uR[0], orgVL = V[o], orgVR = uR[1], orgWL = W[o], orgWR = uR[2];
        double dPN = 0.5 * mpn[f], alpha = al[f];
        if (c->bct[3 * p] == 1) {
            double orgPL = P[o], orgPR = c->bcv[5 * p];
            UnF -= alpha * tmp1 * (orgPR - orgPL) / dPN;
            for (int k = 0; k < 3; ++k) UnF += alpha * tmp1 * gP[3 * o + k] * e[k];
        }
        unf[f] = UnF;
        double dU = 0.0, dV = 0.0, dW = 0.0;
        dU += alpha * (orgUR - orgUL) / dPN;
        dV += alpha * (orgVR - orgVL) / dPN;
        dW += alpha * (orgWR - orgWL) / dPN;
        for (int k = 0; k < 3; ++k) {
            double tv = n[k] - alpha * e[k];
            dU += gU[3 * o + k] * tv; dV += gV[3 * o + k] * tv; dW += gW[3 * o + k] * tv;
        }
        for (int k = 0; k < 3; ++k) { dU += (gU[3 * o + k] * n[k]); dV += (gV[3 * o + k] * n[k]); dW += (gW[3 * o + k] * n[k]); }
        av[o] += cU * (RhoL * UnF * area);
        av[o] += cUd * (muF * alpha / dPN * area);
        B0[o] -= (RhoL * UF * UnF * area + PF * n[0] * area - muF * dU * area);
        B1[o] -= (RhoL * VF_ * UnF * area + PF * n[1] * area - muF * dV * area);
        B2[o] -= (RhoL * WF * UnF * area + PF * n[2] * area - muF * dW * area);
    }
    /* trim the COO arrays to the entries kept */
    orc_arr* a;
    a = find(c, "mom_A_rows"); a->n = nnz;
    a = find(c, "mom_A_cols"); a->n = nnz;
    a = find(c, "mom_A_vals"); a->n = nnz;
    /* COO -> CSR as solveAMGCL.cpp:1129-1172 (in-row order = COO order) */
    int* ptr = ireg(c, "mom_csr_ptr", nc + 1); int* col = ireg(c, "mom_csr_col", nnz);
    double* val = dreg(c, "mom_csr_val", nnz);
    for (int k = 0; k < nnz; ++k) ptr[ar[k]]++;
    for (int i = 0, s2 = 0; i < nc; ++i) { int t = ptr[i]; ptr[i] = s2; s2 += t; }
    ptr[nc] = nnz;
    for (int k = 0; k < nnz; ++k) { int d = ptr[ar[k]]++; col[d] = acl[k]; val[d] = av[k]; }
    for (int i = 0, last = 0; i <= nc; ++i) { int t = ptr[i]; ptr[i] = last; last = t; }
}

/* BiCGStab with a Jacobi preconditioner on the momentum CSR, one right-hand
   side (plane j of mom_B), x0 = 0.  Not AMGCL's FGMRES: the GPU solver's
   algorithm, restated for the CPU baseline and the parity tests. */
static int bicgstab_jacobi(int n, const int* ptr, const int* col, const double* val, const double* b, double tol,
                           int maxiter, double* out_x, double* out_relres);
int orc_solve_momentum(orc_ctx* c, int j, double tol, int maxiter, double* out_x, double* out_relres) {
    int n = c->nc;
    int* ptr = iget(c, "mom_csr_ptr"); int* col = iget(c, "mom_csr_col"); double* val = dget(c, "mom_csr_val");
    double* b = dget(c, "mom_B") + (size_t)j * n;
    return bicgstab_jacobi(n, ptr, col, val, b, tol, maxiter, out_x, out_relres);
}
static int bicgstab_jacobi(int n, const int* ptr, const int* col, const double* val, const double* b, double tol,
                           int maxiter, double* out_x, double* out_relres) {
    double* w = (double*)calloc(8 * (size_t)n, sizeof(double));
    double *r = w, *rh = w + n, *p = w + 2 * (size_t)n, *v = w + 3 * (size_t)n, *s = w + 4 * (size_t)n;
    double *t = w + 5 * (size_t)n, *ph = w + 6 * (size_t)n, *dinv = w + 7 * (size_t)n;
    double* x = out_x;
    for (int i = 0; i < n; ++i) {
        x[i] = 0.0; r[i] = b[i]; rh[i] = b[i];
        double d = 0.0;
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) if (col[k] == i) d += val[k];
        dinv[i] = 1.0 / d;
    }
    double bn = sqrt(dot(b, b, n));
    if (bn == 0.0) { free(w); if (out_relres) *out_relres = 0.0; return 0; }
    double rho = 1.0, alpha = 1.0, omega = 1.0, rn = bn;
    int it = 0;
    while (it < maxiter && rn > tol * bn) {
        double rho1 = dot(rh, r, n);
        double beta = (rho1 / rho) * (alpha / omega);
        rho = rho1;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) { p[i] = r[i] + beta * (p[i] - omega * v[i]); ph[i] = dinv[i] * p[i]; }
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) { double a = 0.0; for (int k = ptr[i]; k < ptr[i + 1]; ++k) a += val[k] * ph[col[k]]; v[i] = a; }
        alpha = rho / dot(rh, v, n);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) { double a = 0.0; for (int k = ptr[i]; k < ptr[i + 1]; ++k) a += val[k] * dinv[col[k]] * s[col[k]]; t[i] = a; }
        double tt = dot(t, t, n);
        omega = (tt > 0.0) ? dot(t, s, n) / tt : 0.0;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) { x[i] += alpha * ph[i] + omega * dinv[i] * s[i]; r[i] = s[i] - omega * t[i]; }
        rn = sqrt(dot(r, r, n));
        ++it;
    }
    /* true residual */
    double tr = 0.0;
    for (int i = 0; i < n; ++i) {
        double a = 0.0; for (int k = ptr[i]; k < ptr[i + 1]; ++k) a += val[k] * x[col[k]];
        tr += (b[i] - a) * (b[i] - a);
    }
    if (out_relres) *out_relres = sqrt(tr) / bn;
    free(w);
    return it;
}

/* eqMomentum.cpp:1029-1119: U += urf x, clamp, norm = |x| / |U| */
double orc_update_momentum(orc_ctx* c, const double* x0, const double* x1, const double* x2) {
    int nc = c->nc;
    double *U = dget(c, "U"), *V = dget(c, "V"), *W = dget(c, "W");
    double nd = 0.0, npn = 0.0;
    for (int i = 0; i < nc; ++i) {
        U[i] += c->urf_mom * x0[i]; V[i] += c->urf_mom * x1[i]; W[i] += c->urf_mom * x2[i];
        if (U[i] <= c->minU) U[i] = c->minU;
        if (U[i] >= c->maxU) U[i] = c->maxU;
        if (V[i] <= c->minV) V[i] = c->minV;
        if (V[i] >= c->maxV) V[i] = c->maxV;
        if (W[i] <= c->minW) W[i] = c->minW;
        if (W[i] >= c->maxW) W[i] = c->maxW;
        nd += x0[i] * x0[i]; nd += x1[i] * x1[i]; nd += x2[i] * x2[i];
        npn += U[i] * U[i]; npn += V[i] * V[i]; npn += W[i] * W[i];
    }
    return sqrt(nd) / sqrt(npn);
}

/* ------------------------------------------------------------------------ */
/* volume fraction: src/solvers/reconIncom.cpp:345-429                        */
/* (setIncomValuesLeftRightFaceWithVfMSTACS: zero-order values, LSQ grad VF,  */
/* MSTACS), src/solvers/NVD.cpp:1098-1790 (calcMSTACS),                        */
/* src/solvers/eqVolfrac.cpp:9-795 (calcVolfracEq, 3-argument overload):      */
/* BDF2 diagonal/RHS :222-260, internal faces :262-606, boundary :611-755,    */
/* update + norm :770-793.  COO order as for the momentum equation (drops of  */
/* |a| < DBL_MIN).  Old (n-1) and second-old VF come from arrays oldVF and    */
/* old2VF (default: the current VF).                                          */
/* ------------------------------------------------------------------------ */
static void mstacs(orc_ctx* c, const double* gVF, double* fl, double* fr) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    double *U = dget(c, "U"), *V = dget(c, "V"), *W = dget(c, "W"), *VF = dget(c, "VF");
    double *fa = dget(c, "face_area"), *vol = dget(c, "cell_vol"), *cc = dget(c, "cell_c");
    double *fn = dget(c, "face_n"), *wc = dget(c, "face_wC"), *sk = dget(c, "face_skew");
    int *cfp = iget(c, "cf_ptr"), *cfi = iget(c, "cf_idx");
    const double eps = 1.e-12;
    double* co = (double*)malloc(sizeof(double) * nc);
    for (int i = 0; i < nc; ++i) {
        double magVel = sqrt(U[i] * U[i] + V[i] * V[i] + W[i] * W[i]);
        double maxA = 0.0;
        for (int k = cfp[i]; k < cfp[i + 1]; ++k) maxA = smax(maxA, fa[cfi[k]]);
        co[i] = 1.0 / 1.0 * magVel * c->dt * maxA / vol[i];
    }
    for (int f = 0; f < ni; ++f) {
        int o = c->own[f], q = c->nei[f];
        double wCL = wc[f], wCR = 1.0 - wCL;
        double L1 = VF[o], R1 = VF[q];
        const double* dL = gVF + 3 * o; const double* dR = gVF + 3 * q;
        double coDDL = co[o], coDDR = co[q];
        double pn[3] = {cc[3 * q] - cc[3 * o], cc[3 * q + 1] - cc[3 * o + 1], cc[3 * q + 2] - cc[3 * o + 2]};
        double L2 = 0.0; for (int k = 0; k < 3; ++k) L2 += dL[k] * pn[k];
        L2 = R1 - 2.0 * L2;
        double R2 = 0.0; for (int k = 0; k < 3; ++k) R2 += dR[k] * pn[k];
        R2 = L1 + 2.0 * R2;
        L2 = smax(0.0, smin(1.0, L2));
        R2 = smax(0.0, smin(1.0, R2));
        double vfL = L1, vfR = R1;
        const double* n = fn + 3 * f; const double* s = sk + 3 * f;
        for (int LR = 0; LR < 2; ++LR) {
            if (LR == 0 && (vfL > 1.0 - eps || vfL < eps)) continue;
            if (LR == 1 && (vfR > 1.0 - eps || vfR < eps)) continue;
            double alpU, alpD, alpA, coDD;
            if (LR == 0) { alpU = L2; alpD = L1; alpA = R1; }
            else { alpU = R2; alpD = R1; alpA = L1; }
            coDD = smax(coDDL, coDDR);
            double m[3] = {wCL * dL[0] + wCR * dR[0], wCL * dL[1] + wCR * dR[1], wCL * dL[2] + wCR * dR[2]};
            double mag = m[0] * m[0]; mag += m[1] * m[1]; mag += m[2] * m[2];
            mag = sqrt(mag);
            for (int k = 0; k < 3; ++k) m[k] = m[k] / (mag + 1.e-200);
            double cosTheta = m[0] * n[0]; cosTheta += m[1] * n[1]; cosTheta += m[2] * n[2];
            cosTheta = fabs(cosTheta);
            double gamF = smin(pow(cosTheta, 4.0), 1.0);
            double tildeCd = (alpD - alpU) / (fabs(alpA - alpU) + 1.e-200) * (alpA > alpU ? 1.0 : -1.0);
            double gamma_f;
            if (tildeCd >= 0.0 && tildeCd < 1.0) {
                if (coDD > 0.0 && coDD <= 0.33) {
                    double tildeCf = smin(1.0, tildeCd / coDD);
                    gamma_f = (tildeCf - tildeCd) / (1.0 - tildeCd);
                } else if (coDD > 0.33 && coDD <= 1.0) {
                    double tildeCf = smin(1.0, 3.0 * tildeCd);
                    gamma_f = (tildeCf - tildeCd) / (1.0 - tildeCd);
                } else gamma_f = 0.0;
            } else gamma_f = 0.0;
            if (LR == 0) gamma_f *= 2.0 * wCR;
            if (LR == 1) gamma_f *= 2.0 * wCL;
            gamma_f = smax(0.0, smin(1.0, gamma_f));
            double vfC = alpD + gamma_f * (alpA - alpD);
            for (int k = 0; k < 3; ++k) vfC += wCL * dL[k] * s[k];
            for (int k = 0; k < 3; ++k) vfC += wCR * dR[k] * s[k];
            vfC = smax(0.0, smin(1.0, vfC));
            if (tildeCd >= 0.0 && tildeCd < 0.2) {
                double tildeCf = smin(1.0, 3.0 * tildeCd);
                gamma_f = (tildeCf - tildeCd) / (1.0 - tildeCd);
            } else if (tildeCd >= 0.2 && tildeCd < 0.5) {
                double tildeCf = 0.5 + 0.5 * tildeCd;
                gamma_f = (tildeCf - tildeCd) / (1.0 - tildeCd);
            } else if (tildeCd >= 0.5 && tildeCd < 0.8333) {
                double tildeCf = 0.375 + 0.75 * tildeCd;
                gamma_f = (tildeCf - tildeCd) / (1.0 - tildeCd);
            } else if (tildeCd >= 0.8333 && tildeCd < 1.0) {
                double tildeCf = 1.0;
                gamma_f = (tildeCf - tildeCd) / (1.0 - tildeCd);
            } else gamma_f = 0.0;
            if (LR == 0) gamma_f *= 2.0 * wCR;
            if (LR == 1) gamma_f *= 2.0 * wCL;
            gamma_f = smax(0.0, smin(1.0, gamma_f));
            double vfD = alpD + gamma_f * (alpA - alpD);
            for (int k = 0; k < 3; ++k) vfD += wCL * dL[k] * s[k];
            for (int k = 0; k < 3; ++k) vfD += wCR * dR[k] * s[k];
            vfD = smax(0.0, smin(1.0, vfD));
            double vf = gamF * vfC + (1.0 - gamF) * vfD;
            if (LR == 0) vfL = vf;
            if (LR == 1) vfR = vf;
        }
        fl[f] = vfL; fr[f] = vfR;
    }
    free(co);
}

void orc_assemble_vof(orc_ctx* c) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    face_values(c);
    gravity_source(c);
    double *P = dget(c, "P"), *U = dget(c, "U"), *V = dget(c, "V"), *W = dget(c, "W"), *VF = dget(c, "VF");
    double *rho = dget(c, "rho"), *sg = dget(c, "src_grav"), *vol = dget(c, "cell_vol");
    double* mm = dreg(c, "vof_minmax_uvw", 6LL * nc);
    double *t1 = (double*)malloc(sizeof(double) * nc), *t2 = (double*)malloc(sizeof(double) * nc);
    minmax(c, U, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i] = t1[i]; mm[6 * i + 1] = t2[i]; }
    minmax(c, V, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i + 2] = t1[i]; mm[6 * i + 3] = t2[i]; }
    minmax(c, W, t1, t2); for (int i = 0; i < nc; ++i) { mm[6 * i + 4] = t1[i]; mm[6 * i + 5] = t2[i]; }
    free(t1); free(t2);
    double *pr = dget(c, "face_pR"), *ur = dget(c, "face_uR"), *vr = dget(c, "face_vfR");
    double* tmp = (double*)malloc(sizeof(double) * nf);
    double* gP = dreg(c, "vof_grad_P", 3LL * nc); lsq_grad(c, P, pr, gP);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f];
    double* gU = dreg(c, "vof_grad_U", 3LL * nc); lsq_grad(c, U, tmp, gU);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f + 1];
    double* gV = dreg(c, "vof_grad_V", 3LL * nc); lsq_grad(c, V, tmp, gV);
    for (int f = 0; f < nf; ++f) tmp[f] = ur[3 * f + 2];
    double* gW = dreg(c, "vof_grad_W", 3LL * nc); lsq_grad(c, W, tmp, gW);
    double* gVF = dreg(c, "vof_grad_VF", 3LL * nc); lsq_grad(c, VF, vr, gVF);
    free(tmp);
    /* MSTACS face values; boundary faces keep the zero-order ones */
    double *fl = dreg(c, "vof_face_vfL", nf), *fr = dreg(c, "vof_face_vfR", nf);
    double* vl0 = dget(c, "face_vfL");
    for (int f = ni; f < nf; ++f) { fl[f] = vl0[f]; fr[f] = vr[f]; }
    mstacs(c, gVF, fl, fr);

    double* oVF = hist(c, "oldVF", VF); double* o2VF = hist(c, "old2VF", VF);
    const double dt = c->dt;
    int cap = nc + 2 * ni;
    int* ar = ireg(c, "vof_A_rows", cap); int* acl = ireg(c, "vof_A_cols", cap);
    double* av = dreg(c, "vof_A_vals", cap);
    double* B = dreg(c, "vof_B", nc);
    for (int i = 0; i < nc; ++i) {
        double volume = vol[i];
        ar[i] = i; acl[i] = i;
        av[i] = 1.5 * volume / dt;
        B[i] = -(1.5 * VF[i] - 2.0 * oVF[i] + 0.5 * o2VF[i]) * volume / dt;
    }
    double *fn = dget(c, "face_n"), *fa = dget(c, "face_area"), *wc = dget(c, "face_wC");
    double *mpn = dget(c, "face_magPN"), *al = dget(c, "face_alphaF"), *epn = dget(c, "face_ePN");
    double *sk = dget(c, "face_skew"), *ul = dget(c, "face_uL"), *rl = dget(c, "face_rhoL");
    double* unf = dreg(c, "vof_face_UnF", nf);
    int nnz = nc;
    for (int f = 0; f < ni; ++f) {
        int o = c->own[f], q = c->nei[f];
        const double* n = fn + 3 * f; const double* e = epn + 3 * f; const double* s = sk + 3 * f;
        double area = fa[f], wCL = wc[f], wCR = 1.0 - wCL;
        double RhoL = rho[o], RhoR = rho[q], PL = P[o], PR = P[q];
        double dPN = mpn[f], alpha = al[f];
        double ULs = U[o], VLs = V[o], WLs = W[o], URs = U[q], VRs = V[q], WRs = W[q];
        for (int k = 0; k < 3; ++k) {
            ULs += gU[3 * o + k] * s[k]; URs += gU[3 * q + k] * s[k];
            VLs += gV[3 * o + k] * s[k]; VRs += gV[3 * q + k] * s[k];
            WLs += gW[3 * o + k] * s[k]; WRs += gW[3 * q + k] * s[k];
        }
        ULs = smax(mm[6 * o + 1], smin(mm[6 * o + 0], ULs)); URs = smax(mm[6 * q + 1], smin(mm[6 * q + 0], URs));
        VLs = smax(mm[6 * o + 3], smin(mm[6 * o + 2], VLs)); VRs = smax(mm[6 * q + 3], smin(mm[6 * q + 2], VRs));
        WLs = smax(mm[6 * o + 5], smin(mm[6 * o + 4], WLs)); WRs = smax(mm[6 * q + 5], smin(mm[6 * q + 4], WRs));
        double UnL = ULs * n[0] + VLs * n[1] + WLs * n[2];
        double UnR = URs * n[0] + VRs * n[1] + WRs * n[2];
        double UnF = wCL * UnL + wCR * UnR;
        double rs = 1.0 / (wCL / RhoL + wCR / RhoR);
        double tt = dt / rs;
        UnF -= alpha * tt * (PR - PL) / dPN;
        for (int k = 0; k < 3; ++k) {
            UnF -= tt * rs * wCL / RhoL * gP[3 * o + k] * (n[k] - alpha * e[k]);
            UnF -= tt * rs * wCR / RhoR * gP[3 * q + k] * (n[k] - alpha * e[k]);
        }
        for (int k = 0; k < 3; ++k) {
            UnF += tt * rs * wCL / RhoL * gP[3 * o + k] * n[k];
            UnF += tt * rs * wCR / RhoR * gP[3 * q + k] * n[k];
        }
        for (int k = 0; k < 3; ++k) UnF += alpha * tt * rs * c->g[k] * alpha * e[k];
        for (int k = 0; k < 3; ++k) {
            UnF += tt * rs * wCL / RhoL * sg[4 * o + k] * (n[k] - alpha * e[k]);
            UnF += tt * rs * wCR / RhoR * sg[4 * q + k] * (n[k] - alpha * e[k]);
        }
        for (int k = 0; k < 3; ++k) {
            UnF -= alpha * tt * rs * wCL / RhoL * sg[4 * o + k] * n[k];
            UnF -= alpha * tt * rs * wCR / RhoR * sg[4 * q + k] * n[k];
        }
        UnF = sft_unf(c, UnF, o, q, RhoL, RhoR, wCL, wCR, alpha, dPN, n, e);
        unf[f] = UnF;
        double weightL = (UnF > 0.0) ? 1.0 : 0.0;
        double weightR = 1.0 - weightL;
        double VFF_HO = weightL * fl[f] + weightR * fr[f];
        av[o] += (weightL * UnF * area);
        {
            double a = (weightR * UnF * area);
            if (!(fabs(a) < 2.2250738585072014e-308)) { ar[nnz] = o; acl[nnz] = q; av[nnz] = a; ++nnz; }
        }
        av[q] -= (weightR * UnF * area);
        {
            double a = -(weightL * UnF * area);
            if (!(fabs(a) < 2.2250738585072014e-308)) { ar[nnz] = q; acl[nnz] = o; av[nnz] = a; ++nnz; }
        }
        B[o] -= (VFF_HO * UnF * area);
        B[q] += (VFF_HO * UnF * area);
    }
    double* pRf = dget(c, "face_pR");
    for (int f = ni; f < nf; ++f) {
        int p = patch_of(c, f), o = c->own[f];
        const double* n = fn + 3 * f; const double* e = epn + 3 * f;
        double area = fa[f];
        double UnL = ul[3 * f] * n[0] + ul[3 * f + 1] * n[1] + ul[3 * f + 2] * n[2];
        double UnR = ur[3 * f] * n[0] + ur[3 * f + 1] * n[1] + ur[3 * f + 2] * n[2];
        double UnF = 0.5 * UnL + 0.5 * UnR;
        double RhoL = rl[f];
        double tmp1 = 1.0 / RhoL * dt;
        double VFF = 0.5 * fl[f] + 0.5 * fr[f];
        double coeffVF = (c->bct[3 * p + 2] == 1) ? 0.0 : 1.0;   /* fixedValue 0, zeroGradient 1 */
        double dPN = 0.5 * mpn[f], alpha = al[f];
        if (c->bct[3 * p] == 1) {
            double orgPL = P[o], orgPR = pRf[f];
            UnF -= alpha * tmp1 * (orgPR - orgPL) / dPN;
            for (int k = 0; k < 3; ++k) UnF += alpha * tmp1 * gP[3 * o + k] * e[k];
        }
        unf[f] = UnF;
        av[o] += coeffVF * (UnF * area);
        B[o] -= (VFF * UnF * area);
    }
    orc_arr* a;
    a = find(c, "vof_A_rows"); a->n = nnz;
    a = find(c, "vof_A_cols"); a->n = nnz;
    a = find(c, "vof_A_vals"); a->n = nnz;
    int* ptr = ireg(c, "vof_csr_ptr", nc + 1); int* col = ireg(c, "vof_csr_col", nnz);
    double* val = dreg(c, "vof_csr_val", nnz);
    for (int k = 0; k < nnz; ++k) ptr[ar[k]]++;
    for (int i = 0, s2 = 0; i < nc; ++i) { int t = ptr[i]; ptr[i] = s2; s2 += t; }
    ptr[nc] = nnz;
    for (int k = 0; k < nnz; ++k) { int d = ptr[ar[k]]++; col[d] = acl[k]; val[d] = av[k]; }
    for (int i = 0, last = 0; i <= nc; ++i) { int t = ptr[i]; ptr[i] = last; last = t; }
}

int orc_solve_vof(orc_ctx* c, double tol, int maxiter, double* out_x, double* out_relres) {
    return bicgstab_jacobi(c->nc, iget(c, "vof_csr_ptr"), iget(c, "vof_csr_col"), dget(c, "vof_csr_val"),
                           dget(c, "vof_B"), tol, maxiter, out_x, out_relres);
}

/* eqVolfrac.cpp:770-793: VF += urf x, clamp to [0, 1]; returns sqrt(sum x^2) */
double orc_update_vof(orc_ctx* c, const double* x) {
    double* VF = dget(c, "VF");
    double nd = 0.0;
    for (int i = 0; i < c->nc; ++i) {
        VF[i] += c->urf_vof * x[i];
        VF[i] = smax(0.0, smin(1.0, VF[i]));
        nd += x[i] * x[i];
    }
    return sqrt(nd);
}

/* ======================================================================== */
/* Compressible coupled 5x5 block system.                                    */
/*                                                                           */
/* The reference's calcCompCoupledEq (src/solvers/compressible/coupled.cpp:  */
/* 8-2711) has its whole body commented out; called by CompCoupled           */
/* (src/solvers/compCoupled.cpp:188) it assembles and solves nothing.  This  */
/* restates the state the body was in when it was last live -- the lines    */
/* under exactly one comment level -- for one species (B_n = 5 unknowns per  */
/* cell: p, u, v, w, T; the mass-fraction row and column of the 6x6 form are */
/* dropped):                                                                 */
/*   cell EOS        eos.cpp:310-437 (calcCellEOSMF, nSp = 1) over           */
/*                   eos.cpp:805-844 (eosIdeal)                              */
/*   face values     zero-order: L = owner, R = neighbour or the boundary    */
/*                   value (reconComp.cpp:1087-1131), face EOS from them     */
/*   gradients       LSQ cellVertex of P, U, V, W (the live calcLeastSquare; */
/*                   the dead body calls the retired calcLeastSquare2nd)     */
/*   cell terms      coupled.cpp:318-625 (diagonal time block, bounded BDF2  */
/*                   right-hand side, gravity)                               */
/*   internal faces  coupled.cpp:631-1936 (AUSM-type face velocity with     */
/*                   Rhie-Chow, upwinded transport, Jacobian blocks, viscous */
/*                   fluxes); the high-order face values equal the zero-     */
/*                   order ones                                              */
/*   boundary faces  coupled.cpp:1945-2368                                   */
/*   update, norm    coupled.cpp:2494-2708                                   */
/* Unpinned: there is no live reference to compare with.  The diagonal time */
/* block is the exact derivative of the first-order part of the right-hand   */
/* side, which the tests check by finite differences; the face blocks are    */
/* the reference's approximate (frozen-coefficient) Jacobian.                */
/*                                                                           */
/* Storage: diagonal blocks cpl_diag[25 i + 5 a + b] (row equation a, column */
/* variable b), off-diagonal blocks per internal face cpl_LR (owner row,     */
/* neighbour column) and cpl_RL (neighbour row, owner column), right-hand    */
/* side field-split cpl_B[a nc + i] as the reference orders it.              */
/* ======================================================================== */
typedef struct { double cv, gam, mu, dt, dto, dto2, g[3], urf; int terms; } cpl_prm_t;
static cpl_prm_t g_cpl = {0, 0, 0, 0, 0, 0, {0, 0, 0}, 0, 7};

/* which parts orc_assemble_coupled adds (tests take them apart):
   1 = cell terms, 2 = internal faces, 4 = boundary faces */
void orc_coupled_terms(int mask) { g_cpl.terms = mask; }

void orc_set_coupled(orc_ctx* c, const double* prm, const int* bct, const double* bcv) {
    g_cpl.cv = prm[0]; g_cpl.gam = prm[1]; g_cpl.mu = prm[2];
    g_cpl.dt = prm[3]; g_cpl.dto = prm[4]; g_cpl.dto2 = prm[5];
    g_cpl.g[0] = prm[6]; g_cpl.g[1] = prm[7]; g_cpl.g[2] = prm[8]; g_cpl.urf = prm[9];
    int* t = ireg(c, "cpl_bct", 3LL * c->npatch); memcpy(t, bct, sizeof(int) * 3 * c->npatch);
    double* v = dreg(c, "cpl_bcv", 5LL * c->npatch); memcpy(v, bcv, sizeof(double) * 5 * c->npatch);
}

/* AUSM split Mach number and pressure polynomials: src/solvers/flux.cpp:924-949 */
static double m_func(double M, double op, double alp) {
    if (fabs(M) > 1.0) return 0.5 * (M + op * fabs(M));
    return op * 0.25 * ((M + op) * (M + op)) + op * alp * ((M * M - 1.0) * (M * M - 1.0));
}
static double pre_func(double M, double op, double alp) {
    if (fabs(M) > 1.0) return 0.5 * (1.0 + op * (M > 0.0 ? 1.0 : -1.0));
    return 0.25 * ((M + op) * (M + op)) * (2.0 - op * M) + op * alp * M * ((M * M - 1.0) * (M * M - 1.0));
}

/* eosIdeal (eos.cpp:805-844) folded through calcCellEOSMF with one species
   (eos.cpp:310-437): out = rho, C, Ht, drho/dp, drho/dT, dHt/dp, dHt/dT */
static void eos_ideal1(double cv, double gam, double P, double U, double V, double W, double T, double* o) {
    double usqrt = U * U + V * V + W * W;
    double ri = 1.0 / ((gam - 1.0) * cv * T / (P));
    double dri_p = ri * ri * (1.0 / ri) / (P);
    double dri_t = -ri * ri * (1.0 / ri) / T;
    double dhi_p = 0.0, dhi_t = gam * cv;
    double hti = gam * cv * T + 0.5 * usqrt;
    double mf = smax(0.0, smin(1.0, 1.0 - 0.0));
    double rho = 0.0; rho += mf / ri; rho = 1.0 / rho;
    double ht = 0.0, drdp = 0.0, drdt = 0.0, dhdp = 0.0, dhdt = 0.0;
    ht += mf * hti;
    drdp += rho * rho * (mf / ri / ri * dri_p);
    drdt += rho * rho * (mf / ri / ri * dri_t);
    dhdp += mf * dhi_p;
    dhdt += mf * dhi_t;
    double cc = drdp + 1.0 / rho * drdt / dhdt * (1.0 - rho * dhdp);
    o[0] = rho; o[1] = sqrt(1.0 / cc); o[2] = ht; o[3] = drdp; o[4] = drdt; o[5] = dhdp; o[6] = dhdt;
}

/* boundary right-state primitives (P, U, V, W, T) of boundary face f */
static void cpl_bvalue(orc_ctx* c, int f, const double* cellv, double* r) {
    int p = patch_of(c, f);
    const int* t = iget(c, "cpl_bct") + 3 * p; const double* bv = dget(c, "cpl_bcv") + 5 * p;
    const double* n = dget(c, "face_n") + 3 * f;
    r[0] = (t[0] == 1) ? bv[0] : cellv[0];
    if (t[1] == 1) { r[1] = bv[1]; r[2] = bv[2]; r[3] = bv[3]; }
    else if (t[1] == 2) { r[1] = 0.0; r[2] = 0.0; r[3] = 0.0; }
    else if (t[1] == 3) {
        double un = cellv[1] * n[0] + cellv[2] * n[1] + cellv[3] * n[2];
        r[1] = cellv[1] - un * n[0]; r[2] = cellv[2] - un * n[1]; r[3] = cellv[3] - un * n[2];
    } else { r[1] = cellv[1]; r[2] = cellv[2]; r[3] = cellv[3]; }
    r[4] = (t[2] == 1) ? bv[4] : cellv[4];
}

void orc_assemble_coupled(orc_ctx* c) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    const cpl_prm_t* q = &g_cpl;
    double *P = dget(c, "cpl_P"), *U = dget(c, "cpl_U"), *V = dget(c, "cpl_V"), *W = dget(c, "cpl_W"), *T = dget(c, "cpl_T");
    double *old = dget(c, "cpl_old"), *old2 = dget(c, "cpl_old2");   /* 5 nc each: P, U, V, W, T planes */
    double *fn = dget(c, "face_n"), *fa = dget(c, "face_area"), *wc = dget(c, "face_wC");
    double *mpn = dget(c, "face_magPN"), *alf = dget(c, "face_alphaF"), *epn = dget(c, "face_ePN");
    double *skw = dget(c, "face_skew"), *vol = dget(c, "cell_vol");
    /* cell EOS */
    double* eos = dreg(c, "cpl_eos", 7LL * nc);
    for (int i = 0; i < nc; ++i) eos_ideal1(q->cv, q->gam, P[i], U[i], V[i], W[i], T[i], eos + 7 * i);
    /* boundary right states + their EOS */
    int nb = nf - ni;
    double* bR = dreg(c, "cpl_bR", 5LL * (nb > 0 ? nb : 1));
    double* bE = dreg(c, "cpl_bE", 7LL * (nb > 0 ? nb : 1));
    for (int f = ni; f < nf; ++f) {
        int o = c->own[f];
        double cv5[5] = {P[o], U[o], V[o], W[o], T[o]};
        double* r = bR + 5 * (f - ni);
        cpl_bvalue(c, f, cv5, r);
        eos_ideal1(q->cv, q->gam, r[0], r[1], r[2], r[3], r[4], bE + 7 * (f - ni));
    }
    /* gradients of P, U, V, W (boundary phi_f = right state) */
    double* phR = (double*)calloc((size_t)nf, sizeof(double));
    double* gr[4]; const char* gn[4] = {"cpl_grad_P", "cpl_grad_U", "cpl_grad_V", "cpl_grad_W"};
    double* fld[4] = {P, U, V, W};
    for (int k = 0; k < 4; ++k) {
        for (int f = ni; f < nf; ++f) phR[f] = bR[5 * (f - ni) + k];
        gr[k] = dreg(c, gn[k], 3LL * nc);
        lsq_grad(c, fld[k], phR, gr[k]);
    }
    free(phR);
    double* D = dreg(c, "cpl_diag", 25LL * nc);
    double* LR = dreg(c, "cpl_LR", 25LL * (ni > 0 ? ni : 1));
    double* RL = dreg(c, "cpl_RL", 25LL * (ni > 0 ? ni : 1));
    double* B = dreg(c, "cpl_B", 5LL * nc);
    const double dt = q->dt; const double* g = q->g;
    /* ---- cell terms: coupled.cpp:318-625 ---- */
    for (int i = 0; i < nc && (g_cpl.terms & 1); ++i) {
        const double* e = eos + 7 * i;
        double Rho = e[0], Ht = e[2], dRhoDP = e[3], dRhoDT = e[4], dHtDP = e[5], dHtDT = e[6];
        double eo[7], eo2[7];
        eos_ideal1(q->cv, q->gam, old[i], old[nc + i], old[2 * nc + i], old[3 * nc + i], old[4 * nc + i], eo);
        eos_ideal1(q->cv, q->gam, old2[i], old2[nc + i], old2[2 * nc + i], old2[3 * nc + i], old2[4 * nc + i], eo2);
        double volume = vol[i], cTime = 1.0;
        double u = U[i], v = V[i], w = W[i];
        double* d = D + 25 * i;
        d[0 * 5 + 0] = cTime * (dRhoDP) * volume / dt;
        d[0 * 5 + 4] = cTime * (dRhoDT) * volume / dt;
        double vel[3] = {u, v, w};
        for (int m = 1; m <= 3; ++m) {
            d[m * 5 + 0] = cTime * (dRhoDP * vel[m - 1]) * volume / dt;
            d[m * 5 + 0] -= dRhoDP * g[m - 1] * volume;
            d[m * 5 + m] = cTime * (Rho) * volume / dt;
            d[m * 5 + 4] = cTime * (dRhoDT * vel[m - 1]) * volume / dt;
            d[m * 5 + 4] -= dRhoDT * g[m - 1] * volume;
        }
        d[4 * 5 + 0] = cTime * (dRhoDP * Ht + dHtDP * Rho - 1.0) * volume / dt;
        d[4 * 5 + 0] -= dRhoDP * (g[0] * u + g[1] * v + g[2] * w) * volume;
        for (int k = 0; k < 3; ++k) {
            d[4 * 5 + 1 + k] = cTime * (Rho * vel[k]) * volume / dt;
            d[4 * 5 + 1 + k] -= Rho * (g[k]) * volume;
        }
        d[4 * 5 + 4] = cTime * (dRhoDT * Ht + dHtDT * Rho) * volume / dt;
        d[4 * 5 + 4] -= dRhoDT * (g[0] * u + g[1] * v + g[2] * w) * volume;
        double cn[5], c1[5], c2[5];
        cn[0] = Rho; c1[0] = eo[0]; c2[0] = eo2[0];
        cn[1] = Rho * u; c1[1] = eo[0] * old[nc + i]; c2[1] = eo2[0] * old2[nc + i];
        cn[2] = Rho * v; c1[2] = eo[0] * old[2 * nc + i]; c2[2] = eo2[0] * old2[2 * nc + i];
        cn[3] = Rho * w; c1[3] = eo[0] * old[3 * nc + i]; c2[3] = eo2[0] * old2[3 * nc + i];
        cn[4] = Rho * Ht - P[i]; c1[4] = eo[0] * eo[2] - old[i]; c2[4] = eo2[0] * eo2[2] - old2[i];
        double beta = 1.0;
        for (int a = 0; a < 5; ++a) {
            double sou = (c1[a] - c2[a]) / (cn[a] - c2[a] + 1.e-200);
            if (0.0 < sou && sou < 1.0) beta = smin(beta, 0.0); else beta = smin(beta, 1.0);
        }
        for (int a = 0; a < 5; ++a) {
            double co1 = q->dto / (dt + q->dto);
            double co2 = q->dto2 / (q->dto + q->dto2);
            double np12 = cn[a] + beta * co1 * (cn[a] - c1[a]);
            double nm12 = c1[a] + beta * co2 * (c1[a] - c2[a]);
            B[(size_t)a * nc + i] = -(np12 - nm12) * volume / dt;
        }
        B[(size_t)1 * nc + i] += Rho * g[0] * volume;
        B[(size_t)2 * nc + i] += Rho * g[1] * volume;
        B[(size_t)3 * nc + i] += Rho * g[2] * volume;
        B[(size_t)4 * nc + i] += Rho * (g[0] * u + g[1] * v + g[2] * w) * volume;
    }
    /* ---- internal faces: coupled.cpp:631-1936 ---- */
    for (int f = 0; f < ni && (g_cpl.terms & 2); ++f) {
        int o = c->own[f], r = c->nei[f];
        const double* n = fn + 3 * f;
        double area = fa[f], wCL = wc[f], wCR = 1.0 - wCL;
        const double *eL = eos + 7 * o, *eR = eos + 7 * r;
        double UL = U[o], VL = V[o], WL = W[o], PL = P[o], RhoL = eL[0], CL = eL[1], HtL = eL[2];
        double dRhoDPL = eL[3], dRhoDTL = eL[4], dHtDPL = eL[5], dHtDTL = eL[6], muL = q->mu;
        double UR = U[r], VR = V[r], WR = W[r], PR = P[r], RhoR = eR[0], CR = eR[1], HtR = eR[2];
        double dRhoDPR = eR[3], dRhoDTR = eR[4], dHtDPR = eR[5], dHtDTR = eR[6], muR = q->mu;
        double UnL = UL * n[0] + VL * n[1] + WL * n[2];
        double UnR = UR * n[0] + VR * n[1] + WR * n[2];
        double UnF = wCL * UnL + wCR * UnR;
        double muF = wCL * muL + wCR * muR;
        double Rho_star = 1.0 / (wCL / RhoL + wCR / RhoR);
        double tmp1 = dt / Rho_star;
        double dPN = mpn[f], alpha = alf[f];
        const double *ep = epn + 3 * f, *sk = skw + 3 * f;
        const double *gPL = gr[0] + 3 * o, *gPR = gr[0] + 3 * r;
        const double *gUL = gr[1] + 3 * o, *gUR = gr[1] + 3 * r;
        const double *gVL = gr[2] + 3 * o, *gVR = gr[2] + 3 * r;
        const double *gWL = gr[3] + 3 * o, *gWR = gr[3] + 3 * r;
        double UnF_RC = 0.0;
        UnF_RC -= alpha * tmp1 * (PR - PL) / dPN;
        for (int ii = 0; ii < 3; ++ii) {
            UnF_RC += alpha * tmp1 * Rho_star * wCL / RhoL * gPL[ii] * ep[ii];
            UnF_RC += alpha * tmp1 * Rho_star * wCR / RhoR * gPR[ii] * ep[ii];
        }
        for (int ii = 0; ii < 3; ++ii) UnF_RC -= alpha * tmp1 * (gPR[ii] - gPL[ii]) * sk[ii] / dPN;
        double Cbar = 0.5 * (CL + CR);
        double ML = UnL / Cbar, MR = UnR / Cbar;
        double MLP = m_func(ML, 1.0, 0.125), MRM = m_func(MR, -1.0, 0.125);
        double PLP = pre_func(ML, 1.0, 0.1875), PRM = pre_func(MR, -1.0, 0.1875);
        double KLR = sqrt(0.5 * (UL * UL + VL * VL + WL * WL + UR * UR + VR * VR + WR * WR));
        double Mdash = smin(1.0, KLR / Cbar);
        double chi = (1.0 - Mdash) * (1.0 - Mdash);
        double rhohat = 0.5 * (RhoL + RhoR);
        UnF = (MLP + MRM) * Cbar + UnF_RC - 0.5 * chi / rhohat / Cbar * (PR - PL);
        double weightL = (UnF > 0.0) ? 1.0 : 0.0, weightR = 1.0 - weightL;
        double WUL, WUR;
        if (fabs(ML) > 1.0) WUL = 0.5 * (1.0 + ((ML > 0.0) ? 1.0 : -1.0));
        else WUL = 0.5 * (ML + 1.0) + 0.125 * 2.0 * 2.0 * (ML * ML - 1.0);
        if (fabs(MR) > 1.0) WUR = 0.5 * (1.0 - ((MR > 0.0) ? 1.0 : -1.0));
        else WUR = -0.5 * (MR - 1.0) - 0.125 * 2.0 * 2.0 * (MR * MR - 1.0);
        double WPL = 0.5 - 0.5 * Mdash * PLP * PRM * 0.5 / Cbar * (UnR - UnL) + 0.5 * Mdash * (PLP + PRM - 1.0) + 0.5 * (PLP - PRM);
        double WPR = 0.5 - 0.5 * Mdash * PLP * PRM * 0.5 / Cbar * (UnR - UnL) + 0.5 * Mdash * (PLP + PRM - 1.0) - 0.5 * (PLP - PRM);
        double diffPDU = 0.0;
        double diffDP = alpha * tmp1 / dPN + 0.5 * chi / rhohat / Cbar;
        double UF = weightL * UL + weightR * UR, VF = weightL * VL + weightR * VR, WF = weightL * WL + weightR * WR;
        double RhoF = weightL * RhoL + weightR * RhoR, HtF = weightL * HtL + weightR * HtR;
        double PF = WPL * PL + WPR * PR;
        double dU[3] = {0, 0, 0}, dV[3] = {0, 0, 0}, dW[3] = {0, 0, 0};
        double dUdn = 0.0, dVdn = 0.0, dWdn = 0.0;
        for (int ii = 0; ii < 3; ++ii) {
            dU[ii] += wCL * gUL[ii]; dU[ii] += wCR * gUR[ii];
            dV[ii] += wCL * gVL[ii]; dV[ii] += wCR * gVR[ii];
            dW[ii] += wCL * gWL[ii]; dW[ii] += wCR * gWR[ii];
            double tvec = n[ii] - alpha * ep[ii];
            dUdn += wCL * gUL[ii] * tvec; dUdn += wCR * gUR[ii] * tvec;
            dVdn += wCL * gVL[ii] * tvec; dVdn += wCR * gVR[ii] * tvec;
            dWdn += wCL * gWL[ii] * tvec; dWdn += wCR * gWR[ii] * tvec;
            dUdn += alpha * (gUR[ii] - gUL[ii]) * sk[ii] / dPN;
            dVdn += alpha * (gVR[ii] - gVL[ii]) * sk[ii] / dPN;
            dWdn += alpha * (gWR[ii] - gWL[ii]) * sk[ii] / dPN;
        }
        dUdn += alpha * (UR - UL) / dPN; dVdn += alpha * (VR - VL) / dPN; dWdn += alpha * (WR - WL) / dPN;
        double dv3 = dU[0] + dV[1] + dW[2];
        double txx = dU[0] - 2.0 / 3.0 * dv3, txy = dV[0], txz = dW[0];
        double tyx = dU[1], tyy = dV[1] - 2.0 / 3.0 * dv3, tyz = dW[1];
        double tzx = dU[2], tzy = dV[2], tzz = dW[2] - 2.0 / 3.0 * dv3;
        double diff_viscous = muF * alpha / dPN;
        double visc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        visc[1] = muF * (txx * n[0] + txy * n[1] + txz * n[2] + dUdn) * area;
        visc[2] = muF * (tyx * n[0] + tyy * n[1] + tyz * n[2] + dVdn) * area;
        visc[3] = muF * (tzx * n[0] + tzy * n[1] + tzz * n[2] + dWdn) * area;
        visc[4] = muF * (txx * UF + txy * VF + txz * WF + dU[0] * UF + dU[1] * VF + dU[2] * WF) * n[0] * area +
                  muF * (tyx * UF + tyy * VF + tyz * WF + dV[0] * UF + dV[1] * VF + dV[2] * WF) * n[1] * area +
                  muF * (tzx * UF + tzy * VF + tzz * WF + dW[0] * UF + dW[1] * VF + dW[2] * WF) * n[2] * area;
        /* high-order values equal the zero-order ones */
        double RhoF_HO = weightL * RhoL + weightR * RhoR, HtF_HO = weightL * HtL + weightR * HtR;
        RhoF = RhoF_HO; HtF = HtF_HO;
        double cL[25], cR[25];
        memset(cL, 0, sizeof cL); memset(cR, 0, sizeof cR);
        cL[0] = (weightL * dRhoDPL * UnF * area + RhoF * diffDP * area);
        cR[0] = (weightR * dRhoDPR * UnF * area - RhoF * diffDP * area);
        for (int k = 0; k < 3; ++k) { cL[1 + k] = (RhoF * WUL * n[k] * area); cR[1 + k] = (RhoF * WUR * n[k] * area); }
        cL[4] = (weightL * dRhoDTL * UnF * area);
        cR[4] = (weightR * dRhoDTR * UnF * area);
        double phF[3] = {UF, VF, WF};
        for (int m = 1; m <= 3; ++m) {
            int k = m - 1; double ph = phF[k];
            cL[5 * m + 0] = (weightL * dRhoDPL * UnF * ph * area + WPL * n[k] * area + RhoF * diffDP * ph * area);
            cR[5 * m + 0] = (weightR * dRhoDPR * UnF * ph * area + WPR * n[k] * area - RhoF * diffDP * ph * area);
            cL[5 * m + m] = (RhoF * WUL * n[k] * ph * area + RhoF * UnF * weightL * area + diff_viscous * area +
                             diffPDU * n[k] * n[k] * area);
            cR[5 * m + m] = (RhoF * WUR * n[k] * ph * area + RhoF * UnF * weightR * area - diff_viscous * area -
                             diffPDU * n[k] * n[k] * area);
            cL[5 * m + 4] = (weightL * dRhoDTL * UnF * ph * area);
            cR[5 * m + 4] = (weightR * dRhoDTR * UnF * ph * area);
        }
        double velL[3] = {UL, VL, WL}, velR[3] = {UR, VR, WR};
        cL[20] = (weightL * dRhoDPL * HtF * UnF * area + RhoF * weightL * dHtDPL * UnF * area + RhoF * diffDP * HtF * area);
        cR[20] = (weightR * dRhoDPR * HtF * UnF * area + RhoF * weightR * dHtDPR * UnF * area - RhoF * diffDP * HtF * area);
        for (int k = 0; k < 3; ++k) {
            cL[21 + k] = (RhoF * WUL * n[k] * HtF * area + RhoF * UnF * weightL * velL[k] * area);
            cR[21 + k] = (RhoF * WUR * n[k] * HtF * area + RhoF * UnF * weightR * velR[k] * area);
        }
        cL[24] = (weightL * dRhoDTL * UnF * HtF * area + RhoF * weightL * dHtDTL * UnF * area);
        cR[24] = (weightR * dRhoDTR * UnF * HtF * area + RhoF * weightR * dHtDTR * UnF * area);
        /* the six cross-momentum entries are absent from the reference's last
           live state: they stay zero and are not accumulated */
        double* dO = D + 25 * o; double* dN = D + 25 * r;
        for (int e = 0; e < 25; ++e) {
            LR[25 * (size_t)f + e] = cR[e]; RL[25 * (size_t)f + e] = -cL[e];
            if (e == 7 || e == 8 || e == 11 || e == 13 || e == 16 || e == 17) continue;
            dO[e] += cL[e]; dN[e] -= cR[e];
        }
        double conv[5];
        conv[0] = RhoF_HO * UnF * area;
        conv[1] = RhoF_HO * UnF * UF * area + PF * n[0] * area;
        conv[2] = RhoF_HO * UnF * VF * area + PF * n[1] * area;
        conv[3] = RhoF_HO * UnF * WF * area + PF * n[2] * area;
        conv[4] = RhoF_HO * UnF * HtF_HO * area;
        for (int a = 0; a < 5; ++a) B[(size_t)a * nc + o] -= (conv[a] - visc[a]);
        for (int a = 0; a < 5; ++a) B[(size_t)a * nc + r] += (conv[a] - visc[a]);
    }
    /* ---- boundary faces: coupled.cpp:1945-2368 ---- */
    int* bct = iget(c, "cpl_bct");
    for (int p = 0; p < c->npatch && (g_cpl.terms & 4); ++p) {
        const int* t = bct + 3 * p;
        double cP = (t[0] == 1) ? 0.0 : 1.0, cPd = (t[0] == 1) ? 1.0 : 0.0;
        double cUVW = (t[1] == 0) ? 1.0 : 0.0, cUVWd = (t[1] == 0) ? 0.0 : 1.0;
        double cT = (t[2] == 1) ? 0.0 : 1.0;
        for (int f = c->pstart[p]; f < c->pstart[p] + c->psize[p]; ++f) {
            int o = c->own[f];
            const double* n = fn + 3 * f;
            const double* eL = eos + 7 * o;
            const double* rv = bR + 5 * (f - ni); const double* eR = bE + 7 * (f - ni);
            double area = fa[f];
            double UnL = U[o] * n[0] + V[o] * n[1] + W[o] * n[2];
            double UnR = rv[1] * n[0] + rv[2] * n[1] + rv[3] * n[2];
            double UnF = 0.5 * UnL + 0.5 * UnR;
            double RhoF = 0.5 * eL[0] + 0.5 * eR[0];
            double UF = 0.5 * U[o] + 0.5 * rv[1], VF = 0.5 * V[o] + 0.5 * rv[2], WF = 0.5 * W[o] + 0.5 * rv[3];
            double PF = 0.5 * P[o] + 0.5 * rv[0];
            double dRhoDPF = 0.5 * eL[3] + 0.5 * eR[3], dRhoDTF = 0.5 * eL[4] + 0.5 * eR[4];
            double dHtDPF = 0.5 * eL[5] + 0.5 * eR[5], dHtDTF = 0.5 * eL[6] + 0.5 * eR[6];
            double HtF = 0.5 * eL[2] + 0.5 * eR[2];
            double dPN = 0.5 * mpn[f], alpha = alf[f];
            double RhoL = eL[0];
            double tmp1 = 1.0 / RhoL * dt;
            const double* ep = epn + 3 * f;
            const double *gP = gr[0] + 3 * o, *gU = gr[1] + 3 * o, *gV = gr[2] + 3 * o, *gW = gr[3] + 3 * o;
            UnF -= cPd * alpha * tmp1 * (rv[0] - P[o]) / dPN;
            for (int ii = 0; ii < 3; ++ii) UnF += cPd * alpha * tmp1 * gP[ii] * ep[ii];
            double muF = 0.5 * q->mu + 0.5 * q->mu;
            double dU[3] = {0, 0, 0}, dV[3] = {0, 0, 0}, dW[3] = {0, 0, 0};
            double dUdn = 0.0, dVdn = 0.0, dWdn = 0.0;
            for (int ii = 0; ii < 3; ++ii) {
                dU[ii] += gU[ii]; dV[ii] += gV[ii]; dW[ii] += gW[ii];
                double tvec = n[ii] - alpha * ep[ii];
                dUdn += gU[ii] * tvec; dVdn += gV[ii] * tvec; dWdn += gW[ii] * tvec;
            }
            dUdn += alpha * (rv[1] - U[o]) / dPN; dVdn += alpha * (rv[2] - V[o]) / dPN; dWdn += alpha * (rv[3] - W[o]) / dPN;
            double dv3 = dU[0] + dV[1] + dW[2];
            double txx = dU[0] - 2.0 / 3.0 * dv3, txy = dV[0], txz = dW[0];
            double tyx = dU[1], tyy = dV[1] - 2.0 / 3.0 * dv3, tyz = dW[1];
            double tzx = dU[2], tzy = dV[2], tzz = dW[2] - 2.0 / 3.0 * dv3;
            double visc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
            visc[1] = muF * (txx * n[0] + txy * n[1] + txz * n[2] + dUdn) * area;
            visc[2] = muF * (tyx * n[0] + tyy * n[1] + tyz * n[2] + dVdn) * area;
            visc[3] = muF * (tzx * n[0] + tzy * n[1] + tzz * n[2] + dWdn) * area;
            visc[4] = muF * (txx * UF + txy * VF + txz * WF + dU[0] * UF + dU[1] * VF + dU[2] * WF) * n[0] * area +
                      muF * (tyx * UF + tyy * VF + tyz * WF + dV[0] * UF + dV[1] * VF + dV[2] * WF) * n[1] * area +
                      muF * (tzx * UF + tzy * VF + tzz * WF + dW[0] * UF + dW[1] * VF + dW[2] * WF) * n[2] * area;
            double* d = D + 25 * o;
            double phF[3] = {UF, VF, WF};
            d[0] += cP * (dRhoDPF * UnF * area);
            d[0] += cPd * (RhoF * tmp1 / dPN * area);
            for (int k = 0; k < 3; ++k) d[1 + k] += cUVW * (RhoF * n[k] * area);
            d[4] += cT * (dRhoDTF * UnF * area);
            for (int m = 1; m <= 3; ++m) {
                int k = m - 1; double ph = phF[k];
                d[5 * m + 0] += cP * (dRhoDPF * UnF * ph * area);
                d[5 * m + 0] += cPd * (RhoF * alpha * tmp1 / dPN * ph * area);
                d[5 * m + m] += cUVW * (RhoF * n[k] * ph * area + RhoF * UnF * area);
                d[5 * m + m] += cUVWd * (alpha * muF / dPN * area);
                d[5 * m + 4] += cT * (dRhoDTF * UnF * ph * area);
            }
            d[20] += cP * (dRhoDPF * UnF * HtF * area + RhoF * UnF * dHtDPF * area);
            d[20] += cPd * (RhoF * alpha * tmp1 / dPN * dHtDPF * area);
            for (int k = 0; k < 3; ++k) d[21 + k] += cUVW * (RhoF * n[k] * HtF * area + RhoF * UnF * phF[k] * area);
            d[24] += cT * (dRhoDTF * UnF * HtF * area + RhoF * UnF * dHtDTF * area);
            double conv[5];
            conv[0] = RhoF * UnF * area;
            conv[1] = RhoF * UnF * UF * area + PF * n[0] * area;
            conv[2] = RhoF * UnF * VF * area + PF * n[1] * area;
            conv[3] = RhoF * UnF * WF * area + PF * n[2] * area;
            conv[4] = RhoF * UnF * HtF * area;
            for (int a = 0; a < 5; ++a) B[(size_t)a * nc + o] -= (conv[a] - visc[a]);
        }
    }
}

/* block CSR on the scalar pattern (row i: diagonal, then the internal faces
   of i in face order), 25 values per slot, row-major (equation, variable) */
static void cpl_bsr(orc_ctx* c, double* val) {
    int* dig = iget(c, "CRS_dig"); int* lr = iget(c, "CRS_LR"); int* rl = iget(c, "CRS_RL");
    double *D = dget(c, "cpl_diag"), *LR = dget(c, "cpl_LR"), *RL = dget(c, "cpl_RL");
    for (int i = 0; i < c->nc; ++i) memcpy(val + 25 * (size_t)dig[i], D + 25 * (size_t)i, 25 * sizeof(double));
    for (int f = 0; f < c->ni; ++f) {
        memcpy(val + 25 * (size_t)lr[f], LR + 25 * (size_t)f, 25 * sizeof(double));
        memcpy(val + 25 * (size_t)rl[f], RL + 25 * (size_t)f, 25 * sizeof(double));
    }
}
void orc_coupled_bsr(orc_ctx* c, double* out_val) { cpl_bsr(c, out_val); }

static void inv5(const double* a, double* x) {
    double m[5][10];
    for (int i = 0; i < 5; ++i) for (int j = 0; j < 5; ++j) { m[i][j] = a[5 * i + j]; m[i][5 + j] = (i == j) ? 1.0 : 0.0; }
    for (int k = 0; k < 5; ++k) {
        int p = k; for (int i = k + 1; i < 5; ++i) if (fabs(m[i][k]) > fabs(m[p][k])) p = i;
        if (p != k) for (int j = 0; j < 10; ++j) { double t = m[k][j]; m[k][j] = m[p][j]; m[p][j] = t; }
        double piv = 1.0 / m[k][k];
        for (int j = 0; j < 10; ++j) m[k][j] *= piv;
        for (int i = 0; i < 5; ++i) if (i != k) { double f = m[i][k]; if (f != 0.0) for (int j = 0; j < 10; ++j) m[i][j] -= f * m[k][j]; }
    }
    for (int i = 0; i < 5; ++i) for (int j = 0; j < 5; ++j) x[5 * i + j] = m[i][5 + j];
}
/* y = A x, x and y field-split (x[b nc + j]) */
static void bsr_mv(int nc, const int* ptr, const int* col, const double* val, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nc; ++i) {
        double s[5] = {0, 0, 0, 0, 0};
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
            int j = col[k]; const double* blk = val + 25 * (size_t)k;
            for (int a = 0; a < 5; ++a)
                for (int b = 0; b < 5; ++b) s[a] += blk[5 * a + b] * x[(size_t)b * nc + j];
        }
        for (int a = 0; a < 5; ++a) y[(size_t)a * nc + i] = s[a];
    }
}
static void bjac(int nc, const double* dinv, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nc; ++i) {
        const double* m = dinv + 25 * (size_t)i;
        double v[5]; for (int b = 0; b < 5; ++b) v[b] = x[(size_t)b * nc + i];
        for (int a = 0; a < 5; ++a) { double s = 0.0; for (int b = 0; b < 5; ++b) s += m[5 * a + b] * v[b]; y[(size_t)a * nc + i] = s; }
    }
}
/* right-preconditioned BiCGStab with block-Jacobi (5x5 inverses) in FP64 */
int orc_solve_coupled(orc_ctx* c, double tol, int maxiter, double* out_x, double* out_relres) {
    int nc = c->nc; size_t n = 5 * (size_t)nc;
    int* ptr = iget(c, "CRS_ptr"); int* col = iget(c, "CRS_col"); int* dig = iget(c, "CRS_dig");
    double* val = (double*)malloc(sizeof(double) * 25 * (size_t)ptr[nc]);
    cpl_bsr(c, val);
    double* b = dget(c, "cpl_B");
    double* dinv = (double*)malloc(sizeof(double) * 25 * (size_t)nc);
    for (int i = 0; i < nc; ++i) inv5(val + 25 * (size_t)dig[i], dinv + 25 * (size_t)i);
    double* w = (double*)calloc(7 * n, sizeof(double));
    double *r = w, *rh = w + n, *p = w + 2 * n, *v = w + 3 * n, *s = w + 4 * n, *t = w + 5 * n, *z = w + 6 * n;
    double* x = out_x;
    for (size_t i = 0; i < n; ++i) { x[i] = 0.0; r[i] = b[i]; rh[i] = b[i]; }
    double bn = sqrt(dot(b, b, (int)n));
    if (bn == 0.0) { free(w); free(val); free(dinv); if (out_relres) *out_relres = 0.0; return 0; }
    double rho = 1.0, alpha = 1.0, omega = 1.0, rn = bn;
    int it = 0;
    while (it < maxiter && rn > tol * bn) {
        double rho1 = dot(rh, r, (int)n);
        double beta = (rho1 / rho) * (alpha / omega);
        rho = rho1;
        for (size_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        bjac(nc, dinv, p, z);
        bsr_mv(nc, ptr, col, val, z, v);
        alpha = rho / dot(rh, v, (int)n);
        for (size_t i = 0; i < n; ++i) { x[i] += alpha * z[i]; s[i] = r[i] - alpha * v[i]; }
        bjac(nc, dinv, s, z);
        bsr_mv(nc, ptr, col, val, z, t);
        double tt = dot(t, t, (int)n);
        omega = (tt > 0.0) ? dot(t, s, (int)n) / tt : 0.0;
        for (size_t i = 0; i < n; ++i) { x[i] += omega * z[i]; r[i] = s[i] - omega * t[i]; }
        rn = sqrt(dot(r, r, (int)n));
        ++it;
    }
    bsr_mv(nc, ptr, col, val, x, t);
    double tr = 0.0;
    for (size_t i = 0; i < n; ++i) tr += (b[i] - t[i]) * (b[i] - t[i]);
    if (out_relres) *out_relres = sqrt(tr) / bn;
    free(w); free(val); free(dinv);
    return it;
}

/* coupled.cpp:2494-2708: primitives += urf x (urf = momVelURF for all five),
   clamps, norm = sqrt(sum x^2) / sqrt(sum prim^2) / B_n */
double orc_update_coupled(orc_ctx* c, const double* x, const double* lim) {
    int nc = c->nc;
    double* f[5] = {dget(c, "cpl_P"), dget(c, "cpl_U"), dget(c, "cpl_V"), dget(c, "cpl_W"), dget(c, "cpl_T")};
    double nd = 0.0, np_ = 0.0, urf = g_cpl.urf;
    for (int i = 0; i < nc; ++i) {
        for (int a = 0; a < 5; ++a) f[a][i] += urf * x[(size_t)a * nc + i];
        for (int a = 0; a < 5; ++a) {
            if (f[a][i] <= lim[2 * a]) f[a][i] = lim[2 * a];
            if (f[a][i] >= lim[2 * a + 1]) f[a][i] = lim[2 * a + 1];
        }
        for (int a = 0; a < 5; ++a) nd += x[(size_t)a * nc + i] * x[(size_t)a * nc + i];
        for (int a = 0; a < 5; ++a) np_ += f[a][i] * f[a][i];
    }
    return sqrt(nd) / sqrt(np_) / 5.0;
}

/* ======================================================================== */
/* Curvature and surface-tension source (once per time step):               */
/* src/solvers/source/curvature.cpp:7-3537 (calcCurvature, the live lines:  */
/* 0.5-shifted level set, interface cells, gradient-normalisation, 4 sweeps */
/* of upwind least-squares re-initialisation, normals, divergence of the    */
/* normals; both smoothing loops run 0 times), and                          */
/* src/solvers/source/surfaceTension.cpp:7-120 (calcSourceSurfaceTension:   */
/* LSQ then Gauss-Green gradient of VF, src = sigma kappa grad VF, and      */
/* sigma kappa grad VF . U).  Arrays: kappa, ls, src_sft[4 i + k].          */
/* ======================================================================== */

/* Singular value decomposition A = U W V^T of a 3x3 matrix by Householder
   bidiagonalisation and implicit-shift QR (Golub & Reinsch 1970, in the
   formulation of Numerical Recipes' svdcmp, which src/math/math.cpp:372-585
   follows); a is replaced by U. */
static double hyp2(double a, double b) {
    double x = fabs(a), y = fabs(b);
    if (x > y) return x * sqrt(1.0 + (y / x) * (y / x));
    return (y == 0.0) ? 0.0 : y * sqrt(1.0 + (x / y) * (x / y));
}
static double signed_sqrt(double s, double f) { return -(f > 0.0 ? fabs(sqrt(s)) : -fabs(sqrt(s))); }
static void svd3(double a[3][3], double w[3], double v[3][3]) {
    const int n = 3;
    double rv1[3] = {0, 0, 0};
    double g = 0.0, scale = 0.0, anorm = 0.0, s, f, h, c, x, y, z;
    int l = 0, i, j, k, nm = 0;
    for (i = 0; i < n; i++) {                       /* bidiagonalisation */
        l = i + 1;
        rv1[i] = scale * g;
        g = s = scale = 0.0;
        for (k = i; k < n; k++) scale += fabs(a[k][i]);
        if (scale != 0.0) {
            for (k = i; k < n; k++) { a[k][i] /= scale; s += a[k][i] * a[k][i]; }
            f = a[i][i];
            g = signed_sqrt(s, f);
            h = f * g - s;
            a[i][i] = f - g;
            for (j = l; j < n; j++) {
                for (s = 0.0, k = i; k < n; k++) s += a[k][i] * a[k][j];
                f = s / h;
                for (k = i; k < n; k++) a[k][j] += f * a[k][i];
            }
            for (k = i; k < n; k++) a[k][i] *= scale;
        }
        w[i] = scale * g;
        g = s = scale = 0.0;
        if (i != n - 1) {
            for (k = l; k < n; k++) scale += fabs(a[i][k]);
            if (scale != 0.0) {
                for (k = l; k < n; k++) { a[i][k] /= scale; s += a[i][k] * a[i][k]; }
                f = a[i][l];
                g = signed_sqrt(s, f);
                h = f * g - s;
                a[i][l] = f - g;
                for (k = l; k < n; k++) rv1[k] = a[i][k] / h;
                for (j = l; j < n; j++) {
                    for (s = 0.0, k = l; k < n; k++) s += a[j][k] * a[i][k];
                    for (k = l; k < n; k++) a[j][k] += s * rv1[k];
                }
                for (k = l; k < n; k++) a[i][k] *= scale;
            }
        }
        anorm = smax(anorm, (fabs(w[i]) + fabs(rv1[i])));
    }
    for (i = n - 1; i >= 0; i--) {                  /* right transformations */
        if (i < n - 1) {
            if (g != 0.0) {
                for (j = l; j < n; j++) v[j][i] = (a[i][j] / a[i][l]) / g;
                for (j = l; j < n; j++) {
                    for (s = 0.0, k = l; k < n; k++) s += a[i][k] * v[k][j];
                    for (k = l; k < n; k++) v[k][j] += s * v[k][i];
                }
            }
            for (j = l; j < n; j++) v[i][j] = v[j][i] = 0.0;
        }
        v[i][i] = 1.0;
        g = rv1[i];
        l = i;
    }
    for (i = n - 1; i >= 0; i--) {                  /* left transformations */
        l = i + 1;
        g = w[i];
        for (j = l; j < n; j++) a[i][j] = 0.0;
        if (g != 0.0) {
            g = 1.0 / g;
            for (j = l; j < n; j++) {
                for (s = 0.0, k = l; k < n; k++) s += a[k][i] * a[k][j];
                f = (s / a[i][i]) * g;
                for (k = i; k < n; k++) a[k][j] += f * a[k][i];
            }
            for (j = i; j < n; j++) a[j][i] *= g;
        } else {
            for (j = i; j < n; j++) a[j][i] = 0.0;
        }
        ++a[i][i];
    }
    for (k = n - 1; k >= 0; k--) {                  /* diagonalisation */
        for (int its = 0; its < 30; its++) {
            int flag = 1;
            for (l = k; l >= 0; l--) {
                nm = l - 1;
                if ((fabs(rv1[l]) + anorm) == anorm) { flag = 0; break; }
                if ((fabs(w[nm]) + anorm) == anorm) break;
            }
            if (flag) {
                c = 0.0; s = 1.0;
                for (i = l; i <= k; i++) {
                    f = s * rv1[i];
                    rv1[i] = c * rv1[i];
                    if ((fabs(f) + anorm) == anorm) break;
                    g = w[i];
                    h = hyp2(f, g);
                    w[i] = h;
                    h = 1.0 / h;
                    c = g * h;
                    s = -f * h;
                    for (j = 0; j < n; j++) {
                        y = a[j][nm]; z = a[j][i];
                        a[j][nm] = y * c + z * s;
                        a[j][i] = z * c - y * s;
                    }
                }
            }
            z = w[k];
            if (l == k) {
                if (z < 0.0) { w[k] = -z; for (j = 0; j < n; j++) v[j][k] = -v[j][k]; }
                break;
            }
            x = w[l];
            nm = k - 1;
            y = w[nm];
            g = rv1[nm];
            h = rv1[k];
            f = ((y - z) * (y + z) + (g - h) * (g + h)) / (2.0 * h * y);
            g = hyp2(f, 1.0);
            f = ((x - z) * (x + z) + h * ((y / (f + (f > 0.0 ? fabs(g) : -fabs(g)))) - h)) / x;
            c = s = 1.0;
            for (j = l; j <= nm; j++) {
                i = j + 1;
                g = rv1[i]; y = w[i];
                h = s * g; g = c * g;
                z = hyp2(f, h);
                rv1[j] = z;
                c = f / z; s = h / z;
                f = x * c + g * s;
                g = g * c - x * s;
                h = y * s;
                y *= c;
                for (int jj = 0; jj < n; jj++) {
                    x = v[jj][j]; z = v[jj][i];
                    v[jj][j] = x * c + z * s;
                    v[jj][i] = z * c - x * s;
                }
                z = hyp2(f, h);
                w[j] = z;
                if (z != 0.0) { z = 1.0 / z; c = f * z; s = h * z; }
                f = c * g + s * y;
                x = c * y - s * g;
                for (int jj = 0; jj < n; jj++) {
                    y = a[jj][j]; z = a[jj][i];
                    a[jj][j] = y * c + z * s;
                    a[jj][i] = z * c - y * s;
                }
            }
            rv1[l] = 0.0;
            rv1[k] = f;
            w[k] = x;
        }
    }
}
/* out = a b for 3x3 (row i, column j, sum over m in order) */
static void mm3(double a[3][3], double b[3][3], double out[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double t = 0.0;
            for (int m = 0; m < 3; ++m) t += a[i][m] * b[m][j];
            out[i][j] = t;
        }
}

/* upwind weight of face f for cell side (owner: sign -1 on the distance) */
static double reinit_weight(double vel0, const double* nv, const double* d, double side) {
    double sgn = (vel0 > 0.0 ? 1.0 : -1.0);
    double wk = 0.0;
    wk += sgn * nv[0] * (side * d[0]);
    wk += sgn * nv[1] * (side * d[1]);
    wk += sgn * nv[2] * (side * d[2]);
    wk = pow(1.0 * wk, 1.0);
    return smax(1.e-5, wk);
}

void orc_curvature(orc_ctx* c) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    double* VF = dget(c, "VF");
    double *wc = dget(c, "face_wC"), *fa = dget(c, "face_area"), *dist = dget(c, "face_dist");
    double *vol = dget(c, "cell_vol"), *cc = dget(c, "cell_c"), *fc = dget(c, "face_c");
    int *cfp = iget(c, "cf_ptr"), *cfi = iget(c, "cf_idx");
    int *sp = iget(c, "stencil_ptr"), *si = iget(c, "stencil_idx");
    double* sa = (double*)malloc(sizeof(double) * nc);        /* smoothAi */
    for (int i = 0; i < nc; ++i) sa[i] = VF[i];
    /* interface cells: the 0.5 level crosses between a cell and one of its faces */
    double* fsa = (double*)malloc(sizeof(double) * nf);
    for (int f = 0; f < nf; ++f) {
        double wL = wc[f], wR = 1.0 - wL;
        fsa[f] = (f < ni) ? wL * sa[c->own[f]] + wR * sa[c->nei[f]] : sa[c->own[f]];
    }
    char* iface = (char*)calloc(nc, 1);
    for (int f = 0; f < nf; ++f) {
        if ((sa[c->own[f]] - 0.5) * (fsa[f] - 0.5) <= 0.0) iface[c->own[f]] = 1;
        if (f < ni && (sa[c->nei[f]] - 0.5) * (fsa[f] - 0.5) <= 0.0) iface[c->nei[f]] = 1;
    }
    for (int i = 0; i < nc; ++i) sa[i] = sa[i] - 0.5;
    double* phiR = (double*)malloc(sizeof(double) * nf);
    double* g = (double*)malloc(sizeof(double) * 3 * nc);
#define LSQ_INPUT(phi, out)                                                    \
    do {                                                                       \
        for (int f_ = ni; f_ < nf; ++f_) phiR[f_] = (phi)[c->own[f_]];         \
        lsq_grad(c, (phi), phiR, (out));                                       \
    } while (0)
    LSQ_INPUT(sa, g);
    for (int i = 0; i < nc; ++i)
        if (iface[i]) {
            double mg = 0.0;
            mg += g[3 * i] * g[3 * i]; mg += g[3 * i + 1] * g[3 * i + 1]; mg += g[3 * i + 2] * g[3 * i + 2];
            if (mg > 1.0) sa[i] = sa[i] / mg;
        }
    double* tau = (double*)malloc(sizeof(double) * nc);
    for (int i = 0; i < nc; ++i) {
        double maxA = 0.0;
        for (int k = cfp[i]; k < cfp[i + 1]; ++k) maxA = smax(maxA, fa[cfi[k]]);
        tau[i] = vol[i] / maxA / 1.0;
        tau[i] = smin(tau[i], pow(vol[i], 0.3));
    }
    double* vel0 = (double*)malloc(sizeof(double) * nc);
    for (int i = 0; i < nc; ++i) {
        double var = sa[i];
        vel0[i] = var / sqrt(var * var + (fabs(var) * pow(vol[i], 0.333)) * (fabs(var) * pow(vol[i], 0.333)));
    }
    double* nrm = (double*)malloc(sizeof(double) * 3 * nc);
    double* vs = (double*)malloc(sizeof(double) * 6 * nc);
    double* gt = (double*)malloc(sizeof(double) * 3 * nc);
    for (int iter = 0; iter < 4; ++iter) {
        LSQ_INPUT(sa, g);
        for (int i = 0; i < nc; ++i) {
            double m = sqrt(g[3 * i] * g[3 * i] + g[3 * i + 1] * g[3 * i + 1] + g[3 * i + 2] * g[3 * i + 2]);
            for (int q = 0; q < 3; ++q) nrm[3 * i + q] = (m != 0.0) ? g[3 * i + q] / m : 0.0;
        }
        memset(vs, 0, sizeof(double) * 6 * nc);
        for (int f = 0; f < nf; ++f) {
            const double* d = dist + 3 * f;
            int o = c->own[f];
            double wk = reinit_weight(vel0[o], nrm + 3 * o, d, -1.0);
            for (int ii = 0, num = 0; ii < 3; ++ii)
                for (int jj = ii; jj < 3; ++jj) vs[6 * o + num++] += wk * d[ii] * d[jj];
            if (f < ni) {
                int q = c->nei[f];
                wk = reinit_weight(vel0[q], nrm + 3 * q, d, 1.0);
                for (int ii = 0, num = 0; ii < 3; ++ii)
                    for (int jj = ii; jj < 3; ++jj) vs[6 * q + num++] += wk * d[ii] * d[jj];
            }
        }
        for (int i = 0; i < nc; ++i) {
            double* v6 = vs + 6 * i;
            double U[3][3] = {{v6[0], v6[1], v6[2]}, {v6[1], v6[3], v6[4]}, {v6[2], v6[4], v6[5]}};
            double D[3], V[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            svd3(U, D, V);
            double iD[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int q = 0; q < 3; ++q) if (fabs(D[q]) > 1.e-25) iD[q][q] = 1.0 / D[q];
            double Ut[3][3], o3[3][3], P[3][3];
            for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) Ut[a][b] = U[b][a];
            mm3(iD, Ut, o3);
            mm3(V, o3, P);
            v6[0] = P[0][0]; v6[1] = P[0][1]; v6[2] = P[0][2]; v6[3] = P[1][1]; v6[4] = P[1][2]; v6[5] = P[2][2];
        }
        memset(gt, 0, sizeof(double) * 3 * nc);
        for (int f = 0; f < nf; ++f) {
            const double* d = dist + 3 * f;
            int o = c->own[f];
            double L = sa[o], R = (f < ni) ? sa[c->nei[f]] : L;
            double DV = R - L;
            double wk = reinit_weight(vel0[o], nrm + 3 * o, d, -1.0);
            for (int q = 0; q < 3; ++q) gt[3 * o + q] += wk * d[q] * DV;
            if (f < ni) {
                int r = c->nei[f];
                wk = reinit_weight(vel0[r], nrm + 3 * r, d, 1.0);
                for (int q = 0; q < 3; ++q) gt[3 * r + q] += wk * d[q] * DV;
            }
        }
        for (int i = 0; i < nc; ++i) {
            const double* v6 = vs + 6 * i; double* t = gt + 3 * i;
            double t0 = v6[0] * t[0] + v6[1] * t[1] + v6[2] * t[2];
            double t1 = v6[1] * t[0] + v6[3] * t[1] + v6[4] * t[2];
            double t2 = v6[2] * t[0] + v6[4] * t[1] + v6[5] * t[2];
            t[0] = t0; t[1] = t1; t[2] = t2;
        }
        for (int i = 0; i < nc; ++i)
            if (!iface[i]) {
                double* t = gt + 3 * i;
                double mg = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
                double resi = 0.1 * tau[i] * vel0[i] * (1.0 - mg);
                sa[i] += resi;
            }
    }
    double* ls = dreg(c, "ls", nc);
    memcpy(ls, sa, sizeof(double) * nc);
    /* normals of the re-initialised level set, then the divergence */
    LSQ_INPUT(sa, g);
    for (int i = 0; i < nc; ++i) {
        double m = 0.0;
        for (int q = 0; q < 3; ++q) m += g[3 * i + q] * g[3 * i + q];
        m = sqrt(m);
        for (int q = 0; q < 3; ++q) nrm[3 * i + q] = (m > 1.e-15) ? g[3 * i + q] / m : 0.0;
    }
    memset(vs, 0, sizeof(double) * 6 * nc);
    memset(gt, 0, sizeof(double) * 3 * nc);
    for (int i = 0; i < nc; ++i)
        for (int k = sp[i]; k < sp[i + 1]; ++k) {
            int j = si[k];
            double d[3] = {cc[3 * j] - cc[3 * i], cc[3 * j + 1] - cc[3 * i + 1], cc[3 * j + 2] - cc[3 * i + 2]};
            for (int ii = 0, num = 0; ii < 3; ++ii)
                for (int jj = ii; jj < 3; ++jj) vs[6 * i + num++] += 1.0 * d[ii] * d[jj];
        }
    for (int p = 0; p < c->npatch; ++p)
        for (int f = c->pstart[p]; f < c->pstart[p] + c->psize[p]; ++f) {
            int o = c->own[f];
            double d[3] = {fc[3 * f] - cc[3 * o], fc[3 * f + 1] - cc[3 * o + 1], fc[3 * f + 2] - cc[3 * o + 2]};
            for (int ii = 0, num = 0; ii < 3; ++ii)
                for (int jj = ii; jj < 3; ++jj) vs[6 * o + num++] += 1.0 * d[ii] * d[jj];
        }
    for (int i = 0; i < nc; ++i) {
        double* v = vs + 6 * i;
        double det = v[0] * v[3] * v[5] + v[1] * v[4] * v[2] + v[2] * v[1] * v[4] - v[0] * v[4] * v[4] -
                     v[2] * v[3] * v[2] - v[1] * v[1] * v[5];
        double t[6];
        t[0] = (v[3] * v[5] - v[4] * v[4]) / det;
        t[1] = (v[2] * v[4] - v[1] * v[5]) / det;
        t[2] = (v[1] * v[4] - v[2] * v[3]) / det;
        t[3] = (v[0] * v[5] - v[2] * v[2]) / det;
        t[4] = (v[2] * v[1] - v[0] * v[4]) / det;
        t[5] = (v[0] * v[3] - v[1] * v[1]) / det;
        memcpy(v, t, sizeof t);
    }
    for (int i = 0; i < nc; ++i)
        for (int k = sp[i]; k < sp[i + 1]; ++k) {
            int j = si[k];
            double d[3] = {cc[3 * j] - cc[3 * i], cc[3 * j + 1] - cc[3 * i + 1], cc[3 * j + 2] - cc[3 * i + 2]};
            for (int q = 0; q < 3; ++q) gt[3 * i + q] += 1.0 * d[q] * (nrm[3 * j + q] - nrm[3 * i + q]);
        }
    double* kappa = dreg(c, "kappa", nc);
    for (int i = 0; i < nc; ++i) {
        const double* v = vs + 6 * i; const double* t = gt + 3 * i;
        double t0 = v[0] * t[0] + v[1] * t[1] + v[2] * t[2];
        double t1 = v[1] * t[0] + v[3] * t[1] + v[4] * t[2];
        double t2 = v[2] * t[0] + v[4] * t[1] + v[5] * t[2];
        kappa[i] = -(t0 + t1 + t2);
    }
#undef LSQ_INPUT
    free(sa); free(fsa); free(iface); free(phiR); free(g); free(tau); free(vel0); free(nrm); free(vs); free(gt);
}

/* calcSourceSurfaceTension (surfaceTension.cpp:7-120) after calcCurvature;
   needs the face values of the pressure pass (face_vfR) */
void orc_surface_tension(orc_ctx* c, double sigma) {
    int nc = c->nc, nf = c->nf, ni = c->ni;
    face_values(c);
    orc_curvature(c);
    double *VF = dget(c, "VF"), *U = dget(c, "U"), *V = dget(c, "V"), *W = dget(c, "W");
    double* kappa = dget(c, "kappa");
    double* g = (double*)malloc(sizeof(double) * 3 * nc);
    lsq_grad(c, VF, dget(c, "face_vfR"), g);
    /* Gauss-Green (gradient.cpp:1778-1975) with the LSQ gradient for the
       skewness correction and the zeroGradient extrapolation */
    double *wc = dget(c, "face_wC"), *fn = dget(c, "face_n"), *fa = dget(c, "face_area");
    double *sk = dget(c, "face_skew"), *vol = dget(c, "cell_vol"), *cc = dget(c, "cell_c"), *fc = dget(c, "face_c");
    double* vr = dget(c, "face_vfR");
    double* gg = (double*)calloc(3 * (size_t)nc, sizeof(double));
    for (int f = 0; f < ni; ++f) {
        int o = c->own[f], q = c->nei[f];
        double wL = wc[f], wR = 1.0 - wL;
        double vf = wL * VF[o] + wR * VF[q];
        vf += wL * g[3 * o] * sk[3 * f]; vf += wL * g[3 * o + 1] * sk[3 * f + 1]; vf += wL * g[3 * o + 2] * sk[3 * f + 2];
        vf += wR * g[3 * q] * sk[3 * f]; vf += wR * g[3 * q + 1] * sk[3 * f + 1]; vf += wR * g[3 * q + 2] * sk[3 * f + 2];
        for (int j = 0; j < 3; ++j) {
            gg[3 * o + j] += vf * fn[3 * f + j] * fa[f] / vol[o];
            gg[3 * q + j] -= vf * fn[3 * f + j] * fa[f] / vol[q];
        }
    }
    for (int p = 0; p < c->npatch; ++p) {
        int t = c->bct[3 * p + 2];
        for (int f = c->pstart[p]; f < c->pstart[p] + c->psize[p]; ++f) {
            int o = c->own[f];
            double vf = VF[o];
            if (t == 1) vf = c->bcv[5 * p + 4];
            else if (t == 0) {
                vf += g[3 * o] * (fc[3 * f] - cc[3 * o]);
                vf += g[3 * o + 1] * (fc[3 * f + 1] - cc[3 * o + 1]);
                vf += g[3 * o + 2] * (fc[3 * f + 2] - cc[3 * o + 2]);
            } else vf = 0.5 * (VF[o] + vr[f]);
            for (int j = 0; j < 3; ++j) gg[3 * o + j] += vf * fn[3 * f + j] * fa[f] / vol[o];
        }
    }
    double* gvf = dreg(c, "sft_grad_VF", 3LL * nc);
    memcpy(gvf, gg, sizeof(double) * 3 * nc);
    double* src = dreg(c, "src_sft", 4LL * nc);
    for (int i = 0; i < nc; ++i) {
        src[4 * i] = (sigma * kappa[i] * gg[3 * i]);
        src[4 * i + 1] = (sigma * kappa[i] * gg[3 * i + 1]);
        src[4 * i + 2] = (sigma * kappa[i] * gg[3 * i + 2]);
        src[4 * i + 3] = sigma * kappa[i] * (gg[3 * i] * U[i] + gg[3 * i + 1] * V[i] + gg[3 * i + 2] * W[i]);
    }
    free(g); free(gg);
    (void)nf;
}
