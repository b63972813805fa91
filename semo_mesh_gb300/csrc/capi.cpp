// C-ABI entry points (include/semo_gb300.h) and host-side mesh preprocessing.
//
// Host work is limited to what SEMO also does once per mesh on the host:
// topology lists, the vertex stencil, RCM and the CSR pattern.  Everything per
// outer iteration runs on the GPU.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <numeric>
#include <string>
#include <vector>

#include "semo_internal.h"

using semo::Error;

namespace semo {
long long g_kernel_launches = 0;
}

namespace {

template <class F>
semo_status guarded(semo_ctx* c, F&& f) {
    if (!c) return SEMO_ERR_ARGUMENT;
    try {
        c->err.clear();
        f();
        return SEMO_OK;
    } catch (const Error& e) {
        c->err = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        c->err = "host allocation failed";
        return SEMO_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        c->err = e.what();
        return SEMO_ERR_CUDA;
    }
}

void need(bool ok, semo_status s, const std::string& msg) {
    if (!ok) throw Error(s, msg);
}

}  // namespace

extern "C" {

void semo_params_default(semo_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->device = 0;
    p->precision = SEMO_PREC_MIXED;
    p->tol = 1e-8;
    p->max_iter = 500;
    p->eps_strong = 0.03;
    p->coarse_enough = 64;
    p->max_levels = 24;
    p->cheb_degree = 2;
    p->reuse_hierarchy = 1;
    p->mom_tol = 1e-9;
    p->mom_max_iter = 1000;
    p->overlap_setup = 1;
    p->smoother = 0;
}

void semo_physics_default(semo_physics* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->dt = 1.0;
    p->rho[0] = p->rho[1] = 1.0;
    p->urf_p = 0.3;
    p->urf_u = 0.3;
    p->p_min = p->u_min = p->v_min = p->w_min = -1e300;
    p->p_max = p->u_max = p->v_max = p->w_max = 1e300;
    p->mu[0] = p->mu[1] = 1e-3;
    p->urf_mom = 0.3;
    p->urf_vof = 0.3;
}

semo_status semo_ctx_create(semo_ctx** out, const semo_params* prm) {
    if (!out) return SEMO_ERR_ARGUMENT;
    *out = nullptr;
    semo_ctx* c = new (std::nothrow) semo_ctx();
    if (!c) return SEMO_ERR_OUT_OF_MEMORY;
    if (prm) c->prm = *prm; else semo_params_default(&c->prm);
    semo_physics_default(&c->phys);
    semo_status st = guarded(c, [&] {
        need(c->prm.tol > 0.0 && c->prm.max_iter > 0 && c->prm.coarse_enough > 0 && c->prm.max_levels > 0 && c->prm.max_levels <= 64 &&
                 c->prm.cheb_degree > 0 && c->prm.cheb_degree <= 16 && c->prm.mom_tol > 0.0 &&
                 (c->prm.smoother == 0 || c->prm.smoother == 1) &&
                 c->prm.mom_max_iter > 0 &&
                 (c->prm.precision == SEMO_PREC_FP64 || c->prm.precision == SEMO_PREC_MIXED),
             SEMO_ERR_ARGUMENT, "invalid semo_params");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(SEMO_ERR_NO_DEVICE, "no CUDA device");
        need(c->prm.device >= 0 && c->prm.device < ndev, SEMO_ERR_ARGUMENT, "device ordinal out of range");
        c->device = c->prm.device;
        SEMO_CUDA(cudaSetDevice(c->device));
        cudaDeviceProp dp;
        SEMO_CUDA(cudaGetDeviceProperties(&dp, c->device));
        if (dp.major * 10 + dp.minor != 103)
            throw Error(SEMO_ERR_NO_DEVICE, "library built for sm_103a, device is sm_" +
                                                std::to_string(dp.major) + std::to_string(dp.minor));
        SEMO_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->setup_s = c->stream;
        // keep freed blocks in the stream-ordered pool instead of returning them
        cudaMemPool_t pool;
        SEMO_CUDA(cudaDeviceGetDefaultMemPool(&pool, c->device));
        uint64_t thr = UINT64_MAX;
        SEMO_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
        // a block freed on one stream is not handed to another stream by making
        // that stream wait for the first (the pressure setup runs on a second
        // stream beside the momentum pass and must not be serialised behind it)
        int no_deps = 0;
        SEMO_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no_deps));
        for (auto& e : c->ev) SEMO_CUDA(cudaEventCreate(&e));
        for (auto& e : c->setup_ev) SEMO_CUDA(cudaEventCreate(&e));
        SEMO_CUDA(cudaMallocHost((void**)&c->hpin, semo::kHostScalars * sizeof(double)));
        SEMO_CUDA(cudaMallocHost((void**)&c->hpin_setup, semo::kHostScalars * sizeof(double)));
        SEMO_CUDA(cudaMallocHost((void**)&c->hpin_scan, semo::kHostInts * sizeof(int)));
        SEMO_CUDA(cudaMallocHost((void**)&c->hpin_int, semo::kHostInts * sizeof(int)));
        c->flag.alloc(16, c->stream);
        c->flag.zero();
    });
    if (st != SEMO_OK) {
        semo_ctx_destroy(c);
        return st;
    }
    *out = c;
    return SEMO_OK;
}

semo_status semo_ctx_destroy(semo_ctx* c) {
    if (!c) return SEMO_ERR_ARGUMENT;
    if (c->stream) {
        cudaSetDevice(c->device);
        cudaStreamSynchronize(c->stream);
    }
    if (c->aux_stream) cudaStreamSynchronize(c->aux_stream);
    for (auto& e : c->ov_ev) if (e) cudaEventDestroy(e);
    c->amg64.clear();
    c->amg32.clear();
    for (auto& e : c->ev) if (e) cudaEventDestroy(e);
    for (auto& e : c->setup_ev) if (e) cudaEventDestroy(e);
    semo::resolve_stage_timers(c);
    for (auto e : c->ev_pool) cudaEventDestroy(e);
    for (auto& e : c->sync_ev) if (e) cudaEventDestroy(e);
    if (c->hpin) cudaFreeHost(c->hpin);
    if (c->hpin_int) cudaFreeHost(c->hpin_int);
    if (c->hpin_setup) cudaFreeHost(c->hpin_setup);
    if (c->hpin_scan) cudaFreeHost(c->hpin_scan);
    cudaStream_t s = c->stream, aux = c->aux_stream;
    delete c;  // DBuf destructors enqueue frees on the (still valid) streams
    if (aux) { cudaStreamSynchronize(aux); cudaStreamDestroy(aux); }
    if (s) { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
    return SEMO_OK;
}

const char* semo_last_error(const semo_ctx* c) { return c ? c->err.c_str() : "null context"; }

void* semo_stream(semo_ctx* c) { return c ? (void*)c->stream : nullptr; }

semo_status semo_mesh_upload(semo_ctx* c, int n_points, const double* points, int n_faces, int n_internal,
                             int n_cells, const int32_t* face_ptr, const int32_t* face_pts, const int32_t* owner,
                             const int32_t* neighbour, int n_patches, const int32_t* patch_start,
                             const int32_t* patch_size) {
    return guarded(c, [&] {
        need(points && face_ptr && face_pts && owner && (neighbour || n_internal == 0) && patch_start &&
                 patch_size,
             SEMO_ERR_ARGUMENT, "null mesh array");
        need(n_points > 0 && n_cells > 0 && n_faces > 0 && n_internal >= 0 && n_internal <= n_faces &&
                 n_patches >= 0,
             SEMO_ERR_ARGUMENT, "bad mesh sizes");
        SEMO_CUDA(cudaSetDevice(c->device));
        const int nf = n_faces, ni = n_internal, nc = n_cells;
        // ---- validation (reference: SEMO_Mesh_Builder::check, build.cpp:8-450) ----
        need(face_ptr[0] == 0, SEMO_ERR_MESH, "face_ptr[0] != 0");
        for (int f = 0; f < nf; ++f) {
            need(face_ptr[f + 1] - face_ptr[f] >= 3, SEMO_ERR_MESH, "face with fewer than 3 points: " + std::to_string(f));
            need(owner[f] >= 0 && owner[f] < nc, SEMO_ERR_MESH, "owner out of range at face " + std::to_string(f));
        }
        for (int k = 0; k < face_ptr[nf]; ++k)
            need(face_pts[k] >= 0 && face_pts[k] < n_points, SEMO_ERR_MESH, "face point out of range");
        for (int f = 0; f < ni; ++f) {
            need(neighbour[f] >= 0 && neighbour[f] < nc, SEMO_ERR_MESH, "neighbour out of range at face " + std::to_string(f));
            need(neighbour[f] != owner[f], SEMO_ERR_MESH, "face " + std::to_string(f) + " has neighbour == owner");
        }
        {
            int expect = ni;
            for (int p = 0; p < n_patches; ++p) {
                need(patch_start[p] == expect && patch_size[p] >= 0, SEMO_ERR_MESH,
                     "patches must tile the boundary faces contiguously");
                expect += patch_size[p];
            }
            need(expect == nf, SEMO_ERR_MESH, "patches do not cover all boundary faces");
        }
        c->np = n_points; c->nf = nf; c->ni = ni; c->nc = nc; c->nb = nf - ni; c->npatch = n_patches;
        c->patch_start.assign(patch_start, patch_start + n_patches);
        c->patch_size.assign(patch_size, patch_size + n_patches);
        c->mesh_ready = c->phys_ready = c->fields_ready = c->assembled = c->mom_assembled = false;
        c->amg32.clear();
        c->amg64.clear();
        c->has_old = c->has_src = c->has_oldvf = false;
        c->pvf_current = c->sg_current = c->sft_current = c->vof_assembled = false;
        c->cpl_phys = c->cpl_fields = c->cpl_assembled = false;
        ++c->mesh_gen;

        // ---- cell -> faces, ascending face index (connectCelltoFaces, build.cpp:587-608) ----
        std::vector<int> cfp(nc + 1, 0), cfi;
        for (int f = 0; f < nf; ++f) { cfp[owner[f] + 1]++; if (f < ni) cfp[neighbour[f] + 1]++; }
        for (int i = 0; i < nc; ++i) cfp[i + 1] += cfp[i];
        cfi.resize(cfp[nc]);
        {
            std::vector<int> fill(cfp.begin(), cfp.end() - 1);
            for (int f = 0; f < nf; ++f) {
                cfi[fill[owner[f]]++] = f;
                if (f < ni) cfi[fill[neighbour[f]]++] = f | (1 << 30);  // bit 30 marks the neighbour side
            }
        }
        // ---- cell -> points, first-touch over the cell's faces (connectCelltoPoints, build.cpp:613-690) ----
        std::vector<int> cpp(nc + 1, 0), cpi;
        {
            std::vector<int> cnt(nc, 0);
#pragma omp parallel for schedule(dynamic, 4096)
            for (int i = 0; i < nc; ++i) {
                int buf[256]; int m = 0; bool over = false;
                for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
                    int f = cfi[k] & 0x3FFFFFFF;
                    for (int q = face_ptr[f]; q < face_ptr[f + 1]; ++q) {
                        int p = face_pts[q];
                        bool seen = false;
                        for (int t = 0; t < m; ++t) if (buf[t] == p) { seen = true; break; }
                        if (!seen) { if (m < 256) buf[m++] = p; else over = true; }
                    }
                }
                cnt[i] = over ? -1 : m;
            }
            for (int i = 0; i < nc; ++i) need(cnt[i] >= 0, SEMO_ERR_MESH, "cell with more than 256 points");
            for (int i = 0; i < nc; ++i) cpp[i + 1] = cpp[i] + cnt[i];
            cpi.resize(cpp[nc]);
#pragma omp parallel for schedule(dynamic, 4096)
            for (int i = 0; i < nc; ++i) {
                int m = cpp[i];
                for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
                    int f = cfi[k] & 0x3FFFFFFF;
                    for (int q = face_ptr[f]; q < face_ptr[f + 1]; ++q) {
                        int p = face_pts[q];
                        bool seen = false;
                        for (int t = cpp[i]; t < m; ++t) if (cpi[t] == p) { seen = true; break; }
                        if (!seen) cpi[m++] = p;
                    }
                }
            }
        }
        // ---- point -> cells (ascending cell), vertex stencil (setStencil, geometric.cpp:1781-1845) ----
        std::vector<int> pcp(n_points + 1, 0), pci;
        for (int k = 0; k < cpp[nc]; ++k) pcp[cpi[k] + 1]++;
        for (int p = 0; p < n_points; ++p) pcp[p + 1] += pcp[p];
        pci.resize(pcp[n_points]);
        {
            std::vector<int> fill(pcp.begin(), pcp.end() - 1);
            for (int i = 0; i < nc; ++i)
                for (int k = cpp[i]; k < cpp[i + 1]; ++k) pci[fill[cpi[k]]++] = i;
        }
        std::vector<int> stp(nc + 1, 0), sti;
        {
            std::vector<int> cnt(nc, 0);
#pragma omp parallel
            {
                std::vector<int> mark;
#pragma omp for schedule(dynamic, 4096)
                for (int i = 0; i < nc; ++i) {
                    int m = 0;
                    int local[1024]; bool over = false;
                    for (int k = cpp[i]; k < cpp[i + 1]; ++k) {
                        int p = cpi[k];
                        for (int q = pcp[p]; q < pcp[p + 1]; ++q) {
                            int j = pci[q];
                            if (j == i) continue;
                            bool seen = false;
                            for (int t = 0; t < m; ++t) if (local[t] == j) { seen = true; break; }
                            if (!seen) { if (m < 1024) local[m++] = j; else over = true; }
                        }
                    }
                    cnt[i] = over ? -1 : m;
                }
            }
            for (int i = 0; i < nc; ++i) need(cnt[i] >= 0, SEMO_ERR_MESH, "vertex stencil larger than 1024");
            for (int i = 0; i < nc; ++i) stp[i + 1] = stp[i] + cnt[i];
            sti.resize(stp[nc]);
#pragma omp parallel for schedule(dynamic, 4096)
            for (int i = 0; i < nc; ++i) {
                int m = stp[i];
                for (int k = cpp[i]; k < cpp[i + 1]; ++k) {
                    int p = cpi[k];
                    for (int q = pcp[p]; q < pcp[p + 1]; ++q) {
                        int j = pci[q];
                        if (j == i) continue;
                        bool seen = false;
                        for (int t = stp[i]; t < m; ++t) if (sti[t] == j) { seen = true; break; }
                        if (!seen) sti[m++] = j;
                    }
                }
            }
        }
        // ---- RCM over the internal-face graph, adjacency in cell.faces order (RCM.cpp:83-118) ----
        {
            std::vector<int> xadj(nc + 1), adj;
            adj.reserve(2 * (size_t)ni + 1);
            xadj[0] = 1;
            for (int i = 0; i < nc; ++i) {
                for (int k = cfp[i]; k < cfp[i + 1]; ++k) {
                    int f = cfi[k] & 0x3FFFFFFF;
                    if (f >= ni) continue;
                    adj.push_back((owner[f] == i ? neighbour[f] : owner[f]) + 1);
                }
                xadj[i + 1] = (int)adj.size() + 1;
            }
            if (adj.empty()) adj.push_back(0);
            semo::genrcm_perm(nc, xadj, adj, c->perm);
            c->iperm.assign(nc, 0);
            for (int r = 0; r < nc; ++r) c->iperm[c->perm[r]] = r;
        }
        const std::vector<int>& perm = c->perm;
        const std::vector<int>& iperm = c->iperm;
        // ---- renumbered lists ----
        std::vector<int> own_r(nf), nei_r(std::max(ni, 1));
        for (int f = 0; f < nf; ++f) own_r[f] = iperm[owner[f]];
        for (int f = 0; f < ni; ++f) nei_r[f] = iperm[neighbour[f]];
        // Faces are stored in an order that follows the RCM cell order
        // (internal faces by new owner then new neighbour, boundary faces by
        // new owner inside their patch) so the cell gathers read per-face
        // arrays coherently.  Cell->face lists keep SEMO's ascending original
        // face order, so every accumulation order is unchanged.
        std::vector<int>& fperm = c->fperm;     // fperm[stored] = caller's face index
        std::vector<int>& fiperm = c->fiperm;
        fperm.assign(nf, 0);
        fiperm.assign(nf, 0);
        {
            std::vector<int> cnt(nc + 1, 0);
            for (int f = 0; f < ni; ++f) cnt[own_r[f] + 1]++;
            for (int i = 0; i < nc; ++i) cnt[i + 1] += cnt[i];
            std::vector<int> pos(cnt.begin(), cnt.end() - 1);
            for (int f = 0; f < ni; ++f) fperm[pos[own_r[f]]++] = f;
            for (int i = 0; i < nc; ++i)
                std::sort(fperm.begin() + cnt[i], fperm.begin() + cnt[i + 1],
                          [&](int a, int b) { return nei_r[a] < nei_r[b] || (nei_r[a] == nei_r[b] && a < b); });
            for (int p = 0; p < n_patches; ++p) {
                const int b0 = patch_start[p], b1 = b0 + patch_size[p];
                for (int f = b0; f < b1; ++f) fperm[f] = f;
                std::stable_sort(fperm.begin() + b0, fperm.begin() + b1,
                                 [&](int a, int b) { return own_r[a] < own_r[b]; });
            }
            for (int k = 0; k < nf; ++k) fiperm[fperm[k]] = k;
        }
        std::vector<int> own_n(nf), nei_n(std::max(ni, 1));
        for (int k = 0; k < nf; ++k) own_n[k] = own_r[fperm[k]];
        for (int k = 0; k < ni; ++k) nei_n[k] = nei_r[fperm[k]];
        for (auto& e : cfi) e = fiperm[e & 0x3FFFFFFF] | (e & (1 << 30));
        std::vector<int> rcfp(nc + 1, 0), rcfi(cfi.size()), rstp(nc + 1, 0), rsti(sti.size());
        for (int r = 0; r < nc; ++r) {
            int o = perm[r];
            rcfp[r + 1] = rcfp[r] + (cfp[o + 1] - cfp[o]);
            rstp[r + 1] = rstp[r] + (stp[o + 1] - stp[o]);
        }
#pragma omp parallel for schedule(static)
        for (int r = 0; r < nc; ++r) {
            int o = perm[r];
            std::copy(cfi.begin() + cfp[o], cfi.begin() + cfp[o + 1], rcfi.begin() + rcfp[r]);
            for (int k = stp[o], d = rstp[r]; k < stp[o + 1]; ++k, ++d) rsti[d] = iperm[sti[k]];
        }
        // ---- CSR pattern in RCM order, SEMO in-row order (cellsGlobal, build.cpp:1319-1424) ----
        c->nnz = (int64_t)nc + 2 * (int64_t)ni;
        need(c->nnz < INT32_MAX, SEMO_ERR_ARGUMENT, "matrix too large for 32-bit indices");
        std::vector<int> aptr(nc + 1), acol(c->nnz), adig(nc), alr(std::max(ni, 1)), arl(std::max(ni, 1));
        for (int r = 0; r < nc; ++r) {
            int o = perm[r];
            int row_len = 1;
            for (int k = cfp[o]; k < cfp[o + 1]; ++k) if ((cfi[k] & 0x3FFFFFFF) < ni) ++row_len;
            aptr[r + 1] = aptr[r] + row_len;
        }
#pragma omp parallel for schedule(static)
        for (int r = 0; r < nc; ++r) {
            int o = perm[r];
            int d = aptr[r];
            acol[d] = r; adig[r] = d; ++d;
            for (int k = cfp[o]; k < cfp[o + 1]; ++k) {
                int fe = cfi[k];
                int f = fe & 0x3FFFFFFF;
                if (f >= ni) continue;
                bool nb_side = (fe >> 30) & 1;
                acol[d] = nb_side ? own_n[f] : nei_n[f];
                if (nb_side) arl[f] = d; else alr[f] = d;
                ++d;
            }
        }
        // boundary face -> patch
        std::vector<int> bp(std::max(c->nb, 1), 0);
        for (int p = 0; p < n_patches; ++p)
            for (int f = patch_start[p]; f < patch_start[p] + patch_size[p]; ++f) bp[f - ni] = p;

        // ---- upload ----
        cudaStream_t s = c->stream;
        c->dperm.upload(perm.data(), nc, s);
        c->own.upload(own_n.data(), nf, s);
        c->nei.upload(nei_n.data(), std::max(ni, 1), s);
        c->cf_ptr.upload(rcfp.data(), nc + 1, s);
        c->cf_idx.upload(rcfi.data(), rcfi.size(), s);
        c->st_ptr.upload(rstp.data(), nc + 1, s);
        c->st_idx.upload(rsti.data(), std::max<size_t>(rsti.size(), 1), s);
        c->st_nnz = (int64_t)rsti.size();
        c->cf_nnz = (int64_t)rcfi.size();
        c->bpatch.upload(bp.data(), bp.size(), s);
        c->A_ptr.upload(aptr.data(), nc + 1, s);
        c->A_col.upload(acol.data(), acol.size(), s);
        c->A_dig.upload(adig.data(), nc, s);
        c->A_lr.upload(alr.data(), alr.size(), s);
        c->A_rl.upload(arl.data(), arl.size(), s);
        c->A_val.alloc(c->nnz, s);
        c->b.alloc(nc, s);
        semo::DBuf<double> d_pts;
        semo::DBuf<int> d_fptr, d_fpts;
        d_pts.upload(points, 3 * (size_t)n_points, s);
        {
            // face point loops in the stored face order
            std::vector<int> pptr(nf + 1, 0), ppts(face_ptr[nf]);
            for (int k = 0; k < nf; ++k) pptr[k + 1] = pptr[k] + (face_ptr[fperm[k] + 1] - face_ptr[fperm[k]]);
            for (int k = 0; k < nf; ++k)
                std::copy(face_pts + face_ptr[fperm[k]], face_pts + face_ptr[fperm[k] + 1], ppts.begin() + pptr[k]);
            d_fptr.upload(pptr.data(), nf + 1, s);
            d_fpts.upload(ppts.data(), ppts.size(), s);
            SEMO_CUDA(cudaStreamSynchronize(s));   // the host vectors go out of scope
        }
        semo::geometry_build(c, d_pts.p, d_fptr.p, d_fpts.p, own_n);
        // field storage
        for (auto* b : {&c->P, &c->U, &c->V, &c->W, &c->VF, &c->rho, &c->irho, &c->x}) b->alloc(nc, s);
        c->grad.alloc(15 * (size_t)nc, s);
        c->mm.alloc(10 * (size_t)nc, s);
        c->sg.alloc(4 * (size_t)nc, s);
        c->gx.alloc(3 * (size_t)nc, s);
        c->bface.alloc(10 * (size_t)std::max(c->nb, 1), s);
        c->fscr.alloc(3 * (size_t)nf, s);
        c->unf.alloc(nf, s);
        c->x.zero();
        SEMO_CUDA(cudaStreamSynchronize(s));
        c->mesh_ready = true;
    });
}

semo_status semo_rcm(semo_ctx* c, int32_t* perm, int32_t* iperm) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        if (perm) std::copy(c->perm.begin(), c->perm.end(), perm);
        if (iperm) std::copy(c->iperm.begin(), c->iperm.end(), iperm);
    });
}

semo_status semo_set_physics(semo_ctx* c, const semo_physics* phys, const int32_t* bc_type, const double* bc_value) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        need(phys && (bc_type || c->npatch == 0) && (bc_value || c->npatch == 0), SEMO_ERR_ARGUMENT, "null argument");
        need(std::isfinite(phys->dt) && phys->dt > 0.0, SEMO_ERR_ARGUMENT, "dt must be positive");
        need(phys->rho[0] > 0.0 && phys->rho[1] > 0.0, SEMO_ERR_ARGUMENT, "densities must be positive");
        need(phys->mu[0] >= 0.0 && phys->mu[1] >= 0.0, SEMO_ERR_ARGUMENT, "viscosities must be non-negative");
        need(std::isfinite(phys->sigma), SEMO_ERR_ARGUMENT, "sigma must be finite");
        for (int p = 0; p < c->npatch; ++p) {
            need(bc_type[3 * p] == SEMO_BC_ZERO_GRADIENT || bc_type[3 * p] == SEMO_BC_FIXED_VALUE, SEMO_ERR_ARGUMENT,
                 "pressure BC must be zeroGradient or fixedValue");
            need(bc_type[3 * p + 1] >= 0 && bc_type[3 * p + 1] <= 3, SEMO_ERR_ARGUMENT, "bad velocity BC");
            need(bc_type[3 * p + 2] == SEMO_BC_ZERO_GRADIENT || bc_type[3 * p + 2] == SEMO_BC_FIXED_VALUE,
                 SEMO_ERR_ARGUMENT, "volume-fraction BC must be zeroGradient or fixedValue");
        }
        c->phys = *phys;
        c->h_bc_type.assign(bc_type, bc_type + 3 * c->npatch);
        c->h_bc_value.assign(bc_value, bc_value + 5 * c->npatch);
        c->bc_type.upload(c->h_bc_type.data(), std::max<size_t>(c->h_bc_type.size(), 1), c->stream);
        c->bc_value.upload(c->h_bc_value.data(), std::max<size_t>(c->h_bc_value.size(), 1), c->stream);
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
        c->phys_ready = true;
        c->assembled = false;
        c->mom_assembled = false;
        c->vof_assembled = false;
        c->pvf_current = false;
        c->sg_current = false;
        c->sft_current = false;
    });
}

static void download_permuted(semo_ctx* c, const double* d, double* h, int planes = 1, bool interleave = false) {
    const int n = c->nc;
    std::vector<double> tmp((size_t)n * planes);
    SEMO_CUDA(cudaMemcpyAsync(tmp.data(), d, sizeof(double) * n * planes, cudaMemcpyDeviceToHost, c->stream));
    SEMO_CUDA(cudaStreamSynchronize(c->stream));
    for (int r = 0; r < n; ++r)
        for (int q = 0; q < planes; ++q) {
            size_t dst = interleave ? (size_t)c->perm[r] * planes + q : (size_t)q * n + c->perm[r];
            h[dst] = tmp[(size_t)q * n + r];
        }
}

// Fields cross the boundary in the caller's cell order: the host arrays are
// copied as they are (a DMA straight from pinned memory when the caller's
// buffers are pinned) and reordered and checked on the GPU.
semo_status semo_set_fields(semo_ctx* c, const double* P, const double* U, const double* V, const double* W,
                            const double* VF) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        need(P && U && V && W && VF, SEMO_ERR_ARGUMENT, "null field");
        const size_t n = (size_t)c->nc;
        cudaStream_t s = c->stream;
        c->stage.alloc(5 * n, s);
        const double* src[5] = {P, U, V, W, VF};
        for (int q = 0; q < 5; ++q)
            SEMO_CUDA(cudaMemcpyAsync(c->stage.p + q * n, src[q], sizeof(double) * n, cudaMemcpyHostToDevice, s));
        double* dst[5] = {c->P.p, c->U.p, c->V.p, c->W.p, c->VF.p};
        if (!semo::fields_from_caller_order(c, c->stage.p, dst, 5))
            throw Error(SEMO_ERR_NAN, "non-finite input field value");
        c->fields_ready = true;
        c->assembled = false;
        c->mom_assembled = false;
        c->vof_assembled = false;
        c->pvf_current = false;
        c->sg_current = false;
        c->sft_current = false;
    });
}

semo_status semo_get_fields(semo_ctx* c, double* P, double* U, double* V, double* W) {
    return guarded(c, [&] {
        need(c->fields_ready, SEMO_ERR_STATE, "no fields set");
        const size_t n = (size_t)c->nc;
        cudaStream_t s = c->stream;
        c->stage.alloc(5 * n, s);
        const double* src[4] = {c->P.p, c->U.p, c->V.p, c->W.p};
        semo::fields_to_caller_order(c, src, c->stage.p, 4);
        double* dst[4] = {P, U, V, W};
        for (int q = 0; q < 4; ++q)
            if (dst[q])
                SEMO_CUDA(cudaMemcpyAsync(dst[q], c->stage.p + q * n, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
    });
}

semo_status semo_source_surface_tension(semo_ctx* c) {
    return guarded(c, [&] {
        need(c->mesh_ready && c->phys_ready && c->fields_ready, SEMO_ERR_STATE,
             "mesh, physics and fields must be set first");
        need(c->phys.sigma != 0.0, SEMO_ERR_STATE, "sigma is 0: no surface tension");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo::assemble_face_values(c, false);
        semo::assemble_gravity(c);
        semo::stencil_pass(c, true);
        semo::assemble_surface_tension(c);
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
        c->pvf_current = false;
    });
}

semo_status semo_get_surface_tension(semo_ctx* c, double* kappa, double* ls, double* src) {
    return guarded(c, [&] {
        need(c->sft_current, SEMO_ERR_STATE, "no surface-tension source computed for the current fields");
        const size_t n = (size_t)c->nc;
        if (kappa) download_permuted(c, c->sft.p, kappa);
        if (ls) download_permuted(c, c->sft.p + n, ls);
        if (src) download_permuted(c, c->sft.p + 2 * n, src, 4, true);
    });
}

semo_status semo_assemble_pressure(semo_ctx* c) {
    return guarded(c, [&] {
        need(c->mesh_ready && c->phys_ready && c->fields_ready, SEMO_ERR_STATE,
             "mesh, physics and fields must be set before assembly");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo::assemble_pressure(c);
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
        c->assembled = true;
    });
}

semo_status semo_get_system_rcm(semo_ctx* c, int32_t* ptr, int32_t* col, double* val, double* b) {
    return guarded(c, [&] {
        need(c->assembled, SEMO_ERR_STATE, "system not assembled");
        cudaStream_t s = c->stream;
        if (ptr) SEMO_CUDA(cudaMemcpyAsync(ptr, c->A_ptr.p, sizeof(int) * (c->nc + 1), cudaMemcpyDeviceToHost, s));
        if (col) SEMO_CUDA(cudaMemcpyAsync(col, c->A_col.p, sizeof(int) * c->nnz, cudaMemcpyDeviceToHost, s));
        if (val) SEMO_CUDA(cudaMemcpyAsync(val, c->A_val.p, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost, s));
        if (b) SEMO_CUDA(cudaMemcpyAsync(b, c->b.p, sizeof(double) * c->nc, cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
    });
}

semo_status semo_get_system_rcm_eq(semo_ctx* c, int eq, int32_t* ptr, int32_t* col, double* val, double* b) {
    return guarded(c, [&] {
        need(eq >= SEMO_EQ_PRESSURE && eq <= SEMO_EQ_COUPLED, SEMO_ERR_ARGUMENT, "unknown equation");
        const double* v = nullptr;
        const double* rhs = nullptr;
        size_t vper = 1, planes = 1;
        switch (eq) {
            case SEMO_EQ_PRESSURE:
                need(c->assembled, SEMO_ERR_STATE, "pressure system not assembled");
                v = c->A_val.p; rhs = c->b.p;
                break;
            case SEMO_EQ_MOMENTUM:
                need(c->mom_assembled, SEMO_ERR_STATE, "momentum system not assembled");
                v = c->Am_val.p; rhs = c->bm.p; planes = 3;
                break;
            case SEMO_EQ_VOF:
                need(c->vof_assembled, SEMO_ERR_STATE, "volume-fraction system not assembled");
                v = c->Av_val.p; rhs = c->bvf.p;
                break;
            default:
                need(c->cpl_assembled, SEMO_ERR_STATE, "coupled system not assembled");
                v = c->cpl_val.p; rhs = c->cpl_b.p; vper = 25; planes = 5;
                break;
        }
        cudaStream_t s = c->stream;
        if (ptr) SEMO_CUDA(cudaMemcpyAsync(ptr, c->A_ptr.p, sizeof(int) * (c->nc + 1), cudaMemcpyDeviceToHost, s));
        if (col) SEMO_CUDA(cudaMemcpyAsync(col, c->A_col.p, sizeof(int) * c->nnz, cudaMemcpyDeviceToHost, s));
        if (val) SEMO_CUDA(cudaMemcpyAsync(val, v, sizeof(double) * vper * c->nnz, cudaMemcpyDeviceToHost, s));
        if (b) SEMO_CUDA(cudaMemcpyAsync(b, rhs, sizeof(double) * planes * c->nc, cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
    });
}

semo_status semo_get_array(semo_ctx* c, const char* name, double* out, int64_t count) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        need(name && out, SEMO_ERR_ARGUMENT, "null argument");
        std::string nm(name);
        const int n = c->nc, nf = c->nf;
        auto cell_planes = [&](const double* d, int planes, bool inter) {
            need(count == (int64_t)n * planes, SEMO_ERR_ARGUMENT, "count mismatch for " + nm);
            download_permuted(c, d, out, planes, inter);
        };
        auto face_planes = [&](const double* d, int planes, int64_t len) {
            need(count == len * planes, SEMO_ERR_ARGUMENT, "count mismatch for " + nm);
            std::vector<double> tmp((size_t)len * planes);
            SEMO_CUDA(cudaMemcpyAsync(tmp.data(), d, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, c->stream));
            SEMO_CUDA(cudaStreamSynchronize(c->stream));
            for (int64_t f = 0; f < len; ++f)   // back to the caller's face order
                for (int q = 0; q < planes; ++q) out[f * planes + q] = tmp[(size_t)q * len + c->fiperm[f]];
        };
        const char* grads[5] = {"grad_P", "grad_U", "grad_V", "grad_W", "grad_VF"};
        for (int g = 0; g < 5; ++g)
            if (nm == grads[g]) {
                need(c->assembled || c->mom_assembled || c->vof_assembled, SEMO_ERR_STATE, "not assembled");
                cell_planes(c->grad.p + (size_t)3 * g * n, 3, true);
                return;
            }
        if (nm == "minmax_uvw") { cell_planes(c->mm.p, 6, true); return; }
        if (nm == "minmax_vf") { cell_planes(c->mm.p + (size_t)6 * n, 2, true); return; }
        if (nm == "minmax_p") { cell_planes(c->mm.p + (size_t)8 * n, 2, true); return; }
        if (nm == "rho") { cell_planes(c->rho.p, 1, false); return; }
        if (nm == "VF") { need(c->fields_ready, SEMO_ERR_STATE, "no fields set"); cell_planes(c->VF.p, 1, false); return; }
        if (nm == "mu") { need(c->mu.n == 2 * (size_t)n, SEMO_ERR_STATE, "no momentum assembly"); cell_planes(c->mu.p, 1, false); return; }
        if (nm == "src_grav") { cell_planes(c->sg.p, 4, true); return; }
        if (nm == "grad_x") { cell_planes(c->gx.p, 3, true); return; }
        if (nm == "face_UnF") { face_planes(c->unf.p, 1, nf); return; }
        if (nm == "face_VF_LR") {
            need(c->vof_assembled, SEMO_ERR_STATE, "no volume-fraction assembly");
            need(count == 2 * (int64_t)nf, SEMO_ERR_ARGUMENT, "count mismatch for " + nm);
            const int ni = c->ni, nb = c->nb;
            std::vector<double> fl((size_t)2 * std::max(ni, 1)), bf((size_t)6 * std::max(nb, 1));
            SEMO_CUDA(cudaMemcpyAsync(fl.data(), c->fvf.p, sizeof(double) * 2 * ni, cudaMemcpyDeviceToHost, c->stream));
            SEMO_CUDA(cudaMemcpyAsync(bf.data(), c->bface.p, sizeof(double) * 6 * nb, cudaMemcpyDeviceToHost, c->stream));
            SEMO_CUDA(cudaStreamSynchronize(c->stream));
            for (int f = 0; f < nf; ++f) {   // the caller's face f is stored at fiperm[f]
                const int sf = c->fiperm[f];
                if (sf < ni) { out[2 * f] = fl[sf]; out[2 * f + 1] = fl[ni + sf]; }
                else { out[2 * f] = out[2 * f + 1] = bf[4 * (size_t)nb + (sf - ni)]; }
            }
            return;
        }

        if (nm == "geometry:cell_vol") { cell_planes(c->vol.p, 1, false); return; }
        if (nm == "geometry:cell_c") { cell_planes(c->cc.p, 3, true); return; }
        if (nm == "geometry:lsq_minv") { cell_planes(c->minv.p, 6, true); return; }
        if (nm == "geometry:face_n") { face_planes(c->fn.p, 3, nf); return; }
        if (nm == "geometry:face_area") { face_planes(c->fa.p, 1, nf); return; }
        if (nm == "geometry:face_c") { face_planes(c->fc.p, 3, nf); return; }
        if (nm == "geometry:face_wC") { face_planes(c->wc.p, 1, nf); return; }
        if (nm == "geometry:face_magPN") { face_planes(c->mpn.p, 1, nf); return; }
        if (nm == "geometry:face_alphaF") { face_planes(c->alf.p, 1, nf); return; }
        if (nm == "geometry:face_ePN") { face_planes(c->epn.p, 3, nf); return; }
        if (nm == "geometry:face_skew") { face_planes(c->skew.p, 3, nf); return; }
        if (nm == "geometry:face_vecPF") { face_planes(c->pf.p, 3, nf); return; }
        if (nm == "geometry:face_vecNF") { face_planes(c->nfv.p, 3, nf); return; }
        throw Error(SEMO_ERR_ARGUMENT, "unknown array " + nm);
    });
}

semo_status semo_solve_pressure(semo_ctx* c, double* x, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(c->assembled, SEMO_ERR_STATE, "system not assembled");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo_solve_info inf{};
        semo::solve_system(c, c->A_ptr.p, c->A_col.p, c->A_val.p, c->nc, c->nnz, c->b.p, c->x.p, &inf, true, true);
        if (info) *info = inf;
        if (x) {
            c->stage.alloc(5 * (size_t)c->nc, c->stream);
            const double* src[1] = {c->x.p};
            semo::fields_to_caller_order(c, src, c->stage.p, 1);
            SEMO_CUDA(cudaMemcpyAsync(x, c->stage.p, sizeof(double) * c->nc, cudaMemcpyDeviceToHost, c->stream));
            SEMO_CUDA(cudaStreamSynchronize(c->stream));
        }
        if (!(inf.rel_residual <= c->prm.tol)) conv = std::isfinite(inf.rel_residual) ? SEMO_ERR_NOT_CONVERGED : SEMO_ERR_NAN;
    });
    if (st == SEMO_OK && conv != SEMO_OK) c->err = "Krylov solve did not reach the tolerance";
    return st != SEMO_OK ? st : conv;
}

namespace {

// calcPressureEq: assemble, solve, update.  Returns the convergence status.
semo_status pressure_pass_impl(semo_ctx* c, double* norm, semo_solve_info* info) {
    need(c->mesh_ready && c->phys_ready && c->fields_ready, SEMO_ERR_STATE,
         "mesh, physics and fields must be set before a pass");
    SEMO_CUDA(cudaSetDevice(c->device));
    semo::assemble_pressure(c);
    c->assembled = true;
    semo_solve_info inf{};
    semo::solve_system(c, c->A_ptr.p, c->A_col.p, c->A_val.p, c->nc, c->nnz, c->b.p, c->x.p, &inf, true, true);
    double nrm = semo::pressure_update(c);
    c->mom_assembled = false;
    if (norm) *norm = nrm;
    if (info) *info = inf;
    if (!(inf.rel_residual <= c->prm.tol)) return std::isfinite(inf.rel_residual) ? SEMO_ERR_NOT_CONVERGED : SEMO_ERR_NAN;
    return SEMO_OK;
}

// calcMomentumEqs: assemble, three solves, update (skipped after a breakdown).
semo_status momentum_pass_impl(semo_ctx* c, double* norm, semo_solve_info* info, bool face_values_done = false) {
    need(c->mesh_ready && c->phys_ready && c->fields_ready, SEMO_ERR_STATE,
         "mesh, physics and fields must be set before a pass");
    SEMO_CUDA(cudaSetDevice(c->device));
    semo::assemble_momentum(c, face_values_done);
    c->mom_assembled = true;
    semo_solve_info inf[3] = {};
    semo_status conv = semo::solve_momentum(c, inf);
    if (info) for (int j = 0; j < 3; ++j) info[j] = inf[j];
    if (conv == SEMO_ERR_BREAKDOWN) return conv;
    double nrm = semo::momentum_update(c);
    c->assembled = false;
    if (norm) *norm = nrm;
    return conv;
}

semo_status finish(semo_ctx* c, semo_status st, semo_status conv, const char* what) {
    if (st == SEMO_OK && conv != SEMO_OK) c->err = what;
    return st != SEMO_OK ? st : conv;
}

}  // namespace

semo_status semo_pressure_pass(semo_ctx* c, double* norm, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] { conv = pressure_pass_impl(c, norm, info); });
    return finish(c, st, conv, "Krylov solve did not reach the tolerance");
}

semo_status semo_set_old_velocity(semo_ctx* c, const double* oU, const double* oV, const double* oW,
                                  const double* o2U, const double* o2V, const double* o2W) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        const double* src[6] = {oU, oV, oW, o2U, o2V, o2W};
        int given = 0;
        for (auto p : src) given += p != nullptr;
        c->mom_assembled = false;
        if (given == 0) { c->has_old = false; return; }
        need(given == 6, SEMO_ERR_ARGUMENT, "give all six old velocity components or none");
        SEMO_CUDA(cudaSetDevice(c->device));
        const size_t n = (size_t)c->nc;
        cudaStream_t s = c->stream;
        c->stage.alloc(5 * n, s);
        c->old.alloc(6 * n, s);
        for (int half = 0; half < 2; ++half) {
            for (int q = 0; q < 3; ++q)
                SEMO_CUDA(cudaMemcpyAsync(c->stage.p + q * n, src[3 * half + q], sizeof(double) * n,
                                          cudaMemcpyHostToDevice, s));
            double* dst[3] = {c->old.p + (3 * half) * n, c->old.p + (3 * half + 1) * n, c->old.p + (3 * half + 2) * n};
            if (!semo::fields_from_caller_order(c, c->stage.p, dst, 3)) {
                c->has_old = false;
                throw Error(SEMO_ERR_NAN, "non-finite old velocity");
            }
        }
        c->has_old = true;
    });
}

semo_status semo_assemble_momentum(semo_ctx* c) {
    return guarded(c, [&] {
        need(c->mesh_ready && c->phys_ready && c->fields_ready, SEMO_ERR_STATE,
             "mesh, physics and fields must be set before assembly");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo::assemble_momentum(c);
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
        c->mom_assembled = true;
    });
}

semo_status semo_momentum_pass(semo_ctx* c, double* norm, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] { conv = momentum_pass_impl(c, norm, info); });
    return finish(c, st, conv, "momentum solve did not reach the tolerance");
}

semo_status semo_solve_momentum(semo_ctx* c, double* x, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(c->mom_assembled, SEMO_ERR_STATE, "momentum system not assembled");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo_solve_info inf[3] = {};
        conv = semo::solve_momentum(c, inf);
        if (info) for (int j = 0; j < 3; ++j) info[j] = inf[j];
        if (x) {
            const size_t n = (size_t)c->nc;
            c->stage.alloc(5 * n, c->stream);
            const double* src[3] = {c->xm.p, c->xm.p + n, c->xm.p + 2 * n};
            semo::fields_to_caller_order(c, src, c->stage.p, 3);
            SEMO_CUDA(cudaMemcpyAsync(x, c->stage.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
            SEMO_CUDA(cudaStreamSynchronize(c->stream));
        }
    });
    return finish(c, st, conv, "momentum solve did not reach the tolerance");
}

namespace {
// The host thread that builds the pressure hierarchy beside the momentum pass,
// kept for the context's lifetime: the setup is the overlapped outer
// iteration's critical path, and a thread started for each outer iteration
// put its creation and its first CUDA call at the head of it.  One job at a
// time; a job's exception is handed to the waiter.
struct SetupWorker {
    std::mutex mu;
    std::condition_variable cv;
    std::function<void()> job;
    bool pending = false, busy = false, quit = false;
    std::exception_ptr err;
    std::thread th;
    explicit SetupWorker(int device) {
        th = std::thread([this, device] { run(device); });
    }
    ~SetupWorker() {
        {
            std::lock_guard<std::mutex> lk(mu);
            quit = true;
        }
        cv.notify_all();
        th.join();
    }
    void run(int device) {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [this] { return pending || quit; });
            if (!pending) return;   // quit with nothing left to do
            std::function<void()> f = std::move(job);
            pending = false;
            busy = true;
            lk.unlock();
            std::exception_ptr e;
            try {
                f();
            } catch (...) {
                e = std::current_exception();
            }
            lk.lock();
            err = e;
            busy = false;
            cv.notify_all();
        }
    }
    void post(std::function<void()> f) {
        {
            std::lock_guard<std::mutex> lk(mu);
            job = std::move(f);
            err = nullptr;
            pending = true;
        }
        cv.notify_all();
    }
    // wait for the posted job; rethrow its exception
    void wait() {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [this] { return !pending && !busy; });
        if (err) {
            std::exception_ptr e = err;
            err = nullptr;
            std::rethrow_exception(e);
        }
    }
};

SetupWorker& setup_worker(semo_ctx* c) {
    if (!c->setup_worker) c->setup_worker = std::make_shared<SetupWorker>(c->device);
    return *static_cast<SetupWorker*>(c->setup_worker.get());
}

// The pressure matrix and its AMG hierarchy built on the second stream, the
// hierarchy from a second host thread, while this thread runs the momentum
// pass and the pressure assembly on the context's stream.  The pressure
// matrix reads only geometry, dt, the cell densities and the boundary
// densities of the face values, which neither of those changes, so it equals
// the one the pressure pass would assemble (the same kernels' roundings) and
// so does its hierarchy.  The destructor joins the thread (also when a pass
// throws) and puts the setup back on the context's stream.
struct SideSetup {
    semo_ctx* c;
    bool waiting = false;   // a job is posted and not yet waited for
    explicit SideSetup(semo_ctx* ctx) : c(ctx) {
        if (!c->aux_stream) {
            // high priority: the setup is a chain of short dependent launches and
            // host round trips, so its blocks go first whenever the momentum
            // pass's kernels would otherwise hold every SM
            int least = 0, greatest = 0;
            SEMO_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            SEMO_CUDA(cudaStreamCreateWithPriority(&c->aux_stream, cudaStreamNonBlocking, greatest));
        }
        for (auto& e : c->ov_ev)
            if (!e) SEMO_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        // host resources the setup creates on first use, made here on this thread
        for (auto& e : c->sync_ev)
            if (!e) SEMO_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        SEMO_CUDA(cudaEventRecord(c->ov_ev[0], c->stream));   // face values (densities) are on the stream
        SEMO_CUDA(cudaStreamWaitEvent(c->aux_stream, c->ov_ev[0], 0));
        semo::pressure_matrix(c, c->aux_stream);
        SEMO_CUDA(cudaEventRecord(c->ov_ev[2], c->aux_stream));   // the face values may be rewritten after this
        c->setup_s = c->aux_stream;
        SetupWorker& w = setup_worker(c);
        semo_ctx* const cc = c;
        w.post([cc] {
            SEMO_CUDA(cudaSetDevice(cc->device));
            const auto t0 = std::chrono::steady_clock::now();
            semo::pressure_setup(cc, cc->A_ptr.p, cc->A_col.p, cc->A_val.p, cc->nc, cc->nnz, true, nullptr);
            SEMO_CUDA(cudaEventRecord(cc->ov_ev[1], cc->aux_stream));
            SEMO_CUDA(cudaEventSynchronize(cc->ov_ev[1]));
            cc->side_setup_ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        });
        waiting = true;
    }
    // wait for the setup; rethrow its failure; the context's stream then waits for the hierarchy
    void finish() {
        waiting = false;
        try {
            setup_worker(c).wait();
        } catch (...) {
            c->setup_s = c->stream;
            throw;
        }
        c->setup_s = c->stream;
        SEMO_CUDA(cudaStreamWaitEvent(c->stream, c->ov_ev[1], 0));
    }
    ~SideSetup() {
        if (waiting) {
            try {
                setup_worker(c).wait();
            } catch (...) {
            }
        }
        c->setup_s = c->stream;
    }
};

// the pressure pass with the side setup: its assembly leaves A_val alone and
// its solve first joins the setup (solve_system calls before_solve)
struct PrebuiltFlag {
    semo_ctx* c;
    PrebuiltFlag(semo_ctx* ctx, SideSetup& ss) : c(ctx) {
        c->matrix_prebuilt = true;
        c->before_solve = [&ss] { ss.finish(); };
    }
    ~PrebuiltFlag() {
        c->matrix_prebuilt = false;
        c->before_solve = nullptr;
    }
};
}  // namespace

semo_status semo_outer_iteration(semo_ctx* c, double* norms, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        semo_solve_info inf[4] = {};
        double nm[2] = {0.0, 0.0};
        if (c->prm.overlap_setup && c->mesh_ready && c->phys_ready && c->fields_ready) {
            SEMO_CUDA(cudaSetDevice(c->device));
            semo::assemble_face_values(c, true);
            SideSetup ss(c);
            const semo_status cm = momentum_pass_impl(c, &nm[0], inf, true);
            if (cm == SEMO_ERR_BREAKDOWN) {
                ss.finish();
                conv = cm;
            } else {
                // the pressure pass rewrites the face values the early matrix read
                SEMO_CUDA(cudaStreamWaitEvent(c->stream, c->ov_ev[2], 0));
                PrebuiltFlag pb(c, ss);
                const semo_status cp = pressure_pass_impl(c, &nm[1], &inf[3]);
                conv = (cp != SEMO_OK) ? cp : cm;
            }
        } else {
            const semo_status cm = momentum_pass_impl(c, &nm[0], inf);
            if (cm == SEMO_ERR_BREAKDOWN) {
                conv = cm;
            } else {
                const semo_status cp = pressure_pass_impl(c, &nm[1], &inf[3]);
                conv = (cp != SEMO_OK) ? cp : cm;
            }
        }
        if (norms) { norms[0] = nm[0]; norms[1] = nm[1]; }
        if (info) for (int j = 0; j < 4; ++j) info[j] = inf[j];
    });
    return finish(c, st, conv, "a solve of the outer iteration did not reach its tolerance");
}

namespace {
// A system held on the context's CSR pattern (RCM rows), written out in SEMO's
// layout: rows back in the caller's numbering, each row in SEMO's in-row order
// with its diagonal first, off-diagonals SEMO leaves out (stored as 0) dropped.
void export_semo_layout(semo_ctx* c, const double* dval, const double* db, int planes, int32_t* ptr, int32_t* col,
                        double* val, double* b, int64_t* nnz_out) {
    cudaStream_t s = c->stream;
    const int n = c->nc;
    std::vector<int> hp(n + 1), hc(c->nnz);
    std::vector<double> hv(c->nnz), hb((size_t)planes * n);
    SEMO_CUDA(cudaMemcpyAsync(hp.data(), c->A_ptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaMemcpyAsync(hc.data(), c->A_col.p, sizeof(int) * c->nnz, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaMemcpyAsync(hv.data(), dval, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaMemcpyAsync(hb.data(), db, sizeof(double) * hb.size(), cudaMemcpyDeviceToHost, s));
    SEMO_CUDA(cudaStreamSynchronize(s));
    int64_t k_out = 0;
    if (ptr) ptr[0] = 0;
    for (int i = 0; i < n; ++i) {
        const int r = c->iperm[i];
        for (int k = hp[r]; k < hp[r + 1]; ++k) {
            if (k != hp[r] && hv[k] == 0.0) continue;
            if (col) col[k_out] = c->perm[hc[k]];
            if (val) val[k_out] = hv[k];
            ++k_out;
        }
        if (ptr) ptr[i + 1] = (int32_t)k_out;
    }
    if (b)
        for (int j = 0; j < planes; ++j)
            for (int r = 0; r < n; ++r) b[(size_t)j * n + c->perm[r]] = hb[(size_t)j * n + r];
    if (nnz_out) *nnz_out = k_out;
}

// calcVolfracEq: reconstruct, assemble, solve, update (skipped after a breakdown).
semo_status vof_pass_impl(semo_ctx* c, double* norm, semo_solve_info* info) {
    need(c->mesh_ready && c->phys_ready && c->fields_ready, SEMO_ERR_STATE,
         "mesh, physics and fields must be set before a pass");
    SEMO_CUDA(cudaSetDevice(c->device));
    semo::assemble_vof(c);
    c->vof_assembled = true;
    semo_solve_info inf{};
    semo_status conv = semo::solve_vof(c, &inf);
    if (info) *info = inf;
    if (conv == SEMO_ERR_BREAKDOWN) return conv;
    const double nrm = semo::vof_update(c);
    if (norm) *norm = nrm;
    return conv;
}
}  // namespace

semo_status semo_get_momentum_system(semo_ctx* c, int32_t* ptr, int32_t* col, double* val, double* b,
                                     int64_t* nnz_out) {
    return guarded(c, [&] {
        need(c->mom_assembled, SEMO_ERR_STATE, "momentum system not assembled");
        export_semo_layout(c, c->Am_val.p, c->bm.p, 3, ptr, col, val, b, nnz_out);
    });
}

semo_status semo_get_vof_system(semo_ctx* c, int32_t* ptr, int32_t* col, double* val, double* b,
                                int64_t* nnz_out) {
    return guarded(c, [&] {
        need(c->vof_assembled, SEMO_ERR_STATE, "volume-fraction system not assembled");
        export_semo_layout(c, c->Av_val.p, c->bvf.p, 1, ptr, col, val, b, nnz_out);
    });
}

semo_status semo_set_old_vf(semo_ctx* c, const double* oldVF, const double* old2VF) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        c->vof_assembled = false;
        if (!oldVF && !old2VF) { c->has_oldvf = false; return; }
        need(oldVF && old2VF, SEMO_ERR_ARGUMENT, "give both old volume fractions or none");
        SEMO_CUDA(cudaSetDevice(c->device));
        const size_t n = (size_t)c->nc;
        cudaStream_t s = c->stream;
        c->stage.alloc(5 * n, s);
        c->oldvf.alloc(2 * n, s);
        SEMO_CUDA(cudaMemcpyAsync(c->stage.p, oldVF, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        SEMO_CUDA(cudaMemcpyAsync(c->stage.p + n, old2VF, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        double* dst[2] = {c->oldvf.p, c->oldvf.p + n};
        if (!semo::fields_from_caller_order(c, c->stage.p, dst, 2)) {
            c->has_oldvf = false;
            throw Error(SEMO_ERR_NAN, "non-finite old volume fraction");
        }
        c->has_oldvf = true;
    });
}

semo_status semo_vof_pass(semo_ctx* c, double* norm, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] { conv = vof_pass_impl(c, norm, info); });
    return finish(c, st, conv, "volume-fraction solve did not reach the tolerance");
}

semo_status semo_assemble_vof(semo_ctx* c) {
    return guarded(c, [&] {
        need(c->mesh_ready && c->phys_ready && c->fields_ready, SEMO_ERR_STATE,
             "mesh, physics and fields must be set before assembly");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo::assemble_vof(c);
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
        c->vof_assembled = true;
    });
}

semo_status semo_solve_vof(semo_ctx* c, double* x, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(c->vof_assembled, SEMO_ERR_STATE, "volume-fraction system not assembled");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo_solve_info inf{};
        conv = semo::solve_vof(c, &inf);
        if (info) *info = inf;
        if (x) {
            const size_t n = (size_t)c->nc;
            c->stage.alloc(5 * n, c->stream);
            const double* src[1] = {c->xvf.p};
            semo::fields_to_caller_order(c, src, c->stage.p, 1);
            SEMO_CUDA(cudaMemcpyAsync(x, c->stage.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
            SEMO_CUDA(cudaStreamSynchronize(c->stream));
        }
    });
    return finish(c, st, conv, "volume-fraction solve did not reach the tolerance");
}

semo_status semo_solve_coo(semo_ctx* c, int n, int64_t nnz, const int32_t* rows, const int32_t* cols,
                           const double* vals, const double* b, double* x, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(n > 0 && nnz >= n && rows && cols && vals && b && x, SEMO_ERR_ARGUMENT, "bad COO system");
        need(nnz < INT32_MAX, SEMO_ERR_ARGUMENT, "nnz too large");
        SEMO_CUDA(cudaSetDevice(c->device));
        // COO -> CSR exactly as solveAMGCL.cpp:206-251 (in-row order = COO order)
        std::vector<int> ptr(n + 1, 0), col(nnz);
        std::vector<double> val(nnz);
        for (int64_t k = 0; k < nnz; ++k) {
            need(rows[k] >= 0 && rows[k] < n && cols[k] >= 0 && cols[k] < n, SEMO_ERR_ARGUMENT, "COO index out of range");
            need(std::isfinite(vals[k]), SEMO_ERR_NAN, "non-finite matrix value");
            ptr[rows[k]]++;
        }
        for (int i = 0, s = 0; i < n; ++i) { int t = ptr[i]; ptr[i] = s; s += t; }
        ptr[n] = (int)nnz;
        for (int64_t k = 0; k < nnz; ++k) { int d = ptr[rows[k]]++; col[d] = cols[k]; val[d] = vals[k]; }
        for (int i = 0, last = 0; i <= n; ++i) { int t = ptr[i]; ptr[i] = last; last = t; }
        for (int i = 0; i < n; ++i) need(std::isfinite(b[i]) && std::isfinite(x[i]), SEMO_ERR_NAN, "non-finite rhs/guess");
        cudaStream_t s = c->stream;
        semo::DBuf<int> dp, dc;
        semo::DBuf<double> dv, db, dx;
        dp.upload(ptr.data(), n + 1, s);
        dc.upload(col.data(), nnz, s);
        dv.upload(val.data(), nnz, s);
        db.upload(b, n, s);
        dx.upload(x, n, s);
        semo_solve_info inf{};
        semo::solve_system(c, dp.p, dc.p, dv.p, n, nnz, db.p, dx.p, &inf, false);
        SEMO_CUDA(cudaMemcpyAsync(x, dx.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
        if (info) *info = inf;
        if (!(inf.rel_residual <= c->prm.tol)) conv = std::isfinite(inf.rel_residual) ? SEMO_ERR_NOT_CONVERGED : SEMO_ERR_NAN;
    });
    if (st == SEMO_OK && conv != SEMO_OK) c->err = "Krylov solve did not reach the tolerance";
    return st != SEMO_OK ? st : conv;
}

semo_status semo_solve_coo_multi(semo_ctx* c, int nrhs, int n, int64_t nnz, const int32_t* rows, const int32_t* cols,
                                 const double* vals, const double* b, double* x, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(nrhs >= 1 && nrhs <= 3, SEMO_ERR_ARGUMENT, "nrhs must be 1, 2 or 3");
        need(n > 0 && nnz >= n && rows && cols && vals && b && x, SEMO_ERR_ARGUMENT, "bad COO system");
        need(nnz < INT32_MAX, SEMO_ERR_ARGUMENT, "nnz too large");
        SEMO_CUDA(cudaSetDevice(c->device));
        // COO -> CSR as solveAMGCL.cpp:1129-1172 (stable: in-row order = COO order)
        std::vector<int> ptr(n + 1, 0), col(nnz), dig(n, -1);
        std::vector<double> val(nnz);
        for (int64_t k = 0; k < nnz; ++k) {
            need(rows[k] >= 0 && rows[k] < n && cols[k] >= 0 && cols[k] < n, SEMO_ERR_ARGUMENT, "COO index out of range");
            need(std::isfinite(vals[k]), SEMO_ERR_NAN, "non-finite matrix value");
            ptr[rows[k]]++;
        }
        for (int i = 0, t = 0; i < n; ++i) { int u = ptr[i]; ptr[i] = t; t += u; }
        ptr[n] = (int)nnz;
        for (int64_t k = 0; k < nnz; ++k) {
            const int d = ptr[rows[k]]++;
            col[d] = cols[k];
            val[d] = vals[k];
            if (cols[k] == rows[k] && dig[rows[k]] < 0) dig[rows[k]] = d;   // each row's first diagonal entry
        }
        for (int i = 0, last = 0; i <= n; ++i) { int t = ptr[i]; ptr[i] = last; last = t; }
        for (int i = 0; i < n; ++i) {
            need(dig[i] >= 0, SEMO_ERR_ARGUMENT, "row " + std::to_string(i) + " has no diagonal entry");
            need(val[dig[i]] != 0.0, SEMO_ERR_ARGUMENT, "row " + std::to_string(i) + " has a zero diagonal");
        }
        bool guess = false;
        for (int64_t i = 0; i < (int64_t)nrhs * n; ++i) {
            need(std::isfinite(b[i]) && std::isfinite(x[i]), SEMO_ERR_NAN, "non-finite rhs/guess");
            guess |= x[i] != 0.0;
        }
        cudaStream_t s = c->stream;
        semo::DBuf<int> dp, dc, dd;
        semo::DBuf<double> dv, db, dx;
        dp.upload(ptr.data(), n + 1, s);
        dc.upload(col.data(), nnz, s);
        dd.upload(dig.data(), n, s);
        dv.upload(val.data(), nnz, s);
        db.upload(b, (size_t)nrhs * n, s);
        dx.upload(x, (size_t)nrhs * n, s);
        semo_solve_info inf[3] = {};
        conv = semo::solve_csr_multi(c, n, dp.p, dc.p, dd.p, dv.p, nrhs, db.p, dx.p, guess, inf);
        SEMO_CUDA(cudaMemcpyAsync(x, dx.p, sizeof(double) * nrhs * n, cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
        if (info) for (int j = 0; j < nrhs; ++j) info[j] = inf[j];
    });
    if (st == SEMO_OK && conv != SEMO_OK) c->err = "a momentum-type solve did not reach the tolerance";
    return st != SEMO_OK ? st : conv;
}

void semo_set_profiling(semo_ctx* c, int on) {
    if (c) c->profiling = on != 0;
}

semo_status semo_stage_time(semo_ctx* c, const char* stage, double* total_ms, int64_t* calls) {
    return guarded(c, [&] {
        need(stage != nullptr, SEMO_ERR_ARGUMENT, "null stage name");
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
        semo::resolve_stage_timers(c);
        for (int k = 0; k < semo::ST_COUNT; ++k)
            if (std::string(stage) == semo::kStageNames[k]) {
                if (total_ms) *total_ms = c->stage_ms[k];
                if (calls) *calls = c->stage_calls[k];
                return;
            }
        throw Error(SEMO_ERR_ARGUMENT, std::string("unknown stage ") + stage);
    });
}

semo_status semo_reset_stats(semo_ctx* c) {
    return guarded(c, [&] {
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
        semo::resolve_stage_timers(c);
        for (int k = 0; k < semo::ST_COUNT; ++k) { c->stage_ms[k] = 0.0; c->stage_calls[k] = 0; }
    });
}

semo_status semo_time_spmv(semo_ctx* c, int which, int reps, double* ms_per_launch) {
    return guarded(c, [&] {
        need(which == 0 || which == 1, SEMO_ERR_ARGUMENT, "which is 0 (finest V-cycle operator) or 1 (FP64 outer)");
        need(reps > 0 && ms_per_launch != nullptr, SEMO_ERR_ARGUMENT, "bad reps or null output");
        SEMO_CUDA(cudaSetDevice(c->device));
        *ms_per_launch = semo::time_pressure_spmv(c, which, reps);
    });
}

semo_status semo_hierarchy_levels(semo_ctx* c, int64_t* out, int max_levels, int* levels) {
    return guarded(c, [&] {
        need(out != nullptr && levels != nullptr && max_levels > 0, SEMO_ERR_ARGUMENT, "bad output");
        *levels = semo::pressure_levels(c, out, max_levels);
    });
}

int64_t semo_kernel_launches(void) { return __atomic_load_n(&semo::g_kernel_launches, __ATOMIC_RELAXED); }

semo_status semo_mesh_info(semo_ctx* c, int64_t* out6) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        need(out6 != nullptr, SEMO_ERR_ARGUMENT, "null output");
        out6[0] = c->nc; out6[1] = c->nf; out6[2] = c->ni; out6[3] = c->nb;
        out6[4] = c->st_nnz; out6[5] = c->nnz;
    });
}

semo_status semo_set_source(semo_ctx* c, const double* src) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        if (!src) { c->has_src = false; c->assembled = false; return; }
        const size_t n = (size_t)c->nc;
        c->src.alloc(n, c->stream);
        c->stage.alloc(5 * n, c->stream);
        SEMO_CUDA(cudaMemcpyAsync(c->stage.p, src, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        double* dst[1] = {c->src.p};
        if (!semo::fields_from_caller_order(c, c->stage.p, dst, 1)) {
            c->has_src = false;
            c->assembled = false;
            throw Error(SEMO_ERR_NAN, "non-finite source");
        }
        c->has_src = true;
        c->assembled = false;
    });
}

semo_status semo_vjp_source(semo_ctx* c, const double* dJ_dx, double* lambda, double* dJ_ds, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(c->assembled, SEMO_ERR_STATE, "no assembled system: run a forward pass first");
        need(dJ_dx != nullptr, SEMO_ERR_ARGUMENT, "null dJ/dx");
        SEMO_CUDA(cudaSetDevice(c->device));
        const size_t n = (size_t)c->nc;
        cudaStream_t s = c->stream;
        semo::DBuf<double> g, lam, djds;
        g.alloc(n, s);
        lam.alloc(n, s);
        djds.alloc(n, s);
        c->stage.alloc(5 * n, s);
        SEMO_CUDA(cudaMemcpyAsync(c->stage.p, dJ_dx, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        double* gdst[1] = {g.p};
        if (!semo::fields_from_caller_order(c, c->stage.p, gdst, 1)) throw Error(SEMO_ERR_NAN, "non-finite dJ/dx");
        semo_solve_info inf{};
        semo::solve_transpose_reuse(c, g.p, lam.p, &inf);
        if (info) *info = inf;
        // dJ/ds_i = V_i lambda_i (s enters the right-hand side as s_i V_i)
        semo::cellwise_product(c, lam.p, c->vol.p, djds.p);
        const double* src[2] = {lam.p, djds.p};
        semo::fields_to_caller_order(c, src, c->stage.p, 2);
        if (lambda) SEMO_CUDA(cudaMemcpyAsync(lambda, c->stage.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        if (dJ_ds) SEMO_CUDA(cudaMemcpyAsync(dJ_ds, c->stage.p + n, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
        if (!(inf.rel_residual <= c->prm.tol)) conv = std::isfinite(inf.rel_residual) ? SEMO_ERR_NOT_CONVERGED : SEMO_ERR_NAN;
    });
    if (st == SEMO_OK && conv != SEMO_OK) c->err = "adjoint solve did not reach the tolerance";
    return st != SEMO_OK ? st : conv;
}

semo_status semo_vjp_fields(semo_ctx* c, const double* dJ_dx, double* lambda, double* dJ_dU, double* dJ_dV,
                            double* dJ_dW, double* dJ_dP, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(c->assembled, SEMO_ERR_STATE, "no assembled system: run a forward pass first");
        need(dJ_dx != nullptr, SEMO_ERR_ARGUMENT, "null dJ/dx");
        SEMO_CUDA(cudaSetDevice(c->device));
        const size_t n = (size_t)c->nc;
        cudaStream_t s = c->stream;
        semo::DBuf<double> g, lam, grads;
        g.alloc(n, s);
        lam.alloc(n, s);
        grads.alloc(4 * n, s);
        c->stage.alloc(5 * n, s);
        SEMO_CUDA(cudaMemcpyAsync(c->stage.p, dJ_dx, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        double* gdst[1] = {g.p};
        if (!semo::fields_from_caller_order(c, c->stage.p, gdst, 1)) throw Error(SEMO_ERR_NAN, "non-finite dJ/dx");
        semo_solve_info inf{};
        semo::solve_transpose_reuse(c, g.p, lam.p, &inf);
        if (info) *info = inf;
        semo::vjp_fields(c, lam.p, grads.p);
        const double* src[5] = {lam.p, grads.p, grads.p + n, grads.p + 2 * n, grads.p + 3 * n};
        semo::fields_to_caller_order(c, src, c->stage.p, 5);
        double* dst[5] = {lambda, dJ_dU, dJ_dV, dJ_dW, dJ_dP};
        for (int q = 0; q < 5; ++q)
            if (dst[q]) SEMO_CUDA(cudaMemcpyAsync(dst[q], c->stage.p + q * n, sizeof(double) * n,
                                                  cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
        if (!(inf.rel_residual <= c->prm.tol)) conv = std::isfinite(inf.rel_residual) ? SEMO_ERR_NOT_CONVERGED : SEMO_ERR_NAN;
    });
    if (st == SEMO_OK && conv != SEMO_OK) c->err = "adjoint solve did not reach the tolerance";
    return st != SEMO_OK ? st : conv;
}

// ---------------------------------------------------------------------------
// compressible coupled system
// ---------------------------------------------------------------------------
semo_status semo_set_coupled_physics(semo_ctx* c, const semo_coupled_physics* phys, const int32_t* bc_type,
                                     const double* bc_value) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        need(phys && bc_type && bc_value, SEMO_ERR_ARGUMENT, "null coupled physics or boundary arrays");
        need(phys->cv > 0.0 && phys->gamma > 1.0 && phys->dt > 0.0 && phys->dt_old > 0.0 && phys->dt_old2 > 0.0,
             SEMO_ERR_ARGUMENT, "coupled physics needs cv > 0, gamma > 1 and positive time steps");
        for (int p = 0; p < c->npatch; ++p)
            for (int q = 0; q < 3; ++q) {
                const int t = bc_type[3 * p + q];
                const bool ok = (q == 1) ? (t >= SEMO_BC_ZERO_GRADIENT && t <= SEMO_BC_SLIP)
                                         : (t == SEMO_BC_ZERO_GRADIENT || t == SEMO_BC_FIXED_VALUE);
                need(ok, SEMO_ERR_ARGUMENT, "bad coupled boundary type");
            }
        SEMO_CUDA(cudaSetDevice(c->device));
        c->cphys = *phys;
        c->cpl_bct.upload(bc_type, 3 * (size_t)c->npatch, c->stream);
        c->cpl_bcv.upload(bc_value, 5 * (size_t)c->npatch, c->stream);
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
        c->cpl_phys = true;
        c->cpl_assembled = false;
    });
}

semo_status semo_set_coupled_fields(semo_ctx* c, const double* P, const double* U, const double* V, const double* W,
                                    const double* T, const double* old, const double* old2) {
    return guarded(c, [&] {
        need(c->mesh_ready, SEMO_ERR_STATE, "no mesh uploaded");
        need(P && U && V && W && T, SEMO_ERR_ARGUMENT, "null coupled field");
        SEMO_CUDA(cudaSetDevice(c->device));
        const size_t n = (size_t)c->nc;
        cudaStream_t s = c->stream;
        c->stage.alloc(5 * n, s);
        c->cpl_f.alloc(15 * n, s);
        c->cpl_fields = false;
        c->cpl_assembled = false;
        const double* cur[5] = {P, U, V, W, T};
        for (int set = 0; set < 3; ++set) {
            const double* h = (set == 0) ? nullptr : (set == 1 ? old : old2);
            for (int q = 0; q < 5; ++q)
                SEMO_CUDA(cudaMemcpyAsync(c->stage.p + q * n, h ? h + q * n : cur[q], sizeof(double) * n,
                                          cudaMemcpyHostToDevice, s));
            double* dst[5];
            for (int q = 0; q < 5; ++q) dst[q] = c->cpl_f.p + (5 * set + q) * n;
            if (!semo::fields_from_caller_order(c, c->stage.p, dst, 5))
                throw Error(SEMO_ERR_NAN, "non-finite coupled field");
        }
        c->cpl_fields = true;
    });
}

semo_status semo_get_coupled_fields(semo_ctx* c, double* P, double* U, double* V, double* W, double* T) {
    return guarded(c, [&] {
        need(c->cpl_fields, SEMO_ERR_STATE, "no coupled fields set");
        const size_t n = (size_t)c->nc;
        cudaStream_t s = c->stream;
        c->stage.alloc(5 * n, s);
        const double* src[5];
        for (int q = 0; q < 5; ++q) src[q] = c->cpl_f.p + q * n;
        semo::fields_to_caller_order(c, src, c->stage.p, 5);
        double* dst[5] = {P, U, V, W, T};
        for (int q = 0; q < 5; ++q)
            if (dst[q])
                SEMO_CUDA(cudaMemcpyAsync(dst[q], c->stage.p + q * n, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaStreamSynchronize(s));
    });
}

semo_status semo_assemble_coupled(semo_ctx* c) {
    return guarded(c, [&] {
        need(c->mesh_ready && c->cpl_phys && c->cpl_fields, SEMO_ERR_STATE,
             "mesh, coupled physics and coupled fields must be set before assembly");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo::coupled_assemble(c);
        SEMO_CUDA(cudaStreamSynchronize(c->stream));
    });
}

semo_status semo_get_coupled_system(semo_ctx* c, int32_t* ptr, int32_t* col, double* val, double* b, int64_t* nnz) {
    return guarded(c, [&] {
        need(c->cpl_assembled, SEMO_ERR_STATE, "coupled system not assembled");
        cudaStream_t s = c->stream;
        const int n = c->nc;
        std::vector<int> hp(n + 1), hc(c->nnz);
        std::vector<double> hv, hb;
        SEMO_CUDA(cudaMemcpyAsync(hp.data(), c->A_ptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
        SEMO_CUDA(cudaMemcpyAsync(hc.data(), c->A_col.p, sizeof(int) * c->nnz, cudaMemcpyDeviceToHost, s));
        if (val) {
            hv.resize(25 * (size_t)c->nnz);
            SEMO_CUDA(cudaMemcpyAsync(hv.data(), c->cpl_val.p, sizeof(double) * hv.size(), cudaMemcpyDeviceToHost, s));
        }
        if (b) {
            hb.resize(5 * (size_t)n);
            SEMO_CUDA(cudaMemcpyAsync(hb.data(), c->cpl_b.p, sizeof(double) * hb.size(), cudaMemcpyDeviceToHost, s));
        }
        SEMO_CUDA(cudaStreamSynchronize(s));
        int64_t k_out = 0;
        if (ptr) ptr[0] = 0;
        for (int i = 0; i < n; ++i) {
            const int r = c->iperm[i];
            for (int k = hp[r]; k < hp[r + 1]; ++k, ++k_out) {
                if (col) col[k_out] = c->perm[hc[k]];
                if (val) std::copy(hv.begin() + 25 * (size_t)k, hv.begin() + 25 * (size_t)k + 25, val + 25 * k_out);
            }
            if (ptr) ptr[i + 1] = (int32_t)k_out;
        }
        if (b)
            for (int a = 0; a < 5; ++a)
                for (int r = 0; r < n; ++r) b[(size_t)a * n + c->perm[r]] = hb[(size_t)a * n + r];
        if (nnz) *nnz = k_out;
    });
}

semo_status semo_solve_coupled(semo_ctx* c, double* x, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(c->cpl_assembled, SEMO_ERR_STATE, "coupled system not assembled");
        SEMO_CUDA(cudaSetDevice(c->device));
        conv = semo::coupled_solve(c, info);
        if (x) {
            const size_t n = (size_t)c->nc;
            cudaStream_t s = c->stream;
            c->stage.alloc(5 * n, s);
            const double* src[5];
            for (int q = 0; q < 5; ++q) src[q] = c->cpl_x.p + q * n;
            semo::fields_to_caller_order(c, src, c->stage.p, 5);
            SEMO_CUDA(cudaMemcpyAsync(x, c->stage.p, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost, s));
            SEMO_CUDA(cudaStreamSynchronize(s));
        }
    });
    return finish(c, st, conv, "coupled solve did not reach the tolerance");
}

semo_status semo_coupled_pass(semo_ctx* c, double* norm, semo_solve_info* info) {
    semo_status conv = SEMO_OK;
    semo_status st = guarded(c, [&] {
        need(c->mesh_ready && c->cpl_phys && c->cpl_fields, SEMO_ERR_STATE,
             "mesh, coupled physics and coupled fields must be set before the coupled pass");
        SEMO_CUDA(cudaSetDevice(c->device));
        semo::coupled_assemble(c);
        conv = semo::coupled_solve(c, info);
        // the reference updates after any solve; a breakdown leaves the fields as they are
        if (conv == SEMO_OK || conv == SEMO_ERR_NOT_CONVERGED) {
            const double nrm = semo::coupled_update(c);
            if (norm) *norm = nrm;
        }
    });
    return finish(c, st, conv, "coupled solve did not reach the tolerance");
}

}  // extern "C"
