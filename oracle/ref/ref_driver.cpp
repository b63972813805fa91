// Drives the reference's own hot-path code (compiled from its sources by
// oracle/ref/Makefile into oracle/_ref/semo_ref) on a mesh and fields read
// from a case file, and dumps every intermediate the GPU path must match.
//
// This file is test infrastructure for the CPU checker.  It contains no
// reference code: it only fills the reference's data structures the way
// SEMO's loader and initialiser do (src/load/loadOpenFoam.cpp:356-374,
// src/solvers/build.cpp:5-41, src/controls/build.cpp:626+) and calls the
// reference functions in the order of one pressure-correction pass of
// src/solvers/pressureBased.cpp:17-31, :139-141, :211-212.  With case flag 2
// the pass is a whole outer iteration instead: cell transport, then the
// momentum equation (:201-202) followed by the pressure correction (:211-212),
// with old and second-old velocities read from the case.  With case flag 4 the
// pass is one volume-fraction sub-iteration instead (:104-112): MSTACS face
// reconstruction and calcVolfracEq, with old and second-old VF from the case.
// With case flag 8 the curvature and the surface-tension source are computed
// after the gravity source (:142) and dumped.
//
// usage: semo_ref <case.bin> <out.bin>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../solvers/build.h"
#include "../load/load.h"
#include "../mesh/geometric.h"
#include "../math/math.h"

using namespace std;

// Set by the capturing stand-in for solveAMGCL (ref_capture.cpp).
struct CapturedSystem {
    vector<int> rows, cols;
    vector<double> vals, b, x;
    double solve_seconds = 0.0;
    int calls = 0;
};
CapturedSystem g_captured;
struct CapturedMomentum {
    vector<int> rows, cols;
    vector<double> vals, b[3], x[3];
    double solve_seconds = 0.0;
    int calls = 0;
};
CapturedMomentum g_momentum;
CapturedSystem g_vof;

// Called from ref_capture.cpp: forwards to the reference's real solver.
void semo_ref_forward_solve(const string& eq, SEMO_Mesh_Builder& mesh, int B_n,
                            vector<int>& r, vector<int>& c, vector<double>& v,
                            vector<double>& b, vector<double>& x) {
    SEMO_Solvers_Builder solver;
    auto t0 = chrono::steady_clock::now();
    solver.solveAMGCL(eq, mesh, B_n, r, c, v, b, x);
    auto t1 = chrono::steady_clock::now();
    g_captured.solve_seconds += chrono::duration<double>(t1 - t0).count();
}
void semo_ref_forward_solve3(const string& eq, SEMO_Mesh_Builder& mesh, int B_n,
                             vector<int>& r, vector<int>& c, vector<double>& v,
                             vector<double>& b0, vector<double>& b1, vector<double>& b2,
                             vector<double>& x0, vector<double>& x1, vector<double>& x2) {
    SEMO_Solvers_Builder solver;
    auto t0 = chrono::steady_clock::now();
    solver.solveAMGCL(eq, mesh, B_n, r, c, v, b0, b1, b2, x0, x1, x2);
    auto t1 = chrono::steady_clock::now();
    g_momentum.solve_seconds += chrono::duration<double>(t1 - t0).count();
}

static FILE* g_out = nullptr;
static void put(const char* name, const double* p, size_t n) {
    int32_t len = (int32_t)strlen(name), dt = 0; int64_t cnt = (int64_t)n;
    fwrite(&len, 4, 1, g_out); fwrite(name, 1, len, g_out); fwrite(&dt, 4, 1, g_out);
    fwrite(&cnt, 8, 1, g_out); if (n) fwrite(p, 8, n, g_out);
}
static void put(const char* name, const int* p, size_t n) {
    int32_t len = (int32_t)strlen(name), dt = 1; int64_t cnt = (int64_t)n;
    fwrite(&len, 4, 1, g_out); fwrite(name, 1, len, g_out); fwrite(&dt, 4, 1, g_out);
    fwrite(&cnt, 8, 1, g_out); if (n) fwrite(p, 4, n, g_out);
}
static void put(const char* name, const vector<double>& v) { put(name, v.data(), v.size()); }
static void put(const char* name, const vector<int>& v) { put(name, v.data(), v.size()); }

template <class T> static void rd(FILE* f, T* p, size_t n) {
    if (n && fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}

// "foam <dir> <out.bin>": load an OpenFOAM polyMesh directory with the
// reference's own loader (src/load/loadOpenFoam.cpp:8-383) and dump what it
// read: points, face point lists, owner, neighbour (internal faces), patches.
static int dump_foam(const char* dir, const char* out) {
    SEMO_Mesh_Builder mesh;
    SEMO_Mesh_Load load;
    load.OpenFoam(mesh, dir);
    FILE* o = fopen(out, "wb");
    if (!o) { perror(out); return 2; }
    auto w32 = [&](int32_t v) { fwrite(&v, 4, 1, o); };
    w32((int32_t)mesh.points.size());
    for (auto& p : mesh.points) { double x[3] = {p.x, p.y, p.z}; fwrite(x, 8, 3, o); }
    w32((int32_t)mesh.faces.size());
    for (auto& f : mesh.faces) {
        w32((int32_t)f.points.size());
        for (int q : f.points) w32(q);
    }
    for (auto& f : mesh.faces) w32(f.owner);
    int32_t ni = 0;
    for (auto& f : mesh.faces) ni += f.neighbour >= 0;
    w32(ni);
    for (auto& f : mesh.faces) if (f.neighbour >= 0) w32(f.neighbour);
    w32((int32_t)mesh.boundary.size());
    for (auto& b : mesh.boundary) {
        w32((int32_t)b.name.size());
        fwrite(b.name.data(), 1, b.name.size(), o);
        w32(b.startFace); w32(b.nFaces);
    }
    fclose(o);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 4 && !strcmp(argv[1], "foam")) return dump_foam(argv[2], argv[3]);
    if (argc < 3) { fprintf(stderr, "usage: %s case.bin out.bin | foam <dir> <out.bin>\n", argv[0]); return 2; }
    FILE* f = fopen(argv[1], "rb");
    if (!f) { perror(argv[1]); return 2; }
    int32_t hdr[8]; rd(f, hdr, 8);
    if (hdr[0] != 0x53454D4F) { fprintf(stderr, "bad magic\n"); return 2; }
    const int np = hdr[1], nf = hdr[2], ni = hdr[3], nc = hdr[4], npatch = hdr[5], nfp = hdr[6], flags = hdr[7];
    vector<double> pts(3 * (size_t)np); rd(f, pts.data(), pts.size());
    vector<int> fptr(nf + 1), fpts(nfp), own(nf), nei(ni);
    rd(f, fptr.data(), fptr.size()); rd(f, fpts.data(), fpts.size());
    rd(f, own.data(), own.size()); rd(f, nei.data(), nei.size());
    vector<int32_t> pint(6 * (size_t)npatch); vector<double> pval(6 * (size_t)npatch);
    for (int p = 0; p < npatch; ++p) { rd(f, &pint[6 * p], 6); rd(f, &pval[6 * p], 6); }
    vector<double> P(nc), U(nc), V(nc), W(nc), VF(nc);
    rd(f, P.data(), nc); rd(f, U.data(), nc); rd(f, V.data(), nc); rd(f, W.data(), nc); rd(f, VF.data(), nc);
    double prm[16]; rd(f, prm, 16);
    // flag 2: old (n-1) and second-old (n-2) velocities for the BDF2 term
    vector<double> old[6];
    if (flags & 2)
        for (int k = 0; k < 6; ++k) { old[k].resize(nc); rd(f, old[k].data(), nc); }
    // flag 4: old and second-old volume fraction
    vector<double> oldvf[2];
    if (flags & 4)
        for (int k = 0; k < 2; ++k) { oldvf[k].resize(nc); rd(f, oldvf[k].data(), nc); }
    fclose(f);

    // ---- species (two incompressible phases; VF[0] is the first) -------
    vector<SEMO_Species> species(2);
    species[0].name = "water"; species[0].rhoType = "const"; species[0].rho = prm[1]; species[0].mu = prm[3]; species[0].sigma = prm[5];
    species[1].name = "air";   species[1].rhoType = "const"; species[1].rho = prm[2]; species[1].mu = prm[4]; species[1].sigma = prm[5];

    SEMO_Controls_Builder controls;
    controls.setValues(species);
    controls.timeStep = prm[0];
    controls.gravityAcceleration = {prm[6], prm[7], prm[8]};
    controls.prePreURF = prm[9];
    controls.preVelURF = prm[10];
    controls.momVelURF = prm[12];
    controls.vofVofURF = prm[13];
    controls.turbType = "laminar";
    controls.oldTimeStep = controls.timeStep;
    controls.old2TimeStep = controls.timeStep;
    controls.minP = -1e300; controls.maxP = 1e300;
    controls.minU = -1e300; controls.maxU = 1e300;
    controls.minV = -1e300; controls.maxV = 1e300;
    controls.minW = -1e300; controls.maxW = 1e300;

    // ---- mesh, as the OpenFOAM loader leaves it -------------------------
    SEMO_Mesh_Builder mesh;
    mesh.points.resize(np);
    for (int i = 0; i < np; ++i) { mesh.points[i].x = pts[3 * i]; mesh.points[i].y = pts[3 * i + 1]; mesh.points[i].z = pts[3 * i + 2]; }
    mesh.faces.resize(nf);
    for (int i = 0; i < nf; ++i) {
        auto& fc = mesh.faces[i];
        fc.points.assign(fpts.begin() + fptr[i], fpts.begin() + fptr[i + 1]);
        fc.owner = own[i];
        fc.neighbour = (i < ni) ? nei[i] : -1;
    }
    static const char* ptype[] = {"zeroGradient", "fixedValue"};
    static const char* utype[] = {"zeroGradient", "fixedValue", "noSlip", "slip"};
    mesh.boundary.resize(npatch);
    for (int p = 0; p < npatch; ++p) {
        auto& b = mesh.boundary[p];
        b.name = "patch" + to_string(p);
        b.startFace = pint[6 * p]; b.nFaces = pint[6 * p + 1];
        b.myProcNo = -1; b.neighbProcNo = -1;
        b.type.assign(6, "zeroGradient"); b.var.assign(6, 0.0);
        b.type[controls.P] = ptype[pint[6 * p + 2]];
        b.type[controls.U] = utype[pint[6 * p + 3]];
        b.type[controls.V] = b.type[controls.U]; b.type[controls.W] = b.type[controls.U];
        b.type[controls.VF[0]] = ptype[pint[6 * p + 4]];
        b.var[controls.P] = pval[6 * p]; b.var[controls.U] = pval[6 * p + 1];
        b.var[controls.V] = pval[6 * p + 2]; b.var[controls.W] = pval[6 * p + 3];
        b.var[controls.VF[0]] = pval[6 * p + 4];
    }
    mesh.buildCells();
    mesh.setFaceTypes();
    mesh.buildLists();
    mesh.connectCelltoFaces();
    mesh.connectCelltoPoints();
    mesh.cellsGlobal();

    SEMO_Mesh_Geometric geometric;
    SEMO_Utility_Math math;
    geometric.init(mesh);
    math.initLeastSquare(mesh);

    SEMO_Solvers_Builder solver;
    solver.setInitValues(mesh, controls);
    mesh.cellsProcVar.resize(controls.nTotalCellVar);
    mesh.cellsProcGradientVar.resize(controls.nTotalCellVar);
    mesh.cellsGradientVar.resize(controls.nTotalCellVar);
    for (int i = 0; i < nc; ++i) {
        auto& c = mesh.cells[i];
        c.var[controls.P] = P[i]; c.var[controls.U] = U[i]; c.var[controls.V] = V[i];
        c.var[controls.W] = W[i]; c.var[controls.VF[0]] = VF[i]; c.var[controls.kappa] = 0.0;
        if (flags & 2) {
            c.var[controls.oldU] = old[0][i]; c.var[controls.oldV] = old[1][i]; c.var[controls.oldW] = old[2][i];
            c.var[controls.Qm[0]] = old[3][i]; c.var[controls.Qm[1]] = old[4][i]; c.var[controls.Qm[2]] = old[5][i];
        }
        if (flags & 4) { c.var[controls.oldVF[0]] = oldvf[0][i]; c.var[controls.Qm[3]] = oldvf[1][i]; }
    }
    auto t0 = chrono::steady_clock::now();
    solver.calcIncomCellEOSVF(mesh, controls, species);
    if (flags & 2) solver.calcCellTransport(mesh, controls, species);
    solver.setIncomValuesLeftRightFace(mesh, controls, species);
    solver.setCellVarMinMax(mesh, controls.VF[0], controls.maximumVF[0], controls.minimumVF[0]);
    if (flags & 1) solver.calcSourceGravity(mesh, controls, species);
    if (flags & 8) solver.calcSourceSurfaceTension(mesh, controls, species);
    auto t1 = chrono::steady_clock::now();

    g_out = fopen(argv[2], "wb");
    if (!g_out) { perror(argv[2]); return 2; }

    // geometry -----------------------------------------------------------
    {
        vector<double> a(nf), n3(3 * nf), c3(3 * nf), wc(nf), mpn(nf), al(nf), e3(3 * nf), s3(3 * nf), pf(3 * nf), nfv(3 * nf), d3(3 * nf);
        for (int i = 0; i < nf; ++i) {
            auto& fc = mesh.faces[i];
            a[i] = fc.area; wc[i] = fc.wC; mpn[i] = fc.magPN; al[i] = fc.alphaF;
            c3[3 * i] = fc.x; c3[3 * i + 1] = fc.y; c3[3 * i + 2] = fc.z;
            for (int k = 0; k < 3; ++k) {
                n3[3 * i + k] = fc.unitNormals[k]; e3[3 * i + k] = fc.unitNomalsPN[k];
                s3[3 * i + k] = fc.vecSkewness[k]; pf[3 * i + k] = fc.vecPF[k];
                nfv[3 * i + k] = fc.vecNF[k]; d3[3 * i + k] = fc.distCells[k];
            }
        }
        put("face_area", a); put("face_n", n3); put("face_c", c3); put("face_wC", wc);
        put("face_magPN", mpn); put("face_alphaF", al); put("face_ePN", e3); put("face_skew", s3);
        put("face_vecPF", pf); put("face_vecNF", nfv); put("face_dist", d3);
        vector<double> vol(nc), cc(3 * nc), minv(6 * nc), rho(nc), sg(4 * nc), mxvf(nc), mnvf(nc);
        vector<int> sptr(nc + 1, 0), sidx;
        for (int i = 0; i < nc; ++i) {
            auto& c = mesh.cells[i];
            vol[i] = c.volume; cc[3 * i] = c.x; cc[3 * i + 1] = c.y; cc[3 * i + 2] = c.z;
            for (int k = 0; k < 6; ++k) minv[6 * i + k] = c.coeffLeastSquare1stCellVetexStencil[k];
            for (int j : c.stencil) sidx.push_back(j);
            sptr[i + 1] = (int)sidx.size();
            rho[i] = c.var[controls.Rho];
            for (int k = 0; k < 4; ++k) sg[4 * i + k] = c.var[controls.sourceGravity[k]];
            mxvf[i] = c.var[controls.maximumVF[0]]; mnvf[i] = c.var[controls.minimumVF[0]];
        }
        put("cell_vol", vol); put("cell_c", cc); put("lsq_minv", minv);
        put("stencil_ptr", sptr); put("stencil_idx", sidx);
        put("rho", rho); put("src_grav", sg); put("max_vf", mxvf); put("min_vf", mnvf);
        if (flags & 8) {   // curvature and surface-tension source (pressureBased.cpp:142)
            vector<double> kap(nc), ls(nc), sst(4 * nc);
            for (int i = 0; i < nc; ++i) {
                auto& c = mesh.cells[i];
                kap[i] = c.var[controls.kappa]; ls[i] = c.var[controls.LS];
                for (int k = 0; k < 4; ++k) sst[4 * i + k] = c.var[controls.sourceSurfaceTension[k]];
            }
            put("kappa", kap); put("ls", ls); put("src_sft", sst);
        }
        vector<double> frl(nf), frr(nf), fpl(nf), fpr(nf), ful(3 * nf), fur(3 * nf);
        for (int i = 0; i < nf; ++i) {
            auto& fc = mesh.faces[i];
            frl[i] = fc.varL[controls.fRho]; frr[i] = fc.varR[controls.fRho];
            fpl[i] = fc.varL[controls.fP]; fpr[i] = fc.varR[controls.fP];
            ful[3 * i] = fc.varL[controls.fU]; ful[3 * i + 1] = fc.varL[controls.fV]; ful[3 * i + 2] = fc.varL[controls.fW];
            fur[3 * i] = fc.varR[controls.fU]; fur[3 * i + 1] = fc.varR[controls.fV]; fur[3 * i + 2] = fc.varR[controls.fW];
        }
        put("face_rhoL", frl); put("face_rhoR", frr); put("face_pL", fpl); put("face_pR", fpr);
        put("face_uL", ful); put("face_uR", fur);
        put("CRS_ptr", mesh.CRS_ptr); put("CRS_col", mesh.CRS_col);
        put("CRS_dig", mesh.CRS_col_ptr_dig); put("CRS_LR", mesh.CRS_col_ptr_LR); put("CRS_RL", mesh.CRS_col_ptr_RL);
    }

    // volume-fraction sub-iteration (flag 4): dump and stop --------------
    if (flags & 4) {
        solver.setIncomValuesLeftRightFaceWithVfMSTACS(mesh, controls, species);
        vector<double> vl(nf), vr(nf);
        for (int i = 0; i < nf; ++i) { vl[i] = mesh.faces[i].varL[controls.fVF[0]]; vr[i] = mesh.faces[i].varR[controls.fVF[0]]; }
        put("vof_face_vfL", vl); put("vof_face_vfR", vr);
        auto v0 = chrono::steady_clock::now();
        double vnorm = solver.calcVolfracEq(mesh, controls, species);
        auto v1 = chrono::steady_clock::now();
        vector<double> g(3 * nc), vfn(nc);
        const int tgt[5] = {controls.P, controls.U, controls.V, controls.W, controls.VF[0]};
        const char* gname[5] = {"vof_grad_P", "vof_grad_U", "vof_grad_V", "vof_grad_W", "vof_grad_VF"};
        for (int t = 0; t < 5; ++t) {
            for (int i = 0; i < nc; ++i) for (int k = 0; k < 3; ++k) g[3 * i + k] = mesh.cellsGradientVar[tgt[t]][i][k];
            put(gname[t], g);
        }
        for (int i = 0; i < nc; ++i) vfn[i] = mesh.cells[i].var[controls.VF[0]];
        put("vof_A_rows", g_vof.rows); put("vof_A_cols", g_vof.cols); put("vof_A_vals", g_vof.vals);
        put("vof_B", g_vof.b); put("vof_x", g_vof.x); put("vof_VF_new", vfn);
        put("vof_norm", &vnorm, 1);
        double tv[2] = {chrono::duration<double>(v1 - v0).count(), 0.0};
        put("vof_timings", tv, 2);
        fclose(g_out);
        return 0;
    }

    // momentum equation (outer iteration only) ---------------------------
    double tmom = 0.0;
    if (flags & 2) {
        vector<double> mu(nc);
        for (int i = 0; i < nc; ++i) mu[i] = mesh.cells[i].var[controls.mu];
        put("mu", mu);
        auto m0 = chrono::steady_clock::now();
        solver.setIncomValuesLeftRightFace(mesh, controls, species);
        double mnorm = solver.calcMomentumEqs(mesh, controls, species);
        auto m1 = chrono::steady_clock::now();
        tmom = chrono::duration<double>(m1 - m0).count();
        vector<double> g(3 * nc);
        const int tgt[5] = {controls.P, controls.U, controls.V, controls.W, controls.VF[0]};
        const char* gname[5] = {"mom_grad_P", "mom_grad_U", "mom_grad_V", "mom_grad_W", "mom_grad_VF"};
        for (int t = 0; t < 5; ++t) {
            for (int i = 0; i < nc; ++i) for (int k = 0; k < 3; ++k) g[3 * i + k] = mesh.cellsGradientVar[tgt[t]][i][k];
            put(gname[t], g);
        }
        vector<double> mmp(2 * nc), un(nc), vn(nc), wn(nc);
        for (int i = 0; i < nc; ++i) {
            auto& c = mesh.cells[i];
            mmp[2 * i] = c.var[controls.maximumP]; mmp[2 * i + 1] = c.var[controls.minimumP];
            un[i] = c.var[controls.U]; vn[i] = c.var[controls.V]; wn[i] = c.var[controls.W];
        }
        put("mom_minmax_p", mmp);
        put("mom_A_rows", g_momentum.rows); put("mom_A_cols", g_momentum.cols); put("mom_A_vals", g_momentum.vals);
        put("mom_B0", g_momentum.b[0]); put("mom_B1", g_momentum.b[1]); put("mom_B2", g_momentum.b[2]);
        put("mom_x0", g_momentum.x[0]); put("mom_x1", g_momentum.x[1]); put("mom_x2", g_momentum.x[2]);
        put("mom_U_new", un); put("mom_V_new", vn); put("mom_W_new", wn);
        put("mom_norm", &mnorm, 1);
        solver.setIncomValuesLeftRightFace(mesh, controls, species);
    }

    // pressure-correction equation ---------------------------------------
    auto t2 = chrono::steady_clock::now();
    double norm = solver.calcPressureEq(mesh, controls, species, 1);
    auto t3 = chrono::steady_clock::now();
    {
        vector<double> g(3 * nc);
        const int tgt[5] = {controls.P, controls.U, controls.V, controls.W, controls.VF[0]};
        const char* gname[5] = {"grad_P", "grad_U", "grad_V", "grad_W", "grad_VF"};
        for (int t = 0; t < 5; ++t) {
            for (int i = 0; i < nc; ++i) for (int k = 0; k < 3; ++k) g[3 * i + k] = mesh.cellsGradientVar[tgt[t]][i][k];
            put(gname[t], g);
        }
        vector<double> mm(6 * nc), pn(nc), un(nc), vn(nc), wn(nc);
        for (int i = 0; i < nc; ++i) {
            auto& c = mesh.cells[i];
            mm[6 * i + 0] = c.var[controls.maximumU]; mm[6 * i + 1] = c.var[controls.minimumU];
            mm[6 * i + 2] = c.var[controls.maximumV]; mm[6 * i + 3] = c.var[controls.minimumV];
            mm[6 * i + 4] = c.var[controls.maximumW]; mm[6 * i + 5] = c.var[controls.minimumW];
            pn[i] = c.var[controls.P]; un[i] = c.var[controls.U]; vn[i] = c.var[controls.V]; wn[i] = c.var[controls.W];
        }
        put("minmax_uvw", mm);
        put("A_rows", g_captured.rows); put("A_cols", g_captured.cols); put("A_vals", g_captured.vals);
        put("B", g_captured.b); put("x", g_captured.x);
        put("P_new", pn); put("U_new", un); put("V_new", vn); put("W_new", wn);
        put("norm", &norm, 1);
    }

    // RCM ------------------------------------------------------------------
    {
        auto t4 = chrono::steady_clock::now();
        math.lib_RCM(mesh);
        auto t5 = chrono::steady_clock::now();
        vector<int> perm(nc), iperm(nc);
        for (int i = 0; i < nc; ++i) { perm[i] = mesh.cells[i].RCM; iperm[i] = mesh.cells[i].invRCM; }
        put("rcm_perm", perm); put("rcm_iperm", iperm);
        double tm[5] = {
            chrono::duration<double>(t1 - t0).count(),                       // EOS + face values + gravity
            chrono::duration<double>(t3 - t2).count() - g_captured.solve_seconds,  // pressure assembly + update
            g_captured.solve_seconds,                                        // AMGCL setup + IDR(4) solve
            chrono::duration<double>(t5 - t4).count(),                       // RCM
            (double)g_captured.calls};
        put("timings", tm, 5);
        if (flags & 2) {
            double tmm[2] = {tmom - g_momentum.solve_seconds, g_momentum.solve_seconds};
            put("mom_timings", tmm, 2);
        }
    }
    fclose(g_out);
    return 0;
}
