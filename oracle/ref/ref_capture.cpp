// Capturing stand-ins for the reference's solveAMGCL overloads.
//
// The Makefile compiles the reference's equation translation units (and this
// file) with -DsolveAMGCL=semo_ref_capture_solveAMGCL, so the calls at
// src/solvers/eqPressure.cpp:677 and src/solvers/eqVolfrac.cpp:766 (scalar)
// and src/solvers/eqMomentum.cpp:1017 (three right-hand sides) land here.  The assembled COO system is copied out
// for the oracle tests and then handed to the real solver, so the reference's pass
// continues exactly as it would.
#include <string>
#include <vector>

#include "../solvers/build.h"

using namespace std;

struct CapturedSystem {
    vector<int> rows, cols;
    vector<double> vals, b, x;
    double solve_seconds = 0.0;
    int calls = 0;
};
extern CapturedSystem g_captured;
struct CapturedMomentum {
    vector<int> rows, cols;
    vector<double> vals, b[3], x[3];
    double solve_seconds = 0.0;
    int calls = 0;
};
extern CapturedMomentum g_momentum;
extern CapturedSystem g_vof;
void semo_ref_forward_solve(const string& eq, SEMO_Mesh_Builder& mesh, int B_n,
                            vector<int>& r, vector<int>& c, vector<double>& v,
                            vector<double>& b, vector<double>& x);
void semo_ref_forward_solve3(const string& eq, SEMO_Mesh_Builder& mesh, int B_n,
                             vector<int>& r, vector<int>& c, vector<double>& v,
                             vector<double>& b0, vector<double>& b1, vector<double>& b2,
                             vector<double>& x0, vector<double>& x1, vector<double>& x2);

void SEMO_Solvers_Builder::semo_ref_capture_solveAMGCL(
    string equation, SEMO_Mesh_Builder& mesh, int B_n,
    vector<int>& A_rows, vector<int>& A_cols, vector<double>& A_vals,
    vector<double>& B_vals, vector<double>& resiVar) {
    CapturedSystem* cap = (equation == "pressure") ? &g_captured
                        : (equation == "volume_fraction") ? &g_vof : nullptr;
    const bool first = cap && cap->calls == 0;
    if (first) {
        cap->rows = A_rows; cap->cols = A_cols; cap->vals = A_vals;
        cap->b = B_vals;
    }
    semo_ref_forward_solve(equation, mesh, B_n, A_rows, A_cols, A_vals, B_vals, resiVar);
    if (first) cap->x = resiVar;
    if (cap) ++cap->calls;
}

void SEMO_Solvers_Builder::semo_ref_capture_solveAMGCL(
    string equation, SEMO_Mesh_Builder& mesh, int B_n,
    vector<int>& A_rows, vector<int>& A_cols, vector<double>& A_vals,
    vector<double>& B0_vals, vector<double>& B1_vals, vector<double>& B2_vals,
    vector<double>& resiVar0, vector<double>& resiVar1, vector<double>& resiVar2) {
    const bool first = g_momentum.calls == 0;
    if (first) {
        g_momentum.rows = A_rows; g_momentum.cols = A_cols; g_momentum.vals = A_vals;
        g_momentum.b[0] = B0_vals; g_momentum.b[1] = B1_vals; g_momentum.b[2] = B2_vals;
    }
    semo_ref_forward_solve3(equation, mesh, B_n, A_rows, A_cols, A_vals, B0_vals, B1_vals, B2_vals,
                            resiVar0, resiVar1, resiVar2);
    if (first) { g_momentum.x[0] = resiVar0; g_momentum.x[1] = resiVar1; g_momentum.x[2] = resiVar2; }
    ++g_momentum.calls;
}
