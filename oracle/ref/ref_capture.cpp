// Capturing stand-in for the reference's scalar solveAMGCL.
//
// The Makefile compiles the reference's equation translation units (and this
// file) with -DsolveAMGCL=semo_ref_capture_solveAMGCL, so the call at
// src/solvers/eqPressure.cpp:677 lands here.  The assembled COO system is
// copied out for the checker and then handed to the real solver, so the
// reference's pass continues exactly as it would.
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
void semo_ref_forward_solve(const string& eq, SEMO_Mesh_Builder& mesh, int B_n,
                            vector<int>& r, vector<int>& c, vector<double>& v,
                            vector<double>& b, vector<double>& x);

void SEMO_Solvers_Builder::semo_ref_capture_solveAMGCL(
    string equation, SEMO_Mesh_Builder& mesh, int B_n,
    vector<int>& A_rows, vector<int>& A_cols, vector<double>& A_vals,
    vector<double>& B_vals, vector<double>& resiVar) {
    if (equation == "pressure" && g_captured.calls == 0) {
        g_captured.rows = A_rows; g_captured.cols = A_cols; g_captured.vals = A_vals;
        g_captured.b = B_vals;
    }
    semo_ref_forward_solve(equation, mesh, B_n, A_rows, A_cols, A_vals, B_vals, resiVar);
    if (equation == "pressure" && g_captured.calls == 0) g_captured.x = resiVar;
    ++g_captured.calls;
}
