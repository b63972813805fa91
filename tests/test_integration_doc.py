"""The C++ replacement of calcPressureEq shown in INTEGRATION.md compiles
against include/semo_gb300.h.

The snippet uses SEMO's mesh, controls and species types; minimal stand-ins
with the members it touches are declared in front of it, so the check is the
library's part: every C-ABI call, struct field and constant the snippet names
exists in the header with a compatible signature.
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STANDINS = r"""
#include <cstdint>
#include <iostream>
#include <string>
#include <vector>
using namespace std;
struct SEMO_Point { double x, y, z; };
namespace SEMO_Types { enum { INTERNAL_FACE = 0, BOUNDARY_FACE = 1 }; }
struct SEMO_Face { vector<int> points; int owner = 0, neighbour = 0; int getType() const { return 0; } };
struct SEMO_Cell { vector<double> var; };
struct SEMO_Boundary { int startFace = 0, nFaces = 0; vector<string> type; vector<double> var; };
struct SEMO_Mesh_Builder { vector<SEMO_Point> points; vector<SEMO_Face> faces; vector<SEMO_Cell> cells;
                           vector<SEMO_Boundary> boundary; };
struct SEMO_Controls_Builder { double timeStep = 0, gravityAcceleration[3] = {}, prePreURF = 0, preVelURF = 0;
                               int P = 0, U = 1, V = 2, W = 3; vector<int> VF; };
struct SEMO_Species { double rho = 0, mu = 0; };
struct SEMO_Solvers_Builder {
    double calcPressureEq(SEMO_Mesh_Builder&, SEMO_Controls_Builder&, vector<SEMO_Species>&, int);
};
typedef int MPI_Comm;
static const MPI_Comm MPI_COMM_WORLD = 0;
inline int MPI_Abort(MPI_Comm, int) { return 0; }
"""


def cpp_blocks(text):
    return re.findall(r"```cpp\n(.*?)```", text, flags=re.S)


def test_integration_snippet_compiles(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        blocks = cpp_blocks(f.read())
    assert blocks, "INTEGRATION.md has no C++ block"
    src = tmp_path / "snippet.cpp"
    src.write_text(STANDINS + "\n".join(blocks))
    out = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"),
                          str(src)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
