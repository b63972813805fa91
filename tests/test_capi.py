"""The C-ABI library: builds for sm_103a, loads, exports every declared symbol.

No compute calls here: these run without a GPU.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "semo_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(semo_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib_path():
    from semo_mesh_gb300.build import build
    return build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("semo_ctx_create", "semo_mesh_upload", "semo_rcm", "semo_pressure_pass", "semo_solve_coo",
              "semo_get_system_rcm", "semo_vjp_source"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_params_defaults(lib_path):
    import semo_mesh_gb300 as S
    L = S.load_library(lib_path)
    p = S.Params()
    L.semo_params_default(ctypes.byref(p))
    assert p.tol == 1e-8 and p.precision == S.PREC_MIXED and p.coarse_enough == 64


def test_no_cpu_fallback_without_device(lib_path):
    """Without a GPU the context refuses to start (no silent CPU path)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import semo_mesh_gb300 as S
    with pytest.raises(S.SemoError):
        S.Context()
