"""The oracle's curvature and surface-tension source against the reference.

Fixtures whose case has sigma != 0 hold what the reference computed in
calcSourceSurfaceTension (src/solvers/source/surfaceTension.cpp:7-215,
called at src/solvers/pressureBased.cpp:142) before the pass: the level set
``ls``, the curvature ``kappa`` and ``src_sft`` (4 per cell).  Their pressure,
momentum and volume-fraction systems carry the calcInterpolVelSurfTens face
terms (src/solvers/surfaceNormalVelocity.cpp:190-221) and are checked bit for
bit by the pass tests of the other oracle test files; here the curvature
itself is checked, and properties of the source that hold for any mesh.
"""
import numpy as np
import pytest

from golden_io import _all, load

SFT = [n for n in _all() if not n.startswith("foam_") and n.endswith("s")]


@pytest.fixture(scope="module", params=SFT)
def sft(request):
    from oracle.oracle import Oracle
    case, ref = load(request.param)
    o = Oracle(case.mesh)
    o.set_case(case)       # sigma != 0: computes ls, kappa and src_sft
    return request.param, case, ref, o


def test_fixtures_present():
    assert len(SFT) >= 3
    for n in SFT:
        case, ref = load(n)
        assert case.sigma != 0.0 and "kappa" in ref, n


@pytest.mark.parametrize("name", ["ls", "kappa", "src_sft"])
def test_bit_exact(sft, name):
    _, _, ref, o = sft
    assert np.array_equal(o.get(name), ref[name])


def test_source_is_linear_in_sigma(sft):
    """src_sft = sigma kappa grad(VF): curvature unchanged, source scaled."""
    _, case, ref, o = sft
    from oracle.oracle import Oracle
    o2 = Oracle(case.mesh)
    o2.set_case(case)
    o2.surface_tension(2.0 * case.sigma)
    assert np.array_equal(o2.get("kappa"), o.get("kappa"))
    s1, s2 = o.get("src_sft").reshape(-1, 4), o2.get("src_sft").reshape(-1, 4)
    np.testing.assert_allclose(s2[:, :3], 2.0 * s1[:, :3], rtol=1e-14, atol=0.0)


def test_uniform_field_has_no_source(sft):
    """With a uniform volume fraction there is no interface: no source, no face terms."""
    _, case, _, _ = sft
    from oracle.oracle import Oracle
    c = load(case.name)[0]
    c.VF = np.full_like(c.VF, 0.5)
    o = Oracle(c.mesh)
    o.set_case(c)
    assert np.all(o.get("src_sft").reshape(-1, 4)[:, :3] == 0.0)
