"""The CPU oracle against golden vectors from the reference's own components.

The fixtures were produced by oracle/ref_harness.cpp (keldu/lbm_mirror's
headers compiled unchanged); the oracle must reproduce them bit for bit:
populations, density and velocity, FP32 and FP64.
"""
import numpy as np
import pytest

from tests import cases
from tests.golden import make_golden as G

NAMES = G.names()


def test_fixture_set_complete():
    assert len(NAMES) >= 18
    for must in ("poiseuille_256x64", "cavity_d3q19", "cavity_d3q27", "mixed2d_psmguo", "mixed3d_d3q27_bgk"):
        assert must in NAMES


@pytest.mark.parametrize("name", [n for n in NAMES if n != "poiseuille_256x64"])
def test_oracle_bit_exact(name):
    case, dfs, rho, vel = G.load(name)
    odfs, orho, ovel = cases.run_oracle(case)
    np.testing.assert_array_equal(odfs, dfs)
    np.testing.assert_array_equal(orho, rho)
    np.testing.assert_array_equal(ovel, vel)


def test_oracle_bit_exact_config1_full():
    """C1 at full size: D2Q9 256x64, 10,000 steps."""
    case, dfs, rho, vel = G.load("poiseuille_256x64")
    odfs, orho, ovel = cases.run_oracle(case)
    np.testing.assert_array_equal(odfs, dfs)
    np.testing.assert_array_equal(orho, rho)
    np.testing.assert_array_equal(ovel, vel)


def test_config1_matches_analytic_parabola():
    """Steady Poiseuille flow: mid-channel u_x(y) close to the inlet parabola."""
    case, dfs, rho, vel = G.load("poiseuille_256x64")
    nx, ny = case["dims"]
    ux = vel[:, 0].reshape(ny, nx)
    prof = case["profile"]
    col = ux[1:-1, nx // 2]
    ref = prof[1:-1]
    err = np.abs(col - ref).max() / np.abs(ref).max()
    assert err < 0.08, err


def test_equilibrium_rest_is_weights():
    """equilibrium.cpp:8-40: f_eq(rho=1, u=0) == w_i exactly (extended to D3Q19/27)."""
    from oracle.oracle import equilibrium_f32
    for q in (9, 19, 27):
        eq = equilibrium_f32(q, 1.0, [0.0, 0.0, 0.0])
        w = cases._weights(q).astype(np.float32)
        np.testing.assert_array_equal(eq, w)


def test_equilibrium_moments_round_trip():
    """macroscopic.cpp:21-112: equilibrium -> moments round trip."""
    from oracle.oracle import equilibrium_f32
    for q in (9, 19, 27):
        D = 2 if q == 9 else 3
        u = np.array([0.03, -0.02, 0.01][:D], dtype=np.float32)
        eq = equilibrium_f32(q, 1.1, u).astype(np.float64)
        c = _dirs(q)
        rho = eq.sum()
        assert abs(rho - 1.1) < 1e-6
        np.testing.assert_allclose((eq[:, None] * c).sum(0) / rho, u, atol=1e-7)


def _dirs(q):
    if q == 9:
        return np.array([[0, 0], [-1, 0], [1, 0], [0, -1], [0, 1], [-1, -1], [1, 1], [-1, 1], [1, -1]])
    if q == 19:
        return np.array([[0, 0, 0], [-1, 0, 0], [1, 0, 0], [0, -1, 0], [0, 1, 0], [0, 0, -1], [0, 0, 1],
                         [-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 1, 0], [-1, 0, -1], [1, 0, -1], [-1, 0, 1],
                         [1, 0, 1], [0, -1, -1], [0, 1, -1], [0, -1, 1], [0, 1, 1]])
    o3 = [0, -1, 1]
    return np.array([[o3[i % 3], o3[(i // 3) % 3], o3[i // 9]] for i in range(27)])
