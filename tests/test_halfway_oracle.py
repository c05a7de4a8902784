"""Half-way bounce-back in the CPU oracle (a restatement: the reference's
walls are full-way).  Known answer: force-driven Poiseuille flow between
half-way walls reaches the parabola whose walls sit half way between the wall
and the first fluid cell.  The reference's BGKGuo drops the half-force
velocity shift (collision.hpp:156-158), so the momentum it adds per step is
(1 - 1/(2 tau)) g, not g: the parabola's amplitude uses that effective force.
BGK reproduces it to a few 1e-3 relative (the viscosity-dependent slip of
half-way walls under BGK)."""
import numpy as np

from tests import cases

from oracle.oracle import build


def test_halfway_poiseuille_profile_matches_analytic():
    build()
    tau, g, nx, ny = 0.8, 1e-6, 8, 22
    case = cases.halfway_poiseuille_2d(nx=nx, ny=ny, steps=3000, tau=tau, g=g, f64=True)
    _, rho, vel = cases.run_oracle(case)
    u = vel[:, 0].reshape(ny, nx)
    nu = (tau - 0.5) / 3.0
    y = np.arange(1, ny - 1)
    g_eff = (1.0 - 0.5 / tau) * g
    exact = g_eff / (2 * nu) * (y - 0.5) * (ny - 1.5 - y)
    got = u[1:ny - 1].mean(axis=1)
    assert np.abs(u[1:ny - 1] - got[:, None]).max() < 1e-12 * exact.max()  # uniform along x
    rel = np.abs(got - exact).max() / exact.max()
    assert rel < 5e-3, rel
