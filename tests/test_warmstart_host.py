"""Host side of the learned warm start: the FP64 reconstruction oracle's
moments (no GPU) and the target normalisation."""
import numpy as np

from lbm_mirror_gb300 import warmstart as WS
from oracle import warmstart_oracle as O


def _field(rng, ny, nx):
    flags = np.full((ny, nx), 2, np.uint8)
    flags[0, :] = flags[-1, :] = 1
    flags[ny // 2 - 2:ny // 2 + 1, nx // 3:nx // 3 + 3] = 1
    pred = np.empty((ny, nx, 3))
    pred[..., :2] = rng.uniform(-1, 1, (ny, nx, 2))
    pred[..., 2] = rng.uniform(-1, 1, (ny, nx))
    return flags, pred


def test_oracle_moments_are_chapman_enskog():
    """Sum f = rho and sum c f = rho u on fluid cells; the second moment of
    f_neq is -rho cs^2 tau (grad u + grad u^T)."""
    rng = np.random.default_rng(5)
    ny, nx, tau = 12, 20, 0.73
    flags, pred = _field(rng, ny, nx)
    scale, offset = (0.05, 0.05, 0.01), (0.0, 0.0, 1.0)
    f = O.warm_start_populations(flags, pred, scale, offset, tau, True).reshape(ny, nx, 9)
    feq = O.warm_start_populations(flags, pred, scale, offset, tau, False).reshape(ny, nx, 9)
    phys = pred * np.array(scale) + np.array(offset)
    fluid = flags != 1
    ux = np.where(fluid, phys[..., 0], 0.0)
    uy = np.where(fluid, phys[..., 1], 0.0)
    for y in range(1, ny - 1):
        for x in range(1, nx - 1):
            if not fluid[y, x]:
                continue
            r = phys[y, x, 2]
            assert abs(f[y, x].sum() - r) < 1e-12
            assert abs((f[y, x] * O.CX).sum() - r * ux[y, x]) < 1e-12
            assert abs((f[y, x] * O.CY).sum() - r * uy[y, x]) < 1e-12
            neq = f[y, x] - feq[y, x]
            dxu = (ux[y, x + 1] - ux[y, x - 1]) / 2
            dyv = (uy[y + 1, x] - uy[y - 1, x]) / 2
            dxv = (uy[y, x + 1] - uy[y, x - 1]) / 2
            dyu = (ux[y + 1, x] - ux[y - 1, x]) / 2
            pxx = (neq * O.CX * O.CX).sum()
            pyy = (neq * O.CY * O.CY).sum()
            pxy = (neq * O.CX * O.CY).sum()
            assert abs(pxx - (-r * tau * 2 * dxu / 3)) < 1e-12
            assert abs(pyy - (-r * tau * 2 * dyv / 3)) < 1e-12
            assert abs(pxy - (-r * tau * (dxv + dyu) / 3)) < 1e-12


def test_oracle_wall_cells_rest_at_neighbour_density():
    rng = np.random.default_rng(6)
    flags, pred = _field(rng, 8, 10)
    f = O.warm_start_populations(flags, pred, (1, 1, 0.1), (0, 0, 1), 0.6).reshape(8, 10, 9)
    # a bottom-wall cell below fluid: mean density of its 3 fluid neighbours
    rho = pred[..., 2] * 0.1 + 1
    x = 5
    want = np.mean([rho[1, x - 1], rho[1, x], rho[1, x + 1]])
    assert np.allclose(f[0, x], O.W * want, rtol=0, atol=1e-14)


def test_targets_normalisation_round_trip():
    rng = np.random.default_rng(7)
    chans = WS.fixed_size_channels(4, seed=11, nx=32, ny=16)
    rho = 1 + 0.01 * rng.standard_normal((4, 16, 32)).astype(np.float32)
    u = 0.05 * rng.standard_normal((4, 16, 32, 2)).astype(np.float32)
    st = WS.SteadyStates(chans, rho, u, np.zeros(4, np.uint64), np.zeros(4), 0.0)
    t, s = WS.targets(st)
    _, u_max, _ = WS.channel_inputs(chans)
    um = u_max[:, None, None]
    assert np.allclose(t[..., 0] * um, u[..., 0], rtol=1e-6, atol=1e-9)
    assert np.allclose(t[..., 2] * um * s + 1, rho, rtol=1e-6, atol=1e-6)
    mask, _, _ = WS.channel_inputs(chans)
    assert mask.shape == (4, 16, 32) and set(np.unique(mask)) <= {0, 1}
    assert abs(np.sqrt(np.mean(t[..., 2][mask == 0] ** 2)) - 1.0) < 1e-5
