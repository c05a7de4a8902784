"""Host side of the learned warm start: the FP64 reconstruction oracle's
moments (no GPU), the target normalisation, and the warm-start bench line's
bookkeeping."""
import numpy as np
import pytest

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


def test_oracle_wall_cells_hold_neighbours_post_collision_populations():
    rng = np.random.default_rng(6)
    flags, pred = _field(rng, 8, 10)
    tau = 0.6
    scale, offset = (1, 1, 0.1), (0, 0, 1)
    f = O.warm_start_populations(flags, pred, scale, offset, tau).reshape(8, 10, 9)
    fneq0 = O.warm_start_populations(flags, pred, scale, offset, tau, with_neq=False).reshape(8, 10, 9)
    rho = pred[..., 2] * 0.1 + 1
    x = 5
    # bottom-wall cell (0, x): slots pointing up from the fluid row above come
    # from there; the others hold the rest state at the neighbours' density
    want_rest = np.mean([rho[1, x - 1], rho[1, x], rho[1, x + 1]])
    for i in range(9):
        if O.CY[i] < 0:  # source (x - cx, 1) is fluid
            post = fneq0[1, x - O.CX[i], i] + (1 - 1 / tau) * (f[1, x - O.CX[i], i] - fneq0[1, x - O.CX[i], i])
            assert abs(f[0, x, i] - post) < 1e-14
        else:
            assert abs(f[0, x, i] - O.W[i] * want_rest) < 1e-14


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
    assert abs(np.sqrt(np.mean(t[..., 2][mask == 0] ** 2)) - 0.25) < 1e-5


def test_lubrication_input_is_the_poiseuille_profile_in_an_empty_channel():
    """Without obstacles the lubrication channel is the inlet's parabola
    (u_x / u_max = 4 eta (1 - eta), halved) and the downstream resistance
    falls linearly to 1 / W at the outlet column."""
    H, W = 10, 12
    mask = np.zeros((1, H, W), np.uint8)
    mask[0, 0, :] = mask[0, -1, :] = 1
    x = O.unet_input(mask, np.array([0.05]), np.array([0.8]))
    eta = (np.arange(1, H - 1) - 0.5) / (H - 2)
    np.testing.assert_allclose(x[0, 1:H - 1, 3, 9], 0.5 * 4 * eta * (1 - eta), rtol=1e-12)
    np.testing.assert_allclose(x[0, 1:H - 1, :, 6][0], (W - np.arange(W)) / W, rtol=1e-12)
    assert (x[0, 0, :, 5:] == 0).all()


def test_lubrication_input_splits_flux_as_gap_cubes():
    """An obstacle splitting a column into gaps of h1 = 3 and h2 = 5 cells:
    each gap's estimate is h^2 / (h1^3 + h2^3) times its own profile, so the
    summed estimates are in the ratio h1^2 S1 : h2^2 S2 (S = the sum of
    4 s (1 - s) over the gap's cell midpoints, about 2 h / 3)."""
    H, W = 12, 4
    mask = np.zeros((1, H, W), np.uint8)
    mask[0, 0, :] = mask[0, -1, :] = 1
    mask[0, 4:6, 2] = 1  # gaps of 3 (y 1..3) and 5 (y 6..10) cells in column 2
    x = O.unet_input(mask, np.array([0.05]), np.array([0.8]))
    u = 2 * x[0, :, 2, 9]  # u_x / u_max estimate
    q1, q2 = u[1:4].sum(), u[6:11].sum()
    s1 = sum(4 * ((k + 0.5) / 3) * (1 - (k + 0.5) / 3) for k in range(3))
    s2 = sum(4 * ((k + 0.5) / 5) * (1 - (k + 0.5) / 5) for k in range(5))
    np.testing.assert_allclose(q1 / q2, (3 ** 2 * s1) / (5 ** 2 * s2), rtol=1e-12)


def test_bench_warm_start_line_for_single_networks_and_ensembles(monkeypatch, capsys):
    """bench.py's warm-start workload assembles its JSON line for one network
    and for an ensemble (`--ensemble K`): the GPU steps (steady states,
    training, the two runs, inference) replaced by fakes, the bookkeeping
    around them run as is."""
    import json
    import types
    torch = pytest.importorskip("torch")
    import bench

    class Net:
        n_params = 1000

        def params(self):
            return np.zeros(3)

    class Model:
        def __init__(self):
            self.net, self.history, self.rho_scale, self.rho_norm = Net(), [(0, 0.5), (1, 0.1)], 2.0, "lubrication"

    class States:
        steps = np.ones(4, np.int64)
        seconds = 1.0
        converged = np.ones(4, bool)
        residual = np.zeros(4)

    keys = ["warm_seconds", "plain_seconds", "speedup", "warm_steps_max", "warm_init_seconds", "plain_steps_mean",
            "warm_steps_mean", "plain_steps_max", "plain_unconverged", "warm_unconverged", "final_u_rel_l2_mean",
            "final_u_rel_l2_max", "prediction_u_rel_l2_mean", "prediction_u_rel_l2_max",
            "prediction_drho_rel_l2_mean", "nonfinite_channels", "warm_fallbacks_to_rest", "steady_init_steps_mean",
            "rho_one_steps_mean", "no_neq_steps_mean", "exact_u_net_rho_steps_mean", "net_u_exact_rho_steps_mean"]
    monkeypatch.setattr(WS, "fixed_size_channels", lambda n, seed, nx, ny: list(range(n)))
    monkeypatch.setattr(WS, "solve", lambda *a, **k: States())
    monkeypatch.setattr(WS, "steady_subset", lambda s: s)
    monkeypatch.setattr(WS, "train", lambda s, **k: Model())
    monkeypatch.setattr(WS, "evaluate", lambda *a, **k: {key: 1.0 for key in keys})
    monkeypatch.setattr(WS, "channel_inputs", lambda ch: (np.zeros(2), np.zeros(2), np.zeros(2)))
    monkeypatch.setattr(WS, "predict", lambda *a, **k: None)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(torch.Tensor, "cuda", lambda self, *a, **k: self)

    def ensemble(s, seeds, **k):
        e = WS.WarmStartEnsemble.__new__(WS.WarmStartEnsemble)
        e.members = [Model() for _ in seeds]
        e.rho_norm, e.rho_scale = "lubrication", 2.0
        return e

    monkeypatch.setattr(WS, "train_ensemble", ensemble)
    for k in (1, 3):
        args = types.SimpleNamespace(workload="d2q9_warm_start_256x64", train=64, test=8, tol=1e-6, max_steps=10,
                                     epochs=1, rho_rms=0.25, residual=False, weight_by_steps=False,
                                     rho_norm="lubrication", rho_residual=False, flip=True, ensemble=k, save_dir="")
        bench.run_warm_start(args, 0, 1)
        line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
        assert line["config"]["ensemble"] == k
        assert line["config"]["params"] == 1000 * k
        assert line["training"]["adam_steps"] == 1 * (64 // 32) * k
        assert line["training"]["loss_last"] == 0.1
