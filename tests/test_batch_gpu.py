"""Batched channels (the batched-channel machinery) on the GPU vs the oracle run channel
by channel.  Bar: reference arithmetic bit-exact per channel; the FP64
convergence residual equal to the numpy FP64 residual of the oracle's
velocities to 1e-12 relative; graph replay identical to plain launches."""
import numpy as np
import pytest

from lbm_mirror_gb300 import Batch
from lbm_mirror_gb300 import capi as K
from oracle.oracle import OracleLattice
from tests import cases

pytestmark = pytest.mark.gpu


def small_batch(n=10, seed=9):
    return cases.batch_channels(n, seed=seed, nx_range=(20, 70), ny_range=(12, 30))


def oracle_channel(c, steps, arithmetic=K.KEL_ARITH_REFERENCE):
    o = OracleLattice(9, (c["nx"], c["ny"]))
    o.set_flags(c["flags"])
    o.set_profile(c["profile"])
    o.run(cases.channel_program(c["tau"], arithmetic), steps)
    return o


@pytest.mark.parametrize("tile", [128, 256, 512])
def test_batch_matches_oracle_per_channel(tile):
    chans = small_batch()
    prog = cases.channel_program(0.8, K.KEL_ARITH_REFERENCE)
    b = Batch(chans, prog, tile=tile)
    b.step(37)
    for i, c in enumerate(chans):
        o = oracle_channel(c, 37)
        np.testing.assert_array_equal(b.populations(i).astype(np.float64), o.populations())
        rho, u = b.macros(i)
        orho, ou = o.macros()
        fl = c["flags"] != 1
        np.testing.assert_array_equal(rho[fl].astype(np.float64), orho[fl])
        np.testing.assert_array_equal(u[fl].astype(np.float64), ou[fl])
    b.close()


def test_residual_and_convergence_bookkeeping():
    chans = small_batch(6, seed=3)
    prog = cases.channel_program(0.8, K.KEL_ARITH_REFERENCE)
    b = Batch(chans, prog)
    steps, res = b.run_until(tol=1e-30, check_every=100, max_steps=200, use_graph=True)
    assert (steps == 200).all()
    for i, c in enumerate(chans):
        o1 = oracle_channel(c, 100)
        o2 = oracle_channel(c, 200)
        u1 = o1.macros()[1]
        u2 = o2.macros()[1]
        ref = np.sqrt(((u2 - u1) ** 2).sum() / (u2 ** 2).sum())
        assert abs(res[i] - ref) <= 1e-12 * ref
    b.close()


def test_graph_replay_equals_plain_launches_and_converged_channels_freeze():
    chans = small_batch(8, seed=5)
    prog = cases.channel_program(0.8)
    a = Batch(chans, prog)
    b = Batch(chans, prog)
    sa, ra = a.run_until(tol=1e-2, check_every=50, max_steps=20000, use_graph=True)
    sb, rb = b.run_until(tol=1e-2, check_every=50, max_steps=20000, use_graph=False)
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(ra, rb)
    for i in range(len(chans)):
        np.testing.assert_array_equal(a.populations(i), b.populations(i))
    assert a.active_count() == 0 and sa.min() < sa.max()  # channels stop at different times
    frozen = a.populations(0)
    a.step(10)
    np.testing.assert_array_equal(a.populations(0), frozen)


def test_autotune_picks_a_tile_and_keeps_results():
    chans = small_batch(5, seed=1)
    prog = cases.channel_program(0.8, K.KEL_ARITH_REFERENCE)
    b = Batch(chans, prog)
    tile, ms = b.autotune(steps=4)
    assert tile in (128, 256, 512) and ms > 0
    assert b.info()[2] == tile
    b.step(12)
    o = oracle_channel(chans[2], 12)
    np.testing.assert_array_equal(b.populations(2).astype(np.float64), o.populations())


def _rel_l2(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def test_shifted_arithmetic_matches_fp64_oracle_closer_than_fast():
    """Shifted FP32 (g = f - w_i) against the FP64 oracle after 2,000 steps:
    relative L2 of u and of rho - 1 <= 1e-5, and the velocity error no larger
    than the fast (unshifted) arithmetic's."""
    chans = small_batch(6, seed=11)
    err = {}
    for mode in (K.KEL_ARITH_FAST, K.KEL_ARITH_SHIFTED):
        b = Batch(chans, cases.channel_program(0.8, mode))
        b.step(2000)
        e_u, e_r = [], []
        for i, c in enumerate(chans):
            o = OracleLattice(9, (c["nx"], c["ny"]), f64=True)
            o.set_flags(c["flags"])
            o.set_profile(c["profile"])
            o.run(cases.channel_program(c["tau"], K.KEL_ARITH_FAST), 2000)
            orho, ou = o.macros()
            rho, u = b.macros(i)
            fl = c["flags"] != 1
            e_u.append(_rel_l2(u[fl].astype(np.float64), ou[fl]))
            e_r.append(_rel_l2(rho[fl].astype(np.float64) - 1, orho[fl] - 1))
        err[mode] = (max(e_u), max(e_r))
        b.close()
    assert err[K.KEL_ARITH_SHIFTED][0] <= 1e-5 and err[K.KEL_ARITH_SHIFTED][1] <= 1e-5, err
    assert err[K.KEL_ARITH_SHIFTED][0] <= err[K.KEL_ARITH_FAST][0] * 1.5, err


def test_shifted_populations_round_trip_and_switch_back():
    """Downloads add the weights back: at rest every population is w_i; a
    switch to shifted arithmetic and back leaves the populations unchanged."""
    chans = small_batch(3, seed=12)
    b = Batch(chans, cases.channel_program(0.8, K.KEL_ARITH_SHIFTED))
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, np.float32)
    assert np.array_equal(b.populations(1), np.tile(w, (chans[1]["nx"] * chans[1]["ny"], 1)))
    b.step(50)
    before = b.populations(2)
    b.close()
    b2 = Batch(chans, cases.channel_program(0.8, K.KEL_ARITH_SHIFTED))
    b2.step(50)
    np.testing.assert_array_equal(b2.populations(2), before)
    b2.lib.kel_batch_set_program(b2._h, cases.channel_program(0.8, K.KEL_ARITH_FAST))
    b2.lib.kel_batch_set_program(b2._h, cases.channel_program(0.8, K.KEL_ARITH_SHIFTED))
    np.testing.assert_allclose(b2.populations(2), before, rtol=0, atol=1e-7)
    b2.close()


def test_shifted_reaches_1e6_where_fp32_rounding_stalls():
    """A 256x64 channel (tau 0.67, u_max 0.021) whose unshifted FP32 run stalls
    above a relative velocity change of 1e-6 per 1000 steps (the FP64 oracle
    converges in about 41,000 steps) converges in shifted arithmetic."""
    from lbm_mirror_gb300.workloads import batch_channels
    c = batch_channels(n=10, seed=5, nx_range=(256, 256), ny_range=(64, 64))[8]
    b = Batch([c], cases.channel_program(0.8, K.KEL_ARITH_SHIFTED))
    steps, res = b.run_until(tol=1e-6, check_every=1000, max_steps=150_000)
    assert res[0] < 1e-6 and steps[0] <= 100_000, (steps, res)
    b.close()
