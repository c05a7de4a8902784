"""Batched channels (config C4 machinery) on the GPU vs the oracle run channel
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
