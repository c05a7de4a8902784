"""Half-way bounce-back walls (KEL_BC_HALFWAY_WALL) on the GPU against the
oracle's restatement.  Bars: reference arithmetic bit-exact on every
computed cell (populations stored at wall cells are undefined and left out),
for D2Q9 / D3Q19 / D3Q27, periodic and bounded rows, every launch shape
(shapes other than one cell per thread fall back to it), chunked stepping
from both parities; fast arithmetic reaches the analytic Poiseuille profile
of the oracle's known-answer test."""
import numpy as np
import pytest

from lbm_mirror_gb300 import capi as K
from tests import cases
from tests.gpu_util import run_gpu, with_arith

pytestmark = pytest.mark.gpu

ROWS = K.KEL_LAUNCH_ROWS


def computed(case):
    wall = {fl for fl, o in enumerate(case["program"].ops) if o.bc == K.KEL_BC_HALFWAY_WALL}
    return ~np.isin(case["flags"], list(wall))


@pytest.mark.parametrize("periodic", [False, True], ids=["bounded", "periodic"])
@pytest.mark.parametrize("q,dims", [(9, (40, 18)), (19, (16, 12, 10)), (27, (16, 12, 10))])
def test_reference_arithmetic_bit_exact_vs_oracle(q, dims, periodic):
    case = cases.halfway_mixed(q, dims, steps=23, periodic=periodic)
    of, orho, ovel = cases.run_oracle(case)
    keep = computed(case)
    for launch in [None, (4, 256), (ROWS, 3)]:
        f, r, v = run_gpu(case, K.KEL_ARITH_REFERENCE, launch=launch)
        np.testing.assert_array_equal(f[keep], of[keep])
        fluid = case["flags"] == 2
        np.testing.assert_array_equal(v[fluid], ovel[fluid])
        np.testing.assert_array_equal(r[fluid], orho[fluid])


@pytest.mark.parametrize("chunks", [[1, 1, 1, 20], [2, 7, 14], [23]])
def test_chunked_steps_same_bits(chunks):
    case = cases.halfway_mixed(19, (16, 12, 10), steps=23)
    of, _, _ = cases.run_oracle(case)
    f, _, _ = run_gpu(case, K.KEL_ARITH_REFERENCE, chunks=chunks)
    keep = computed(case)
    np.testing.assert_array_equal(f[keep], of[keep])


def test_fast_arithmetic_poiseuille_profile():
    # g = 1e-5: the Guo increment per step (~3 w_i g) stays well above the
    # FP32 rounding of the rest populations (~6e-8 x 4/9)
    tau, g, nx, ny = 0.8, 1e-5, 8, 22
    case = cases.halfway_poiseuille_2d(nx=nx, ny=ny, steps=8000, tau=tau, g=g)
    _, _, v = run_gpu(case, K.KEL_ARITH_FAST)
    u = v[:, 0].reshape(ny, nx)[1:ny - 1].mean(axis=1)
    nu = (tau - 0.5) / 3.0
    y = np.arange(1, ny - 1)
    exact = (1.0 - 0.5 / tau) * g / (2 * nu) * (y - 0.5) * (ny - 1.5 - y)
    err = np.abs(u - exact).max() / exact.max()
    assert err < 5e-3, err


def test_fp16s_halfway_cavity_vs_fp64():
    """FP16-shifted storage with half-way walls: a D3Q19 lid-driven cavity
    whose side walls are half-way walls, against the FP64 oracle of the same
    case, relative L2 velocity error <= 1e-3 (the FP16S bar of the other
    cavities).  A slow force-driven steady flow is no FP16S case: its
    per-step momentum input falls below the half-precision rounding of the
    populations' deviation from rest, which biases the steady profile by a
    few per cent."""
    case = cases.cavity_3d(19, dims=(32, 32, 32), steps=400)
    d = K.program_to_dict(case["program"])
    d["ops"][1] = dict(bc=K.KEL_BC_HALFWAY_WALL, collide=0, east=0, use_profile=0, rho=1.0, u=[0, 0, 0])
    case["program"] = K.program_from_dict(d)
    _, _, vel64 = cases.run_oracle(dict(case, f64=True))
    _, _, v16 = run_gpu(case, K.KEL_ARITH_FAST, storage="fp16s")
    fluid = case["flags"] == 2
    err = np.linalg.norm(v16[fluid] - vel64[fluid]) / np.linalg.norm(vel64[fluid])
    assert err < 1e-3, err
