"""GPU sweep vs the reference (golden vectors) and vs the CPU oracle.

Bar: KEL_ARITH_REFERENCE (the reference's rounding sequence, FP64 equilibrium
bracket) is bit-exact against the reference's own outputs.  KEL_ARITH_FAST
(float-float equilibrium bracket, fused BGK relaxation) stays within 1e-5
relative L2 error (||a - b|| / ||b||, the norm of the reference's
scripts/python/csv_l2_norm.py) on populations, density and velocity.
FP16-shifted storage is within 1e-3 relative L2 velocity error of FP64.
"""
import numpy as np
import pytest

from lbm_mirror_gb300 import capi as K
from tests import cases
from tests.golden import make_golden as G
from tests.gpu_util import make_lattice, rel_err, rel_l2, run_gpu, with_arith

pytestmark = pytest.mark.gpu

FAST_TOL = 1e-5
F32_NAMES = [n for n in G.names() if not n.endswith("_f64")]


# (cells per thread, threads per block); (KEL_LAUNCH_ROWS, stages) is the row pipeline
ROWS = K.KEL_LAUNCH_ROWS
LAUNCHES = [(1, 256), (2, 256), (4, 256), (1, 64), (2, 64), (4, 128), (ROWS, 2), (ROWS, 4)]


def launch_id(l):
    return f"rows_{l[1]}stages" if l[0] == ROWS else f"{l[0]}cell_{l[1]}thr"


@pytest.mark.parametrize("launch", LAUNCHES, ids=launch_id)
@pytest.mark.parametrize("name", F32_NAMES)
def test_reference_arithmetic_bit_exact(name, launch):
    """Bit-exact for every launch shape (one or four cells per thread, row pipeline)."""
    case, dfs, rho, vel = G.load(name)
    f, r, v = run_gpu(case, K.KEL_ARITH_REFERENCE, launch=launch)
    np.testing.assert_array_equal(f, dfs)
    np.testing.assert_array_equal(r, rho)
    np.testing.assert_array_equal(v, vel)


@pytest.mark.parametrize("launch", [None, (ROWS, 3)], ids=lambda l: "default" if l is None else launch_id(l))
@pytest.mark.parametrize("name", F32_NAMES)
def test_fast_arithmetic_within_1e5(name, launch):
    case, dfs, rho, vel = G.load(name)
    f, r, v = run_gpu(case, K.KEL_ARITH_FAST, launch=launch)
    assert rel_l2(f, dfs) < FAST_TOL
    assert rel_l2(r, rho) < FAST_TOL
    assert rel_l2(v, vel) < FAST_TOL
    assert rel_err(v, vel) < 5 * FAST_TOL  # max-norm stays in the same range


@pytest.mark.parametrize("launch", [None, (ROWS, 3)], ids=lambda l: "default" if l is None else launch_id(l))
@pytest.mark.parametrize("chunks", [[1, 1, 1, 18], [2, 7, 12], [21]])
def test_step_chunking_and_parity(chunks, launch):
    """Stepping 1, 2, 7 ... at a time (odd and even entry parities) gives the
    same bits as one call."""
    case, dfs, rho, vel = G.load("mixed3d_d3q19_guo")
    f, r, v = run_gpu(case, K.KEL_ARITH_REFERENCE, chunks=chunks, launch=launch)
    np.testing.assert_array_equal(f, dfs)


def test_upload_at_odd_time_step():
    """Download at odd t, upload into a fresh lattice advanced to odd t, and
    continue: identical to the uninterrupted run."""
    case = G.normalise(cases.mixed_2d(K.KEL_COLL_BGK_GUO, steps=0))
    prog = with_arith(case["program"], K.KEL_ARITH_REFERENCE)
    a = make_lattice(case)
    a.step(prog, 5)
    mid = a.populations(np.float64)
    a.step(prog, 6)
    ref = a.populations(np.float64)
    b = make_lattice(case)
    b.step(prog, 5)
    b.upload_populations(mid)
    b.step(prog, 6)
    np.testing.assert_array_equal(b.populations(np.float64), ref)


@pytest.mark.parametrize("launch", [(1, 256), (2, 128), (4, 256), (ROWS, 3)], ids=launch_id)
@pytest.mark.parametrize("q", [9, 27])
def test_periodic_x_matches_oracle(q, launch):
    if q == 9:
        case = G.normalise(cases.mixed_2d(K.KEL_COLL_PSM_GUO, dims=(48, 20), periodic=True, steps=23))
    else:
        case = G.normalise(cases.mixed_3d(27, K.KEL_COLL_BGK_GUO, dims=(16, 12, 10), periodic=True, steps=15))
    odfs, orho, ovel = cases.run_oracle(case)
    f, r, v = run_gpu(case, K.KEL_ARITH_REFERENCE, launch=launch)
    np.testing.assert_array_equal(f, odfs)
    np.testing.assert_array_equal(v, ovel)


@pytest.mark.parametrize("launch", [(1, 64), (2, 64), (4, 256), (ROWS, 4)], ids=launch_id)
@pytest.mark.parametrize("nx", [5, 37, 130, 131])
def test_ragged_widths_match_oracle(nx, launch):
    """Row widths that are not multiples of 4 or of a warp's 128 cells."""
    case = G.normalise(cases.mixed_2d(K.KEL_COLL_BGK, dims=(nx, 9), steps=9, seed=7))
    odfs, orho, ovel = cases.run_oracle(case)
    f, r, v = run_gpu(case, K.KEL_ARITH_REFERENCE, launch=launch)
    np.testing.assert_array_equal(f, odfs)
    np.testing.assert_array_equal(r, orho)


def test_config1_full_size_bit_exact():
    """C1 at full size: D2Q9 256x64 Poiseuille, 10,000 steps."""
    case, dfs, rho, vel = G.load("poiseuille_256x64")
    f, r, v = run_gpu(case, K.KEL_ARITH_REFERENCE)
    np.testing.assert_array_equal(v, vel)
    np.testing.assert_array_equal(r, rho)
    f2, r2, v2 = run_gpu(case, K.KEL_ARITH_FAST)
    assert rel_l2(v2, vel) < FAST_TOL
    assert rel_l2(r2, rho) < FAST_TOL


@pytest.mark.parametrize("launch", [None, (2, 128), (ROWS, 4)], ids=lambda l: "default" if l is None else launch_id(l))
@pytest.mark.parametrize("q", [19, 27])
def test_fp16s_velocity_error_vs_fp64(q, launch):
    """FP16-shifted storage: relative L2 velocity error against the FP64 oracle
    of the same cavity below 1e-3."""
    case = cases.cavity_3d(q, dims=(32, 32, 32), steps=400)
    c64 = dict(case, f64=True)
    _, rho64, vel64 = cases.run_oracle(c64)
    _, r16, v16 = run_gpu(case, K.KEL_ARITH_FAST, storage="fp16s", launch=launch)
    err = np.linalg.norm(v16 - vel64) / np.linalg.norm(vel64)
    assert err < 1e-3, err
    _, r32, v32 = run_gpu(case, K.KEL_ARITH_FAST, storage="fp32", launch=launch)
    assert np.linalg.norm(v32 - vel64) / np.linalg.norm(vel64) < 1e-4


@pytest.mark.parametrize("storage", ["fp32", "fp16s"])
@pytest.mark.parametrize("q", [19, 27])
def test_row_pipeline_and_two_cell_sweep_same_bits_as_one_cell_sweep(q, storage):
    """The row pipeline and the two-cell sweep run the same per-cell
    arithmetic as the one-cell sweep: fast arithmetic, FP32 and FP16S
    storage, identical populations,
    with rows of 72 cells (FP16S rows padded to 16 bytes) and
    boundary rows in every direction."""
    case = cases.cavity_3d(q, dims=(72, 20, 13), steps=31)
    a = run_gpu(case, K.KEL_ARITH_FAST, storage=storage, launch=(1, 128))
    for launch in [(ROWS, 2), (ROWS, 3), (ROWS, 6), (2, 64), (2, 256)]:
        b = run_gpu(case, K.KEL_ARITH_FAST, storage=storage, launch=launch)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("periodic", [False, True], ids=["bounded", "periodic"])
@pytest.mark.parametrize("coll", [K.KEL_COLL_BGK, K.KEL_COLL_BGK_GUO, K.KEL_COLL_PSM, K.KEL_COLL_PSM_GUO])
def test_two_cell_fp16s_same_bits_mixed(coll, periodic):
    """FP16S two-cell sweep (packed half pairs) against the one-cell sweep:
    every boundary op, random populations and fields, rows of 2-3 warps of
    pairs, bounded and periodic x, identical populations and macros."""
    for case in (G.normalise(cases.mixed_2d(coll, dims=(160, 20), periodic=periodic, steps=23)),
                 G.normalise(cases.mixed_3d(19, coll, dims=(72, 12, 10), periodic=periodic, steps=15)),
                 G.normalise(cases.mixed_3d(27, coll, dims=(136, 6, 5), periodic=periodic, steps=15))):
        a = run_gpu(case, K.KEL_ARITH_FAST, storage="fp16s", launch=(1, 128))
        for launch in [(2, 64), (2, 256)]:
            b = run_gpu(case, K.KEL_ARITH_FAST, storage="fp16s", launch=launch)
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y)


def test_closed_box_mass_conservation_and_determinism():
    """Full-size property (C2 extents): 256^3 D3Q19 closed box, all walls
    full-way bounce-back, walls start empty so no population ever leaves the
    lattice.  Total mass is conserved to float accuracy and two runs give
    identical bits."""
    dims = (256, 256, 256)
    case = cases.cavity_3d(19, dims=dims, steps=20)
    d = K.program_to_dict(case["program"])
    d["ops"][5] = dict(bc=K.KEL_BC_BOUNCE_BACK, collide=0, east=1, use_profile=0, rho=1.0, u=[0, 0, 0])
    prog = K.program_from_dict(d)
    rng = np.random.default_rng(5)
    w = cases._weights(19).astype(np.float32)
    init = w[None, :] * (1 + 0.01 * rng.standard_normal((dims[0] * dims[1] * dims[2], 19), dtype=np.float32))
    init[case["flags"] != 2] = 0.0
    m0 = init.sum(dtype=np.float64)
    sums = []
    digests = []
    for _ in range(2):
        lat = make_lattice(case)
        lat.upload_populations(init)
        lat.step(prog, 20)
        f = lat.populations(np.float32)
        sums.append(f.sum(dtype=np.float64))
        digests.append(hash(f.tobytes()))
        del f
        lat.close()
    assert abs(sums[0] - m0) / m0 < 1e-5
    assert digests[0] == digests[1]


def test_invalid_arguments_return_errors():
    from lbm_mirror_gb300 import KelError, Lattice
    with pytest.raises(KelError):
        Lattice("D2Q9", (8, 8, 2))
    with pytest.raises(KelError):
        Lattice("D2Q9", (10, 8), periodic_x=True)
    lat = Lattice("D3Q19", (8, 8, 8))
    bad = K.make_program(0.8, K.KEL_COLL_BGK, {3: dict(bc=K.KEL_BC_ZOUHE_VELOCITY_X, collide=1)})
    lat.step(bad, 1)  # no cell carries flag 3 yet: nothing to reject
    flags = np.full(8 * 8 * 8, 2, dtype=np.uint8)
    flags[0] = 3
    lat.upload_flags(flags)
    with pytest.raises(KelError) as e:
        lat.step(bad, 1)
    assert e.value.code == K.KEL_ERR_UNSUPPORTED
    with pytest.raises(KelError):
        lat.step(K.make_program(-1.0), 1)
    with pytest.raises(KelError):
        lat.set_launch(3, 256)
    with pytest.raises(KelError):
        lat.set_launch(ROWS, 7)
    with pytest.raises(KelError):
        lat.set_launch(1, 100)
    lat.set_launch(ROWS, 2)
    lat.close()
    wide = Lattice("D2Q9", (300, 4))  # rows longer than 256 cells: no row pipeline
    with pytest.raises(KelError):
        wide.set_launch(ROWS, 3)
    wide.close()


def test_autotune_restores_state_and_keeps_results():
    case, dfs, rho, vel = G.load("cavity_d3q19")
    prog = with_arith(case["program"], K.KEL_ARITH_REFERENCE)
    lat = make_lattice(case)
    lat.step(prog, 7)
    before = lat.populations(np.float64)
    t = lat.t
    cpt, block, ms = lat.autotune(prog, steps=4)
    assert (cpt, block) in [(1, 64), (1, 128), (1, 256), (2, 64), (2, 128), (2, 256), (4, 64), (4, 128), (4, 256),
                            (ROWS, 3), (ROWS, 4), (ROWS, 6)] and ms > 0
    assert lat.t == t and lat.launch() == (cpt, block)
    np.testing.assert_array_equal(lat.populations(np.float64), before)
    lat.step(prog, case["steps"] - 7)
    np.testing.assert_array_equal(lat.populations(np.float64), dfs)


@pytest.mark.parametrize("chunks", [[10000], [3, 9997], [1, 130, 9869]])
def test_graph_replay_on_a_stream_bit_exact(chunks):
    """On a non-default stream, long kel_step calls replay a captured graph
    of sweeps (entered at even or odd steps): config C1 at full size stays
    bit-exact against the reference."""
    torch = pytest.importorskip("torch")
    from lbm_mirror_gb300 import Lattice
    case, dfs, rho, vel = G.load("poiseuille_256x64")
    prog = with_arith(case["program"], K.KEL_ARITH_REFERENCE)
    st = torch.cuda.Stream()
    lat = Lattice("D2Q9", case["dims"], stream=st.cuda_stream)
    lat.upload_flags(case["flags"])
    if case["profile"] is not None:
        lat.upload_inlet_profile(case["profile"])
    for c in chunks:
        lat.step(prog, c)
    f = lat.populations(np.float64)
    r, v = lat.macros()
    lat.close()
    np.testing.assert_array_equal(f, dfs)
    np.testing.assert_array_equal(v.astype(np.float64), vel)


def test_caller_captured_kel_step_bit_exact():
    """A caller may capture kel_step into a CUDA graph of its own.  kel_step
    then launches its sweeps into that capture one by one (it neither nests a
    capture of its own nor synchronises), and replays of the caller's graph
    (an even number of steps, so the AA parity the host records stays right)
    give config C1 bit for bit."""
    torch = pytest.importorskip("torch")
    from lbm_mirror_gb300 import Lattice
    case, dfs, rho, vel = G.load("poiseuille_256x64")
    prog = with_arith(case["program"], K.KEL_ARITH_REFERENCE)
    st = torch.cuda.Stream()
    lat = Lattice("D2Q9", case["dims"], stream=st.cuda_stream)
    lat.upload_flags(case["flags"])
    lat.upload_inlet_profile(case["profile"])
    lat.step(prog, 16, write_macros=False)  # the program is uploaded outside the capture
    lat.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=st, capture_error_mode="global"):
        lat.step(prog, 256, write_macros=False)
    with torch.cuda.stream(st):
        for _ in range(38):
            g.replay()
    lat.step(prog, case["steps"] - 16 - 38 * 256)
    f = lat.populations(np.float64)
    r, v = lat.macros()
    lat.close()
    np.testing.assert_array_equal(f, dfs)
    np.testing.assert_array_equal(v.astype(np.float64), vel)
