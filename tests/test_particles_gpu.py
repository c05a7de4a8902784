"""GPU particle kernels vs the oracle and vs the reference's golden vectors.

Bar: couple porosity within 1e-7 (FP64 ramp stored as float; sin() may differ
in the last bit) with the solid/coupled cell masks bit-exact, and bit-exact
for 4x4 sub-cell sampling; per-cell momentum-exchange forces bit-exact; FP64
force/torque sums within 1e-12 of sum |cell force| (reduction order);
contact and integration bit-exact (FP64, unfused); against the reference's
own float gather within 1e-5 of sum |cell force|.
"""
import numpy as np
import pytest

from lbm_mirror_gb300 import Lattice, Particles
from lbm_mirror_gb300 import capi as K
from oracle import oracle as O
from tests import cases
from tests.golden import make_golden as G
from tests.test_particles_oracle import golden_params, initial_states

pytestmark = pytest.mark.gpu


def gpu_lattice(init, dims=G.PART_DIMS, periodic=False):
    lat = Lattice("D2Q9", dims, periodic_x=periodic)
    lat.upload_populations(init.astype(np.float32))
    return lat


def oracle_lattice(init, dims=G.PART_DIMS, periodic=False):
    o = O.OracleLattice(9, dims, f64=False, periodic_x=periodic)
    o.set_populations(init.astype(np.float64))
    return o


@pytest.mark.parametrize("mode", [K.KEL_POROSITY_RAMP, K.KEL_POROSITY_SUBCELL])
def test_couple_gather_vs_oracle(mode):
    g = G.load_particles("particles_gather_f64")
    prm = golden_params(g)
    prm.porosity_mode = mode
    st0 = initial_states(g)
    lat = gpu_lattice(g["init"])
    ps = Particles(lat, st0)
    ps.reset()
    ps.couple(prm)
    por_gpu = lat.download_field(K.KEL_FIELD_POROSITY, 1).astype(np.float64)
    cf_gpu = ps.gather(prm, cell_force=True).astype(np.float64)
    got = ps.download()

    o = oracle_lattice(g["init"])
    st = K.states_from_array(st0)
    O.particles_reset(st)
    o.particles_couple(st, prm)
    por_o = o.porosity()
    cf_o = o.particles_gather(st, prm, want_cell_force=True)
    ref = K.states_to_array(st)

    np.testing.assert_array_equal(por_gpu < 1.0, por_o < 1.0)
    np.testing.assert_array_equal(por_gpu == 0.0, por_o == 0.0)
    if mode == K.KEL_POROSITY_SUBCELL:
        np.testing.assert_array_equal(por_gpu, por_o)
    else:
        assert np.abs(por_gpu - por_o).max() <= 1e-7
    scale = np.abs(cf_o).reshape(-1, 2).sum(0).max()
    assert np.abs(cf_gpu - cf_o).max() <= 1e-6 * scale
    assert np.abs(got[:, 18:20] - ref[:, 18:20]).max() <= 1e-12 * max(scale, 1.0) + 1e-7 * scale
    assert np.abs(got[:, 21] - ref[:, 21]).max() <= 1e-6 * scale * 10
    ps.close()
    lat.close()


def test_gather_vs_reference_float_path():
    """Against the reference's own T = Float32 gather (float sums)."""
    g32 = G.load_particles("particles_gather_f32")
    prm = golden_params(g32)
    lat = gpu_lattice(g32["init"])
    ps = Particles(lat, initial_states(g32))
    ps.reset()
    ps.couple(prm)
    cf = ps.gather(prm, cell_force=True).astype(np.float64)
    got = ps.download()
    scale = np.abs(g32["force_field"]).reshape(-1, 2).sum(0).max()
    assert np.abs(got[:, 18:20] - g32["after_gather"][:, 18:20]).max() <= 1e-5 * scale
    assert np.abs(cf - g32["force_field"]).max() <= 1e-5 * scale
    np.testing.assert_array_equal(lat.download_field(K.KEL_FIELD_POROSITY, 1) < 1.0, g32["porosity"] < 1.0)


@pytest.mark.parametrize("name", ["particles_gather_f64", "particles_contact_f64"])
def test_contact_integrate_bit_exact_vs_reference(name):
    g = G.load_particles(name)
    prm = golden_params(g)
    lat = Lattice("D2Q9", G.PART_DIMS)
    ps = Particles(lat, g["after_gather"])
    ps.contact(prm)
    np.testing.assert_array_equal(ps.download(), g["after_contact"])
    ps.integrate(prm)
    np.testing.assert_array_equal(ps.download(), g["after_integrate"])


def test_contact_known_answer():
    from tests.test_particles_oracle import _pair
    lat = Lattice("D2Q9", (64, 32))
    ps = Particles(lat, _pair(20.0, 23.0))
    ps.reset()
    ps.contact(K.make_particle_params(k_n=4.0, zeta_n=0.0, wall_axes=0b11))
    a = ps.download()
    assert abs(a[0, 18] + 4.0) < 1e-12 and a[0, 18] == -a[1, 18]


def _periodic_bodies():
    st = np.zeros((4, 28))
    bodies = [(1.5, 20.3, 6.0), (70.2, 40.7, 5.0), (40.0, 12.0, 5.5), (88.9, 30.2, 6.5)]
    for i, (x, y, r) in enumerate(bodies):
        st[i, 0:2] = (x, y)
        st[i, 3:5] = (x - 0.003 * (i + 1), y + 0.002)
        st[i, 26] = r
        st[i, 27] = 1.5
        st[i, 24] = np.pi * r * r * 1.5
        st[i, 25] = 0.5 * st[i, 24] * r * r
    return st


@pytest.mark.parametrize("launch", [None, (K.KEL_LAUNCH_ROWS, 3)], ids=["default", "rows"])
def test_coupled_periodic_run_vs_oracle(launch):
    """Config-3 shape in small: periodic x, walls in y, PSM + Guo gravity,
    bodies straddling the periodic seam, 40 coupled steps (reset, couple,
    gather, contact, integrate, sweep) against the oracle stepping the same."""
    dims = (96, 64)
    nx, ny = dims
    x, y, _ = cases.cell_grid(dims)
    flags = np.full(nx * ny, 2, dtype=np.uint8)
    flags[(y == 0) | (y == ny - 1)] = 1
    ops = {1: dict(bc=K.KEL_BC_BOUNCE_BACK), 2: dict(bc=K.KEL_BC_FLUID, collide=1)}
    prog = K.make_program(0.7, K.KEL_COLL_PSM_GUO, ops, global_force=(0.0, -1e-5, 0.0),
                          arithmetic=K.KEL_ARITH_REFERENCE)
    prm = K.make_particle_params(K.KEL_POROSITY_SUBCELL, sub_steps=1, k_n=100.0, zeta_n=0.1,
                                 body_acceleration=(0.0, -1e-5), wall_axes=0b10)
    st0 = _periodic_bodies()
    lat = Lattice("D2Q9", dims, periodic_x=True)
    if launch is not None:
        lat.set_launch(*launch)
    lat.upload_flags(flags)
    ps = Particles(lat, st0)
    ps.step(prm, prog, 40)
    got = ps.download()
    f_gpu = lat.populations(np.float64)

    o = O.OracleLattice(9, dims, periodic_x=True)
    o.set_flags(flags)
    st = K.states_from_array(st0)
    for _ in range(40):
        O.particles_reset(st)
        o.particles_couple(st, prm)
        o.particles_gather(st, prm)
        O.particles_contact(st, 2, prm, dims, periodic_x=True)
        O.particles_integrate(st, 2, prm, dims, periodic_x=True)
        o.run(prog, 1)
    ref = K.states_to_array(st)
    assert np.abs(got[:, 0:2] - ref[:, 0:2]).max() < 1e-9
    assert np.abs(f_gpu - o.populations()).max() < 1e-5
    assert np.all((got[:, 0] >= 0) & (got[:, 0] < nx))


def _config3(nsteps_seed=7):
    """Config C3 at its stated size: 2048 x 512 periodic channel, walls in y,
    PSM + Guo gravity (g = 1e-6 in -y), tau 0.7, 64 seeded discs R = 8 of
    density 1.5, 4x4 sub-cell solid fraction, DEM k = 100, damping 0.1.  The
    real run starts from rest, where 500 steps move nothing; here the bodies
    get seeded velocities and spins and the populations a seeded
    perturbation of the rest state, so that forces, contacts and moving
    porosity are all exercised."""
    from lbm_mirror_gb300.workloads import particle_channel
    dims = (2048, 512)
    flags, st = particle_channel(*dims)
    rng = np.random.default_rng(nsteps_seed)
    v = rng.uniform(-0.05, 0.05, (st.shape[0], 2))
    st[:, 3:5] = st[:, 0:2] - v                         # position_old: velocity v
    st[:, 9] = st[:, 6] - rng.uniform(-0.01, 0.01, st.shape[0])  # rotation_old: spin
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    init = w[None, :] * (1.0 + rng.uniform(-0.02, 0.02, (dims[0] * dims[1], 9)))
    ops = {1: dict(bc=K.KEL_BC_BOUNCE_BACK), 2: dict(bc=K.KEL_BC_FLUID, collide=1)}
    prog = K.make_program(0.7, K.KEL_COLL_PSM_GUO, ops, global_force=(0.0, -1e-6, 0.0),
                          arithmetic=K.KEL_ARITH_REFERENCE)
    prm = K.make_particle_params(K.KEL_POROSITY_SUBCELL, sub_steps=1, k_n=100.0, zeta_n=0.1,
                                 body_acceleration=(0.0, -1e-6), wall_axes=0b10)
    return dims, flags, st, init.astype(np.float32), prog, prm


def _gpu_config3(dims, flags, st, init, prog, prm, steps, stream=None):
    lat = Lattice("D2Q9", dims, periodic_x=True, stream=stream)
    lat.upload_flags(flags)
    lat.upload_populations(init)
    ps = Particles(lat, st)
    ps.step(prm, prog, steps)
    out = (ps.download(), lat.populations(np.float64), lat.download_field(K.KEL_FIELD_POROSITY, 1))
    ps.close()
    lat.close()
    return out


def test_config3_full_size_vs_oracle():
    """500 coupled steps of config C3 at 2048 x 512 with 64 bodies, in the
    reference's arithmetic, on a stream (the captured two-step graph and the
    incremental couple) against the oracle stepping the same: body positions
    and velocities within 1e-9, populations within 1e-5, the porosity field
    (4x4 sub-cell counts) bit-exact."""
    torch = pytest.importorskip("torch")
    dims, flags, st0, init, prog, prm = _config3()
    steps = 500
    stream = torch.cuda.Stream()
    got, f_gpu, por_gpu = _gpu_config3(dims, flags, st0, init, prog, prm, steps, stream.cuda_stream)

    o = O.OracleLattice(9, dims, periodic_x=True)
    o.set_flags(flags)
    o.set_populations(init.astype(np.float64))
    st = K.states_from_array(st0)
    for _ in range(steps):
        O.particles_reset(st)
        o.particles_couple(st, prm)
        o.particles_gather(st, prm)
        O.particles_contact(st, 2, prm, dims, periodic_x=True)
        O.particles_integrate(st, 2, prm, dims, periodic_x=True)
        o.run(prog, 1)
    ref = K.states_to_array(st)
    moved = np.abs(ref[:, 0:2] - st0[:, 0:2]).max()
    assert moved > 1.0  # the bodies did travel
    np.testing.assert_array_equal(por_gpu.astype(np.float64), o.porosity())
    assert np.abs(got[:, 0:2] - ref[:, 0:2]).max() < 1e-9
    vel_gpu, vel_ref = got[:, 0:2] - got[:, 3:5], ref[:, 0:2] - ref[:, 3:5]
    assert np.abs(vel_gpu - vel_ref).max() < 1e-9
    assert np.abs(f_gpu - o.populations()).max() < 1e-5


def test_coupled_graph_replay_equals_plain_launches():
    """kel_particles_step on a stream replays a captured graph of two coupled
    steps; on the legacy stream every launch is issued one by one.  Both give
    the same bits (64 bodies, 2048 x 512, 61 steps: odd count, macro step)."""
    torch = pytest.importorskip("torch")
    dims, flags, st0, init, prog, prm = _config3(11)
    a = _gpu_config3(dims, flags, st0, init, prog, prm, 61, torch.cuda.Stream().cuda_stream)
    b = _gpu_config3(dims, flags, st0, init, prog, prm, 61, None)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_couple_after_porosity_upload_recomputes_every_cell():
    """The couple only revisits the bodies' current and previous boxes while
    the porosity field is the one its last couple left; after an upload of
    the field it recomputes every cell (equal to the oracle's full pass)."""
    dims, flags, st0, init, prog, prm = _config3(5)
    lat = Lattice("D2Q9", dims, periodic_x=True)
    lat.upload_flags(flags)
    ps = Particles(lat, st0)
    ps.couple(prm)
    st1 = st0.copy()
    st1[:, 0] = (st1[:, 0] + 37.5) % dims[0]
    ps.upload(st1)
    ps.couple(prm)  # incremental: the old boxes go back to 1
    lat.upload_porosity(np.full(dims[0] * dims[1], 0.25, dtype=np.float32))
    ps.couple(prm)  # after the upload: every cell
    por = lat.download_field(K.KEL_FIELD_POROSITY, 1).astype(np.float64)
    o = O.OracleLattice(9, dims, periodic_x=True)
    o.particles_couple(K.states_from_array(st1), prm)
    np.testing.assert_array_equal(por, o.porosity())
    ps.close()
    lat.close()
