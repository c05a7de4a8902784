"""HLBM coupling on the GPU (KEL_COUPLING_HLBM, KEL_COLL_HLBM) against the
oracle's FP32 restatement on the reference's HLBM case (tests/golden/
hlbm_d2q9_f32_48x40x3.npz).  Bars: porosity and per-cell HLBM momentum
bit-exact; body forces within 1e-12 of sum |cell momentum| (FP64 reduction
order); N / D after the stamp within 1e-6; one HLBM sweep in reference
arithmetic bit-exact given the same N, D and porosity; 25 coupled steps
(kel_particles_step) within 1e-5 relative L2 of the populations."""
import numpy as np
import pytest

from lbm_mirror_gb300 import Lattice, Particles
from lbm_mirror_gb300 import capi as K
from oracle import oracle as O
from tests.golden import make_golden as G
from tests.test_hlbm_oracle import initial_states, load, params

pytestmark = pytest.mark.gpu

OPS = {1: dict(bc=K.KEL_BC_BOUNCE_BACK), 2: dict(bc=K.KEL_BC_FLUID, collide=1)}


def setup(g, launch=None):
    prm, P = params(g)
    prm.coupling = K.KEL_COUPLING_HLBM
    lat = Lattice("D2Q9", G.HLBM_DIMS)
    if launch is not None:
        lat.set_launch(*launch)
    lat.upload_flags(g["flags"])
    lat.upload_populations(g["init"].astype(np.float32))
    ps = Particles(lat, initial_states(g))
    o = O.OracleLattice(9, G.HLBM_DIMS, f64=False)
    o.set_flags(g["flags"])
    o.set_populations(g["init"].astype(np.float64))
    st = K.states_from_array(initial_states(g))
    return prm, P, lat, ps, o, st


@pytest.mark.parametrize("launch", [None, (K.KEL_LAUNCH_ROWS, 3)], ids=["default", "rows"])
def test_hlbm_phases_vs_oracle(launch):
    g = load("hlbm_d2q9_f32_48x40x3")
    prm, P, lat, ps, o, st = setup(g, launch)
    ps.reset()
    ps.couple(prm)
    cf = ps.gather(prm, cell_force=True).astype(np.float64)
    por = lat.download_field(K.KEL_FIELD_POROSITY, 1).astype(np.float64)
    got = ps.download()
    o.hlbm_couple(st, prm)
    O.particles_reset(st)
    cf_o = o.hlbm_gather(st, prm, want_cell_force=True)
    np.testing.assert_array_equal(por, o.porosity())
    np.testing.assert_array_equal(cf, cf_o)
    scale = np.abs(cf_o).reshape(-1, 2).sum()
    ref = K.states_to_array(st)
    assert np.abs(got[:, 18:20] - ref[:, 18:20]).max() <= 1e-12 * scale
    ps.integrate(prm)
    O.particles_integrate(st, 2, prm, G.HLBM_DIMS)
    ps.stamp(prm)
    o.hlbm_stamp(st, prm)
    N = lat.download_field(K.KEL_FIELD_HLBM_N, 2).astype(np.float64).reshape(-1, 2)
    Dv = lat.download_field(K.KEL_FIELD_HLBM_D, 1).astype(np.float64)
    N_o, D_o = o.hlbm_fields()
    np.testing.assert_allclose(N, N_o, rtol=0, atol=1e-6 * max(np.abs(N_o).max(), 1e-30))
    np.testing.assert_allclose(Dv, D_o, rtol=0, atol=1e-6)
    assert (Dv > 0).sum() > 100
    # one sweep from the same fields, reference arithmetic: bit-exact
    o.set_hlbm_fields(N.astype(np.float32).astype(np.float64), Dv.astype(np.float32).astype(np.float64))
    prog = K.make_program(P["tau"], K.KEL_COLL_HLBM, OPS, arithmetic=K.KEL_ARITH_REFERENCE)
    lat.step(prog, 1)
    o.run(prog, 1)
    np.testing.assert_array_equal(lat.populations(np.float64), o.populations())
    rho, u = lat.macros()
    orho, ou = o.macros()
    fl = g["flags"] == 2
    np.testing.assert_array_equal(u[fl].astype(np.float64), ou[fl])


@pytest.mark.parametrize("launch", [None, (K.KEL_LAUNCH_ROWS, 4)], ids=["default", "rows"])
def test_hlbm_coupled_steps_vs_oracle(launch):
    g = load("hlbm_d2q9_f32_48x40x3")
    prm, P, lat, ps, o, st = setup(g, launch)
    prog = K.make_program(P["tau"], K.KEL_COLL_HLBM, OPS, arithmetic=K.KEL_ARITH_REFERENCE)
    ps.step(prm, prog, 25)
    for _ in range(25):
        o.hlbm_couple(st, prm)
        O.particles_reset(st)
        o.hlbm_gather(st, prm)
        O.particles_contact(st, 2, prm, G.HLBM_DIMS)
        O.particles_integrate(st, 2, prm, G.HLBM_DIMS)
        o.hlbm_stamp(st, prm)
        o.run(prog, 1)
    f, fo = lat.populations(np.float64), o.populations()
    assert np.linalg.norm(f - fo) / np.linalg.norm(fo) <= 1e-5
    np.testing.assert_allclose(ps.download()[:, 0:2], K.states_to_array(st)[:, 0:2], rtol=0, atol=1e-6)


def test_hlbm_needs_d2q9_and_the_hlbm_collision():
    g = load("hlbm_d2q9_f32_48x40x3")
    prm, P, lat, ps, o, st = setup(g)
    bgk = K.make_program(P["tau"], K.KEL_COLL_BGK, OPS)
    with pytest.raises(Exception):
        ps.step(prm, bgk, 1)
    lat3 = Lattice("D3Q19", (8, 8, 8))
    with pytest.raises(Exception):
        lat3.step(K.make_program(0.8, K.KEL_COLL_HLBM, {2: dict(bc=K.KEL_BC_FLUID, collide=1)}), 1)
