"""FPLBM coupling on the GPU (KEL_COUPLING_FPLBM / _OWN, KEL_COLL_FPLBM)
against the reference's own components (golden vectors of
oracle/ref_harness.cpp, fplbm.hpp: FpLbmReset, FpLbmOneParticle, FpLbm)
and against the oracle stepping the same coupled run.

Bars, FP32 lattice, FP64 bodies: FpLbmReset's density and momentum bit-exact
(the same float sums); porosity within 1e-6 with the solid / coupled masks
bit-exact (the device sinf may differ from the host's in the last bit);
coupling forces within 5e-6 absolute and accelerations / positions within
1e-5 of the reference's float bodies (the float rounding of a body velocity
formed from float positions near 20); over 25 coupled steps against the
oracle's FP64 bodies, positions and accelerations within 1e-6 (the device
sinf differs from the host's in the last bit, porosities by ~1e-7) and
populations within 1e-5; one step's populations within 1e-6."""
import json

import numpy as np
import pytest

from lbm_mirror_gb300 import Lattice, Particles
from lbm_mirror_gb300 import capi as K
from oracle import oracle as O
from tests.golden import make_golden as G

pytestmark = pytest.mark.gpu

OPS = {1: dict(bc=K.KEL_BC_BOUNCE_BACK), 2: dict(bc=K.KEL_BC_FLUID, collide=1)}


def bodies_from_fixture(g):
    b = np.zeros((g["bodies"].shape[0], 28))
    for k, (x, y, xo, yo, rot, roto, r, rho) in enumerate(g["bodies"]):
        b[k, [0, 1, 3, 4, 6, 9, 26, 27]] = x, y, xo, yo, rot, roto, r, rho
        b[k, 24] = np.pi * r * r * rho
        b[k, 25] = 0.5 * b[k, 24] * r * r
    return b


def setup(g, coupling=K.KEL_COUPLING_FPLBM):
    P = json.loads(str(g["params"]))
    prm = K.make_particle_params(sub_steps=P["sub_steps"], body_acceleration=tuple(P["gravity"]), coupling=coupling)
    prog = K.make_program(P["tau"], K.KEL_COLL_FPLBM, OPS, arithmetic=K.KEL_ARITH_REFERENCE)
    lat = Lattice("D2Q9", G.HLBM_DIMS)
    lat.upload_flags(g["flags"])
    lat.upload_populations(g["init"].astype(np.float32))
    return lat, Particles(lat, bodies_from_fixture(g)), prm, prog


@pytest.mark.parametrize("name", ["fplbm_d2q9_f32_48x40x1", "fplbm_d2q9_f32_48x40x3"])
def test_fplbm_one_step_vs_reference(name):
    g = G.load_particles(name)
    lat, ps, prm, prog = setup(g)
    ps.couple(prm)
    rho, mom = lat.macros()
    np.testing.assert_array_equal(rho.astype(np.float64), g["reset_rho"])
    np.testing.assert_array_equal(mom.ravel().astype(np.float64), g["reset_mom"])
    por = lat.download_field(K.KEL_FIELD_POROSITY, 1).astype(np.float64)
    np.testing.assert_array_equal(por < 1.0, g["porosity"] < 1.0)
    np.testing.assert_array_equal(por == 0.0, g["porosity"] == 0.0)
    assert np.abs(por - g["porosity"]).max() <= 1e-6
    force = lat.download_field(K.KEL_FIELD_FORCE, 2).astype(np.float64).ravel()
    assert np.abs(force - g["force_field"]).max() <= 5e-6
    ps.gather(prm)
    ps.integrate(prm)
    got, ref = ps.download(), g["after_particle"]
    assert np.abs(got[:, 12:14] - ref[:, 12:14]).max() <= 1e-5
    assert np.abs(got[:, [0, 1, 3, 4]] - ref[:, [0, 1, 3, 4]]).max() <= 1e-5
    lat.step(prog, 1)
    assert np.abs(lat.populations(np.float64).ravel() - g["dfs"]).max() <= 1e-6
    ps.close()
    lat.close()


@pytest.mark.parametrize("coupling", [K.KEL_COUPLING_FPLBM, K.KEL_COUPLING_FPLBM_OWN], ids=["body0_box", "own_box"])
def test_fplbm_coupled_run_vs_oracle(coupling):
    """25 coupled steps (kel_particles_step) against the oracle stepping the
    same: FpLbmReset, the particle pass with its integration, the sweep."""
    g = G.load_particles("fplbm_d2q9_f32_48x40x3")
    lat, ps, prm, prog = setup(g, coupling)
    steps = 25
    ps.step(prm, prog, steps)
    got = ps.download()
    f_gpu = lat.populations(np.float64)

    o = O.OracleLattice(9, G.HLBM_DIMS)
    o.set_flags(g["flags"])
    o.set_populations(g["init"].astype(np.float32).astype(np.float64))
    st = K.states_from_array(bodies_from_fixture(g))
    for _ in range(steps):
        o.fplbm_reset(1 << 2)
        o.fplbm_particles(st, prm, own=coupling == K.KEL_COUPLING_FPLBM_OWN)
        o.run(prog, 1)
    ref = K.states_to_array(st)
    moved = np.abs(ref[:, 0:2] - bodies_from_fixture(g)[:, 0:2]).max()
    assert moved > 0.05
    assert np.abs(got[:, 0:2] - ref[:, 0:2]).max() < 1e-6
    assert np.abs(got[:, 12:14] - ref[:, 12:14]).max() < 1e-6
    assert np.abs(f_gpu - o.populations()).max() < 1e-5
    ps.close()
    lat.close()


def test_fplbm_rejects_bad_setups():
    g = G.load_particles("fplbm_d2q9_f32_48x40x1")
    lat, ps, prm, prog = setup(g)
    psm_prog = K.make_program(0.8, K.KEL_COLL_PSM, OPS)
    with pytest.raises(Exception):
        ps.step(prm, psm_prog, 1)  # FPLBM coupling needs the FPLBM collision
    grav = K.make_program(0.8, K.KEL_COLL_FPLBM, OPS, global_force=(0.0, -1e-5, 0.0))
    with pytest.raises(Exception):
        lat.step(grav, 1)  # no global force with FPLBM
    ps.close()
    lat.close()
    lat3 = Lattice("D3Q19", (8, 8, 8))
    with pytest.raises(Exception):
        lat3.step(K.make_program(0.8, K.KEL_COLL_FPLBM, OPS), 1)
    lat3.close()
