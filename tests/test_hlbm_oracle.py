"""The HLBM restatement of the oracle (particles_oracle.c ko_particles_hlbm_*,
the HLBM collision of lbm_oracle_impl.h) against the reference's own
components run on the same inputs (tests/golden/hlbm_*.npz from
oracle/ref_harness.cpp: HlbmReset, HlbmOneParticleGather, ParticleIntegrate,
HlbmOneParticleStamp, Hlbm collision, BounceBack, Stream), bit for bit with
T = Float64; with T = Float32 the particle sums (kept in FP64 here) agree to
1e-5 relative."""
import json

import numpy as np
import pytest

from lbm_mirror_gb300 import capi as K
from oracle import oracle as O
from tests.golden import make_golden as G


def load(name):
    z = np.load(f"{G.GOLDEN}/{name}.npz")
    return {k: z[k] for k in z.files}


def params(g):
    P = json.loads(str(g["params"]))
    return K.make_particle_params(K.KEL_POROSITY_RAMP, P["sub_steps"], 1.5, 0.0, 0.0, 0.0, 0.0,
                                  tuple(P["gravity"]) + (0.0,), 0), P


def initial_states(g):
    b, ag = g["bodies"], g["after_gather"]
    st = np.zeros((b.shape[0], 28))
    st[:, 0:2] = b[:, 0:2]
    st[:, 3:5] = b[:, 2:4]
    st[:, 6] = b[:, 4]
    st[:, 9] = b[:, 5]
    st[:, 24:26] = ag[:, 24:26]
    st[:, 26] = b[:, 6]
    st[:, 27] = b[:, 7]
    return st


def run_oracle_step(g, f64):
    prm, P = params(g)
    lat = O.OracleLattice(9, G.HLBM_DIMS, f64=f64)
    lat.set_flags(g["flags"])
    lat.set_populations(g["init"].astype(np.float64))
    st = K.states_from_array(initial_states(g))
    lat.hlbm_couple(st, prm)
    por = lat.porosity()
    O.particles_reset(st)
    cf = lat.hlbm_gather(st, prm, want_cell_force=True)
    after_gather = K.states_to_array(st)
    O.particles_integrate(st, 2, prm, G.HLBM_DIMS)
    after_integrate = K.states_to_array(st)
    lat.hlbm_stamp(st, prm)
    N, Dv = lat.hlbm_fields()
    ops = {1: dict(bc=K.KEL_BC_BOUNCE_BACK), 2: dict(bc=K.KEL_BC_FLUID, collide=1)}
    lat.run(K.make_program(P["tau"], K.KEL_COLL_HLBM, ops, arithmetic=K.KEL_ARITH_REFERENCE), 1)
    rho, vel = lat.macros()
    return dict(porosity=por, force_field=cf, after_gather=after_gather, after_integrate=after_integrate,
                hlbm_N=N.reshape(-1), hlbm_D=Dv, dfs=lat.populations().reshape(-1), rho=rho, vel=vel.reshape(-1))


def test_hlbm_step_bit_exact_f64():
    g = load("hlbm_d2q9_f64_48x40x3")
    o = run_oracle_step(g, True)
    for k in ("porosity", "force_field", "hlbm_N", "hlbm_D", "dfs"):
        np.testing.assert_array_equal(o[k], g[k], err_msg=k)
    fl = g["flags"] == 2
    np.testing.assert_array_equal(o["rho"][fl], g["rho"][fl])
    np.testing.assert_array_equal(o["vel"].reshape(-1, 2)[fl], g["vel"].reshape(-1, 2)[fl])
    np.testing.assert_array_equal(o["after_gather"][:, 18:22], g["after_gather"][:, 18:22])
    np.testing.assert_array_equal(o["after_integrate"], g["after_integrate"])
    # the case exercises the coupling: overlapping AABBs, moving bodies
    assert (g["hlbm_D"] > 0).sum() > 100 and np.abs(g["hlbm_N"]).max() > 0


def test_hlbm_step_f32_close():
    g = load("hlbm_d2q9_f32_48x40x3")
    o = run_oracle_step(g, False)
    # the reference evaluates the ramp in float, the restatement in double
    np.testing.assert_allclose(o["porosity"], g["porosity"], rtol=0, atol=1e-5)
    rel = np.linalg.norm(o["dfs"] - g["dfs"]) / np.linalg.norm(g["dfs"])
    assert rel <= 1e-5, rel
    f_o, f_g = o["after_gather"][:, 18:20], g["after_gather"][:, 18:20]
    assert np.abs(f_o - f_g).max() <= 1e-5 * np.abs(f_g).max()
