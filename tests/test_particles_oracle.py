"""The particle restatement of the oracle against the reference's own
components (golden vectors from oracle/ref_harness.cpp: PsmOneParticleGather,
ParticleContact, ParticleIntegrate, T = Float64), bit for bit; plus the
reference's own known-answer tests for contact and integration
(modules/core/tests/component_instantiation.cpp:95-200)."""
import json

import numpy as np
import pytest

from lbm_mirror_gb300 import capi as K
from oracle import oracle as O
from tests.golden import make_golden as G


def golden_params(g):
    P = json.loads(str(g["params"]))
    return K.make_particle_params(K.KEL_POROSITY_RAMP, P["sub_steps"], 1.5, P["k_n"], P["zeta_n"], P["gamma_t"],
                                  P["mu"], tuple(P["gravity"]) + (0.0,), 0b11 if P["walls"] else 0)


def initial_states(g):
    b, ag = g["bodies"], g["after_gather"]
    st = np.zeros((b.shape[0], 28))
    st[:, 0:2] = b[:, 0:2]
    st[:, 3:5] = b[:, 2:4]
    st[:, 6] = b[:, 4]
    st[:, 9] = b[:, 5]
    st[:, 24:26] = ag[:, 24:26]  # mass, inertia as the reference's group factory made them
    st[:, 26] = b[:, 6]
    st[:, 27] = b[:, 7]
    return st


def test_gather_and_porosity_bit_exact():
    g = G.load_particles("particles_gather_f64")
    prm = golden_params(g)
    lat = O.OracleLattice(9, G.PART_DIMS, f64=True)
    lat.set_populations(g["init"].astype(np.float64))
    st = K.states_from_array(initial_states(g))
    O.particles_reset(st)
    lat.particles_couple(st, prm)
    np.testing.assert_array_equal(lat.porosity(), g["porosity"])
    cf = lat.particles_gather(st, prm, want_cell_force=True)
    np.testing.assert_array_equal(cf, g["force_field"])
    got = K.states_to_array(st)
    np.testing.assert_array_equal(got[:, 18:20], g["after_gather"][:, 18:20])
    assert np.abs(got[:, 21]).max() > 0  # the restated PSM torque is non-trivial


@pytest.mark.parametrize("name", ["particles_gather_f64", "particles_contact_f64"])
def test_contact_and_integrate_bit_exact(name):
    g = G.load_particles(name)
    prm = golden_params(g)
    st = K.states_from_array(g["after_gather"])
    O.particles_contact(st, 2, prm, G.PART_DIMS)
    np.testing.assert_array_equal(K.states_to_array(st), g["after_contact"])
    O.particles_integrate(st, 2, prm, G.PART_DIMS)
    np.testing.assert_array_equal(K.states_to_array(st), g["after_integrate"])


def test_contact_case_has_contacts():
    g = G.load_particles("particles_contact_f64")
    d = g["after_contact"][:, 18:20] - g["after_gather"][:, 18:20]
    assert (np.abs(d).sum(1) > 1e-3).sum() >= 4  # two pairs and two walls


def _pair(x0, x1, r=2.0, y=16.0):
    st = np.zeros((2, 28))
    for i, x in enumerate((x0, x1)):
        st[i, 0:2] = (x, y)
        st[i, 3:5] = (x, y)
        st[i, 26] = r
        st[i, 27] = 1.0
        st[i, 24] = np.pi * r * r
        st[i, 25] = 0.5 * st[i, 24] * r * r
    return st


def test_known_answer_contact_k4_overlap1():
    """component_instantiation.cpp:121-153: k = 4, overlap 1 -> |F| = 4, halves cancel exactly."""
    st = K.states_from_array(_pair(20.0, 23.0))
    prm = K.make_particle_params(k_n=4.0, zeta_n=0.0, wall_axes=0b11)
    O.particles_contact(st, 2, prm, (64, 32))
    a = K.states_to_array(st)
    assert abs(a[0, 18] + 4.0) < 1e-12
    assert a[0, 18] == -a[1, 18]


def test_known_answer_wall_push():
    """component_instantiation.cpp:155-178: wall pushes +x by k * depth."""
    st = K.states_from_array(_pair(1.5, 50.0))
    prm = K.make_particle_params(k_n=6.0, zeta_n=0.0, wall_axes=0b11)
    O.particles_contact(st, 2, prm, (64, 32))
    assert abs(K.states_to_array(st)[0, 18] - 6.0 * 0.5) < 1e-12
    st = K.states_from_array(_pair(1.5, 50.0))
    O.particles_contact(st, 2, K.make_particle_params(k_n=6.0, zeta_n=0.0, wall_axes=0), (64, 32))
    assert K.states_to_array(st)[0, 18] == 0.0


def test_known_answer_integrate_unit_acceleration():
    """component_instantiation.cpp:95-119: force = mass -> a_x = 1, gravity added."""
    a = _pair(0.0, 40.0)
    a[0, 18] = a[0, 24]
    st = K.states_from_array(a)
    O.particles_integrate(st, 2, K.make_particle_params(sub_steps=1, body_acceleration=(0.0, -0.5)), (64, 32))
    b = K.states_to_array(st)
    assert abs(b[0, 12] - 1.0) < 1e-12 and abs(b[0, 13] + 0.5) < 1e-12
    assert b[0, 0] > 0.0
