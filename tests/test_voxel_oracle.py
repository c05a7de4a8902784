"""The voxel signed-distance restatement (oracle/voxel_oracle.c) against the
reference's own mask, porosity and voxel narrow-phase functions
(particle/mask.hpp, particle/porosity.hpp:24-54, particle/voxel_narrow.hpp),
run by the reference harness into tests/golden/voxel_*.npz (T = Float64).
Also the properties the reference's tests check (modules/core/tests/mask.cpp,
voxel_narrow.cpp, particle_consistency.cpp, particle_gaps.cpp) on the
restatement."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["voxel_2d_sphere", "voxel_2d_cube", "voxel_3d_sphere", "voxel_3d_cube"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    return d


@pytest.mark.parametrize("name", CASES)
def test_mask_fill_matches_reference(name):
    g = load(name)
    P = g["params"]
    mask, com = O.mask_fill(P["dim"], P["resolution"], P["kind"])
    assert np.array_equal(mask, g["mask"])
    assert np.max(np.abs(com - g["com"])) <= 1e-15


@pytest.mark.parametrize("name", CASES)
def test_samples_transforms_and_porosity_match_reference(name):
    g = load(name)
    P = g["params"]
    D, R, eps = P["dim"], P["resolution"], P["eps"]
    mask, com = g["mask"], g["com"]
    samp = np.array([O.mask_sample_local(D, R, mask, u) for u in g["locals"]])
    assert np.array_equal(samp, g["sample"])
    st = O.voxel_states(g["bodies"])
    glob = np.array([O.mask_local_to_global(D, st[b], com, u) for b in range(len(st)) for u in g["locals"]])
    assert np.max(np.abs(glob - g["global"])) <= 1e-12
    sdf = np.array([O.mask_signed_distance(D, R, mask, com, st[b], x) for b in range(len(st)) for x in g["points"]])
    assert np.max(np.abs(sdf - g["sdf"])) <= 1e-12
    por = np.array([O.voxel_porosity(D, R, mask, com, st[b], x, eps) for b in range(len(st)) for x in g["points"]])
    assert np.max(np.abs(por - g["porosity"])) <= 1e-12
    sol = np.array([O.solid_fraction(s, eps) for s in g["sdfs"]])
    assert np.max(np.abs(sol - g["solid"])) <= 1e-15


@pytest.mark.parametrize("name", CASES)
def test_voxel_contact_matches_reference(name):
    g = load(name)
    P = g["params"]
    D, R, eps = P["dim"], P["resolution"], P["eps"]
    st = O.voxel_states(g["bodies"])
    got = np.array([O.voxel_contact(D, R, g["mask"], g["com"], st[int(a)], st[int(b)], P["extent"][:D], eps)
                    for a, b in g["pairs"]])
    want = g["contacts"]
    assert np.array_equal(got[:, 0], want[:, 0])
    assert np.max(np.abs(got - want)) <= 1e-12


def test_fixtures_cover_hits_and_misses():
    for name in CASES:
        hits = load(name)["contacts"][:, 0]
        assert hits.any() and not hits.all(), name


def test_reference_properties_on_the_restatement():
    """mask.cpp: signed distance -1 at the centre, 0 on the surface, -0.5
    halfway; centroid at the origin; porosity within 0.35 of the analytic
    sphere; voxel_narrow.cpp: antisymmetric under pair swap, depth within
    1.6 of the analytic depth."""
    D, R = 2, 32
    mask, com = O.mask_fill(D, R, 0)
    assert abs(O.mask_sample_local(D, R, mask, [0, 0]) + 1) < 0.05
    assert abs(O.mask_sample_local(D, R, mask, [1, 0])) < 0.05
    assert abs(O.mask_sample_local(D, R, mask, [0.5, 0]) + 0.5) < 0.05
    assert np.all(np.abs(com) < 0.02)
    st = O.voxel_states([[16, 16, 0, 0, 0, 0, 5.0]])
    worst = 0.0
    for i in range(41):
        x = 16.0 + 10.0 * (i / 40.0) - 5.0
        s = abs(x - 16.0)
        lo, hi = 5.0 - 0.75, 5.0 + 0.75
        ana = 0.0 if s <= lo else (1.0 if s >= hi else np.sin(np.pi / 3.0 * (s - lo)) ** 2)
        worst = max(worst, abs(ana - O.voxel_porosity(D, R, mask, com, st[0], [x, 16.0], 1.5)))
    assert worst < 0.35
    pair = O.voxel_states([[29, 30, 0, 0, 0, 0, 5.0], [36, 33.5, 0, 0, 0, 0, 5.0]])
    a = O.voxel_contact(D, R, mask, com, pair[0], pair[1], [64, 64], 1.0)
    b = O.voxel_contact(D, R, mask, com, pair[1], pair[0], [64, 64], 1.0)
    assert a[0] == 1 and b[0] == 1 and a[1] == b[1]
    assert np.array_equal(a[2:5], -b[2:5]) and np.array_equal(a[5:8], b[5:8])
    for step in range(1, 5):
        sep = 12.0 - step * 1.5
        p = O.voxel_states([[32 - sep / 2, 32, 0, 0, 0, 0, 6.0], [32 + sep / 2, 32, 0, 0, 0, 0, 6.0]])
        m = O.voxel_contact(D, R, mask, com, p[0], p[1], [64, 64], 1.0)
        assert m[0] == 1 and abs(m[1] - (12.0 - sep)) < 1.6


def test_voxel_couple_is_one_outside_the_boxes_and_product_inside():
    """The FP32 voxel couple: 1 away from every body; where one body covers
    a cell, the factor of that body alone; the FP64 porosity within 1e-5."""
    D, R, eps = 2, 32, 1.5
    mask, com = O.mask_fill(D, R, 1)
    reach = O.mask_reach(D, R, mask)
    assert 1.35 < reach < 1.6  # the cube's corner sqrt(2) plus a voxel diagonal
    st = O.voxel_states([[20.3, 21.6, 0, 0.4, 0, 0, 5.0], [44.1, 40.2, 0, -0.9, 0, 0, 6.0]])
    por = O.voxel_couple(D, R, mask, com, reach, st, [64, 64], eps).reshape(64, 64)
    assert por[0, 63] == 1.0 and por[63, 0] == 1.0
    for b in range(2):
        y, x = int(round(st[b].position[1])), int(round(st[b].position[0]))
        assert por[y, x] == 0.0
        for dy in range(-8, 9):
            for dx in range(-8, 9):
                xx, yy = x + dx, y + dy
                want = O.voxel_porosity(D, R, mask, com, st[b], [xx, yy], eps)
                assert abs(por[yy, xx] - want) <= 1e-5, (b, xx, yy)
