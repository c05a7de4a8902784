"""Voxel signed-distance bodies on the GPU against the reference's fixtures
(tests/golden/voxel_*.npz, made by the reference's own mask.hpp / porosity.hpp
/ voxel_narrow.hpp functions in T = Float64) and against the oracle.

Bars: masks bit-exact (host fill, same operations); FP64 signed distances
and contact manifolds within 1e-12 / 1e-10 of the reference (cos/sin and the
block's summation order may differ in the last bits), the hit flags exact,
a swapped pair's normal the exact negation; the FP32 voxel couple within
2e-6 of the oracle's FP32 restatement (cosf) and 1e-4 of the FP64 porosity;
coupled steps with voxel porosity within 1e-9 (bodies) and 1e-5
(populations) of the oracle stepping the same.
"""
import json
import os

import numpy as np
import pytest

from lbm_mirror_gb300 import Lattice, Particles, Shape
from lbm_mirror_gb300 import capi as K
from oracle import oracle as O
from tests import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["voxel_2d_sphere", "voxel_2d_cube", "voxel_3d_sphere", "voxel_3d_cube"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    return d


def states(bodies):
    return K.states_to_array(O.voxel_states(bodies))


def setup(g):
    P = g["params"]
    D = P["dim"]
    ext = P["extent"]
    lat = Lattice("D2Q9" if D == 2 else "D3Q19", tuple(ext[:D]))
    ps = Particles(lat, states(g["bodies"]))
    sh = Shape(D, P["resolution"], P["kind"])
    ps.set_shape(sh)
    return lat, ps, sh


@pytest.mark.parametrize("name", CASES)
def test_shape_fill_matches_reference(name):
    g = load(name)
    P = g["params"]
    sh = Shape(P["dim"], P["resolution"], P["kind"])
    mask, com, reach = sh.info()
    assert np.array_equal(mask, g["mask"])
    assert np.max(np.abs(com - g["com"])) <= 1e-14
    assert reach == O.mask_reach(P["dim"], P["resolution"], g["mask"])
    sh2 = Shape.from_mask(P["dim"], P["resolution"], g["mask"], g["com"])
    m2, c2, r2 = sh2.info()
    assert np.array_equal(m2, g["mask"]) and np.array_equal(c2, g["com"]) and r2 == reach


@pytest.mark.parametrize("name", CASES)
def test_voxel_distance_matches_reference(name):
    g = load(name)
    D = g["params"]["dim"]
    lat, ps, sh = setup(g)
    n = len(g["bodies"])
    got = np.concatenate([ps.voxel_distance(b, g["points"][:, :D]) for b in range(n)])
    assert np.max(np.abs(got - g["sdf"])) <= 1e-12


@pytest.mark.parametrize("name", CASES)
def test_voxel_contact_matches_reference(name):
    g = load(name)
    P = g["params"]
    lat, ps, sh = setup(g)
    got = ps.voxel_contact(g["pairs"].astype(np.int32), P["eps"])
    want = g["contacts"]
    assert np.array_equal(got[:, 0], want[:, 0])
    assert np.max(np.abs(got - want)) <= 1e-10
    # pairs 0/1 and 2/3 are the same pair in both orders
    for a, b in ((0, 1), (2, 3)):
        assert got[a, 1] == got[b, 1]
        assert np.array_equal(got[a, 2:5], -got[b, 2:5])
        assert np.array_equal(got[a, 5:8], got[b, 5:8])
    # bitwise reproducible
    assert np.array_equal(got, ps.voxel_contact(g["pairs"].astype(np.int32), P["eps"]))


@pytest.mark.parametrize("name", CASES)
def test_voxel_couple_matches_oracle(name):
    g = load(name)
    P = g["params"]
    D, R, eps = P["dim"], P["resolution"], P["eps"]
    ext = P["extent"][:D]
    lat, ps, sh = setup(g)
    prm = K.make_particle_params(K.KEL_POROSITY_VOXEL, eps=eps)
    ps.couple(prm)
    por = lat.download_field(K.KEL_FIELD_POROSITY, 1).astype(np.float64)
    mask, com, reach = sh.info()
    st = O.voxel_states(g["bodies"])
    want = O.voxel_couple(D, R, mask, com, reach, st, ext, eps)
    assert np.max(np.abs(por - want)) <= 2e-6
    assert (por < 1.0).sum() > 100 and (por == 0.0).sum() > 10
    # against the FP64 porosity of the reference's formula, where one body covers the cell
    cells = np.arange(por.size)[:: max(1, por.size // 4000)]
    for c in cells:
        x = [c % ext[0], (c // ext[0]) % ext[1]] + ([c // (ext[0] * ext[1])] if D == 3 else [])
        f = [O.voxel_porosity(D, R, mask, com, st[b], x, eps) for b in range(len(st))]
        if sum(v < 1.0 for v in f) == 1:
            assert abs(por[c] - min(f)) <= 1e-4, (c, por[c], f)


def test_voxel_bodies_reject_bad_use():
    from lbm_mirror_gb300.lattice import KelError
    g = load("voxel_2d_sphere")
    lat = Lattice("D2Q9", (64, 64))
    ps = Particles(lat, states(g["bodies"]))
    prm = K.make_particle_params(K.KEL_POROSITY_VOXEL, eps=1.0)
    with pytest.raises(KelError) as e:
        ps.couple(prm)  # no shape yet
    assert e.value.code == K.KEL_ERR_STATE
    with pytest.raises(KelError) as e:
        ps.set_shape(Shape(3, 8))  # 3D shape on a 2D lattice
    assert e.value.code == K.KEL_ERR_INVALID_ARGUMENT
    ps.set_shape(Shape(2, 16))
    with pytest.raises(KelError) as e:
        ps.couple(K.make_particle_params(K.KEL_POROSITY_VOXEL, eps=1.0, coupling=K.KEL_COUPLING_HLBM))
    assert e.value.code == K.KEL_ERR_UNSUPPORTED
    with pytest.raises(KelError) as e:
        ps.voxel_contact(np.array([[0, 9]], np.int32), 1.0)
    assert e.value.code == K.KEL_ERR_INVALID_ARGUMENT
    with pytest.raises(KelError):
        Shape(2, 1)


@pytest.mark.parametrize("kind", [K.KEL_SHAPE_SPHERE, K.KEL_SHAPE_CUBE])
def test_coupled_voxel_run_vs_oracle(kind):
    """40 coupled steps (couple with the voxel porosity, gather over the voxel
    boxes, DEM contact, integrate, PSM + Guo sweep) of rotating discs in a
    periodic channel, on a stream (captured two-step graph, incremental
    couple), against the oracle stepping the same."""
    torch = pytest.importorskip("torch")
    dims = (96, 64)
    nx, ny = dims
    x, y, _ = cases.cell_grid(dims)
    flags = np.full(nx * ny, 2, dtype=np.uint8)
    flags[(y == 0) | (y == ny - 1)] = 1
    ops = {1: dict(bc=K.KEL_BC_BOUNCE_BACK), 2: dict(bc=K.KEL_BC_FLUID, collide=1)}
    prog = K.make_program(0.7, K.KEL_COLL_PSM_GUO, ops, global_force=(0.0, -1e-5, 0.0),
                          arithmetic=K.KEL_ARITH_REFERENCE)
    eps = 1.5
    prm = K.make_particle_params(K.KEL_POROSITY_VOXEL, eps=eps, sub_steps=1, k_n=100.0, zeta_n=0.1,
                                 body_acceleration=(0.0, -1e-5), wall_axes=0b10)
    st0 = np.zeros((4, 28))
    bodies = [(3.5, 20.3, 6.0), (70.2, 40.7, 5.0), (40.0, 14.0, 5.5), (86.9, 30.2, 6.5)]
    for i, (bx, by, r) in enumerate(bodies):
        st0[i, 0:2] = (bx, by)
        st0[i, 3:5] = (bx - 0.003 * (i + 1), by + 0.002)
        st0[i, 6] = 0.3 * i
        st0[i, 9] = 0.3 * i - 0.01
        st0[i, 26] = r
        st0[i, 27] = 1.5
        st0[i, 24] = np.pi * r * r * 1.5
        st0[i, 25] = 0.5 * st0[i, 24] * r * r
    sh = Shape(2, 32, kind)
    mask, com, reach = sh.info()
    stream = torch.cuda.Stream()
    lat = Lattice("D2Q9", dims, periodic_x=True, stream=stream.cuda_stream)
    lat.upload_flags(flags)
    ps = Particles(lat, st0)
    ps.set_shape(sh)
    ps.step(prm, prog, 40)
    got = ps.download()
    f_gpu = lat.populations(np.float64)
    por_gpu = lat.download_field(K.KEL_FIELD_POROSITY, 1).astype(np.float64)

    o = O.OracleLattice(9, dims, periodic_x=True)
    o.set_flags(flags)
    O.particles_set_voxel_box(reach, eps / 2)
    st = K.states_from_array(st0)
    for _ in range(40):
        O.particles_reset(st)
        last_por = O.voxel_couple(2, 32, mask, com, reach, st, dims, eps, periodic_x=True)
        o.set_porosity(last_por)
        o.particles_gather(st, prm)
        O.particles_contact(st, 2, prm, dims, periodic_x=True)
        O.particles_integrate(st, 2, prm, dims, periodic_x=True)
        o.run(prog, 1)
    O.particles_set_voxel_box(1.0, 0.0)
    ref = K.states_to_array(st)
    assert np.abs(por_gpu - last_por).max() <= 2e-6
    assert np.abs(got[:, 0:2] - ref[:, 0:2]).max() < 1e-9
    assert np.abs(got[:, 6] - ref[:, 6]).max() < 1e-9
    assert np.abs(f_gpu - o.populations()).max() < 1e-5
    ps.close()
    lat.close()
