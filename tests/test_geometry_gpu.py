"""Device-side geometry and initial state (kel_lattice_paint,
kel_lattice_init_equilibrium): the painted flag fields equal the host
builders of the reference drivers' layouts, and the equilibrium start equals
the reference-rounded equilibrium of the oracle cell by cell (bit-exact)."""
import numpy as np
import pytest

from lbm_mirror_gb300 import Lattice
from lbm_mirror_gb300 import capi as K
from oracle import oracle as O
from tests import cases

pytestmark = pytest.mark.gpu

BIG = 1 << 40


def channel_ops(dims):
    nx, ny = dims[0], dims[1]
    nz = dims[2] if len(dims) > 2 else 1
    zi = (1, nz - 1) if nz > 1 else (0, 1)
    return [dict(flag=1),
            dict(flag=2, lo=(1, 1, zi[0]), hi=(nx - 1, ny - 1, zi[1])),
            dict(flag=3, lo=(0, 1, zi[0]), hi=(1, ny - 1, zi[1])),
            dict(flag=4, lo=(nx - 1, 1, zi[0]), hi=(nx, ny - 1, zi[1]))]


def cavity_ops(dims):
    nx, ny = dims[0], dims[1]
    nz = dims[2] if len(dims) > 2 else 1
    zi = (1, nz - 1) if nz > 1 else (0, 1)
    return [dict(flag=1),
            dict(flag=2, lo=(1, 1, zi[0]), hi=(nx - 1, ny - 1, zi[1])),
            dict(flag=5, lo=(1, ny - 1, zi[0]), hi=(nx - 1, ny, zi[1]))]


@pytest.mark.parametrize("dims", [(37, 19), (12, 10, 8)])
def test_painted_channel_and_cavity_equal_host_layouts(dims):
    q = "D2Q9" if len(dims) == 2 else "D3Q19"
    lat = Lattice(q, dims)
    lat.paint(channel_ops(dims))
    np.testing.assert_array_equal(lat.flags(), cases.channel_flags(dims))
    lat.paint(cavity_ops(dims))
    np.testing.assert_array_equal(lat.flags(), cases.cavity_flags(dims))
    lat.close()


def test_painted_disks_clipped_like_the_channel_generator():
    nx, ny = 64, 32
    lat = Lattice("D2Q9", (nx, ny))
    disks = [(20.3, 15.2, 6.1), (44.0, 9.5, 4.0), (3.5, 16.0, 5.0)]
    ops = channel_ops((nx, ny)) + [dict(shape="sphere", flag=1, lo=(3, 0, 0), hi=(nx - 3, ny, 1), center=(cx, cy, 0),
                                        radius=r) for cx, cy, r in disks]
    lat.paint(ops)
    x, y, _ = cases.cell_grid((nx, ny))
    want = cases.channel_flags((nx, ny))
    for cx, cy, r in disks:
        want[((x - cx) ** 2 + (y - cy) ** 2 <= r * r) & (x > 2) & (x < nx - 3)] = 1
    np.testing.assert_array_equal(lat.flags(), want)
    lat.close()


@pytest.mark.parametrize("q,dims", [(9, (20, 11)), (19, (7, 6, 5)), (27, (6, 5, 4))])
def test_equilibrium_init_bit_exact(q, dims):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(q)
    lat = Lattice({9: "D2Q9", 19: "D3Q19", 27: "D3Q27"}[q], dims)
    n = int(np.prod(dims))
    D = 2 if q == 9 else 3
    lat.init_equilibrium(1.02, (0.03, -0.01, 0.02))
    f = lat.populations(np.float64)
    want = O.equilibrium_f32(q, np.float32(1.02), np.array([0.03, -0.01, 0.02][:D], np.float32))
    np.testing.assert_array_equal(f, np.tile(want.astype(np.float64), (n, 1)))
    rho = (1 + 0.05 * rng.standard_normal(n)).astype(np.float32)
    u = (0.05 * rng.standard_normal((D, n))).astype(np.float32)
    d_rho = torch.from_numpy(rho).cuda()
    d_u = torch.from_numpy(u).cuda()
    torch.cuda.synchronize()
    lat.step(K.make_program(0.8, K.KEL_COLL_BGK, {}), 1)  # an odd time step: slots placed by parity
    lat.init_equilibrium(d_rho=d_rho.data_ptr(), d_u=d_u.data_ptr())
    f = lat.populations(np.float64)
    # at an odd time step a boundary cell's populations from outside have no
    # slot (they are the ghost ring's zeros): compare interior cells
    x, y, z = cases.cell_grid(dims)
    inner = (x > 0) & (x < dims[0] - 1) & (y > 0) & (y < dims[1] - 1)
    if D == 3:
        inner &= (z > 0) & (z < dims[2] - 1)
    for c in np.flatnonzero(inner)[::max(1, inner.sum() // 97)]:
        want = O.equilibrium_f32(q, rho[c], u[:, c])
        np.testing.assert_array_equal(f[c], want.astype(np.float64), err_msg=str(c))
    lat.close()


def test_paint_revalidates_the_program():
    lat = Lattice("D3Q19", (8, 8, 8))
    lat.paint([dict(flag=2)])
    zh = K.make_program(0.8, K.KEL_COLL_BGK, {2: dict(bc=K.KEL_BC_FLUID, collide=1),
                                               3: dict(bc=K.KEL_BC_ZOUHE_VELOCITY_X, collide=1)})
    lat.step(zh, 1)  # no cell carries flag 3: allowed
    lat.paint([dict(flag=3, lo=(0, 0, 0), hi=(1, BIG, BIG))])
    with pytest.raises(Exception):
        lat.step(zh, 1)
    lat.close()
