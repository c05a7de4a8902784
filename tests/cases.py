"""Seeded sweep cases shared by the golden-vector generator and the tests.

Each builder returns a dict:
  q, dims, f64, periodic, steps, program (StepProgram), flags (uint8 per cell),
  init (AoS float64 or None), profile (per-y float64 or None),
  porosity / force (per-cell float64 or None).

Flag layouts follow the reference drivers: walls on the rim, fluid inside,
inlet flag 3 at x = 0 and outlet flag 4 at x = nx-1 over y in [1, ny-2]
(examples/stdkr_2d_bgk/init.hpp:16-54); the cavity lid is flag 5 on the top
row with the corners left as walls (examples/cavity_2d_gpu/cavity_2d_gpu.cpp:63-91).
"""
from __future__ import annotations

import numpy as np

from lbm_mirror_gb300 import capi as K

SEED = 0x4B454C


def cell_grid(dims):
    nx, ny = dims[0], dims[1]
    nz = dims[2] if len(dims) > 2 else 1
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return x.reshape(-1), y.reshape(-1), z.reshape(-1)


def channel_flags(dims):
    """Rim walls, fluid interior, inlet 3 at x=0, outlet 4 at x=nx-1."""
    nx, ny = dims[0], dims[1]
    nz = dims[2] if len(dims) > 2 else 1
    x, y, z = cell_grid(dims)
    f = np.full(x.shape, 1, dtype=np.uint8)
    inner_y = (y >= 1) & (y <= ny - 2)
    inner_z = (z >= 1) & (z <= nz - 2) if nz > 1 else np.ones_like(inner_y)
    f[(x >= 1) & (x <= nx - 2) & inner_y & inner_z] = 2
    f[(x == 0) & inner_y & inner_z] = 3
    f[(x == nx - 1) & inner_y & inner_z] = 4
    return f


def cavity_flags(dims):
    """All faces walls, lid 5 on y = ny-1 over the interior of the other axes."""
    nx, ny = dims[0], dims[1]
    nz = dims[2] if len(dims) > 2 else 1
    x, y, z = cell_grid(dims)
    f = np.full(x.shape, 1, dtype=np.uint8)
    ix = (x >= 1) & (x <= nx - 2)
    iz = ((z >= 1) & (z <= nz - 2)) if nz > 1 else np.ones_like(ix)
    f[ix & (y >= 1) & (y <= ny - 2) & iz] = 2
    f[ix & (y == ny - 1) & iz] = 5
    return f


def parabolic_profile(ny, u_max):
    """u_x(y) = 4 u_max eta (1 - eta), eta = (y - 1/2)/(ny - 2): zero on the
    half-way wall positions y = 1/2 and y = ny - 3/2."""
    y = np.arange(ny, dtype=np.float64)
    eta = (y - 0.5) / (ny - 2)
    u = 4.0 * u_max * eta * (1.0 - eta)
    u[0] = 0.0
    u[-1] = 0.0
    return u


def _weights(q):
    from itertools import product
    if q == 9:
        return np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    if q == 19:
        return np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    w = []
    for i in range(27):
        a, b, g = i % 3, (i // 3) % 3, i // 9
        n = (a != 0) + (b != 0) + (g != 0)
        w.append([8 / 27, 2 / 27, 1 / 54, 1 / 216][n])
    return np.array(w)


def random_populations(q, n, rng, amp=0.02):
    """Equilibrium-like positive populations with a seeded perturbation."""
    w = _weights(q)
    return (w[None, :] * (1.0 + amp * rng.standard_normal((n, q)))).astype(np.float64)


def poiseuille_2d(nx=256, ny=64, steps=10000, tau=0.8, u_max=0.05, arithmetic=K.KEL_ARITH_FAST, f64=False):
    """Config C1: D2Q9 BGK Poiseuille channel, Zou-He velocity inlet with a
    parabolic profile, Zou-He pressure outlet rho = 1, rest-equilibrium init."""
    dims = (nx, ny)
    ops = {
        1: dict(bc=K.KEL_BC_BOUNCE_BACK),
        2: dict(bc=K.KEL_BC_FLUID, collide=1),
        3: dict(bc=K.KEL_BC_ZOUHE_VELOCITY_X, collide=1, east=1, use_profile=1, u=(u_max, 0.0, 0.0)),
        4: dict(bc=K.KEL_BC_ZOUHE_PRESSURE_X, collide=1, east=0, rho=1.0),
    }
    return dict(q=9, dims=dims, f64=f64, periodic=False, steps=steps,
                program=K.make_program(tau, K.KEL_COLL_BGK, ops, arithmetic=arithmetic),
                flags=channel_flags(dims), init=None, profile=parabolic_profile(ny, u_max),
                porosity=None, force=None)


def cavity_3d(q, dims=(16, 12, 10), steps=60, tau=0.55, lid=(0.1, 0.0, 0.0), arithmetic=K.KEL_ARITH_FAST,
              f64=False):
    """Config C2: BGK lid-driven cavity, moving bounce-back lid, rest init."""
    ops = {
        1: dict(bc=K.KEL_BC_BOUNCE_BACK),
        2: dict(bc=K.KEL_BC_FLUID, collide=1),
        5: dict(bc=K.KEL_BC_MOVING_WALL, u=lid),
    }
    return dict(q=q, dims=tuple(dims), f64=f64, periodic=False, steps=steps,
                program=K.make_program(tau, K.KEL_COLL_BGK, ops, arithmetic=arithmetic),
                flags=cavity_flags(dims), init=None, profile=None, porosity=None, force=None)


def mixed_2d(collision, dims=(48, 20), steps=37, seed=1, arithmetic=K.KEL_ARITH_FAST, f64=False,
             periodic=False):
    """Every D2Q9 boundary op on one lattice, random populations and fields."""
    rng = np.random.default_rng(SEED + seed)
    nx, ny = dims
    x, y, _ = cell_grid(dims)
    flags = np.full(nx * ny, 2, dtype=np.uint8)
    flags[(y == 0) | (y == ny - 1)] = 1
    if not periodic:
        flags[(x == 0) & (y > 0) & (y < ny - 1)] = 4          # pressure inlet (east = 1)
        flags[(x == nx - 1) & (y > 0) & (y < ny - 1)] = 3     # velocity outlet (east = 0)
    flags[(y == ny - 1) & (x > 2) & (x < nx - 3)] = 5         # lid
    flags[(y == 0) & (x > 5) & (x < 12)] = 6                  # anti bounce-back stripe
    flags[(x > 20) & (x < 24) & (y > 6) & (y < 10)] = 7       # equilibrium block
    flags[(x > 30) & (x < 34) & (y > 8) & (y < 13)] = 1       # obstacle
    ops = {
        1: dict(bc=K.KEL_BC_BOUNCE_BACK),
        2: dict(bc=K.KEL_BC_FLUID, collide=1),
        3: dict(bc=K.KEL_BC_ZOUHE_VELOCITY_X, collide=1, east=0, u=(0.03, 0.01, 0.0)),
        4: dict(bc=K.KEL_BC_ZOUHE_PRESSURE_X, collide=1, east=1, rho=1.01),
        5: dict(bc=K.KEL_BC_MOVING_WALL, u=(0.08, 0.02, 0.0)),
        6: dict(bc=K.KEL_BC_ANTI_BOUNCE_BACK),
        7: dict(bc=K.KEL_BC_EQUILIBRIUM, rho=1.02, u=(0.01, -0.02, 0.0)),
    }
    por = None
    if collision in (K.KEL_COLL_PSM, K.KEL_COLL_PSM_GUO):
        por = rng.uniform(0.0, 1.0, nx * ny)
        por[rng.uniform(size=nx * ny) < 0.3] = 1.0
        por[rng.uniform(size=nx * ny) < 0.1] = 0.0
    force = None
    if collision in (K.KEL_COLL_BGK_GUO, K.KEL_COLL_PSM_GUO):
        force = 1e-4 * rng.standard_normal(nx * ny * 2)
    return dict(q=9, dims=dims, f64=f64, periodic=periodic, steps=steps,
                program=K.make_program(0.7, collision, ops, global_force=(2e-5, -1e-5, 0.0), arithmetic=arithmetic),
                flags=flags, init=random_populations(9, nx * ny, rng), profile=None,
                porosity=por, force=force)


def mixed_3d(q, collision, dims=(16, 12, 10), steps=21, seed=2, arithmetic=K.KEL_ARITH_FAST, f64=False,
             periodic=False):
    """3D walls, fluid, lid, equilibrium block and (D3Q27) Zou-He pressure faces."""
    rng = np.random.default_rng(SEED + seed)
    nx, ny, nz = dims
    x, y, z = cell_grid(dims)
    n = nx * ny * nz
    flags = np.full(n, 2, dtype=np.uint8)
    flags[(y == 0) | (y == ny - 1) | (z == 0) | (z == nz - 1)] = 1
    if q == 27 and not periodic:
        inner = (y > 0) & (y < ny - 1) & (z > 0) & (z < nz - 1)
        flags[(x == 0) & inner] = 3   # pressure inlet, east = 1
        flags[(x == nx - 1) & inner] = 4  # pressure outlet, east = 0
    elif not periodic:
        flags[(x == 0) | (x == nx - 1)] = 1
    flags[(y == ny - 1) & (x > 2) & (x < nx - 3) & (z > 1) & (z < nz - 2)] = 5
    flags[(x > 8) & (x < 11) & (y > 3) & (y < 6) & (z > 5) & (z < 9)] = 7
    ops = {
        1: dict(bc=K.KEL_BC_BOUNCE_BACK),
        2: dict(bc=K.KEL_BC_FLUID, collide=1),
        3: dict(bc=K.KEL_BC_ZOUHE_PRESSURE_X, collide=1, east=1, rho=1.01),
        4: dict(bc=K.KEL_BC_ZOUHE_PRESSURE_X, collide=1, east=0, rho=1.0),
        5: dict(bc=K.KEL_BC_MOVING_WALL, u=(0.07, 0.0, -0.03)),
        7: dict(bc=K.KEL_BC_EQUILIBRIUM, rho=0.99, u=(0.02, 0.01, -0.01)),
    }
    por = None
    if collision in (K.KEL_COLL_PSM, K.KEL_COLL_PSM_GUO):
        por = rng.uniform(0.0, 1.0, n)
        por[rng.uniform(size=n) < 0.3] = 1.0
    force = None
    if collision in (K.KEL_COLL_BGK_GUO, K.KEL_COLL_PSM_GUO):
        force = 1e-4 * rng.standard_normal(n * 3)
    return dict(q=q, dims=dims, f64=f64, periodic=periodic, steps=steps,
                program=K.make_program(0.62, collision, ops, global_force=(1e-5, -2e-5, 3e-6), arithmetic=arithmetic),
                flags=flags, init=random_populations(q, n, rng), profile=None,
                porosity=por, force=force)


def run_oracle(case):
    """Run a case on the CPU oracle; returns (populations AoS, rho, vel)."""
    from oracle.oracle import OracleLattice
    lat = OracleLattice(case["q"], case["dims"], f64=case["f64"], periodic_x=case["periodic"])
    lat.set_flags(case["flags"])
    if case["init"] is not None:
        lat.set_populations(case["init"])
    if case["profile"] is not None:
        lat.set_profile(case["profile"])
    if case["porosity"] is not None:
        lat.set_porosity(case["porosity"])
    if case["force"] is not None:
        lat.set_force(case["force"])
    lat.run(case["program"], case["steps"])
    rho, vel = lat.macros()
    return lat.populations(), rho, vel


def channel_geometry(nx, ny, rng):
    """One config-C4 channel: rim walls, inlet 3 at x = 0, outlet 4 at
    x = nx-1, and 1..8 seeded obstacles (disks r in [3, 12] or axis-aligned
    rectangles) kept clear of the inlet/outlet columns and of the channel
    height, so that the channel never closes."""
    x, y, _ = cell_grid((nx, ny))
    f = channel_flags((nx, ny))
    n_obs = int(rng.integers(1, 9))
    for _ in range(n_obs):
        if rng.uniform() < 0.5:
            r = float(rng.uniform(3.0, 12.0))
            r = max(1.5, min(r, (ny - 6) / 2.0 - 1.0, (nx - 14) / 2.0))
            cx = float(rng.uniform(r + 6, nx - r - 6))
            cy = float(rng.uniform(r + 1, ny - r - 2))
            solid = (x - cx) ** 2 + (y - cy) ** 2 <= r * r
        else:
            w = int(rng.integers(2, max(3, nx // 8)))
            h = int(rng.integers(2, max(3, ny // 2)))
            x0 = int(rng.integers(6, max(7, nx - w - 6)))
            y0 = int(rng.integers(1, max(2, ny - h - 1)))
            solid = (x >= x0) & (x < x0 + w) & (y >= y0) & (y < y0 + h)
        f[solid & (x > 2) & (x < nx - 3)] = 1
    return f


def batch_channels(n=1024, seed=4, nx_range=(64, 512), ny_range=(32, 128)):
    """Config C4: n independent D2Q9 channels of uneven size, u_max ~ U[0.01,
    0.08], tau ~ U[0.55, 1.0].  Returns a list of dicts (nx, ny, tau, u_max,
    flags, profile)."""
    rng = np.random.default_rng(SEED + 1000 + seed)
    out = []
    for _ in range(n):
        nx = int(rng.integers(nx_range[0], nx_range[1] + 1))
        ny = int(rng.integers(ny_range[0], ny_range[1] + 1))
        u_max = float(rng.uniform(0.01, 0.08))
        tau = float(rng.uniform(0.55, 1.0))
        out.append(dict(nx=nx, ny=ny, tau=tau, u_max=u_max, flags=channel_geometry(nx, ny, rng),
                        profile=parabolic_profile(ny, u_max)))
    return out


def channel_program(tau, arithmetic=K.KEL_ARITH_FAST):
    """The per-flag program of a C4 channel (the stdkr_2d_bgk switch)."""
    ops = {
        1: dict(bc=K.KEL_BC_BOUNCE_BACK),
        2: dict(bc=K.KEL_BC_FLUID, collide=1),
        3: dict(bc=K.KEL_BC_ZOUHE_VELOCITY_X, collide=1, east=1, use_profile=1),
        4: dict(bc=K.KEL_BC_ZOUHE_PRESSURE_X, collide=1, east=0, rho=1.0),
    }
    return K.make_program(tau, K.KEL_COLL_BGK, ops, arithmetic=arithmetic)


def particle_channel(nx=2048, ny=512, n_particles=64, radius=8.0, density=1.5, seed=3):
    """Config C3: periodic-x channel with walls at y = 0 and y = ny-1 and
    n_particles discs of radius R placed by seeded uniform rejection sampling
    (no overlap, at least one cell between discs and from the walls), at rest.
    Returns (flags, states (P, 28))."""
    rng = np.random.default_rng(SEED + 3000 + seed)
    x, y, _ = cell_grid((nx, ny))
    flags = np.full(nx * ny, 2, dtype=np.uint8)
    flags[(y == 0) | (y == ny - 1)] = 1
    pos = []
    while len(pos) < n_particles:
        px = rng.uniform(0.0, nx)
        py = rng.uniform(radius + 2.0, ny - 1 - radius - 2.0)
        ok = True
        for (qx, qy) in pos:
            dx = abs(px - qx)
            dx = min(dx, nx - dx)
            if dx * dx + (py - qy) ** 2 < (2 * radius + 1.0) ** 2:
                ok = False
                break
        if ok:
            pos.append((px, py))
    st = np.zeros((n_particles, 28))
    m = np.pi * radius * radius * density
    for i, (px, py) in enumerate(pos):
        st[i, 0:2] = (px, py)
        st[i, 3:5] = (px, py)
        st[i, 24] = m
        st[i, 25] = 0.5 * m * radius * radius
        st[i, 26] = radius
        st[i, 27] = density
    return flags, st
