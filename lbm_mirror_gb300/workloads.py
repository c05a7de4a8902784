"""Seeded workload generators: the channel, cavity, batched-channel and
particle-laden layouts the drivers of keldu/lbm_mirror set up, and the
per-flag program of a pressure-driven channel.

Flag layouts follow the reference drivers: walls on the rim, fluid inside,
inlet flag 3 at x = 0 and outlet flag 4 at x = nx-1 over y in [1, ny-2]
(examples/stdkr_2d_bgk/init.hpp:16-54); the cavity lid is flag 5 on the top
row with the corners left as walls (examples/cavity_2d_gpu/cavity_2d_gpu.cpp:63-91).
Cells are numbered x fastest.
"""
from __future__ import annotations

import numpy as np

from . import capi as K

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


def _open_passage(f, nx, ny):
    """True when (a) every column keeps at least half of its ny - 2 interior
    cells open (blockage at most 50%, so the mean velocity through the
    narrowest section stays within twice the channel's) and (b) fluid
    connects the inlet column to the outlet column through a passage at
    least 3 cells wide (the fluid eroded by one cell stays 4-connected from
    x = 1 to x = nx-2)."""
    from scipy import ndimage
    fluid = (f.reshape(ny, nx) != 1)
    if np.min(fluid[1:ny - 1].sum(axis=0)) * 2 < ny - 2:
        return False
    core = ndimage.binary_erosion(fluid, structure=np.ones((3, 3), bool), border_value=0)
    lab, _ = ndimage.label(core)
    a = set(np.unique(lab[:, 1])) - {0}
    b = set(np.unique(lab[:, nx - 2])) - {0}
    return bool(a & b)


def channel_geometry(nx, ny, rng):
    """One channel of the batched-channel workload: rim walls, inlet 3 at
    x = 0, outlet 4 at x = nx-1, and up to 8 seeded obstacles (disks r in
    [3, 12] or axis-aligned rectangles) kept clear of the inlet/outlet
    columns.  An obstacle that would block more than half of a column, or
    leave no passage at least 3 cells wide from inlet to outlet, is dropped:
    a closed channel fed by a velocity inlet gains mass without bound, and a
    narrow gap drives the flow to Mach numbers where BGK diverges."""
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
        g = f.copy()
        g[solid & (x > 2) & (x < nx - 3)] = 1
        if _open_passage(g, nx, ny):
            f = g
    return f


def batch_channels(n=1024, seed=4, nx_range=(64, 512), ny_range=(32, 128)):
    """The batched-channel workload: n independent D2Q9 channels of uneven size, u_max ~ U[0.01,
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
    """Particle-laden channel: periodic in x, with walls at y = 0 and y = ny-1 and
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
