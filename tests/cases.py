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
from lbm_mirror_gb300.workloads import (SEED, batch_channels, cavity_flags, cell_grid,  # noqa: F401
                                        channel_flags, channel_geometry, channel_program,
                                        parabolic_profile, particle_channel)


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
    """D2Q9 BGK Poiseuille channel, Zou-He velocity inlet with a
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
    """BGK lid-driven cavity, moving bounce-back lid, rest init."""
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


def halfway_poiseuille_2d(nx=8, ny=22, steps=6000, tau=0.8, g=1e-6, arithmetic=K.KEL_ARITH_FAST, f64=False):
    """Force-driven D2Q9 channel, periodic in x, half-way bounce-back walls
    at y = 0 and y = ny - 1 (the wall planes sit at y = 1/2 and y = ny - 3/2),
    BGK + Guo body force g along x, rest start.  Steady state:
    u_x(y) = g_eff / (2 nu) (y - 1/2) (ny - 3/2 - y), nu = (tau - 1/2) / 3,
    g_eff = (1 - 1/(2 tau)) g (the reference's Guo term without the
    half-force velocity shift)."""
    dims = (nx, ny)
    x, y, _ = cell_grid(dims)
    flags = np.full(nx * ny, 2, dtype=np.uint8)
    flags[(y == 0) | (y == ny - 1)] = 1
    ops = {1: dict(bc=K.KEL_BC_HALFWAY_WALL), 2: dict(bc=K.KEL_BC_FLUID, collide=1)}
    return dict(q=9, dims=dims, f64=f64, periodic=True, steps=steps,
                program=K.make_program(tau, K.KEL_COLL_BGK_GUO, ops, global_force=(g, 0.0, 0.0),
                                       arithmetic=arithmetic),
                flags=flags, init=None, profile=None, porosity=None, force=None)


def halfway_mixed(q, dims, steps=23, seed=3, arithmetic=K.KEL_ARITH_REFERENCE, f64=False, periodic=False):
    """Half-way walls (flag 6: the rim in y and z, an obstacle block and an
    isolated wall cell) beside full-way walls (flag 1: the x ends), a moving
    lid (flag 5), fluid, random populations."""
    rng = np.random.default_rng(SEED + seed)
    x, y, z = cell_grid(dims)
    nx, ny = dims[0], dims[1]
    nz = dims[2] if len(dims) == 3 else 1
    n = nx * ny * nz
    flags = np.full(n, 2, dtype=np.uint8)
    rim = (y == 0) | (y == ny - 1)
    if q != 9:
        rim |= (z == 0) | (z == nz - 1)
    flags[rim] = 6
    if not periodic:
        flags[(x == 0) | (x == nx - 1)] = 1
    flags[(y == ny - 1) & (x > 2) & (x < nx - 3) & ((z > 1) & (z < nz - 2) if q != 9 else True)] = 5
    blk = (x > 5) & (x < 9) & (y > 3) & (y < 7)
    if q != 9:
        blk &= (z > 2) & (z < 6)
    flags[blk] = 6
    flags[(x == nx - 5) & (y == ny // 2) & (z == nz // 2)] = 6
    ops = {
        1: dict(bc=K.KEL_BC_BOUNCE_BACK),
        2: dict(bc=K.KEL_BC_FLUID, collide=1),
        5: dict(bc=K.KEL_BC_MOVING_WALL, u=(0.06, 0.0, 0.02) if q != 9 else (0.06, 0.0, 0.0)),
        6: dict(bc=K.KEL_BC_HALFWAY_WALL),
    }
    return dict(q=q, dims=tuple(dims), f64=f64, periodic=periodic, steps=steps,
                program=K.make_program(0.7, K.KEL_COLL_BGK_GUO, ops, global_force=(2e-5, -1e-5, 0.0),
                                       arithmetic=arithmetic),
                flags=flags, init=random_populations(q, n, rng), profile=None, porosity=None, force=None)


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
