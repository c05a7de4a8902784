"""Generate the golden sweep vectors from keldu/lbm_mirror's own components.

Runs oracle/_ref/ref_harness (built by oracle/Makefile from the reference's
headers, unchanged) on every case below and stores inputs + outputs as
tests/golden/<name>.npz.  Needs the reference tree, named by the environment
variable KEL_REFERENCE_ROOT (the harness is built from
$KEL_REFERENCE_ROOT/modules/core/c++), so it runs only where the reference is
mounted; the committed .npz files are what the tests read.

    KEL_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py [--only NAME] [--check]

--check regenerates every selected fixture and compares it array for array
with the committed file instead of writing it (exit status 1 on a difference).

Inputs are rounded to float32 before use so that the stored float32 copy is
exactly what both the reference and the implementations under test consume.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lbm_mirror_gb300 import capi as K  # noqa: E402
from tests import cases  # noqa: E402

GOLDEN = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def registry():
    """name -> (harness case id, case dict)."""
    r = {}
    r["poiseuille_48x20"] = ("d2q9_f32_48x20", cases.poiseuille_2d(48, 20, steps=301, u_max=0.05))
    r["poiseuille_48x20_f64"] = ("d2q9_f64_48x20", cases.poiseuille_2d(48, 20, steps=301, f64=True))
    r["poiseuille_256x64"] = ("d2q9_f32_256x64", cases.poiseuille_2d(256, 64, steps=10000))
    for nm, coll in (("bgk", K.KEL_COLL_BGK), ("guo", K.KEL_COLL_BGK_GUO), ("psm", K.KEL_COLL_PSM),
                     ("psmguo", K.KEL_COLL_PSM_GUO)):
        r[f"mixed2d_{nm}"] = ("d2q9_f32_48x20", cases.mixed_2d(coll))
    r["mixed2d_guo_f64"] = ("d2q9_f64_48x20", cases.mixed_2d(K.KEL_COLL_BGK_GUO, f64=True))
    for q in (19, 27):
        r[f"cavity_d3q{q}"] = (f"d3q{q}_f32_16x12x10", cases.cavity_3d(q))
        r[f"cavity_d3q{q}_f64"] = (f"d3q{q}_f64_16x12x10", cases.cavity_3d(q, f64=True))
        r[f"mixed3d_d3q{q}_bgk"] = (f"d3q{q}_f32_16x12x10", cases.mixed_3d(q, K.KEL_COLL_BGK))
        r[f"mixed3d_d3q{q}_guo"] = (f"d3q{q}_f32_16x12x10", cases.mixed_3d(q, K.KEL_COLL_BGK_GUO, seed=3))
        r[f"mixed3d_d3q{q}_psmguo"] = (f"d3q{q}_f32_16x12x10", cases.mixed_3d(q, K.KEL_COLL_PSM_GUO, seed=4))
    return r


def _f32_round(a):
    return None if a is None else np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


def normalise(case):
    """Round every floating input to float32 (the stored precision)."""
    c = dict(case)
    for k in ("init", "profile", "porosity", "force"):
        c[k] = _f32_round(c[k])
    return c


def run_harness(hcase, case, workdir):
    ind = os.path.join(workdir, "in")
    outd = os.path.join(workdir, "out")
    os.makedirs(ind, exist_ok=True)
    os.makedirs(outd, exist_ok=True)
    p = case["program"]
    lines = [f"steps {case['steps']}", f"tau {p.tau!r}", f"collision {p.collision}",
             "gforce " + " ".join(repr(float(v)) for v in p.global_force)]
    for i, o in enumerate(p.ops):
        lines.append(f"op {i} {o.bc} {o.collide} {o.east} {o.rho!r} {o.u[0]!r} {o.u[1]!r} {o.u[2]!r} {o.use_profile}")
    open(os.path.join(ind, "params.txt"), "w").write("\n".join(lines) + "\n")
    case["flags"].astype(np.uint8).tofile(os.path.join(ind, "flags.u8"))
    for k, fn in (("init", "init.f64"), ("profile", "profile.f64"), ("porosity", "porosity.f64"),
                  ("force", "force.f64")):
        if case[k] is not None:
            np.asarray(case[k], dtype=np.float64).tofile(os.path.join(ind, fn))
    subprocess.check_call([HARNESS, hcase, ind, outd])
    q, n = case["q"], case["flags"].size
    D = 2 if q == 9 else 3
    dfs = np.fromfile(os.path.join(outd, "dfs.f64")).reshape(n, q)
    rho = np.fromfile(os.path.join(outd, "rho.f64"))
    vel = np.fromfile(os.path.join(outd, "vel.f64")).reshape(n, D)
    return dfs, rho, vel


CHECK = {"on": False, "bad": []}


def emit(name, **arrays):
    """Write tests/golden/<name>.npz, or with --check compare with it."""
    path = os.path.join(GOLDEN, name + ".npz")
    if not CHECK["on"]:
        np.savez_compressed(path, **arrays)
        return
    old = np.load(path)
    same = set(old.files) == set(arrays) and all(
        np.array_equal(np.asarray(arrays[k]), old[k]) for k in arrays)
    if not same:
        CHECK["bad"].append(name)
    print(f"{name:28s} check: {'identical' if same else 'DIFFERS'}")


def build_harness():
    ref = os.environ.get("KEL_REFERENCE_ROOT", "")
    if not ref:
        raise SystemExit("set KEL_REFERENCE_ROOT to the reference checkout (modules/core/c++ below it)")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={ref}"])


def save(name, case, dfs, rho, vel):
    odt = np.float64 if case["f64"] else np.float32
    arrays = dict(
        meta=np.array(json.dumps(dict(
            q=case["q"], dims=list(case["dims"]), f64=bool(case["f64"]), periodic=bool(case["periodic"]),
            steps=int(case["steps"]), program=K.program_to_dict(case["program"])))),
        flags=case["flags"].astype(np.uint8),
        dfs=dfs.astype(odt), rho=rho.astype(odt), vel=vel.astype(odt))
    for k in ("init", "profile", "porosity", "force"):
        if case[k] is not None:
            arrays[k] = np.asarray(case[k]).astype(np.float32)
    emit(name, **arrays)


def load(name):
    """Fixture -> (case dict, dfs, rho, vel) with float64 arrays."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    case = dict(q=meta["q"], dims=tuple(meta["dims"]), f64=meta["f64"], periodic=meta["periodic"],
                steps=meta["steps"], program=K.program_from_dict(meta["program"]), flags=z["flags"])
    for k in ("init", "profile", "porosity", "force"):
        case[k] = z[k].astype(np.float64) if k in z.files else None
    return case, z["dfs"].astype(np.float64), z["rho"].astype(np.float64), z["vel"].astype(np.float64)


# ---- particle path ------------------------------------------------------------

PART_DIMS = (64, 48)
PART_PARAMS = dict(sub_steps=2, k_n=100.0, zeta_n=0.1, gamma_t=0.5, mu=0.3, gravity=(0.0, -1e-4), walls=1)


def particle_inputs(kind, seed=11):
    """Bodies (x, y, x_old, y_old, rot, rot_old, radius, density) and AoS
    populations.  'gather': well separated bodies (no ramp overlaps);
    'contact': two overlapping pairs and bodies pressed into two walls."""
    rng = np.random.default_rng(cases.SEED + seed)
    if kind == "gather":
        xy = [(12.3, 11.7, 5.0), (33.6, 14.2, 4.5), (51.1, 30.4, 6.0), (14.8, 35.5, 5.5), (38.2, 35.9, 4.0)]
    else:
        xy = [(20.2, 20.4, 6.0), (30.1, 21.3, 5.5), (44.6, 4.1, 5.0), (58.2, 30.3, 6.5), (23.9, 31.0, 5.0)]
    bodies = []
    for (x, y, r) in xy:
        vx, vy = 0.01 * rng.standard_normal(2)
        rot = 0.05 * rng.standard_normal()
        bodies.append([x, y, x - vx, y - vy, rot, rot - 0.002 * rng.standard_normal(), r, 1.5])
    bodies = np.array(bodies, dtype=np.float64)
    n = PART_DIMS[0] * PART_DIMS[1]
    init = cases.random_populations(9, n, rng, amp=0.05)
    init = init.astype(np.float32).astype(np.float64)
    return bodies, init


def run_particle_harness(hcase, bodies, init, workdir):
    ind = os.path.join(workdir, "in")
    outd = os.path.join(workdir, "out")
    os.makedirs(ind, exist_ok=True)
    os.makedirs(outd, exist_ok=True)
    P = PART_PARAMS
    open(os.path.join(ind, "pparams.txt"), "w").write(
        f"{P['sub_steps']} {P['k_n']!r} {P['zeta_n']!r} {P['gamma_t']!r} {P['mu']!r} "
        f"{P['gravity'][0]!r} {P['gravity'][1]!r} {P['walls']}\n")
    bodies.astype(np.float64).tofile(os.path.join(ind, "particles.f64"))
    init.astype(np.float64).tofile(os.path.join(ind, "init.f64"))
    subprocess.check_call([HARNESS, hcase, ind, outd])
    out = {}
    for k in ("porosity", "force_field", "after_gather", "after_contact", "after_integrate"):
        a = np.fromfile(os.path.join(outd, k + ".f64"))
        out[k] = a.reshape(-1, 28) if k.startswith("after") else a
    return out


HLBM_DIMS = (48, 40)
HLBM_PARAMS = dict(sub_steps=2, gravity=(0.0, -1e-4), tau=0.8)
HLBM_CASES = {"hlbm_d2q9_f64_48x40x3": np.float64, "hlbm_d2q9_f32_48x40x3": np.float32}


def hlbm_inputs(seed=31):
    """Three moving discs in a walled 48x40 box (rim flag 1, fluid 2), two of
    them with overlapping AABBs (the last body's porosity wins there), and
    near-equilibrium populations."""
    rng = np.random.default_rng(cases.SEED + seed)
    xy = [(14.3, 13.6, 5.0), (22.8, 15.1, 4.5), (33.4, 27.2, 6.0)]
    bodies = []
    for (x, y, r) in xy:
        vx, vy = 0.02 * rng.standard_normal(2)
        rot = 0.05 * rng.standard_normal()
        bodies.append([x, y, x - vx, y - vy, rot, rot - 0.002 * rng.standard_normal(), r, 1.5])
    bodies = np.array(bodies, dtype=np.float64)
    nx, ny = HLBM_DIMS
    x, y, _ = cases.cell_grid(HLBM_DIMS)
    flags = np.full(nx * ny, 2, np.uint8)
    flags[(x == 0) | (x == nx - 1) | (y == 0) | (y == ny - 1)] = 1
    init = cases.random_populations(9, nx * ny, rng, amp=0.05).astype(np.float32).astype(np.float64)
    return bodies, init, flags


def run_hlbm_harness(hcase, bodies, init, flags, workdir):
    ind, outd = os.path.join(workdir, "in"), os.path.join(workdir, "out")
    os.makedirs(ind, exist_ok=True)
    os.makedirs(outd, exist_ok=True)
    P = HLBM_PARAMS
    open(os.path.join(ind, "pparams.txt"), "w").write(
        f"{P['sub_steps']} {P['gravity'][0]!r} {P['gravity'][1]!r} {P['tau']!r}\n")
    bodies.astype(np.float64).tofile(os.path.join(ind, "particles.f64"))
    init.astype(np.float64).tofile(os.path.join(ind, "init.f64"))
    flags.astype(np.uint8).tofile(os.path.join(ind, "flags.u8"))
    subprocess.check_call([HARNESS, hcase, ind, outd])
    out = {}
    for k in ("porosity", "force_field", "after_gather", "after_integrate", "hlbm_N", "hlbm_D", "dfs", "rho", "vel"):
        a = np.fromfile(os.path.join(outd, k + ".f64"))
        out[k] = a.reshape(-1, 28) if k.startswith("after") else a
    return out


FPLBM_PARAMS = dict(sub_steps=2, gravity=(0.0, -1e-4), tau=0.8)
# name -> (harness case, bodies used)
FPLBM_CASES = {"fplbm_d2q9_f64_48x40x1": ("fplbm_d2q9_f64_48x40x1", 1),
               "fplbm_d2q9_f32_48x40x1": ("fplbm_d2q9_f32_48x40x1", 1),
               "fplbm_d2q9_f32_48x40x3": ("fplbm_d2q9_f32_48x40x3", 3)}


def fplbm_inputs(nbodies, seed=37):
    """The HLBM box and populations; the first `nbodies` of its moving discs."""
    bodies, init, flags = hlbm_inputs(seed)
    return bodies[:nbodies].copy(), init, flags


def run_fplbm_harness(hcase, bodies, init, flags, workdir):
    ind, outd = os.path.join(workdir, "in"), os.path.join(workdir, "out")
    os.makedirs(ind, exist_ok=True)
    os.makedirs(outd, exist_ok=True)
    P = FPLBM_PARAMS
    open(os.path.join(ind, "pparams.txt"), "w").write(
        f"{P['sub_steps']} {P['gravity'][0]!r} {P['gravity'][1]!r} {P['tau']!r}\n")
    bodies.astype(np.float64).tofile(os.path.join(ind, "particles.f64"))
    init.astype(np.float64).tofile(os.path.join(ind, "init.f64"))
    flags.astype(np.uint8).tofile(os.path.join(ind, "flags.u8"))
    subprocess.check_call([HARNESS, hcase, ind, outd])
    out = {}
    for k in ("reset_rho", "reset_mom", "porosity", "force_field", "after_particle", "dfs", "rho", "vel"):
        a = np.fromfile(os.path.join(outd, k + ".f64"))
        out[k] = a.reshape(-1, 28) if k.startswith("after") else a
    return out


# Voxel signed-distance bodies: harness case, dimension, mask resolution,
# shape (0 sphere, 1 cube), eps, lattice extent.
VOXEL_CASES = {"voxel_2d_sphere": ("voxel_2d_f64_4", 2, 32, 0, 1.0, (64, 64, 1)),
               "voxel_2d_cube": ("voxel_2d_f64_4", 2, 32, 1, 1.5, (64, 64, 1)),
               "voxel_3d_sphere": ("voxel_3d_f64_4", 3, 16, 0, 1.0, (40, 40, 40)),
               "voxel_3d_cube": ("voxel_3d_f64_4", 3, 16, 1, 1.5, (40, 40, 40))}


def voxel_inputs(dim, ext, seed=43):
    """Four bodies (position, rotation, radius): 0 and 1 overlap off-axis, 2
    touches 1, 3 stands apart; local points inside and outside the mask box;
    lattice points around the bodies; pairs in both orders; distances across
    the ramp."""
    rng = np.random.default_rng(seed + dim)
    if dim == 2:
        pos = np.array([[29.0, 30.0, 0], [36.0, 33.5, 0], [42.3, 24.7, 0], [16.2, 47.9, 0]])
        rot = np.array([[0.0, 0, 0], [0.7, 0, 0], [-1.3, 0, 0], [2.9, 0, 0]])
        rad = np.array([5.0, 5.0, 6.0, 4.5])
    else:
        pos = np.array([[18.0, 19.0, 20.0], [23.0, 21.5, 20.5], [27.2, 14.6, 22.3], [9.1, 30.2, 28.4]])
        rot = np.array([[0.0, 0.0, 0.0], [0.3, -0.5, 0.2], [1.1, 0.4, -0.7], [-0.2, 0.9, 1.6]])
        rad = np.array([4.5, 4.5, 5.0, 3.5])
    bodies = np.concatenate([pos, rot, rad[:, None]], axis=1)
    locals_ = np.zeros((48, 3))
    locals_[:40, :dim] = rng.uniform(-1.3, 1.3, (40, dim))
    fixed = [[0, 0, 0], [1, 0, 0], [0.5, 0, 0], [-1, -1, 0], [0.99, 0.99, 0], [1.2, -1.25, 0], [-0.3, 0.4, 0],
             [0.0, 1.0, 0]]
    locals_[40:, :2] = np.array(fixed)[:, :2]
    if dim == 3:
        locals_[40:, 2] = rng.uniform(-1, 1, 8)
    pts = np.zeros((160, 3))
    for k in range(160):
        b = k % 4
        pts[k, :dim] = pos[b, :dim] + rng.uniform(-1.6, 1.6, dim) * rad[b]
    pairs = np.array([[0, 1], [1, 0], [1, 2], [2, 1], [0, 2], [0, 3], [3, 2]], np.float64)
    sdfs = np.concatenate([np.linspace(-1.0, 1.0, 41), [-5.0, 5.0]])
    return dict(bodies=bodies, locals=locals_, points=pts, pairs=pairs, sdfs=sdfs)


def run_voxel_harness(hcase, R, kind, eps, ext, inp, workdir):
    ind, outd = os.path.join(workdir, "in"), os.path.join(workdir, "out")
    os.makedirs(ind)
    os.makedirs(outd)
    open(os.path.join(ind, "vparams.txt"), "w").write(f"{R} {kind} {eps!r} {ext[0]} {ext[1]} {ext[2]}\n")
    for k, f in (("bodies", "bodies"), ("locals", "locals"), ("points", "points"), ("pairs", "pairs"),
                 ("sdfs", "sdfs")):
        inp[k].astype(np.float64).tofile(os.path.join(ind, f + ".f64"))
    subprocess.check_call([HARNESS, hcase, ind, outd])
    out = {}
    for k in ("mask", "com", "sample", "global", "sdf", "porosity", "solid", "contacts"):
        out[k] = np.fromfile(os.path.join(outd, k + ".f64"))
    out["contacts"] = out["contacts"].reshape(-1, 8)
    out["global"] = out["global"].reshape(-1, 3)
    return out


def particle_registry():
    return {
        "particles_gather_f64": ("particles_d2q9_f64_64x48x5", "gather"),
        "particles_gather_f32": ("particles_d2q9_f32_64x48x5", "gather"),
        "particles_contact_f64": ("particles_d2q9_f64_64x48x5", "contact"),
    }


def load_particles(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and not f.startswith(("particles_", "writers_", "cavity256_", "hlbm_", "fplbm_",
                                                               "voxel_")))


WRITER_CASES = {"writers_d2q9_f32_12x7": (9, (12, 7), np.float32),
                "writers_d3q19_f64_5x4x3": (19, (5, 4, 3), np.float64)}
WRITER_FILES = ("vtk/m_37.vtk", "vtk/initial_state_0.vtk", "csv/m_velocity_37.csv", "csv/m_density_37.csv",
                "m.forst", "lattice.forst")


def writer_inputs(q, dims, dtype, seed=21):
    """Values that exercise the number formatting: magnitudes from 1e-9 to 1e3,
    both signs, exact zeros and integers."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(dims))
    d = 2 if q == 9 else 3

    def vals(shape):
        v = rng.standard_normal(shape) * 10.0 ** rng.integers(-9, 4, shape)
        v[rng.random(shape) < 0.05] = 0.0
        v[rng.random(shape) < 0.05] = 1.0
        v[rng.random(shape) < 0.05] = -250.0
        return v.astype(dtype).astype(np.float64)

    flags = rng.integers(0, 6, n).astype(np.uint8)
    return dict(flags=flags, dfs=vals((n, q)), rho=1.0 + vals(n), vel=vals((n, d)))


def run_writer_harness(name, inp, workdir):
    ind, outd = os.path.join(workdir, "in"), os.path.join(workdir, "out")
    os.makedirs(ind)
    os.makedirs(outd)
    inp["flags"].tofile(os.path.join(ind, "flags.u8"))
    for k in ("dfs", "rho", "vel"):
        inp[k].astype(np.float64).tofile(os.path.join(ind, k + ".f64"))
    subprocess.check_call([HARNESS, name, ind, outd])
    return {f: np.frombuffer(open(os.path.join(outd, f), "rb").read(), np.uint8) for f in WRITER_FILES}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    ap.add_argument("--check", action="store_true", help="compare with the committed fixtures, write nothing")
    args = ap.parse_args()
    CHECK["on"] = args.check
    if not os.path.exists(HARNESS):
        build_harness()
    for name, (hcase, kind) in particle_registry().items():
        if args.only and args.only not in name:
            continue
        bodies, init = particle_inputs(kind)
        with tempfile.TemporaryDirectory() as td:
            out = run_particle_harness(hcase, bodies, init, td)
        emit(name, bodies=bodies, init=init.astype(np.float32),
                            params=np.array(json.dumps(PART_PARAMS)), **out)
        print(f"{name:28s} particles: force after gather {out['after_gather'][:, 18:20].ravel()[:4]}")
    for name in HLBM_CASES:
        if args.only and args.only not in name:
            continue
        bodies, init, flags = hlbm_inputs()
        with tempfile.TemporaryDirectory() as td:
            out = run_hlbm_harness(name, bodies, init, flags, td)
        emit(name, bodies=bodies, init=init, flags=flags,
                            params=np.array(json.dumps(HLBM_PARAMS)), **out)
        print(f"{name:28s} hlbm: body force after gather {out['after_gather'][:, 18:20].ravel()[:4]}")
    for name, (hcase, nb) in FPLBM_CASES.items():
        if args.only and args.only not in name:
            continue
        bodies, init, flags = fplbm_inputs(nb)
        with tempfile.TemporaryDirectory() as td:
            out = run_fplbm_harness(hcase, bodies, init, flags, td)
        emit(name, bodies=bodies, init=init, flags=flags, params=np.array(json.dumps(FPLBM_PARAMS)), **out)
        print(f"{name:28s} fplbm: acceleration {out['after_particle'][:, 12:14].ravel()[:4]}")
    for name, (hcase, dim, R, kind, eps, ext) in VOXEL_CASES.items():
        if args.only and args.only not in name:
            continue
        inp = voxel_inputs(dim, ext)
        with tempfile.TemporaryDirectory() as td:
            out = run_voxel_harness(hcase, R, kind, eps, ext, inp, td)
        emit(name, **inp, params=np.array(json.dumps(dict(dim=dim, resolution=R, kind=kind, eps=eps,
                                                             extent=list(ext)))), **out)
        print(f"{name:28s} voxel: hits {out['contacts'][:, 0].astype(int).tolist()} com {out['com']}")
    for name, (q, dims, dtype) in WRITER_CASES.items():
        if args.only and args.only not in name:
            continue
        inp = writer_inputs(q, dims, dtype)
        with tempfile.TemporaryDirectory() as td:
            files = run_writer_harness(name, inp, td)
        emit(name, **inp,
                            **{"file:" + f: v for f, v in files.items()})
        print(f"{name:28s} writers: " + ", ".join(f"{f} {len(v)} B" for f, v in files.items()))
    for name, (hcase, case) in registry().items():
        if args.only and args.only not in name:
            continue
        case = normalise(case)
        with tempfile.TemporaryDirectory() as td:
            dfs, rho, vel = run_harness(hcase, case, td)
        save(name, case, dfs, rho, vel)
        odfs, orho, ovel = cases.run_oracle(case)
        same = np.array_equal(odfs, dfs) and np.array_equal(orho, rho) and np.array_equal(ovel, vel)
        print(f"{name:28s} steps={case['steps']:6d}  oracle bit-exact: {same}  "
              f"max|dfs diff|={np.abs(odfs - dfs).max():.3e}")
    if CHECK["bad"]:
        print("differing fixtures: " + ", ".join(CHECK["bad"]))
        raise SystemExit(1)


if __name__ == "__main__":
    main()
