"""ctypes binding of the CPU oracle (oracle/lbm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  The oracle is a
plain-C restatement of keldu/lbm_mirror's two-lattice sweep; see the header of
lbm_oracle.c for the reference lines each part follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libkel_oracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")

_lib = None


def build(force: bool = False) -> str:
    """Compile the restatement with gcc (no FMA contraction, OpenMP)."""
    src = [os.path.join(HERE, "lbm_oracle.c"), os.path.join(HERE, "lbm_oracle_impl.h"),
           os.path.join(HERE, "particles_oracle.c"), os.path.join(HERE, "voxel_oracle.c")]
    src = [s for s in src if os.path.exists(s)]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in src):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    cfiles = [s for s in src if s.endswith(".c")]
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB + ".tmp"] + cfiles + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, i64, u64 = C.c_void_p, C.c_int64, C.c_uint64
        L.ko_create.argtypes = [C.c_int, C.c_int, i64, i64, i64, C.c_int]
        L.ko_create.restype = vp
        L.ko_destroy.argtypes = [vp]
        L.ko_set_flags.argtypes = [vp, vp]
        L.ko_set_profile.argtypes = [vp, vp]
        L.ko_set_populations.argtypes = [vp, vp]
        L.ko_get_populations.argtypes = [vp, vp]
        L.ko_set_porosity.argtypes = [vp, vp]
        L.ko_set_force.argtypes = [vp, vp]
        L.ko_get_macros.argtypes = [vp, vp, vp]
        L.ko_run.argtypes = [vp, vp, u64]
        L.ko_run.restype = C.c_int
        L.ko_run_rows.argtypes = [vp, vp, i64, i64]
        L.ko_run_rows.restype = C.c_int
        L.ko_time_step.argtypes = [vp]
        L.ko_time_step.restype = u64
        L.ko_equilibrium_f32.argtypes = [C.c_int, C.c_float, vp, vp]
        L.ko_program_size.restype = C.c_size_t
        L.ko_get_porosity.argtypes = [vp, vp]
        L.ko_particles_couple.argtypes = [vp, vp, C.c_int, vp]
        L.ko_particles_gather.argtypes = [vp, vp, C.c_int, vp, vp]
        L.ko_particles_reset.argtypes = [vp, C.c_int]
        L.ko_particles_contact.argtypes = [vp, C.c_int, C.c_int, vp, vp, C.c_int]
        L.ko_particles_integrate.argtypes = [vp, C.c_int, C.c_int, vp, vp, C.c_int]
        L.ko_particles_hlbm_couple.argtypes = [vp, vp, C.c_int, vp]
        L.ko_particles_hlbm_gather.argtypes = [vp, vp, C.c_int, vp, vp]
        L.ko_particles_hlbm_stamp.argtypes = [vp, vp, C.c_int, vp]
        L.ko_get_hlbm.argtypes = [vp, vp, vp]
        L.ko_set_hlbm.argtypes = [vp, vp, vp]
        L.ko_fplbm_reset.argtypes = [vp, C.c_uint32]
        L.ko_fplbm_particles.argtypes = [vp, vp, C.c_int, vp, C.c_int]
        L.ko_get_force.argtypes = [vp, vp]
        d = C.c_double
        L.ko_solid_fraction.argtypes = [d, d]
        L.ko_solid_fraction.restype = d
        L.ko_mask_fill.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp]
        L.ko_mask_reach.argtypes = [C.c_int, C.c_int, vp]
        L.ko_mask_reach.restype = d
        L.ko_mask_sample_local.argtypes = [C.c_int, C.c_int, vp, vp]
        L.ko_mask_sample_local.restype = d
        L.ko_mask_local_to_global.argtypes = [C.c_int, vp, vp, vp, vp]
        L.ko_mask_signed_distance.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp]
        L.ko_mask_signed_distance.restype = d
        L.ko_voxel_porosity.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, d]
        L.ko_voxel_porosity.restype = d
        L.ko_voxel_contact.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, vp, d, vp]
        L.ko_voxel_contact.restype = C.c_int
        L.ko_voxel_couple.argtypes = [C.c_int, C.c_int, vp, vp, d, vp, C.c_int, vp, C.c_int, d, vp]
        L.ko_particles_set_voxel_box.argtypes = [d, d]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleLattice:
    """Two-lattice AoS+ghost restatement of the reference sweep (float or double)."""

    def __init__(self, q, dims, f64=False, periodic_x=False):
        nx, ny = dims[0], dims[1]
        nz = dims[2] if len(dims) > 2 else 1
        self.q, self.dims, self.f64 = q, (nx, ny, nz), f64
        self.D = 2 if q == 9 else 3
        self.n = nx * ny * nz
        self._h = lib().ko_create(q, int(f64), nx, ny, nz, int(periodic_x))
        if not self._h:
            raise ValueError("oracle: bad lattice arguments")
        self._keep = []

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ko_destroy(self._h)
            self._h = None

    def set_flags(self, flags):
        a = np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1)
        assert a.size == self.n
        lib().ko_set_flags(self._h, _ptr(a))

    def set_profile(self, prof):
        a = np.ascontiguousarray(prof, dtype=np.float64)
        self._keep.append(a)
        lib().ko_set_profile(self._h, _ptr(a))

    def set_populations(self, aos):
        a = np.ascontiguousarray(aos, dtype=np.float64).reshape(-1)
        assert a.size == self.n * self.q
        lib().ko_set_populations(self._h, _ptr(a))

    def populations(self):
        out = np.empty(self.n * self.q, dtype=np.float64)
        lib().ko_get_populations(self._h, _ptr(out))
        return out.reshape(self.n, self.q)

    def set_porosity(self, v):
        a = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        lib().ko_set_porosity(self._h, _ptr(a))

    def set_force(self, v):
        a = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        lib().ko_set_force(self._h, _ptr(a))

    def macros(self):
        rho = np.empty(self.n, dtype=np.float64)
        vel = np.empty(self.n * self.D, dtype=np.float64)
        lib().ko_get_macros(self._h, _ptr(rho), _ptr(vel))
        return rho, vel.reshape(self.n, self.D)

    def run(self, program, steps):
        rc = lib().ko_run(self._h, C.byref(program), steps)
        if rc != 0:
            raise RuntimeError("oracle: program not supported for this descriptor")

    def run_rows(self, program, r0, r1):
        """One collide+stream pass over rows [r0, r1) only (timing sample)."""
        rc = lib().ko_run_rows(self._h, C.byref(program), r0, r1)
        if rc != 0:
            raise RuntimeError("oracle: program not supported for this descriptor")

    @property
    def t(self):
        return lib().ko_time_step(self._h)

    def porosity(self):
        out = np.empty(self.n, dtype=np.float64)
        lib().ko_get_porosity(self._h, _ptr(out))
        return out

    # ---- particle restatement (particles_oracle.c) -------------------------
    def particles_couple(self, states, params):
        lib().ko_particles_couple(self._h, C.byref(states), len(states), C.byref(params))

    def particles_gather(self, states, params, want_cell_force=False):
        cf = np.zeros(self.n * self.D, dtype=np.float64) if want_cell_force else None
        lib().ko_particles_gather(self._h, C.byref(states), len(states), C.byref(params),
                                  _ptr(cf) if cf is not None else None)
        return cf


    def fplbm_reset(self, plain_mask):
        """FpLbmReset on every cell; cells whose flag is in plain_mask (bit
        per flag value) get their density and momentum."""
        lib().ko_fplbm_reset(self._h, int(plain_mask))

    def fplbm_particles(self, states, params, own=False):
        """FpLbmOneParticle for every body (body 0's AABB and radius unless own)."""
        lib().ko_fplbm_particles(self._h, C.byref(states), len(states), C.byref(params), int(bool(own)))

    def force(self):
        out = np.empty(self.n * self.D, dtype=np.float64)
        lib().ko_get_force(self._h, _ptr(out))
        return out

    def hlbm_couple(self, states, params):
        lib().ko_particles_hlbm_couple(self._h, C.byref(states), len(states), C.byref(params))

    def hlbm_gather(self, states, params, want_cell_force=False):
        cf = np.zeros(self.n * self.D, dtype=np.float64) if want_cell_force else None
        lib().ko_particles_hlbm_gather(self._h, C.byref(states), len(states), C.byref(params),
                                       _ptr(cf) if cf is not None else None)
        return cf

    def hlbm_stamp(self, states, params):
        lib().ko_particles_hlbm_stamp(self._h, C.byref(states), len(states), C.byref(params))

    def hlbm_fields(self):
        N = np.empty(self.n * self.D, dtype=np.float64)
        Dv = np.empty(self.n, dtype=np.float64)
        lib().ko_get_hlbm(self._h, _ptr(N), _ptr(Dv))
        return N.reshape(self.n, self.D), Dv

    def set_hlbm_fields(self, N, Dv):
        N = np.ascontiguousarray(N, dtype=np.float64).reshape(-1)
        Dv = np.ascontiguousarray(Dv, dtype=np.float64)
        lib().ko_set_hlbm(self._h, _ptr(N), _ptr(Dv))


def particles_reset(states):
    lib().ko_particles_reset(C.byref(states), len(states))


def particles_contact(states, D, params, extent, periodic_x=False):
    ext = np.zeros(3, dtype=np.int64)
    ext[:len(extent)] = extent
    lib().ko_particles_contact(C.byref(states), len(states), D, C.byref(params), _ptr(ext), int(periodic_x))


def particles_integrate(states, D, params, extent, periodic_x=False):
    ext = np.zeros(3, dtype=np.int64)
    ext[:len(extent)] = extent
    lib().ko_particles_integrate(C.byref(states), len(states), D, C.byref(params), _ptr(ext), int(periodic_x))


def equilibrium_f32(q, rho, u):
    u3 = np.zeros(3, dtype=np.float32)
    u3[:len(u)] = u
    out = np.zeros(q, dtype=np.float32)
    lib().ko_equilibrium_f32(q, C.c_float(rho), _ptr(u3), _ptr(out))
    return out


# ---- voxel signed-distance bodies (voxel_oracle.c) ----------------------------

def voxel_states(bodies):
    """(n, 7) rows of position[3], rotation[3], radius -> kel_particle_state array."""
    from lbm_mirror_gb300 import capi as K
    b = np.asarray(bodies, dtype=np.float64).reshape(-1, 7)
    a = np.zeros((b.shape[0], 28))
    a[:, 0:3] = b[:, 0:3]
    a[:, 6:9] = b[:, 3:6]
    a[:, 26] = b[:, 6]
    return K.states_from_array(a)


def solid_fraction(sdf, eps):
    return lib().ko_solid_fraction(float(sdf), float(eps))


def mask_fill(D, R, kind):
    mask = np.zeros(R ** D)
    com = np.zeros(3)
    lib().ko_mask_fill(D, R, kind, _ptr(mask), _ptr(com))
    return mask, com


def mask_reach(D, R, mask):
    m = np.ascontiguousarray(mask, dtype=np.float64)
    return lib().ko_mask_reach(D, R, _ptr(m))


def mask_sample_local(D, R, mask, u):
    m = np.ascontiguousarray(mask, dtype=np.float64)
    u3 = np.zeros(3)
    u3[:D] = np.asarray(u)[:D]
    return lib().ko_mask_sample_local(D, R, _ptr(m), _ptr(u3))


def mask_local_to_global(D, state, com, u):
    c = np.ascontiguousarray(com, dtype=np.float64)
    u3 = np.zeros(3)
    u3[:D] = np.asarray(u)[:D]
    x = np.zeros(3)
    lib().ko_mask_local_to_global(D, C.byref(state), _ptr(c), _ptr(u3), _ptr(x))
    return x


def mask_signed_distance(D, R, mask, com, state, x):
    m = np.ascontiguousarray(mask, dtype=np.float64)
    c = np.ascontiguousarray(com, dtype=np.float64)
    x3 = np.zeros(3)
    x3[:D] = np.asarray(x)[:D]
    return lib().ko_mask_signed_distance(D, R, _ptr(m), _ptr(c), C.byref(state), _ptr(x3))


def voxel_porosity(D, R, mask, com, state, x, eps):
    m = np.ascontiguousarray(mask, dtype=np.float64)
    c = np.ascontiguousarray(com, dtype=np.float64)
    x3 = np.zeros(3)
    x3[:D] = np.asarray(x)[:D]
    return lib().ko_voxel_porosity(D, R, _ptr(m), _ptr(c), C.byref(state), _ptr(x3), float(eps))


def voxel_contact(D, R, mask, com, lo, hi, extent, eps):
    """Manifold of voxel_contact(lo, hi) as (hit, depth, normal[3], point[3])."""
    from lbm_mirror_gb300 import capi as K
    m = np.ascontiguousarray(mask, dtype=np.float64)
    c = np.ascontiguousarray(com, dtype=np.float64)
    ext = np.ones(3, dtype=np.int64)
    ext[:len(extent)] = extent
    out = K.ContactManifold()
    hit = lib().ko_voxel_contact(D, R, _ptr(m), _ptr(c), C.byref(lo), C.byref(hi), _ptr(ext), float(eps),
                                 C.byref(out))
    return np.array([float(hit), out.depth, *out.normal, *out.point])


def voxel_couple(D, R, mask, com, reach, states, extent, eps, periodic_x=False):
    """Porosity field (x fastest) of the FP32 voxel couple."""
    m = np.ascontiguousarray(mask, dtype=np.float64)
    c = np.ascontiguousarray(com, dtype=np.float64)
    ext = np.ones(3, dtype=np.int64)
    ext[:len(extent)] = extent
    por = np.zeros(int(np.prod(ext[:D])))
    lib().ko_voxel_couple(D, R, _ptr(m), _ptr(c), float(reach), C.byref(states), len(states), _ptr(ext),
                          int(periodic_x), float(eps), _ptr(por))
    return por


def particles_set_voxel_box(mul, add):
    """Box growth of the gather for KEL_POROSITY_VOXEL bodies (radius * mul + add)."""
    lib().ko_particles_set_voxel_box(float(mul), float(add))
