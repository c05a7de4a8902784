"""Python host mirror of the reference's lattice/component interface.

A reference driver builds components (``component<T,Desc,cmpt::BGK>{tau}``,
``cmpt::BounceBack``, ``cmpt::ZouHeVelocityX<true>{u}``, ...) and applies
them per cell through ``switch(info)`` (e.g.
examples/poiseulle_2d_gpu/poiseulle_2d_gpu.cpp:169-224).  Here the same
components are plain descriptions; ``program_from_switch`` lowers a
``{flag: [components]}`` switch into the C ABI's kel_step_program and a
``Lattice`` runs it on the GPU through libkel_lbm_cuda.so.  There is no CPU
path: constructing a Lattice without the built library raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import capi as K

DESCRIPTORS = {"D2Q9": K.KEL_D2Q9, "D3Q19": K.KEL_D3Q19, "D3Q27": K.KEL_D3Q27}


class KelError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{msg} (status {code})")
        self.code = code


def _check(rc, lib):
    if rc != K.KEL_OK:
        raise KelError(rc, lib.kel_last_error_string().decode())


# ---- components (parameter carriers, reference spellings) -------------------
@dataclass
class BGK:
    """cmpt::BGK (collision.hpp:19-97)."""
    tau: float
    collision = K.KEL_COLL_BGK


@dataclass
class BGKGuo:
    """cmpt::BGKGuo (collision.hpp:99-205); adds the cell "force" field."""
    tau: float
    global_force: tuple = (0.0, 0.0, 0.0)
    collision = K.KEL_COLL_BGK_GUO


@dataclass
class Psm:
    """cmpt::Psm (psm.hpp:37-90); reads the cell "porosity" field."""
    tau: float
    collision = K.KEL_COLL_PSM


@dataclass
class PsmGuo:
    """cmpt::Psm followed by the BGKGuo forcing term (no reference component)."""
    tau: float
    global_force: tuple = (0.0, 0.0, 0.0)
    collision = K.KEL_COLL_PSM_GUO


@dataclass
class BounceBack:
    """cmpt::BounceBack, full-way (boundary.hpp:32-76)."""
    bc = K.KEL_BC_BOUNCE_BACK


@dataclass
class AntiBounceBack:
    """cmpt::AntiBounceBack<0>, D2Q9 (boundary.hpp:81-133)."""
    bc = K.KEL_BC_ANTI_BOUNCE_BACK


@dataclass
class Equilibrium:
    """cmpt::Equilibrium(rho, u) (boundary.hpp:135-161)."""
    rho: float
    u: tuple
    bc = K.KEL_BC_EQUILIBRIUM


@dataclass
class ZouHePressureX:
    """cmpt::ZouHePressureX<East>(rho) (boundary.hpp:175-756)."""
    east: bool
    rho: float
    bc = K.KEL_BC_ZOUHE_PRESSURE_X


@dataclass
class ZouHeVelocityX:
    """cmpt::ZouHeVelocityX<East>(u) (boundary.hpp:759-805); ``u`` may be
    "profile" to take u_x(y) from the uploaded inlet profile."""
    east: bool
    u: object
    bc = K.KEL_BC_ZOUHE_VELOCITY_X


@dataclass
class MovingWall:
    """Lid: f_i = f_opp + 2 w_i (c_i.u_w)/cs^2 (cavity_2d_gpu.cpp:204-235)."""
    u: tuple
    bc = K.KEL_BC_MOVING_WALL


def program_from_switch(switch, arithmetic=K.KEL_ARITH_FAST):
    """Lower ``{flag: [boundary?, collision?]}`` into a StepProgram.

    Every collision in the switch must be the same operator (one per step, as
    in every reference driver)."""
    coll = None
    ops = {}
    for flag, comps in switch.items():
        if not 0 < flag < K.KEL_MAX_FLAGS:
            raise ValueError(f"flag {flag} out of range 1..{K.KEL_MAX_FLAGS - 1}")
        op = dict(bc=K.KEL_BC_FLUID, collide=0)
        for c in comps:
            if hasattr(c, "collision"):
                if coll is not None and (type(c) is not type(coll) or c != coll):
                    raise ValueError("one collision operator per program")
                coll = c
                op["collide"] = 1
            else:
                op["bc"] = c.bc
                if isinstance(c, (ZouHePressureX, ZouHeVelocityX)):
                    op["east"] = int(c.east)
                if isinstance(c, (ZouHePressureX, Equilibrium)):
                    op["rho"] = c.rho
                if isinstance(c, ZouHeVelocityX):
                    if isinstance(c.u, str):
                        op["use_profile"] = 1
                    else:
                        op["u"] = tuple(c.u)
                if isinstance(c, (MovingWall, Equilibrium)):
                    op["u"] = tuple(c.u)
        ops[flag] = op
    if coll is None:
        coll = BGK(1.0)
    return K.make_program(coll.tau, coll.collision, ops, getattr(coll, "global_force", (0.0, 0.0, 0.0)),
                          arithmetic)


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


class Lattice:
    """One lattice in HBM (structure of arrays, AA in-place), driven through
    the C ABI.  ``dims`` = (nx, ny) for D2Q9, (nx, ny, nz) for D3Q*."""

    def __init__(self, descriptor, dims, storage="fp32", periodic_x=False, stream=None):
        self.lib = K.load_library()
        q = DESCRIPTORS[descriptor] if isinstance(descriptor, str) else int(descriptor)
        self.q = q
        self.D = 2 if q == K.KEL_D2Q9 else 3
        nx, ny = int(dims[0]), int(dims[1])
        nz = int(dims[2]) if len(dims) > 2 else 1
        self.dims = (nx, ny, nz)
        self.n = nx * ny * nz
        d = K.LatticeDesc()
        d.descriptor = q
        d.storage = {"fp32": K.KEL_STORAGE_FP32, "fp16s": K.KEL_STORAGE_FP16S}[storage]
        d.nx, d.ny, d.nz = nx, ny, nz
        d.flags = K.KEL_LATTICE_PERIODIC_X if periodic_x else 0
        h = C.c_void_p()
        _check(self.lib.kel_lattice_create(C.byref(d), C.byref(h)), self.lib)
        self._h = h
        if stream is not None:
            self.set_stream(stream)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.kel_lattice_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_handle: int):
        _check(self.lib.kel_lattice_set_stream(self._h, C.c_void_p(stream_handle)), self.lib)

    @property
    def t(self):
        v = C.c_uint64()
        _check(self.lib.kel_lattice_time_step(self._h, C.byref(v)), self.lib)
        return v.value

    def upload_flags(self, flags):
        a = np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1)
        if a.size != self.n:
            raise ValueError("flags: wrong size")
        _check(self.lib.kel_upload_flags(self._h, _ptr(a)), self.lib)

    def upload_populations(self, f, layout="aos"):
        a = np.ascontiguousarray(f)
        if a.dtype not in (np.float32, np.float64):
            a = a.astype(np.float64)
        if a.size != self.n * self.q:
            raise ValueError("populations: wrong size")
        dt = K.KEL_DTYPE_F32 if a.dtype == np.float32 else K.KEL_DTYPE_F64
        lay = K.KEL_LAYOUT_AOS if layout == "aos" else K.KEL_LAYOUT_SOA
        _check(self.lib.kel_upload_populations(self._h, _ptr(a), dt, lay), self.lib)

    def populations(self, dtype=np.float32, layout="aos"):
        out = np.empty(self.n * self.q, dtype=dtype)
        dt = K.KEL_DTYPE_F32 if out.dtype == np.float32 else K.KEL_DTYPE_F64
        lay = K.KEL_LAYOUT_AOS if layout == "aos" else K.KEL_LAYOUT_SOA
        _check(self.lib.kel_download_populations(self._h, _ptr(out), dt, lay), self.lib)
        return out.reshape(self.n, self.q) if layout == "aos" else out.reshape(self.q, self.n)

    def macros(self):
        rho = np.empty(self.n, dtype=np.float32)
        u = np.empty(self.n * self.D, dtype=np.float32)
        _check(self.lib.kel_download_macros(self._h, _ptr(rho), _ptr(u)), self.lib)
        return rho, u.reshape(self.n, self.D)

    def upload_porosity(self, por):
        a = np.ascontiguousarray(por, dtype=np.float32).reshape(-1)
        _check(self.lib.kel_upload_field(self._h, K.KEL_FIELD_POROSITY, _ptr(a)), self.lib)

    def upload_force(self, force):
        a = np.ascontiguousarray(force, dtype=np.float32).reshape(-1)
        _check(self.lib.kel_upload_field(self._h, K.KEL_FIELD_FORCE, _ptr(a)), self.lib)

    def download_field(self, field_id, comps):
        out = np.empty(self.n * comps, dtype=np.float32)
        _check(self.lib.kel_download_field(self._h, field_id, _ptr(out)), self.lib)
        return out

    def upload_inlet_profile(self, ux):
        a = np.ascontiguousarray(ux, dtype=np.float64)
        _check(self.lib.kel_upload_inlet_profile(self._h, _ptr(a), a.size), self.lib)

    def step(self, program, n_steps=1, write_macros=True, all_macros=False):
        fl = (K.KEL_STEP_WRITE_MACROS if write_macros else 0) | (K.KEL_STEP_ALL_MACROS if all_macros else 0)
        _check(self.lib.kel_step(self._h, C.byref(program), n_steps, fl), self.lib)

    def paint(self, ops):
        """Flag painting on the device: ops are dicts with shape ("box" or
        "sphere"), flag, lo, hi (cell bounds, lo <= x < hi) and, for spheres,
        center and radius; applied in order."""
        arr = (K.PaintOp * len(ops))()
        for a, o in zip(arr, ops):
            a.shape = K.KEL_PAINT_SPHERE if o.get("shape", "box") == "sphere" else K.KEL_PAINT_BOX
            a.flag = int(o["flag"])
            big = 1 << 40
            lo = list(o.get("lo", (0, 0, 0))) + [0] * 3
            hi = list(o.get("hi", (big, big, big))) + [big] * 3
            for d in range(3):
                a.lo[d], a.hi[d] = int(lo[d]), int(hi[d])
            c = list(o.get("center", (0.0, 0.0, 0.0))) + [0.0] * 3
            for d in range(3):
                a.center[d] = float(c[d])
            a.radius = float(o.get("radius", 0.0))
        _check(self.lib.kel_lattice_paint(self._h, arr, len(ops)), self.lib)

    def flags(self):
        out = np.empty(self.n, dtype=np.uint8)
        _check(self.lib.kel_download_flags(self._h, _ptr(out)), self.lib)
        return out

    def init_equilibrium(self, rho=1.0, u=(0.0, 0.0, 0.0), d_rho=None, d_u=None):
        """Populations = equilibrium(rho, u) on the device (reference rounding);
        d_rho / d_u: optional device pointers to per-cell fields."""
        u3 = (C.c_double * 3)(*(list(u) + [0.0] * 3)[:3])
        _check(self.lib.kel_lattice_init_equilibrium(self._h, C.c_void_p(d_rho) if d_rho else None,
                                                     C.c_void_p(d_u) if d_u else None, float(rho), u3), self.lib)

    def write_fields(self, out_dir, file_name, t, formats=K.KEL_WRITE_VTK):
        """The macro output (velocity, density) as the reference's VTK / CSV /
        Forst files under out_dir (kel_lattice_write_fields)."""
        _check(self.lib.kel_lattice_write_fields(self._h, int(formats), str(out_dir).encode(),
                                                 str(file_name).encode(), int(t)), self.lib)

    def save(self, path):
        """Checkpoint (Forst: time step, flags, populations)."""
        _check(self.lib.kel_lattice_save(self._h, str(path).encode()), self.lib)

    def load(self, path):
        """Restore a checkpoint written by save() (same descriptor and extents)."""
        _check(self.lib.kel_lattice_load(self._h, str(path).encode()), self.lib)

    def set_launch(self, cells_per_thread, block_threads=256):
        """Sweep launch shape: (1, 2 or 4 cells per thread, 64/128/256 threads per
        block), or (KEL_LAUNCH_ROWS, row stages 2-6) for the row pipeline."""
        _check(self.lib.kel_lattice_set_launch(self._h, cells_per_thread, block_threads), self.lib)

    def autotune(self, program, steps=6):
        """Time every launch shape on the current state (restored after each
        trial) and keep the fastest; returns (cells_per_thread, block, ms)."""
        a, b, ms = C.c_int32(), C.c_int32(), C.c_float()
        _check(self.lib.kel_lattice_autotune(self._h, C.byref(program), steps, C.byref(a), C.byref(b), C.byref(ms)),
               self.lib)
        return a.value, b.value, ms.value

    def launch(self):
        a, b = C.c_int32(), C.c_int32()
        _check(self.lib.kel_lattice_get_launch(self._h, C.byref(a), C.byref(b)), self.lib)
        return a.value, b.value

    def synchronize(self):
        _check(self.lib.kel_lattice_synchronize(self._h), self.lib)


class Particles:
    """Rigid spheres/discs on a Lattice (C ABI kel_particles_*): PSM porosity
    couple, FP64 momentum-exchange force/torque gather, DEM contact and
    position-Verlet integration -- the per-particle components of the
    reference (psm.hpp, particle/contact.hpp, particle/integrate.hpp)."""

    def __init__(self, lattice: Lattice, states):
        self.lat = lattice
        self.lib = lattice.lib
        self.n = len(states)
        h = C.c_void_p()
        _check(self.lib.kel_particles_create(lattice.handle, self.n, C.byref(h)), self.lib)
        self._h = h
        self.upload(states)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.kel_particles_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, states):
        arr = states if isinstance(states, C.Array) else K.states_from_array(states)
        _check(self.lib.kel_particles_upload(self._h, arr), self.lib)

    def download(self):
        arr = (K.ParticleState * self.n)()
        _check(self.lib.kel_particles_download(self._h, arr), self.lib)
        return K.states_to_array(arr)

    def reset(self):
        _check(self.lib.kel_particles_reset(self._h), self.lib)

    def couple(self, params):
        _check(self.lib.kel_particles_couple(self._h, C.byref(params)), self.lib)

    def gather(self, params, cell_force=False):
        out = np.empty(self.lat.n * self.lat.D, dtype=np.float32) if cell_force else None
        _check(self.lib.kel_particles_gather(self._h, C.byref(params), _ptr(out) if out is not None else None),
               self.lib)
        return out

    def contact(self, params):
        _check(self.lib.kel_particles_contact(self._h, C.byref(params)), self.lib)

    def stamp(self, params):
        """HLBM coupling: the particle_N / particle_D accumulators (after integrate)."""
        _check(self.lib.kel_particles_stamp(self._h, C.byref(params)), self.lib)

    def integrate(self, params):
        _check(self.lib.kel_particles_integrate(self._h, C.byref(params)), self.lib)

    def step(self, params, program, n_steps=1, write_macros=True):
        fl = K.KEL_STEP_WRITE_MACROS if write_macros else 0
        _check(self.lib.kel_particles_step(self._h, C.byref(params), C.byref(program), n_steps, fl), self.lib)

    def set_shape(self, shape):
        """The voxel shape every body takes (KEL_POROSITY_VOXEL, voxel queries); None detaches."""
        self._shape = shape
        _check(self.lib.kel_particles_set_shape(self._h, shape.handle if shape is not None else None), self.lib)

    def voxel_distance(self, body, points):
        """mask_signed_distance (particle/mask.hpp:270-282) of one body at lattice points, FP64 on the device."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, self.lat.D)
        out = np.empty(pts.shape[0])
        _check(self.lib.kel_particles_voxel_distance(self._h, int(body), _ptr(pts), pts.shape[0], _ptr(out)), self.lib)
        return out

    def voxel_contact(self, pairs, eps):
        """voxel_contact (particle/voxel_narrow.hpp:78-259) of body pairs (lo, hi), FP64 on the device.
        Returns (n, 8): hit, depth, normal[3], point[3]."""
        pr = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        out = (K.ContactManifold * pr.shape[0])()
        _check(self.lib.kel_particles_voxel_contact(self._h, _ptr(pr), pr.shape[0], float(eps), out), self.lib)
        return np.array([[m.hit, m.depth, *m.normal, *m.point] for m in out], dtype=np.float64).reshape(-1, 8)


class Shape:
    """A voxel signed-distance body shape (C ABI kel_shape_*; particle/mask.hpp):
    ``Shape(dim, resolution, kind)`` fills a built-in sphere or cube mask
    (fill_mask_from_sdf); ``Shape.from_mask(dim, resolution, mask, com)`` takes
    a caller's R^D mask (last axis fastest)."""

    def __init__(self, dim, resolution, kind=K.KEL_SHAPE_SPHERE, _mask=None, _com=None):
        self.lib = K.load_library()
        self.dim, self.resolution = int(dim), int(resolution)
        h = C.c_void_p()
        if _mask is None:
            _check(self.lib.kel_shape_create(self.dim, self.resolution, int(kind), C.byref(h)), self.lib)
        else:
            m = np.ascontiguousarray(_mask, dtype=np.float64).reshape(-1)
            c = np.zeros(3)
            c[:len(_com)] = _com
            _check(self.lib.kel_shape_create_from_mask(self.dim, self.resolution, _ptr(m), _ptr(c), C.byref(h)),
                   self.lib)
        self._h = h

    @classmethod
    def from_mask(cls, dim, resolution, mask, com):
        return cls(dim, resolution, _mask=mask, _com=np.asarray(com, dtype=np.float64)[:dim])

    @property
    def handle(self):
        return self._h

    def info(self):
        """(mask (R^D doubles), center of mass (3), reach)."""
        mask = np.empty(self.resolution ** self.dim)
        com = np.empty(3)
        reach = C.c_double()
        _check(self.lib.kel_shape_info(self._h, _ptr(mask), _ptr(com), C.byref(reach)), self.lib)
        return mask, com, reach.value

    def close(self):
        if getattr(self, "_h", None):
            self.lib.kel_shape_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent D2Q9 channels of uneven size in one launch
    (C ABI kel_batch_*).  ``channels``: dicts with nx, ny, tau, u_max, flags."""

    def __init__(self, channels, program, tile=0):
        self.lib = K.load_library()
        self.n = len(channels)
        arr = (K.ChannelDesc * self.n)()
        for a, c in zip(arr, channels):
            a.nx, a.ny, a.tau, a.u_max = int(c["nx"]), int(c["ny"]), float(c["tau"]), float(c["u_max"])
        h = C.c_void_p()
        _check(self.lib.kel_batch_create(self.n, arr, int(tile), C.byref(h)), self.lib)
        self._h = h
        self.dims = [(int(c["nx"]), int(c["ny"])) for c in channels]
        packed = np.concatenate([np.ascontiguousarray(c["flags"], dtype=np.uint8).reshape(-1) for c in channels])
        _check(self.lib.kel_batch_upload_flags(self._h, _ptr(packed)), self.lib)
        _check(self.lib.kel_batch_set_program(self._h, C.byref(program)), self.lib)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.kel_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def autotune(self, steps=6):
        t, ms = C.c_int32(), C.c_float()
        _check(self.lib.kel_batch_autotune(self._h, steps, C.byref(t), C.byref(ms)), self.lib)
        return t.value, ms.value

    def step(self, n=1):
        _check(self.lib.kel_batch_step(self._h, n), self.lib)

    def run_until(self, tol=1e-6, check_every=1000, max_steps=10**7, use_graph=True):
        steps = np.zeros(self.n, dtype=np.uint64)
        res = np.zeros(self.n, dtype=np.float64)
        _check(self.lib.kel_batch_run_until(self._h, tol, check_every, max_steps, int(use_graph), _ptr(steps),
                                            _ptr(res)), self.lib)
        return steps, res

    def active_count(self):
        v = C.c_int32()
        _check(self.lib.kel_batch_active_count(self._h, C.byref(v)), self.lib)
        return v.value

    def info(self):
        a, b, t = C.c_int64(), C.c_int64(), C.c_int32()
        _check(self.lib.kel_batch_info(self._h, C.byref(a), C.byref(b), C.byref(t)), self.lib)
        return a.value, b.value, t.value

    def time_step(self, channel):
        v = C.c_uint64()
        _check(self.lib.kel_batch_channel_time_step(self._h, channel, C.byref(v)), self.lib)
        return v.value

    def populations(self, channel):
        nx, ny = self.dims[channel]
        out = np.empty(nx * ny * 9, dtype=np.float32)
        _check(self.lib.kel_batch_download_populations(self._h, channel, _ptr(out)), self.lib)
        return out.reshape(nx * ny, 9)

    def macros(self, channel):
        nx, ny = self.dims[channel]
        out = np.empty(nx * ny * 3, dtype=np.float32)
        _check(self.lib.kel_batch_download_macros(self._h, channel, _ptr(out)), self.lib)
        out = out.reshape(nx * ny, 3)
        return out[:, 0].copy(), out[:, 1:3].copy()

    def warm_start(self, first, count, d_pred, pred_stride, d_scale, d_offset, with_neq=True):
        """Populations of channels [first, first + count) from a predicted
        (u_x, u_y, rho) field (device pointers; see kel_batch_warm_start)."""
        _check(self.lib.kel_batch_warm_start(self._h, int(first), int(count), C.c_void_p(d_pred), int(pred_stride),
                                             C.c_void_p(d_scale), C.c_void_p(d_offset), int(bool(with_neq))),
               self.lib)

    def warm_refine(self, first, count, d_pred, pred_stride, d_scale, d_offset, iterations, keep_rho=False):
        """Refinement after warm_start (see kel_batch_warm_refine): `iterations`
        times two sweeps, then the predicted field is put back while the
        non-equilibrium part the sweeps produced is kept."""
        _check(self.lib.kel_batch_warm_refine(self._h, int(first), int(count), C.c_void_p(d_pred), int(pred_stride),
                                              C.c_void_p(d_scale), C.c_void_p(d_offset), int(iterations),
                                              int(bool(keep_rho))), self.lib)

    def synchronize(self):
        _check(self.lib.kel_batch_synchronize(self._h), self.lib)


class UNet:
    """The warm-start U-Net (C ABI kel_unet_*): bf16 tensor-core convolutions,
    FP32 accumulate, FP32 master weights and Adam.  Device buffers passed in
    are raw device pointers (e.g. torch tensors' data_ptr())."""

    def __init__(self, height=64, width=256, widths=(32, 64, 128, 128), out_channels=3, max_batch=32, seed=1):
        self.lib = K.load_library()
        d = K.UnetDesc()
        d.height, d.width, d.in_channels, d.out_channels = height, width, 16, out_channels
        for i in range(4):
            d.widths[i] = widths[i]
        d.max_batch = max_batch
        h = C.c_void_p()
        _check(self.lib.kel_unet_create(C.byref(d), seed, C.byref(h)), self.lib)
        self._h = h
        self.shape = (height, width, out_channels)
        self.widths = tuple(widths)
        self.max_batch = max_batch
        n = C.c_int64()
        _check(self.lib.kel_unet_param_count(self._h, C.byref(n)), self.lib)
        self.n_params = n.value
        self.step_count = 0

    def close(self):
        if getattr(self, "_h", None):
            self.lib.kel_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        out = np.empty(self.n_params, dtype=np.float32)
        _check(self.lib.kel_unet_get_params(self._h, _ptr(out)), self.lib)
        return out

    def set_params(self, p):
        a = np.ascontiguousarray(p, dtype=np.float32)
        _check(self.lib.kel_unet_set_params(self._h, _ptr(a)), self.lib)

    def grads(self):
        out = np.empty(self.n_params, dtype=np.float32)
        _check(self.lib.kel_unet_get_grads(self._h, _ptr(out)), self.lib)
        return out

    def set_conv_kernel(self, kind):
        """K.KEL_UNET_CONV_TCGEN05 (default) or K.KEL_UNET_CONV_MMA_SYNC."""
        _check(self.lib.kel_unet_set_conv_kernel(self._h, int(kind)), self.lib)

    def set_residual(self, out_channel, in_channel=0, scale=1.0):
        """Output channel out_channel = head + scale * input plane in_channel
        (out_channel < 0: off)."""
        _check(self.lib.kel_unet_set_residual(self._h, int(out_channel), int(in_channel), float(scale)), self.lib)

    def set_stream(self, stream):
        _check(self.lib.kel_unet_set_stream(self._h, C.c_void_p(stream)), self.lib)

    def synchronize(self):
        _check(self.lib.kel_unet_synchronize(self._h), self.lib)

    def make_input(self, d_mask, d_umax, d_tau, n):
        _check(self.lib.kel_unet_make_input(self._h, C.c_void_p(d_mask), C.c_void_p(d_umax), C.c_void_p(d_tau), n),
               self.lib)

    def get_input(self, d_out_bf16, n):
        _check(self.lib.kel_unet_get_input(self._h, C.c_void_p(d_out_bf16), n), self.lib)

    def set_input(self, d_input_bf16, n):
        _check(self.lib.kel_unet_set_input(self._h, C.c_void_p(d_input_bf16), n), self.lib)

    def forward(self, n, d_out=None):
        _check(self.lib.kel_unet_forward(self._h, n, C.c_void_p(d_out) if d_out else None), self.lib)

    def backward(self, d_target, n):
        loss = C.c_double()
        _check(self.lib.kel_unet_backward(self._h, C.c_void_p(d_target), n, C.byref(loss)), self.lib)
        return loss.value

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        _check(self.lib.kel_unet_adam_step(self._h, lr, beta1, beta2, eps, self.step_count), self.lib)

    def train_step(self, d_target, n, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        """forward + backward + Adam in one call without a host synchronisation,
        replayed as a captured CUDA graph (kel_unet_train_step); the loss stays
        on the device (last_loss reads it)."""
        self.step_count += 1
        _check(self.lib.kel_unet_train_step(self._h, C.c_void_p(d_target), n, lr, beta1, beta2, eps,
                                            self.step_count, None), self.lib)

    def last_loss(self):
        loss = C.c_double()
        _check(self.lib.kel_unet_last_loss(self._h, C.byref(loss)), self.lib)
        return loss.value
