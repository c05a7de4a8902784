"""ctypes mirror of include/kel_lbm_cuda.h (the C ABI of the sweep).

Only plain-old-data types, constants and the library loader live here.  The
library is the in-tree build ``lbm_mirror_gb300/_build/libkel_lbm_cuda.so``;
if it is missing the import of the loader raises instead of falling back to
anything else.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libkel_lbm_cuda.so")

# ---- status codes --------------------------------------------------------
KEL_OK = 0
KEL_ERR_INVALID_ARGUMENT = -1
KEL_ERR_OUT_OF_MEMORY = -2
KEL_ERR_CUDA = -3
KEL_ERR_DEVICE_CHECK = -4
KEL_ERR_TIMEOUT = -5
KEL_ERR_UNSUPPORTED = -6
KEL_ERR_STATE = -7

# ---- descriptors / storage -----------------------------------------------
KEL_D2Q9, KEL_D3Q19, KEL_D3Q27 = 9, 19, 27
KEL_STORAGE_FP32, KEL_STORAGE_FP16S = 0, 1
KEL_LATTICE_PERIODIC_X = 1
# kel_lattice_set_launch: cells_per_thread value of the row pipeline (block_threads = row stages)
KEL_LAUNCH_ROWS = -1

# ---- boundary ops (values of kel_flag_op.bc) -------------------------------
KEL_BC_NONE = 0
KEL_BC_BOUNCE_BACK = 1
KEL_BC_FLUID = 2
KEL_BC_ZOUHE_VELOCITY_X = 3
KEL_BC_ZOUHE_PRESSURE_X = 4
KEL_BC_MOVING_WALL = 5
KEL_BC_ANTI_BOUNCE_BACK = 6
KEL_BC_EQUILIBRIUM = 7
KEL_BC_HALFWAY_WALL = 8

KEL_COLL_BGK, KEL_COLL_BGK_GUO, KEL_COLL_PSM, KEL_COLL_PSM_GUO, KEL_COLL_HLBM, KEL_COLL_FPLBM = 0, 1, 2, 3, 4, 5
KEL_ARITH_FAST, KEL_ARITH_REFERENCE, KEL_ARITH_SHIFTED = 0, 1, 2
KEL_MAX_FLAGS = 8

KEL_DTYPE_F32, KEL_DTYPE_F64 = 0, 1
KEL_LAYOUT_AOS, KEL_LAYOUT_SOA = 0, 1
KEL_FIELD_POROSITY, KEL_FIELD_FORCE, KEL_FIELD_HLBM_N, KEL_FIELD_HLBM_D = 1, 2, 3, 4
KEL_STEP_WRITE_MACROS, KEL_STEP_ALL_MACROS = 1, 2
KEL_UNET_CONV_TCGEN05, KEL_UNET_CONV_MMA_SYNC = 0, 1
KEL_VALUE_U8, KEL_VALUE_F32, KEL_VALUE_F64 = 0, 1, 2
KEL_PAINT_BOX, KEL_PAINT_SPHERE = 0, 1
KEL_WRITE_VTK, KEL_WRITE_CSV, KEL_WRITE_FORST = 1, 2, 4


class FlagOp(C.Structure):
    _fields_ = [
        ("bc", C.c_int32),
        ("collide", C.c_int32),
        ("east", C.c_int32),
        ("use_profile", C.c_int32),
        ("rho", C.c_double),
        ("u", C.c_double * 3),
    ]


class StepProgram(C.Structure):
    _fields_ = [
        ("collision", C.c_int32),
        ("arithmetic", C.c_int32),
        ("tau", C.c_double),
        ("global_force", C.c_double * 3),
        ("ops", FlagOp * KEL_MAX_FLAGS),
    ]


class LatticeDesc(C.Structure):
    _fields_ = [
        ("descriptor", C.c_int32),
        ("storage", C.c_int32),
        ("nx", C.c_int64),
        ("ny", C.c_int64),
        ("nz", C.c_int64),
        ("flags", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


def make_program(tau, collision=KEL_COLL_BGK, ops=None, global_force=(0.0, 0.0, 0.0),
                 arithmetic=KEL_ARITH_FAST):
    """Build a StepProgram.

    ``ops`` maps a flag value (0..7) to a dict with keys bc, collide, east,
    use_profile, rho, u -- the per-flag ``switch(info)`` of a reference driver.
    """
    p = StepProgram()
    p.collision = collision
    p.arithmetic = arithmetic
    p.tau = float(tau)
    for k in range(3):
        p.global_force[k] = float(global_force[k]) if k < len(global_force) else 0.0
    for flag, op in (ops or {}).items():
        o = p.ops[flag]
        o.bc = int(op.get("bc", KEL_BC_NONE))
        o.collide = int(op.get("collide", 0))
        o.east = int(op.get("east", 1))
        o.use_profile = int(op.get("use_profile", 0))
        o.rho = float(op.get("rho", 1.0))
        u = list(op.get("u", (0.0, 0.0, 0.0))) + [0.0, 0.0, 0.0]
        for k in range(3):
            o.u[k] = float(u[k])
    return p


def program_to_dict(p):
    """Plain-Python view of a StepProgram (for fixtures and logging)."""
    return {
        "collision": p.collision,
        "arithmetic": p.arithmetic,
        "tau": p.tau,
        "global_force": list(p.global_force),
        "ops": {
            i: {"bc": o.bc, "collide": o.collide, "east": o.east, "use_profile": o.use_profile,
                "rho": o.rho, "u": list(o.u)}
            for i, o in enumerate(p.ops) if o.bc != KEL_BC_NONE or o.collide
        },
    }


def program_from_dict(d):
    return make_program(d["tau"], d["collision"], {int(k): v for k, v in d["ops"].items()},
                        d["global_force"], d.get("arithmetic", KEL_ARITH_FAST))


KEL_POROSITY_RAMP, KEL_POROSITY_SUBCELL, KEL_POROSITY_VOXEL = 0, 1, 2
KEL_SHAPE_SPHERE, KEL_SHAPE_CUBE = 0, 1
KEL_COUPLING_PSM, KEL_COUPLING_HLBM, KEL_COUPLING_FPLBM, KEL_COUPLING_FPLBM_OWN = 0, 1, 2, 3


class ParticleState(C.Structure):
    """kel_particle_state: 28 doubles (particle/schema.hpp:51-115 + radius)."""
    _fields_ = [
        ("position", C.c_double * 3),
        ("position_old", C.c_double * 3),
        ("rotation", C.c_double * 3),
        ("rotation_old", C.c_double * 3),
        ("acceleration", C.c_double * 3),
        ("angular_acceleration", C.c_double * 3),
        ("force", C.c_double * 3),
        ("torque", C.c_double * 3),
        ("mass", C.c_double),
        ("inertia", C.c_double),
        ("radius", C.c_double),
        ("density", C.c_double),
    ]


class ParticleParams(C.Structure):
    _fields_ = [
        ("porosity_mode", C.c_int32),
        ("sub_steps", C.c_int32),
        ("eps", C.c_double),
        ("k_n", C.c_double),
        ("zeta_n", C.c_double),
        ("gamma_t", C.c_double),
        ("mu", C.c_double),
        ("body_acceleration", C.c_double * 3),
        ("wall_axes", C.c_uint32),
        ("coupling", C.c_int32),
    ]


class ContactManifold(C.Structure):
    """kel_contact_manifold (sch::ContactManifold, particle/contact.hpp:20-25, plus the hit flag)."""
    _fields_ = [
        ("hit", C.c_int32),
        ("pad", C.c_int32),
        ("normal", C.c_double * 3),
        ("point", C.c_double * 3),
        ("depth", C.c_double),
    ]


def make_particle_params(porosity_mode=KEL_POROSITY_RAMP, sub_steps=1, eps=1.5, k_n=1.0, zeta_n=0.3, gamma_t=0.0,
                         mu=0.0, body_acceleration=(0.0, 0.0, 0.0), wall_axes=0, coupling=KEL_COUPLING_PSM):
    p = ParticleParams()
    p.coupling = coupling
    p.porosity_mode, p.sub_steps, p.eps = porosity_mode, sub_steps, eps
    p.k_n, p.zeta_n, p.gamma_t, p.mu = k_n, zeta_n, gamma_t, mu
    for k in range(3):
        p.body_acceleration[k] = body_acceleration[k] if k < len(body_acceleration) else 0.0
    p.wall_axes = wall_axes
    return p


def states_to_array(states):
    """ctypes array of ParticleState -> (P, 28) float64 numpy array (copy)."""
    import numpy as np
    return np.frombuffer(bytes(states), dtype=np.float64).reshape(len(states), 28).copy()


def states_from_array(a):
    import numpy as np
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 28)
    arr = (ParticleState * a.shape[0])()
    C.memmove(arr, a.ctypes.data, a.nbytes)
    return arr


class UnetDesc(C.Structure):
    _fields_ = [("height", C.c_int32), ("width", C.c_int32), ("in_channels", C.c_int32),
                ("out_channels", C.c_int32), ("widths", C.c_int32 * 4), ("max_batch", C.c_int32),
                ("reserved", C.c_int32)]


class PaintOp(C.Structure):
    _fields_ = [("shape", C.c_int32), ("flag", C.c_int32), ("lo", C.c_int64 * 3), ("hi", C.c_int64 * 3),
                ("center", C.c_double * 3), ("radius", C.c_double)]


class FieldView(C.Structure):
    _fields_ = [("name", C.c_char_p), ("value_type", C.c_int32), ("components", C.c_int32), ("ghost", C.c_int32),
                ("vector", C.c_int32), ("data", C.c_void_p)]


class ChannelDesc(C.Structure):
    _fields_ = [("nx", C.c_int64), ("ny", C.c_int64), ("tau", C.c_double), ("u_max", C.c_double)]


_lib = None


def load_library(path: str | None = None):
    """Load the CUDA library and declare its signatures.  Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"CUDA extension not built: {p} is missing (run __graft_entry__.build() "
            "or python -m lbm_mirror_gb300.build)")
    lib = C.CDLL(p)
    vp, i32, i64, u32, u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64
    sigs = {
        "kel_lattice_create": ([C.POINTER(LatticeDesc), C.POINTER(vp)], C.c_int),
        "kel_lattice_destroy": ([vp], C.c_int),
        "kel_lattice_set_stream": ([vp, vp], C.c_int),
        "kel_lattice_time_step": ([vp, C.POINTER(u64)], C.c_int),
        "kel_upload_flags": ([vp, vp], C.c_int),
        "kel_upload_populations": ([vp, vp, i32, i32], C.c_int),
        "kel_download_populations": ([vp, vp, i32, i32], C.c_int),
        "kel_download_macros": ([vp, vp, vp], C.c_int),
        "kel_upload_field": ([vp, i32, vp], C.c_int),
        "kel_download_field": ([vp, i32, vp], C.c_int),
        "kel_upload_inlet_profile": ([vp, vp, i64], C.c_int),
        "kel_step": ([vp, C.POINTER(StepProgram), u64, u32], C.c_int),
        "kel_lattice_synchronize": ([vp], C.c_int),
        "kel_lattice_set_launch": ([vp, i32, i32], C.c_int),
        "kel_batch_create": ([i32, C.POINTER(ChannelDesc), i32, C.POINTER(vp)], C.c_int),
        "kel_velocity_residual_noalloc": ([vp, vp, i64, i32, vp, vp], C.c_int),
        "kel_unet_create": ([C.POINTER(UnetDesc), u64, C.POINTER(vp)], C.c_int),
        "kel_unet_destroy": ([vp], C.c_int),
        "kel_unet_param_count": ([vp, C.POINTER(i64)], C.c_int),
        "kel_unet_get_params": ([vp, vp], C.c_int),
        "kel_unet_set_params": ([vp, vp], C.c_int),
        "kel_unet_get_grads": ([vp, vp], C.c_int),
        "kel_unet_set_stream": ([vp, vp], C.c_int),
        "kel_unet_synchronize": ([vp], C.c_int),
        "kel_unet_make_input": ([vp, vp, vp, vp, i32], C.c_int),
        "kel_unet_set_input": ([vp, vp, i32], C.c_int),
        "kel_unet_get_input": ([vp, vp, i32], C.c_int),
        "kel_unet_forward": ([vp, i32, vp], C.c_int),
        "kel_unet_backward": ([vp, vp, i32, C.POINTER(C.c_double)], C.c_int),
        "kel_unet_adam_step": ([vp, C.c_float, C.c_float, C.c_float, C.c_float, i32], C.c_int),
        "kel_unet_train_step": ([vp, vp, i32, C.c_float, C.c_float, C.c_float, C.c_float, i32, vp], C.c_int),
        "kel_unet_last_loss": ([vp, C.POINTER(C.c_double)], C.c_int),
        "kel_unet_set_conv_kernel": ([vp, i32], C.c_int),
        "kel_unet_set_residual": ([vp, i32, i32, C.c_float], C.c_int),
        "kel_batch_destroy": ([vp], C.c_int),
        "kel_batch_upload_flags": ([vp, vp], C.c_int),
        "kel_batch_set_program": ([vp, C.POINTER(StepProgram)], C.c_int),
        "kel_batch_autotune": ([vp, i32, C.POINTER(i32), C.POINTER(C.c_float)], C.c_int),
        "kel_batch_step": ([vp, u64], C.c_int),
        "kel_batch_run_until": ([vp, C.c_double, u64, u64, i32, vp, vp], C.c_int),
        "kel_batch_active_count": ([vp, C.POINTER(i32)], C.c_int),
        "kel_batch_channel_time_step": ([vp, i32, C.POINTER(u64)], C.c_int),
        "kel_batch_info": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i32)], C.c_int),
        "kel_batch_download_populations": ([vp, i32, vp], C.c_int),
        "kel_batch_download_macros": ([vp, i32, vp], C.c_int),
        "kel_batch_warm_start": ([vp, i32, i32, vp, i64, vp, vp, i32], C.c_int),
        "kel_batch_warm_refine": ([vp, i32, i32, vp, i64, vp, vp, i32, i32], C.c_int),
        "kel_batch_synchronize": ([vp], C.c_int),
        "kel_write_vtk": ([C.c_char_p, C.c_char_p, u64, C.POINTER(i64), i32, C.POINTER(FieldView), i32], C.c_int),
        "kel_write_csv": ([C.c_char_p, C.c_char_p, u64, C.POINTER(i64), i32, C.POINTER(FieldView), i32], C.c_int),
        "kel_write_forst": ([C.c_char_p, C.POINTER(i64), i32, C.POINTER(FieldView), i32], C.c_int),
        "kel_read_forst": ([C.c_char_p, C.POINTER(i64), i32, C.POINTER(FieldView), i32], C.c_int),
        "kel_lattice_write_fields": ([vp, i32, C.c_char_p, C.c_char_p, u64], C.c_int),
        "kel_lattice_save": ([vp, C.c_char_p], C.c_int),
        "kel_lattice_load": ([vp, C.c_char_p], C.c_int),
        "kel_lattice_paint": ([vp, C.POINTER(PaintOp), i32], C.c_int),
        "kel_download_flags": ([vp, vp], C.c_int),
        "kel_lattice_init_equilibrium": ([vp, vp, vp, C.c_double, C.POINTER(C.c_double)], C.c_int),
        "kel_particles_stamp": ([vp, C.POINTER(ParticleParams)], C.c_int),
        "kel_lattice_get_launch": ([vp, C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "kel_lattice_autotune": ([vp, C.POINTER(StepProgram), i32, C.POINTER(i32), C.POINTER(i32),
                                  C.POINTER(C.c_float)], C.c_int),
        "kel_particles_create": ([vp, i32, C.POINTER(vp)], C.c_int),
        "kel_particles_destroy": ([vp], C.c_int),
        "kel_particles_upload": ([vp, vp], C.c_int),
        "kel_particles_download": ([vp, vp], C.c_int),
        "kel_particles_reset": ([vp], C.c_int),
        "kel_particles_couple": ([vp, C.POINTER(ParticleParams)], C.c_int),
        "kel_particles_gather": ([vp, C.POINTER(ParticleParams), vp], C.c_int),
        "kel_particles_contact": ([vp, C.POINTER(ParticleParams)], C.c_int),
        "kel_particles_integrate": ([vp, C.POINTER(ParticleParams)], C.c_int),
        "kel_particles_step": ([vp, C.POINTER(ParticleParams), C.POINTER(StepProgram), u64, u32], C.c_int),
        "kel_shape_create": ([i32, i32, i32, C.POINTER(vp)], C.c_int),
        "kel_shape_create_from_mask": ([i32, i32, vp, vp, C.POINTER(vp)], C.c_int),
        "kel_shape_info": ([vp, vp, vp, vp], C.c_int),
        "kel_shape_destroy": ([vp], C.c_int),
        "kel_particles_set_shape": ([vp, vp], C.c_int),
        "kel_particles_voxel_distance": ([vp, i32, vp, i32, vp], C.c_int),
        "kel_particles_voxel_contact": ([vp, vp, i32, C.c_double, vp], C.c_int),
        "kel_last_error_string": ([], C.c_char_p),
        "kel_version": ([], C.c_char_p),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def header_symbols(header_path: str | None = None):
    """Names of every function declared in include/kel_lbm_cuda.h."""
    import re
    hp = header_path or os.path.join(os.path.dirname(HERE), "include", "kel_lbm_cuda.h")
    text = open(hp).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(kel_[a-z_0-9]+)\s*\(", text, flags=re.M)))
