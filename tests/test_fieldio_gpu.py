"""Checkpoint / resume and the lattice's field output on the GPU.  A run
saved at step t (even or odd) and resumed in a fresh lattice continues with
the same bits as the uninterrupted run; the lattice's VTK / CSV / Forst
output equals the host writers' on its downloaded macros."""
import ctypes as C
import os

import numpy as np
import pytest

from lbm_mirror_gb300 import capi as K
from tests import cases
from tests.gpu_util import make_lattice, with_arith

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("t_save", [20, 21])
@pytest.mark.parametrize("storage", ["fp32", "fp16s"])
def test_save_load_resumes_bit_exact(tmp_path, t_save, storage):
    case = cases.mixed_2d(K.KEL_COLL_BGK_GUO, dims=(37, 19), steps=0, seed=4)
    prog = with_arith(case["program"], K.KEL_ARITH_FAST)
    a = make_lattice(case, storage)
    a.step(prog, t_save)
    p = os.path.join(tmp_path, "ck.forst")
    a.save(p)
    a.step(prog, 17)
    want = a.populations(np.float64)
    b = make_lattice(case, storage)
    b.load(p)
    assert b.t == t_save
    b.step(prog, 17)
    assert np.array_equal(b.populations(np.float64), want)
    a.close()
    b.close()


def test_write_fields_equals_host_writers(tmp_path):
    case = cases.cavity_3d(19, dims=(12, 10, 8), steps=0)
    lat = make_lattice(case)
    lat.step(case["program"], 30, write_macros=True)
    lat.write_fields(tmp_path / "gpu", "m", 30, K.KEL_WRITE_VTK | K.KEL_WRITE_CSV | K.KEL_WRITE_FORST)
    rho, u = lat.macros()
    lat.close()
    lib = K.load_library()
    dims = (C.c_int64 * 3)(12, 10, 8)
    u = np.ascontiguousarray(u, np.float32)
    rho = np.ascontiguousarray(rho, np.float32)
    fv = (K.FieldView * 2)()
    fv[0].name, fv[0].value_type, fv[0].components, fv[0].vector, fv[0].data = b"velocity", K.KEL_VALUE_F32, 3, 1, \
        u.ctypes.data
    fv[1].name, fv[1].value_type, fv[1].components, fv[1].data = b"density", K.KEL_VALUE_F32, 1, rho.ctypes.data
    host = str(tmp_path / "host").encode()
    assert lib.kel_write_vtk(host, b"m", 30, dims, 3, fv, 2) == 0
    assert lib.kel_write_csv(host, b"m", 30, dims, 3, fv, 2) == 0
    for f in ("vtk/m_30.vtk", "csv/m_velocity_30.csv", "csv/m_density_30.csv"):
        assert open(tmp_path / "gpu" / f, "rb").read() == open(tmp_path / "host" / f, "rb").read(), f
    raw = open(tmp_path / "gpu" / "forst" / "m_30.forst", "rb").read()
    assert raw == u.tobytes() + rho.tobytes()
