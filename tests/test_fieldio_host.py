"""Field writers (C ABI kel_write_vtk / kel_write_csv / kel_write_forst /
kel_read_forst) byte for byte against the reference's own writers run on the
same values (tests/golden/writers_*.npz from oracle/_ref/ref_harness:
write_vtk.hpp, write_csv.hpp, abstract/forst.hpp + forst_chunk.hpp).  Host
code only: no GPU needed."""
import ctypes as C
import os

import numpy as np
import pytest

from lbm_mirror_gb300 import capi as K

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = {"writers_d2q9_f32_12x7": (9, (12, 7), np.float32, K.KEL_VALUE_F32),
         "writers_d3q19_f64_5x4x3": (19, (5, 4, 3), np.float64, K.KEL_VALUE_F64)}


def lib():
    try:
        return K.load_library()
    except RuntimeError as e:
        pytest.skip(str(e))


def views(specs):
    """specs: (name, array, value_type, ghost, vector) -> (FieldView array, keep-alive)."""
    arr = (K.FieldView * len(specs))()
    keep = []
    for v, (name, a, vt, ghost, vector) in zip(arr, specs):
        a = np.ascontiguousarray(a)
        keep.append(a)
        comps = 1 if a.ndim == 1 else a.shape[1]
        v.name, v.value_type, v.components, v.ghost, v.vector = name.encode(), vt, comps, ghost, vector
        v.data = a.ctypes.data
    return arr, keep


def fixture(name):
    p = os.path.join(HERE, "golden", name + ".npz")
    return np.load(p)


def specs_for(name):
    q, dims, dt, vt = CASES[name]
    z = fixture(name)
    macros = [("velocity", z["vel"].astype(dt), vt, 0, 1), ("density", z["rho"].astype(dt), vt, 0, 0)]
    dfs = z["dfs"].astype(dt)
    lattice = [("info", z["flags"], K.KEL_VALUE_U8, 0, 0), ("dfs", dfs, vt, 1, 0), ("dfs_old", -dfs, vt, 1, 0)]
    return z, dims, macros, lattice


@pytest.mark.parametrize("name", sorted(CASES))
def test_vtk_and_csv_match_reference_bytes(name, tmp_path):
    L = lib()
    z, dims, macros, lattice = specs_for(name)
    d = (C.c_int64 * len(dims))(*dims)
    fm, k1 = views(macros)
    fl, k2 = views(lattice)
    out = str(tmp_path).encode()
    assert L.kel_write_vtk(out, b"m", 37, d, len(dims), fm, 2) == 0
    assert L.kel_write_csv(out, b"m", 37, d, len(dims), fm, 2) == 0
    assert L.kel_write_vtk(out, b"initial_state", 0, d, len(dims), fl, 3) == 0
    for f in ("vtk/m_37.vtk", "vtk/initial_state_0.vtk", "csv/m_velocity_37.csv", "csv/m_density_37.csv"):
        got = open(os.path.join(tmp_path, f), "rb").read()
        assert got == bytes(z["file:" + f]), f


@pytest.mark.parametrize("name", sorted(CASES))
def test_forst_matches_reference_bytes_and_round_trips(name, tmp_path):
    L = lib()
    z, dims, macros, lattice = specs_for(name)
    d = (C.c_int64 * len(dims))(*dims)
    for key, specs in (("m.forst", macros), ("lattice.forst", lattice)):
        fv, keep = views(specs)
        p = os.path.join(tmp_path, key)
        assert L.kel_write_forst(p.encode(), d, len(dims), fv, len(specs)) == 0
        assert open(p, "rb").read() == bytes(z["file:" + key]), key
        back = [(n, np.zeros_like(a), vt, g, v) for (n, a, vt, g, v) in specs]
        bv, keep2 = views(back)
        assert L.kel_read_forst(p.encode(), d, len(dims), bv, len(back)) == 0
        for (n, a, *_), b in zip(specs, keep2):
            assert np.array_equal(np.asarray(a).reshape(b.shape), b), n


def test_read_forst_rejects_a_wrong_size(tmp_path):
    L = lib()
    p = os.path.join(tmp_path, "short.forst")
    open(p, "wb").write(b"\0" * 10)
    a = np.zeros(12, np.float32)
    fv, keep = views([("density", a, K.KEL_VALUE_F32, 0, 0)])
    d = (C.c_int64 * 1)(12)
    assert L.kel_read_forst(p.encode(), d, 1, fv, 1) == K.KEL_ERR_INVALID_ARGUMENT
    assert b"48" in L.kel_last_error_string()
