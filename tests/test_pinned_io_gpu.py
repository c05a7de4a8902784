"""Transfers through page-locked host buffers: kel_upload_populations,
kel_download_populations and kel_download_macros read / write such buffers
in place from the conversion kernels (no staging copy).  Results must equal,
bit for bit, those of the staged path taken for ordinary (pageable) host
memory, for FP32 and FP64 host data, AoS and SoA layouts, at even and odd
time steps."""
import ctypes as C

import numpy as np
import pytest

from lbm_mirror_gb300 import capi as K
from tests import cases
from tests.gpu_util import make_lattice, with_arith

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def pinned_like(a):
    t = torch.empty(a.size, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
    out = t.numpy()
    out[:] = a.reshape(-1)
    return t, out


@pytest.mark.parametrize("storage", ["fp32", "fp16s"])
@pytest.mark.parametrize("steps", [6, 7])
def test_pinned_transfers_equal_staged(storage, steps):
    case = cases.cavity_3d(19, dims=(40, 24, 18), steps=steps)
    prog = with_arith(case["program"], K.KEL_ARITH_FAST)
    rng = np.random.default_rng(3)
    w = cases._weights(19)
    init = (w[None, :] * (1 + 0.01 * rng.standard_normal((40 * 24 * 18, 19)))).astype(np.float32)
    init[case["flags"] != 2] = 0.0

    a = make_lattice(case, storage)
    a.upload_populations(init)
    a.step(prog, steps, write_macros=True)

    b = make_lattice(case, storage)
    keep, pin = pinned_like(init)
    b.upload_populations(pin)
    b.step(prog, steps, write_macros=True)

    for dtype in (np.float32, np.float64):
        for layout in ("aos", "soa"):
            ref = a.populations(dtype, layout)
            t = torch.empty(ref.size, dtype=getattr(torch, str(np.dtype(dtype))), pin_memory=True)
            out = t.numpy()
            dt = K.KEL_DTYPE_F32 if dtype == np.float32 else K.KEL_DTYPE_F64
            lay = K.KEL_LAYOUT_AOS if layout == "aos" else K.KEL_LAYOUT_SOA
            assert b.lib.kel_download_populations(b.handle, C.c_void_p(out.ctypes.data), dt, lay) == 0
            np.testing.assert_array_equal(out.reshape(ref.shape), ref)
    rho_a, u_a = a.macros()
    tr = torch.empty(rho_a.size, dtype=torch.float32, pin_memory=True)
    tu = torch.empty(u_a.size, dtype=torch.float32, pin_memory=True)
    assert b.lib.kel_download_macros(b.handle, C.c_void_p(tr.numpy().ctypes.data), C.c_void_p(tu.numpy().ctypes.data)) == 0
    np.testing.assert_array_equal(tr.numpy(), rho_a)
    np.testing.assert_array_equal(tu.numpy().reshape(u_a.shape), u_a)
    a.close()
    b.close()
