"""kel_velocity_residual_noalloc -- the convergence residual for callers that
may not allocate device memory while they run -- against the residual the
batched runner computes itself (kel_batch_run_until), on two calls in a row.

The caller owns every buffer (allocated here through torch before the calls);
the entry point only launches kernels on its fixed device scratch.  Collected
last so that a stop at the first failure has run everything else first; it
also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from lbm_mirror_gb300 import Batch
from lbm_mirror_gb300 import capi as K
from tests import cases

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _planes(u_aos):
    """(n, 2) host velocities -> device planes [u_x..., u_y...]."""
    return torch.tensor(np.ascontiguousarray(u_aos.T), dtype=torch.float32, device="cuda").contiguous()


def test_noalloc_residual_matches_batch_residual_twice():
    lib = K.load_library()
    chan = cases.batch_channels(1, seed=21, nx_range=(200, 256), ny_range=(48, 64))
    b = Batch(chan, cases.channel_program(chan[0]["tau"]))
    us, res = [], []
    for _ in range(3):
        _, r = b.run_until(tol=0.0, check_every=100, max_steps=100, use_graph=False)
        us.append(b.macros(0)[1].astype(np.float32))
        res.append(float(r[0]))
    n = us[0].shape[0]
    stream = torch.cuda.current_stream().cuda_stream
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    planes = [(_planes(us[k]), _planes(us[k - 1])) for k in (1, 2)]
    torch.cuda.synchronize()
    free_before = None
    for k in (1, 2):  # two calls in a row, scratch shared between them
        ua, ub = planes[k - 1]
        rc = lib.kel_velocity_residual_noalloc(C.c_void_p(ua.data_ptr()), C.c_void_p(ub.data_ptr()), n, 2,
                                               C.c_void_p(out.data_ptr() + 8 * (k - 1)), C.c_void_p(stream))
        assert rc == K.KEL_OK, lib.kel_last_error_string().decode()
        torch.cuda.synchronize()
        if k == 1:  # the first call may load the module that holds the scratch
            free_before = torch.cuda.mem_get_info()[0]
    # the second call allocated no device memory
    assert torch.cuda.mem_get_info()[0] == free_before
    got = out.cpu().numpy()
    for k in (1, 2):
        assert abs(got[k - 1] - res[k]) <= 1e-12 * res[k], (got[k - 1], res[k])
        assert 0.0 < got[k - 1] < 1.0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = K.load_library()
    x = torch.zeros(4, dtype=torch.float32, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = lib.kel_velocity_residual_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), 16_777_217, 1,
                                           C.c_void_p(out.data_ptr()), None)
    assert rc == K.KEL_ERR_INVALID_ARGUMENT
    assert "16777216" in lib.kel_last_error_string().decode()
