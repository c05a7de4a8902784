"""The C++ face run as a reference-style driver (the 256x64 Poiseuille channel in small) on the
GPU: with reference arithmetic its macros equal the reference's bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from tests.golden import make_golden as G

pytestmark = pytest.mark.gpu


def test_cpp_driver_matches_reference(tmp_path):
    from tests.cpp_driver import build_driver
    exe = build_driver(str(tmp_path))
    case, dfs, rho, vel = G.load("poiseuille_48x20")
    out = os.path.join(str(tmp_path), "m.bin")
    subprocess.check_call([exe, "48", "20", str(case["steps"]), out, "reference"])
    raw = np.fromfile(out, dtype=np.float32)
    n = 48 * 20
    np.testing.assert_array_equal(raw[:n].astype(np.float64), rho)
    np.testing.assert_array_equal(raw[n:].reshape(n, 2).astype(np.float64), vel)
