"""FP64 oracle run of the lid-driven cavity at full size (256^3, D3Q19 and
D3Q27, tau = 0.55, lid u = (0.1, 0, 0), rest start, 5,000 steps), kept as a
sub-sampled golden fixture: rho and u at every 8th cell along each axis
(32^3 cells, offset 4), float64.  The GPU FP32 and FP16-shifted runs of the
same case are compared against it at those cells (tests/test_cavity_fp64.py).

Runs on the host cores through the C oracle (OpenMP); about an hour per
descriptor on 8 cores.

    python tests/golden/make_cavity_fp64.py [19|27 ...]
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import OracleLattice, build  # noqa: E402
from tests import cases  # noqa: E402

N, STEPS, STRIDE, OFF = 256, 5000, 8, 4


def run(q):
    c = cases.cavity_3d(q, dims=(N, N, N), steps=STEPS, f64=True)
    o = OracleLattice(q, c["dims"], f64=True)
    o.set_flags(c["flags"])
    t0 = time.time()
    for k in range(STEPS // 500):
        o.run(c["program"], 500)
        print(f"D3Q{q}: {(k + 1) * 500} steps, {time.time() - t0:.0f} s", flush=True)
    rho, u = o.macros()
    rho = rho.reshape(N, N, N)
    u = u.reshape(N, N, N, 3)
    sl = (slice(OFF, N, STRIDE),) * 3
    out = os.path.join(HERE, f"cavity256_d3q{q}_fp64_5000_sub8.npz")
    np.savez_compressed(out, rho=rho[sl], u=u[sl], stride=STRIDE, offset=OFF, steps=STEPS, n=N,
                        tau=0.55, lid=np.array([0.1, 0.0, 0.0]))
    print("wrote", out, flush=True)


if __name__ == "__main__":
    build()
    for q in (int(a) for a in (sys.argv[1:] or ["19", "27"])):
        run(q)
