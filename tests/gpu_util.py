"""Helpers for the GPU parity tests: run a case through the C ABI."""
from __future__ import annotations

import numpy as np

from lbm_mirror_gb300 import Lattice
from lbm_mirror_gb300 import capi as K

QNAME = {9: "D2Q9", 19: "D3Q19", 27: "D3Q27"}


def make_lattice(case, storage="fp32", launch=None):
    lat = Lattice(QNAME[case["q"]], case["dims"], storage=storage, periodic_x=case["periodic"])
    if launch is not None:
        lat.set_launch(*launch)
    lat.upload_flags(case["flags"])
    if case["init"] is not None:
        lat.upload_populations(case["init"].astype(np.float32))
    if case["profile"] is not None:
        lat.upload_inlet_profile(case["profile"])
    if case["porosity"] is not None:
        lat.upload_porosity(case["porosity"])
    if case["force"] is not None:
        lat.upload_force(case["force"])
    return lat


def with_arith(program, arithmetic):
    d = K.program_to_dict(program)
    d["arithmetic"] = arithmetic
    return K.program_from_dict(d)


def run_gpu(case, arithmetic=K.KEL_ARITH_REFERENCE, storage="fp32", chunks=None, launch=None):
    """Run ``case`` on the GPU; returns (populations AoS f64, rho, vel)."""
    lat = make_lattice(case, storage, launch)
    prog = with_arith(case["program"], arithmetic)
    steps = case["steps"]
    if chunks:
        done = 0
        for c in chunks:
            lat.step(prog, c)
            done += c
        assert done == steps
    else:
        lat.step(prog, steps)
    f = lat.populations(np.float64)
    rho, vel = lat.macros()
    lat.close()
    return f, rho.astype(np.float64), vel.astype(np.float64)


def rel_l2(a, b):
    """||a - b||_2 / ||b||_2: the field comparison of the reference's own
    tooling (scripts/python/csv_l2_norm.py prints ||a - b||_2)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    return 0.0 if num == 0 else num / max(den, 1e-300)


def rel_err(a, b):
    """max |a - b| / max |b| (0 when both vanish)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).max()
    num = np.abs(a - b).max()
    return 0.0 if num == 0 else num / max(den, 1e-300)
