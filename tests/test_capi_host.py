"""CPU-side checks of the C ABI boundary and the Python host mirror (no GPU calls)."""
import ctypes as C
import os
import subprocess

import pytest

from lbm_mirror_gb300 import capi as K
from lbm_mirror_gb300 import lattice as LL


def _lib_path():
    if not os.path.exists(K.LIB_PATH):
        from lbm_mirror_gb300 import build
        build.build()
    return K.LIB_PATH


def test_library_exports_every_header_symbol():
    names = K.header_symbols()
    assert "kel_step" in names and "kel_lattice_create" in names
    lib = C.CDLL(_lib_path())
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", _lib_path()], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln and ln.split()[-1].startswith("kel_")}
    assert set(names) <= exported
    assert exported <= set(names), exported - set(names)


def test_struct_layouts_match_header():
    assert C.sizeof(K.FlagOp) == 48
    assert C.sizeof(K.StepProgram) == 8 + 8 + 24 + 48 * K.KEL_MAX_FLAGS
    assert C.sizeof(K.LatticeDesc) == 40
    from oracle.oracle import lib as olib
    assert olib().ko_program_size() == C.sizeof(K.StepProgram)


def test_program_from_switch_mirrors_driver_switch():
    """examples/stdkr_2d_bgk/step.hpp:22-69 as a switch description."""
    prog = LL.program_from_switch({
        1: [LL.BounceBack()],
        2: [LL.BGK(0.8)],
        3: [LL.ZouHeVelocityX(True, "profile"), LL.BGK(0.8)],
        4: [LL.ZouHePressureX(False, 1.0), LL.BGK(0.8)],
    })
    assert prog.collision == K.KEL_COLL_BGK and abs(prog.tau - 0.8) < 1e-15
    assert prog.ops[1].bc == K.KEL_BC_BOUNCE_BACK and prog.ops[1].collide == 0
    assert prog.ops[2].bc == K.KEL_BC_FLUID and prog.ops[2].collide == 1
    assert prog.ops[3].use_profile == 1 and prog.ops[3].east == 1
    assert prog.ops[4].east == 0 and prog.ops[4].rho == 1.0
    with pytest.raises(ValueError):
        LL.program_from_switch({2: [LL.BGK(0.8)], 3: [LL.BGK(0.9)]})
    with pytest.raises(ValueError):
        LL.program_from_switch({9: [LL.BGK(0.8)]})


def test_program_dict_round_trip():
    from tests import cases
    c = cases.mixed_2d(K.KEL_COLL_PSM_GUO)
    d = K.program_to_dict(c["program"])
    p2 = K.program_from_dict(d)
    assert bytes(p2) == bytes(c["program"])


def test_cpp_facade_driver_compiles_and_links(tmp_path):
    """The reference-style C++ driver builds against the header-only face and
    links the CUDA library (running it needs a GPU: tests/test_cpp_facade.py)."""
    from tests.cpp_driver import build_driver
    exe = build_driver(str(tmp_path))
    assert os.path.exists(exe)
