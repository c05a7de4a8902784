"""Build helper for the C++ driver written against include/kel/lbm/cuda/lbm_cuda.hpp."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_driver(out_dir):
    from lbm_mirror_gb300 import capi as K
    if not os.path.exists(K.LIB_PATH):
        from lbm_mirror_gb300 import build
        build.build()
    exe = os.path.join(out_dir, "poiseuille_driver")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"),
           os.path.join(HERE, "cpp", "poiseuille_driver.cpp"), "-o", exe, "-L" + K.BUILD_DIR, "-lkel_lbm_cuda",
           "-Wl,-rpath," + K.BUILD_DIR]
    subprocess.check_call(cmd)
    return exe
