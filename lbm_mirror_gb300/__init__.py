"""GB300-native lattice-Boltzmann hot path with keldu/lbm_mirror's component API.

The compute path is libkel_lbm_cuda.so (hand-written sm_103a CUDA kernels behind
the C ABI of include/kel_lbm_cuda.h); this package is the Python host mirror.
"""
from . import capi
from .lattice import (BGK, Batch, UNet, AntiBounceBack, BGKGuo, BounceBack, Equilibrium, KelError, Lattice, MovingWall, Particles, Psm,
                      PsmGuo, Shape, ZouHePressureX, ZouHeVelocityX, program_from_switch)

__all__ = ["capi", "Lattice", "Particles", "Shape", "Batch", "UNet", "KelError", "program_from_switch", "BGK", "BGKGuo", "Psm", "PsmGuo", "BounceBack",
           "AntiBounceBack", "Equilibrium", "ZouHePressureX", "ZouHeVelocityX", "MovingWall"]
