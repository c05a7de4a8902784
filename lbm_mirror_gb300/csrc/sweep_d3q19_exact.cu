// Sweep kernels for the D3Q19 descriptor, FP32 storage, the reference's arithmetic: every launch shape,
// parity and collision variant.
#include "sweep_launch.cuh"

namespace kel {
namespace gb {
template cudaError_t launch_sweep_part<D3Q19, PART_EXACT32>(const SweepParams &, bool, int, cudaStream_t);
} // namespace gb
} // namespace kel
