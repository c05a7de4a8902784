// Sweep kernels for the D2Q9 descriptor, FP32 storage, fast arithmetic: every launch shape,
// parity and collision variant.
#include "sweep_launch.cuh"

namespace kel {
namespace gb {
template cudaError_t launch_sweep_part<D2Q9, PART_FAST32>(const SweepParams &, bool, int, cudaStream_t);
} // namespace gb
} // namespace kel
