// Sweep kernels for the D2Q9 descriptor (all storage / parity / collision /
// arithmetic variants).
#include "sweep_launch.cuh"

namespace kel {
namespace gb {
template cudaError_t launch_sweep<D2Q9>(const SweepParams &, int, bool, int, bool, cudaStream_t);
} // namespace gb
} // namespace kel
