// Host-side dispatch of a sweep launch to the translation unit that holds the
// variant: one per descriptor x {FP32 fast, FP32 reference arithmetic, FP16S}
// (sweep_<descriptor>_<part>.cu), so that the nine compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "sweep.cuh"

namespace kel {
namespace gb {

enum : int { PART_FAST32 = 0, PART_EXACT32 = 1, PART_FP16S = 2 };

template <class L, int PART>
cudaError_t launch_sweep_part(const SweepParams &p, bool odd, int coll, cudaStream_t st);

template <class L>
cudaError_t launch_sweep(const SweepParams &p, int storage, bool odd, int coll, bool exact, cudaStream_t st) {
	if (storage == STORE_FP32)
		return exact ? launch_sweep_part<L, PART_EXACT32>(p, odd, coll, st) : launch_sweep_part<L, PART_FAST32>(p, odd, coll, st);
	if (exact) return cudaErrorInvalidValue; // FP16S has no reference arithmetic
	return launch_sweep_part<L, PART_FP16S>(p, odd, coll, st);
}

} // namespace gb
} // namespace kel
