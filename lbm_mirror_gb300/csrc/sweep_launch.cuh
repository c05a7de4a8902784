// Instantiation and launch of the sweep kernel for one descriptor; included
// once per descriptor translation unit (sweep_d2q9.cu, sweep_d3q19.cu,
// sweep_d3q27.cu) so the three compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "sweep.cuh"

namespace kel {
namespace gb {

template <class L, int STORE, bool ODD, int COLL, bool EXACT>
static cudaError_t launch_variant(const SweepParams &p, cudaStream_t st) {
	const int block = p.block > 0 ? p.block : 256;
	if constexpr (COLL == COLL_HLBM) { // one cell per thread only
		dim3 grid((p.nxp + block - 1) / block, p.ny, p.nz);
		sweep1_kernel<L, STORE, ODD, COLL, EXACT><<<grid, block, 0, st>>>(p);
	} else if (p.cpt == 1) {
		dim3 grid((p.nxp + block - 1) / block, p.ny, p.nz);
		sweep1_kernel<L, STORE, ODD, COLL, EXACT><<<grid, block, 0, st>>>(p);
	} else {
		const int64_t threads = static_cast<int64_t>(p.ny) * p.nz * p.wpr * 32;
		const int64_t blocks = (threads + block - 1) / block;
		sweep_kernel<L, STORE, ODD, COLL, EXACT><<<static_cast<unsigned>(blocks), block, 0, st>>>(p);
	}
	return cudaGetLastError();
}

template <class L, int STORE, bool ODD, bool EXACT>
static cudaError_t launch_coll(const SweepParams &p, int coll, cudaStream_t st) {
	switch (coll) {
	case COLL_BGK: return launch_variant<L, STORE, ODD, COLL_BGK, EXACT>(p, st);
	case COLL_BGK_GUO: return launch_variant<L, STORE, ODD, COLL_BGK_GUO, EXACT>(p, st);
	case COLL_PSM: return launch_variant<L, STORE, ODD, COLL_PSM, EXACT>(p, st);
	case COLL_PSM_GUO: return launch_variant<L, STORE, ODD, COLL_PSM_GUO, EXACT>(p, st);
	case COLL_HLBM:
		if constexpr (L::Q == 9) return launch_variant<L, STORE, ODD, COLL_HLBM, EXACT>(p, st);
		return cudaErrorInvalidValue;
	}
	return cudaErrorInvalidValue;
}

template <class L>
cudaError_t launch_sweep(const SweepParams &p, int storage, bool odd, int coll, bool exact, cudaStream_t st) {
	if (storage == STORE_FP32) {
		if (exact) return odd ? launch_coll<L, STORE_FP32, true, true>(p, coll, st)
							  : launch_coll<L, STORE_FP32, false, true>(p, coll, st);
		return odd ? launch_coll<L, STORE_FP32, true, false>(p, coll, st)
				   : launch_coll<L, STORE_FP32, false, false>(p, coll, st);
	}
	if (exact) return cudaErrorInvalidValue;
	return odd ? launch_coll<L, STORE_FP16S, true, false>(p, coll, st)
			   : launch_coll<L, STORE_FP16S, false, false>(p, coll, st);
}

} // namespace gb
} // namespace kel
