// Launch of the sweep kernels; included by the nine translation units
// sweep_<descriptor>_<fast|exact|fp16s>.cu, each of which instantiates one
// part (sweep_dispatch.cuh picks the part at run time).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "sweep.cuh"
#include "sweep_dispatch.cuh"
#include "sweep_rows.cuh"

namespace kel {
namespace gb {

// Row pipeline: persistent grid of (resident CTAs per SM) x SMs, capped at the
// row count.  The shared-memory opt-in and the occupancy query run once per
// kernel variant, device, row length and stage count (one cached entry).
// Any grid size is correct (rows are dealt round-robin to the CTAs); the
// occupancy only makes all CTAs resident at once.
template <class L, int STORE, bool ODD, int COLL, bool EXACT>
static cudaError_t launch_rows(const SweepParams &p, cudaStream_t st) {
	auto kern = sweep_rows_kernel<L, STORE, ODD, COLL, EXACT>;
	const int smem = rows_smem_bytes(L::Q, p.nxp, (int)sizeof(typename Store<STORE>::T), p.stages);
	const int threads = ((p.nxp + 31) & ~31) + 32; // consumers (one per cell) + the producer warp
	// one atomic word: device + 1 (bits 48-63), stages (40-47), nxp (16-39), CTAs per SM (0-15)
	static std::atomic<uint64_t> cached{0};
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	const uint64_t key = (static_cast<uint64_t>(dev + 1) << 48) | (static_cast<uint64_t>(p.stages & 0xff) << 40) |
						 (static_cast<uint64_t>(p.nxp & 0xffffff) << 16);
	const uint64_t hit = cached.load();
	int per_sm = 0;
	if ((hit & ~static_cast<uint64_t>(0xffff)) == key) {
		per_sm = static_cast<int>(hit & 0xffff);
	} else {
		// opt in to the device's whole per-block shared memory, so that no
		// later call with a smaller footprint can lower it under another thread
		int optin = 0;
		if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
		if (smem > optin) return cudaErrorInvalidConfiguration;
		if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin)) != cudaSuccess) return e;
		if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem)) != cudaSuccess) return e;
		if (per_sm < 1) return cudaErrorInvalidConfiguration;
		cached.store(key | static_cast<uint64_t>(per_sm & 0xffff));
	}
	const int64_t rows = static_cast<int64_t>(p.ny) * p.nz;
	const int64_t slots = static_cast<int64_t>(per_sm) * (p.sms > 0 ? p.sms : 1);
	const unsigned grid = static_cast<unsigned>(rows < slots ? rows : slots);
	kern<<<grid, threads, smem, st>>>(p);
	return cudaGetLastError();
}

template <class L, int STORE, bool ODD, int COLL, bool EXACT>
static cudaError_t launch_variant(const SweepParams &p, cudaStream_t st) {
	const int block = p.block > 0 ? p.block : 256;
	if (p.hw_mask) { // half-way walls: the one-cell sweep only (other shapes fall back to it)
		const int b1 = p.cpt == 1 ? block : 256;
		dim3 grid((p.nxp + b1 - 1) / b1, p.ny, p.nz);
		sweep1_kernel<L, STORE, ODD, COLL, EXACT, true><<<grid, b1, 0, st>>>(p);
		return cudaGetLastError();
	}
	if (p.cpt == CPT_ROWS) return launch_rows<L, STORE, ODD, COLL, EXACT>(p, st);
	if (p.cpt == 2) {
		const int64_t threads = static_cast<int64_t>(p.ny) * p.nz * p.wpr2 * 32;
		const int64_t blocks = (threads + block - 1) / block;
		if constexpr (STORE == STORE_FP16S) // nxp is even in FP16S storage
			sweep2h_kernel<L, ODD, COLL, EXACT><<<static_cast<unsigned>(blocks), block, 0, st>>>(p);
		else
			sweep2_kernel<L, STORE, ODD, COLL, EXACT><<<static_cast<unsigned>(blocks), block, 0, st>>>(p);
		return cudaGetLastError();
	}
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

// One part of the variant set (the translation units compile one part each,
// in parallel): FP32 fast arithmetic, FP32 reference arithmetic, FP16S.
template <class L, int PART>
cudaError_t launch_sweep_part(const SweepParams &p, bool odd, int coll, cudaStream_t st) {
	if constexpr (PART == PART_FAST32)
		return odd ? launch_coll<L, STORE_FP32, true, false>(p, coll, st) : launch_coll<L, STORE_FP32, false, false>(p, coll, st);
	else if constexpr (PART == PART_EXACT32)
		return odd ? launch_coll<L, STORE_FP32, true, true>(p, coll, st) : launch_coll<L, STORE_FP32, false, true>(p, coll, st);
	else
		return odd ? launch_coll<L, STORE_FP16S, true, false>(p, coll, st)
				   : launch_coll<L, STORE_FP16S, false, false>(p, coll, st);
}

} // namespace gb
} // namespace kel
