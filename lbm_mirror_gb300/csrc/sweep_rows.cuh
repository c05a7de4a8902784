// Row-pipeline sweep: the same fused collide + boundary + stream time step as
// sweep1_kernel (AA pattern, in place), with whole rows moved between HBM and
// shared memory by the TMA engine and a producer warp that keeps several rows
// in flight.
//
// A CTA is C = nxp rounded up to 32 consumer threads (one per cell of a row,
// nxp <= 256) plus one producer warp, and owns the rows blockIdx.x,
// blockIdx.x + gridDim.x, ... (a persistent grid sized to the resident CTAs).
// Shared memory holds `stages` row stages; a stage is Q population rows plus
// the row's flags, with two mbarriers: `full` (bytes landed) and `done`
// (consumers finished the row).
//   producer warp, per row k of the CTA (stage s = k % stages):
//     wait done[s]; lane i issues the bulk store (cp.async.bulk shared ->
//     global, bulk_group) of population row i to its destination; every lane
//     waits until its stores have read the stage; then lane i issues the bulk
//     load of population row i of row k + stages into the same stage, lane Q
//     the flag row, lane 0 having armed full[s] with the byte count;
//   consumer threads, per row k:
//     wait full[s] (bounded); read the cell's populations from the stage (odd
//     steps: shifted by -c_i in x, from the row at y - c_y, z - c_z, zero
//     where that lies outside); the same cell_update as the other sweeps;
//     one consumer barrier (which also makes a failed wait uniform); write
//     the post-collision populations back into the same stage (odd steps:
//     shifted by +c_i in x); fence.proxy.async; each warp arrives on done[s].
// The slots a row reads and writes in one step are touched by no other row
// (every AA location is read and written by the same cell), so rows need no
// ordering among CTAs.  Slots whose source lies outside the lattice get the
// zero population: x edges inside the stored row, whole rows (source row
// outside in y or z) by plain stores from the consumers.
//
// Requirements checked on the host: nxp * sizeof(element) is a multiple of
// 16 bytes (bulk-copy alignment of every row start), nxp <= 256, the flags
// allocation extends at least 16 bytes past the last row (the flag copy is
// widened to 16-byte boundaries).
#pragma once

#include "sweep.cuh"

namespace kel {
namespace gb {

constexpr int ROWS_MAX_NXP = 256;
constexpr int ROWS_MAX_STAGES = 6;
constexpr int ROWS_HEADER = 128; // 2 x stages mbarriers at the start of dynamic shared memory

__device__ __forceinline__ uint32_t rows_saddr(const void *p) {
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool rows_mbar_try(uint32_t addr, uint32_t parity) {
	uint32_t ok;
	asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
				 : "=r"(ok)
				 : "r"(addr), "r"(parity)
				 : "memory");
	return ok != 0;
}

// Bounded wait (about one second at the maximum SM clock); false on timeout.
__device__ __forceinline__ bool rows_mbar_wait(uint32_t addr, uint32_t parity) {
	const long long t0 = clock64();
	while (!rows_mbar_try(addr, parity))
		if (clock64() - t0 > 2000000000ll) return false;
	return true;
}

__device__ __forceinline__ void rows_bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
				 "l"(src), "r"(bytes), "r"(mbar)
				 : "memory");
}

__device__ __forceinline__ void rows_bulk_store(void *dst, uint32_t src, uint32_t bytes) {
	asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst), "r"(src), "r"(bytes)
				 : "memory");
}

template <class ST>
__device__ __forceinline__ float rows_from(ST v, float s);
template <>
__device__ __forceinline__ float rows_from<float>(float v, float) { return v; }
template <>
__device__ __forceinline__ float rows_from<__half>(__half v, float s) { return __half2float(v) + s; }

template <class ST>
__device__ __forceinline__ ST rows_to(float v, float s);
template <>
__device__ __forceinline__ float rows_to<float>(float v, float) { return v; }
template <>
__device__ __forceinline__ __half rows_to<__half>(float v, float s) { return __float2half_rn(v - s); }

// Host and device agree on the stage layout through these two functions.
__host__ __device__ inline int rows_stage_bytes(int Q, int nxp, int elem) {
	const int pops = Q * nxp * elem;
	const int flags = ((nxp + 15) / 16) * 16 + 16;
	return (pops + flags + 127) / 128 * 128;
}
__host__ __device__ inline int rows_smem_bytes(int Q, int nxp, int elem, int stages) {
	return ROWS_HEADER + stages * rows_stage_bytes(Q, nxp, elem);
}

// Direction components of a runtime direction index (producer lanes).
template <class L>
__device__ __forceinline__ void rows_dir(int i, int &cx, int &cy, int &cz, int &op) {
	cx = cy = cz = 0;
	op = 0;
#pragma unroll
	for (int j = 0; j < L::Q; ++j)
		if (j == i) {
			cx = L::cx(j);
			cy = L::cy(j);
			cz = L::cz(j);
			op = L::opp(j);
		}
}

// Consumer barrier (named barrier 1 over the C consumer threads) that also
// ORs a predicate across them.
__device__ __forceinline__ bool rows_consumer_bar_or(bool v, int nthreads) {
	uint32_t r;
	asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}\n"
				 : "=r"(r)
				 : "r"((uint32_t)v), "r"(nthreads)
				 : "memory");
	return r != 0;
}

template <class L, int STORE, bool ODD, int COLL, bool EXACT>
__global__ void __launch_bounds__(ROWS_MAX_NXP + 32, 2) sweep_rows_kernel(const __grid_constant__ SweepParams p) {
	using ST = typename Store<STORE>::T;
	constexpr int Q = L::Q;
	extern __shared__ __align__(128) unsigned char rows_smem[];
	const int nxp = p.nxp, ny = p.ny, nz = p.nz, NS = p.stages;
	const int C = (nxp + 31) & ~31; // consumer threads
	const int tid = threadIdx.x;
	const uint32_t row_bytes = static_cast<uint32_t>(nxp) * sizeof(ST);
	const uint32_t stage_bytes = static_cast<uint32_t>(rows_stage_bytes(Q, nxp, sizeof(ST)));
	uint64_t *full = reinterpret_cast<uint64_t *>(rows_smem);
	uint64_t *done = full + NS;
	unsigned char *stage0 = rows_smem + ROWS_HEADER;
	const int64_t R = static_cast<int64_t>(ny) * nz;
	const int64_t G = gridDim.x;
	const int64_t K = static_cast<int64_t>(blockIdx.x) < R ? (R - 1 - blockIdx.x) / G + 1 : 0;
	ST *const f = static_cast<ST *>(p.f);

	if (blockDim.x != static_cast<unsigned>(C + 32) || NS < 1 || NS > ROWS_MAX_STAGES) { // launch does not match the layout
		if (tid == 0) atomicOr(p.err, 2u);
		return;
	}
	if (tid == 0) {
		for (int s = 0; s < NS; ++s) {
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(rows_saddr(full + s)));
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(rows_saddr(done + s)), "r"(C / 32));
		}
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	}
	__syncthreads();

	if (tid >= C) {
		// ---------------- producer warp ----------------
		const int lane = tid - C;
		int dcx = 0, dcy = 0, dcz = 0, dop = 0;
		if (lane < Q) rows_dir<L>(lane, dcx, dcy, dcz, dop);
		auto issue_loads = [&](int64_t k) {
			const int s = static_cast<int>(k % NS);
			const int64_t r = blockIdx.x + k * G;
			const int y = static_cast<int>(r % ny), z = static_cast<int>(r / ny);
			unsigned char *st = stage0 + static_cast<size_t>(s) * stage_bytes;
			const uint32_t mb = rows_saddr(full + s);
			const int64_t f0 = r * nxp, a0 = f0 & ~static_cast<int64_t>(15);
			const uint32_t fbytes = static_cast<uint32_t>((f0 - a0 + nxp + 15) & ~static_cast<int64_t>(15));
			const int sy = ODD ? y - dcy : y, sz = ODD ? z - dcz : z;
			const bool valid = lane < Q && sy >= 0 && sy < ny && sz >= 0 && sz < nz;
			const uint32_t n = __popc(__ballot_sync(0xffffffffu, valid));
			if (lane == 0)
				asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb),
							 "r"(n * row_bytes + fbytes)
							 : "memory");
			__syncwarp();
			if (valid) {
				const int plane = ODD ? dop : lane;
				const ST *src = f + static_cast<int64_t>(plane) * p.plane + (static_cast<int64_t>(sz) * ny + sy) * nxp;
				rows_bulk_load(rows_saddr(st + static_cast<size_t>(lane) * row_bytes), src, row_bytes, mb);
			}
			if (lane == Q) rows_bulk_load(rows_saddr(st + static_cast<size_t>(Q) * row_bytes), p.flags + a0, fbytes, mb);
		};
		int64_t issued = 0;
		for (; issued < K && issued < NS; ++issued) issue_loads(issued);
		bool failed = false;
		int64_t k = 0;
		for (; k < K; ++k) {
			const int s = static_cast<int>(k % NS);
			const bool ok = rows_mbar_wait(rows_saddr(done + s), static_cast<uint32_t>((k / NS) & 1));
			if (!__all_sync(0xffffffffu, ok)) {
				failed = true;
				break;
			}
			const int64_t r = blockIdx.x + k * G;
			const int y = static_cast<int>(r % ny), z = static_cast<int>(r / ny);
			const int dy = ODD ? y + dcy : y, dz = ODD ? z + dcz : z;
			if (lane < Q && dy >= 0 && dy < ny && dz >= 0 && dz < nz)
				rows_bulk_store(f + static_cast<int64_t>(lane) * p.plane + (static_cast<int64_t>(dz) * ny + dy) * nxp,
								rows_saddr(stage0 + static_cast<size_t>(s) * stage_bytes +
										   static_cast<size_t>(lane) * row_bytes),
								row_bytes);
			asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
			asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
			__syncwarp();
			if (issued < K) {
				issue_loads(issued); // issued == k + NS: the stage just stored
				++issued;
			}
		}
		if (failed) {
			if (lane == 0) atomicOr(p.err, 1u);
			// let the loads still in flight land before the CTA's shared memory goes away
			for (int64_t j = k; j < issued; ++j)
				rows_mbar_wait(rows_saddr(full + (j % NS)), static_cast<uint32_t>((j / NS) & 1));
		}
		asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
		return;
	}

	// ---------------- consumer threads ----------------
	const int x = tid;
	const bool active = x < nxp;
	for (int64_t k = 0; k < K; ++k) {
		const int s = static_cast<int>(k % NS);
		const int64_t r = blockIdx.x + k * G;
		const int y = static_cast<int>(r % ny), z = static_cast<int>(r / ny);
		unsigned char *st = stage0 + static_cast<size_t>(s) * stage_bytes;
		const int64_t cell = r * nxp + x;

		// per-cell fields of the collision, from global memory
		float por = 1.f;
		float Fc[3] = {0.f, 0.f, 0.f};
		if (active) {
			if (COLL == COLL_PSM || COLL == COLL_PSM_GUO || COLL == COLL_HLBM) por = p.por[cell];
			if (COLL == COLL_BGK_GUO || COLL == COLL_PSM_GUO) {
#pragma unroll
				for (int d = 0; d < L::D; ++d) Fc[d] = p.force[d * p.plane + cell];
			}
			if (COLL == COLL_HLBM) {
				Fc[0] = p.hN[cell];
				Fc[1] = p.hN[p.plane + cell];
				Fc[2] = p.hD[cell];
			}
		}
		const bool ok = rows_mbar_wait(rows_saddr(full + s), static_cast<uint32_t>((k / NS) & 1));
		float fv[Q];
		if (active) {
			const int flag = st[static_cast<size_t>(Q) * row_bytes + (r * nxp & 15) + x];
#pragma unroll
			for (int i = 0; i < Q; ++i) {
				const ST *slot = reinterpret_cast<const ST *>(st + static_cast<size_t>(i) * row_bytes);
				if (!ODD) {
					fv[i] = rows_from<ST>(slot[x], p.wshift[i]);
				} else {
					const int cx = L::cx(i), sy = y - L::cy(i), sz = z - L::cz(i);
					bool in = sy >= 0 && sy < ny && sz >= 0 && sz < nz;
					int sx = x - cx;
					if (cx != 0) {
						if (p.periodic) sx = sx < 0 ? sx + nxp : (sx >= nxp ? sx - nxp : sx);
						else in = in && sx >= 0 && sx < nxp;
					}
					fv[i] = in ? rows_from<ST>(slot[sx], p.wshift[i]) : 0.f;
				}
			}
			float rho = 1.f, u[3] = {0.f, 0.f, 0.f};
			const bool col = cell_update<L, COLL, EXACT>(fv, flag, y, cell_ctx(p), por, Fc, rho, u);
			if (p.write_macros && col) {
				p.rho[cell] = rho;
#pragma unroll
				for (int d = 0; d < L::D; ++d) p.u[d * p.plane + cell] = u[d];
			}
		}
		// every read of this stage is done (and a failed wait is seen by all)
		if (rows_consumer_bar_or(!ok, C)) {
			if (tid == 0) atomicOr(p.err, 1u);
			break;
		}
		if (active) {
#pragma unroll
			for (int i = 0; i < Q; ++i) {
				if (!ODD) {
					ST *slot = reinterpret_cast<ST *>(st + static_cast<size_t>(L::opp(i)) * row_bytes);
					slot[x] = rows_to<ST>(fv[i], p.wshift[i]);
				} else {
					ST *slot = reinterpret_cast<ST *>(st + static_cast<size_t>(i) * row_bytes);
					const int cx = L::cx(i);
					if (cx == 0) {
						slot[x] = rows_to<ST>(fv[i], p.wshift[i]);
					} else if (p.periodic) {
						int dx = x + cx;
						dx = dx < 0 ? dx + nxp : (dx >= nxp ? dx - nxp : dx);
						slot[dx] = rows_to<ST>(fv[i], p.wshift[i]);
					} else {
						const int dx = x + cx;
						if (dx >= 0 && dx < nxp) slot[dx] = rows_to<ST>(fv[i], p.wshift[i]);
						// the edge slot whose source x - c_i lies outside
						if (cx > 0 && x == 0) slot[0] = rows_to<ST>(0.f, p.wshift[i]);
						if (cx < 0 && x == nxp - 1) slot[nxp - 1] = rows_to<ST>(0.f, p.wshift[i]);
					}
					// whole row of plane i whose source row lies outside in y or z
					const int sy = y - L::cy(i), sz = z - L::cz(i);
					if (!(sy >= 0 && sy < ny && sz >= 0 && sz < nz))
						f[static_cast<int64_t>(i) * p.plane + cell] = rows_to<ST>(0.f, p.wshift[i]);
				}
			}
		}
		asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
		__syncwarp();
		if ((tid & 31) == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(rows_saddr(done + s)) : "memory");
	}
}

} // namespace gb
} // namespace kel
