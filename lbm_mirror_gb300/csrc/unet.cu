// Warm-start U-Net: training and inference kernels (C ABI kel_unet_*).
//
// No counterpart in keldu/lbm_mirror (it has no learned component).  The
// network maps an obstacle mask and the inlet amplitude / relaxation time of
// a channel to (u_x, u_y, rho) on the lattice, which initialises the LBM.
//
// Layout: activations NHWC in bf16, channels a multiple of 16 (the input is
// padded to 16); conv weights [c_out][ky][kx][c_in] with an FP32 master copy,
// a bf16 copy for the forward GEMM and a flipped/transposed bf16 copy
// [c_in][2-ky][2-kx][c_out] for the data gradient.  Architecture as in
// oracle/unet_oracle.py (4 levels, concat skips, 1x1 head).
//
// Convolutions on the fifth-generation tensor cores (tcgen05.mma, bf16 in,
// FP32 accumulators in TMEM, operands staged by TMA; the default):
//   conv_rows        forward and data gradient of layers 128+ pixels wide
//                    whose weights stay in shared memory: input rows stream
//                    once each, one MMA feeds three output-row accumulators;
//   conv_halo        the other layers: per chunk of input channels a TMA halo
//                    tile, the nine taps as shifted descriptors;
//   conv_wgrad_halo  weight gradients from TMA-loaded halo rows, FP32
//                    partials per pixel chunk reduced in fixed order;
//   conv_tc, conv_wgrad_tc  im2col forms for levels narrower than the halo
//                    kernels take.
// The same GEMMs on warp-level mma.sync m16n8k16 (kel_unet_set_conv_kernel):
//   conv_igemm  implicit GEMM, M = pixels, N = c_out, K = 9 c_in; also the
//               data gradient (same kernel on dY with the flipped weights);
//               bias + ReLU fused into the epilogue;
//   conv_wgrad  M = c_out, N = 9 c_in, K = pixels, split over pixel chunks
//               into FP32 partial sums, reduced in fixed order (deterministic).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lattice_internal.cuh"

using namespace kel::gb;

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
	asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
				 "{%0,%1,%2,%3};\n"
				 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
				 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// ---- implicit-GEMM 3x3 convolution (forward and data gradient) -----------------

constexpr int CB_M = 64, CB_N = 64, CB_K = 16, CPAD = 24; // tile + padded row pitch (bf16)

struct ConvArgs {
	const bf16 *x; // (N,H,W,Ci)
	const bf16 *w; // (Co,3,3,Ci)
	const float *bias;
	bf16 *y;       // (N,H,W,Co)
	int N, H, W, Ci, Co;
	int relu, use_bias;
};

__global__ void __launch_bounds__(128) conv_igemm(ConvArgs a) {
	__shared__ __align__(16) bf16 As[2][CB_M][CPAD];
	__shared__ __align__(16) bf16 Bs[2][CB_N][CPAD];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int wm = warp >> 1, wn = warp & 1;
	const int g = lane >> 2, t = lane & 3;
	const int64_t M = (int64_t)a.N * a.H * a.W;
	const int64_t m0 = (int64_t)blockIdx.x * CB_M;
	const int n0 = blockIdx.y * CB_N;
	const int K = 9 * a.Ci;
	const int ksteps = K / CB_K;
	// this thread's load slots: one 16-byte vector of A and one of B per k-step
	const int lrow = tid >> 1, lhalf = tid & 1;
	const int64_t lm = m0 + lrow;
	int ln = 0, ly = 0, lx = 0;
	if (lm < M) {
		ln = (int)(lm / ((int64_t)a.H * a.W));
		const int r = (int)(lm - (int64_t)ln * a.H * a.W);
		ly = r / a.W;
		lx = r - ly * a.W;
	}
	const int lco = n0 + lrow;
	auto load_a = [&](int ks) -> uint4 {
		const int k0 = ks * CB_K;
		const int tap = k0 / a.Ci, ci0 = k0 - tap * a.Ci + lhalf * 8;
		const int yy = ly + tap / 3 - 1, xx = lx + tap % 3 - 1;
		uint4 v = make_uint4(0, 0, 0, 0);
		if (lm < M && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W)
			v = *reinterpret_cast<const uint4 *>(a.x + (((int64_t)ln * a.H + yy) * a.W + xx) * a.Ci + ci0);
		return v;
	};
	auto load_b = [&](int ks) -> uint4 {
		uint4 v = make_uint4(0, 0, 0, 0);
		if (lco < a.Co) v = *reinterpret_cast<const uint4 *>(a.w + (int64_t)lco * K + ks * CB_K + lhalf * 8);
		return v;
	};
	float acc[2][4][4];
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j)
#pragma unroll
			for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
	uint4 ra = load_a(0), rb = load_b(0);
	*reinterpret_cast<uint4 *>(&As[0][lrow][lhalf * 8]) = ra;
	*reinterpret_cast<uint4 *>(&Bs[0][lrow][lhalf * 8]) = rb;
	__syncthreads();
	for (int ks = 0; ks < ksteps; ++ks) {
		const int cur = ks & 1;
		if (ks + 1 < ksteps) {
			ra = load_a(ks + 1);
			rb = load_b(ks + 1);
		}
		uint32_t af[2][4], bfr[4][2];
#pragma unroll
		for (int i = 0; i < 2; ++i) {
			const int r = wm * 32 + i * 16 + g;
			af[i][0] = *reinterpret_cast<const uint32_t *>(&As[cur][r][2 * t]);
			af[i][1] = *reinterpret_cast<const uint32_t *>(&As[cur][r + 8][2 * t]);
			af[i][2] = *reinterpret_cast<const uint32_t *>(&As[cur][r][2 * t + 8]);
			af[i][3] = *reinterpret_cast<const uint32_t *>(&As[cur][r + 8][2 * t + 8]);
		}
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const int c = wn * 32 + j * 8 + g;
			bfr[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[cur][c][2 * t]);
			bfr[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[cur][c][2 * t + 8]);
		}
#pragma unroll
		for (int i = 0; i < 2; ++i)
#pragma unroll
			for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
		if (ks + 1 < ksteps) {
			*reinterpret_cast<uint4 *>(&As[cur ^ 1][lrow][lhalf * 8]) = ra;
			*reinterpret_cast<uint4 *>(&Bs[cur ^ 1][lrow][lhalf * 8]) = rb;
		}
		__syncthreads();
	}
	// epilogue: bias, ReLU, bf16 store
#pragma unroll
	for (int i = 0; i < 2; ++i) {
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const int co = n0 + wn * 32 + j * 8 + 2 * t;
			if (co >= a.Co) continue;
			const float b0 = a.use_bias ? a.bias[co] : 0.f, b1 = a.use_bias ? a.bias[co + 1] : 0.f;
#pragma unroll
			for (int h = 0; h < 2; ++h) {
				const int64_t m = m0 + wm * 32 + i * 16 + g + h * 8;
				if (m >= M) continue;
				float v0 = acc[i][j][2 * h] + b0, v1 = acc[i][j][2 * h + 1] + b1;
				if (a.relu) {
					v0 = fmaxf(v0, 0.f);
					v1 = fmaxf(v1, 0.f);
				}
				*reinterpret_cast<__nv_bfloat162 *>(a.y + m * a.Co + co) = __floats2bfloat162_rn(v0, v1);
			}
		}
	}
}

// ---- the same implicit-GEMM convolution on the 5th-generation tensor cores ------
//
// One CTA (4 warps) computes a 128-pixel x Co tile (M = 128 rows of the
// accumulator in TMEM, N = Co columns, Co <= 256).  K = 9 Ci runs in chunks of
// 64 through a TC_STAGES-deep ring of shared-memory stages filled by cp.async
// (16-byte vectors; taps outside the image and rows past M are zero-filled).
// One thread issues tcgen05.mma (kind::f16, bf16 x bf16 -> FP32, both operands
// K-major, no swizzle) per 16-wide K step and commits each chunk to that
// stage's mbarrier; a stage is refilled only after its mbarrier shows the MMAs
// that read it are done.  The epilogue reads TMEM with tcgen05.ld, adds bias,
// applies ReLU and stores bf16.  Every wait is bounded: on timeout the CTA
// records the failure in *err, stops issuing, and still frees its TMEM.
//
// Shared-memory operand layout (K-major, no swizzle): 8-row x 16-byte core
// matrices; element (r, k) at (r / 8) * 1024 + (k / 8) * 128 + (r % 8) * 16 +
// (k % 8) * 2, i.e. leading-dimension (K) core-matrix stride 128 B and
// stride-dimension (M/N) 8-row-group stride 1024 B.  The B stages come first
// in shared memory so that every address a descriptor can form stays inside
// the CTA's allocation.

constexpr int TC_M = 128, TC_K = 64;

struct TcArgs {
	const bf16 *x; // (N,H,W,Ci)
	const bf16 *w; // (Co,3,3,Ci)
	const float *bias;
	bf16 *y;       // (N,H,W,Co)
	int N, H, W, Ci, Co;
	int relu, use_bias;
	int stages;
	uint32_t tmem_cols;
	int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor, no swizzle: start address, leading and
// stride byte offsets (16-byte units), version 1 (tcgen05), base offset 0.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo = 128u, uint32_t sbo = 1024u) {
	uint64_t d = 0;
	d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
	d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
	d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
	d |= (uint64_t)1 << 46;
	return d;
}

// Descriptor of a shared-memory operand at 16-byte unit addr16 = address >> 4:
// the address field is the low 14 bits, so adding n to the descriptor moves
// the operand by 16 n bytes (shared addresses stay below 2^18).
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
	asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
				 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
				 "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void *g, bool valid) {
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(g), "r"(valid ? 16 : 0));
}

// the same through L1: the nine taps of an implicit-GEMM tile re-read the same
// input rows, which L1 then serves
__device__ __forceinline__ void cp_async16_l1(uint32_t saddr, const void *g, bool valid) {
	asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(g), "r"(valid ? 16 : 0));
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
	asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t parity) {
	uint32_t ok;
	asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
				 : "=r"(ok)
				 : "r"(addr), "r"(parity)
				 : "memory");
	return ok != 0;
}

// Bounded wait (about a second of SM clock); false on timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
	const long long t0 = clock64();
	while (!mbar_try(addr, parity))
		if (clock64() - t0 > 2000000000ll) return false;
	return true;
}

__global__ void __launch_bounds__(128) conv_tc(TcArgs a) {
	extern __shared__ __align__(1024) uint8_t sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int S = a.stages;
	const uint32_t b_bytes = (uint32_t)a.Co * 128u; // one B stage: Co rows x 64 K
	const uint32_t a_bytes = TC_M * 128u;           // one A stage
	uint8_t *Bs = sm;
	uint8_t *As = sm + (size_t)S * b_bytes;
	uint64_t *mbar = reinterpret_cast<uint64_t *>(As + (size_t)S * a_bytes);
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + S);

	const int64_t M = (int64_t)a.N * a.H * a.W;
	const int64_t m0 = (int64_t)blockIdx.x * TC_M;
	const int K = 9 * a.Ci;
	const int nk = (K + TC_K - 1) / TC_K;

	if (tid == 0) {
		for (int s = 0; s < S; ++s)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar + s)));
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
					 "r"(a.tmem_cols));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	const uint32_t tmem = *tmem_slot;

	// this thread's 8 A vectors per stage: v = tid + 128 i -> row v / 8, group v % 8
	int64_t a_pix[8];
	int a_y[8], a_x[8];
#pragma unroll
	for (int i = 0; i < 8; ++i) {
		const int v = tid + 128 * i;
		const int64_t m = m0 + (v >> 3);
		a_pix[i] = -1;
		a_y[i] = a_x[i] = 0;
		if (m < M) {
			const int64_t n = m / ((int64_t)a.H * a.W);
			const int r = (int)(m - n * a.H * a.W);
			a_y[i] = r / a.W;
			a_x[i] = r - a_y[i] * a.W;
			a_pix[i] = n * a.H * a.W;
		}
	}
	auto load_chunk = [&](int c, int s) {
		const uint32_t abase = smem_u32(As + (size_t)s * a_bytes);
		const uint32_t bbase = smem_u32(Bs + (size_t)s * b_bytes);
#pragma unroll
		for (int i = 0; i < 8; ++i) {
			const int v = tid + 128 * i, row = v >> 3, g = v & 7;
			const int k = c * TC_K + g * 8;
			if (k >= K) continue;
			const int tap = k / a.Ci, ci = k - tap * a.Ci;
			const int yy = a_y[i] + tap / 3 - 1, xx = a_x[i] + tap % 3 - 1;
			const bool ok = a_pix[i] >= 0 && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
			const bf16 *src = ok ? a.x + (a_pix[i] + (int64_t)yy * a.W + xx) * a.Ci + ci : a.x;
			cp_async16_l1(abase + (row >> 3) * 1024 + g * 128 + (row & 7) * 16, src, ok);
		}
		for (int v = tid; v < a.Co * 8; v += 128) {
			const int row = v >> 3, g = v & 7;
			const int k = c * TC_K + g * 8;
			if (k >= K) continue;
			cp_async16(bbase + (row >> 3) * 1024 + g * 128 + (row & 7) * 16, a.w + (int64_t)row * K + k, true);
		}
	};

	// instruction descriptor: D f32, A bf16, B bf16, both K-major, N = Co, M = 128
	const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(a.Co >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

	for (int c = 0; c < S - 1; ++c) {
		if (c < nk) load_chunk(c, c);
		cp_async_commit();
	}
	int issued = -1;  // last chunk whose MMAs were issued (the same in every thread)
	int my_fail = 0;  // this thread saw a wait time out
	for (int c = 0; c < nk; ++c) {
		const int s = c % S;
		// chunk c has landed once at most S - 2 younger groups are pending
		if (S == 2) cp_async_wait<0>();
		else if (S == 3) cp_async_wait<1>();
		else cp_async_wait<2>();
		asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
		if (__syncthreads_or(my_fail)) break; // the same decision in every thread
		issued = c;
		if (tid == 0) {
			asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
			const int ksteps = (K - c * TC_K < TC_K ? K - c * TC_K : TC_K) / 16;
			const uint32_t abase = smem_u32(As + (size_t)s * a_bytes);
			const uint32_t bbase = smem_u32(Bs + (size_t)s * b_bytes);
			for (int j = 0; j < ksteps; ++j) {
				const uint64_t ad = umma_desc(abase + j * 256), bd = umma_desc(bbase + j * 256);
				const uint32_t acc = (c > 0 || j > 0) ? 1u : 0u;
				asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
							 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
							 "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
			}
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
				smem_u32(mbar + s)));
		}
		// refill the stage chunk c - 1 used, once its MMAs are done
		const int cn = c + S - 1;
		if (cn < nk) {
			if (c >= 1 && !mbar_wait(smem_u32(mbar + (c - 1) % S), (uint32_t)(((c - 1) / S) & 1))) my_fail = 1;
			else load_chunk(cn, cn % S);
		}
		cp_async_commit();
	}
	cp_async_wait<0>();
	// the commit of the last issued chunk covers every MMA issued before it;
	// wait for it (bounded) even after a failure, before TMEM is freed
	if (issued >= 0 && !mbar_wait(smem_u32(mbar + issued % S), (uint32_t)((issued / S) & 1))) my_fail = 1;
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	const int failed = __syncthreads_or(my_fail || issued != nk - 1);
	if (failed) {
		if (tid == 0) atomicExch(a.err, 1);
	} else {
		// epilogue: warp w owns TMEM lanes (= tile rows) 32 w .. 32 w + 31
		const int row = warp * 32 + lane;
		const int64_t m = m0 + row;
		for (int c0 = 0; c0 < a.Co; c0 += 16) {
			uint32_t r[16];
			const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
			asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
						 "[%16];\n"
						 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
						   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
						   "=r"(r[14]), "=r"(r[15])
						 : "r"(taddr));
			asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
			if (m < M) {
				__align__(16) __nv_bfloat162 o[8];
#pragma unroll
				for (int q = 0; q < 8; ++q) {
					float v0 = __uint_as_float(r[2 * q]), v1 = __uint_as_float(r[2 * q + 1]);
					if (a.use_bias) {
						v0 += a.bias[c0 + 2 * q];
						v1 += a.bias[c0 + 2 * q + 1];
					}
					if (a.relu) {
						v0 = fmaxf(v0, 0.f);
						v1 = fmaxf(v1, 0.f);
					}
					o[q] = __floats2bfloat162_rn(v0, v1);
				}
				uint4 *dst = reinterpret_cast<uint4 *>(a.y + m * a.Co + c0);
				dst[0] = *reinterpret_cast<const uint4 *>(&o[0]);
				dst[1] = *reinterpret_cast<const uint4 *>(&o[4]);
			}
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	if (warp == 0) {
		asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tmem_cols));
	}
}

// ---- the convolution from a TMA-loaded halo ----------------------------------------
//
// One CTA computes RT M tiles of 128 pixels by all Co outputs, each tile in
// its own TMEM accumulator; the weights of a chunk of CK input channels serve
// all RT tiles.  For a layer whose width is a multiple of 128 a tile is 128
// consecutive pixels of one image row (MR = 1) and the CTA takes RT
// consecutive rows; the chunk's input reaches shared memory as one halo, a
// TMA tile of RT + 2 rows x 130 pixels x CK channels at (x0 - 1 .. x0 + 128,
// y0 - 1 .. y0 + RT), zero-filled by the copy outside the image, laid out
// channel-group major: element (row r, pixel p, channel 8 g + e) at
// ((g * rows + r) * P + p) * 16 + 2 e with P = 130.  Pixels are 16 bytes
// apart within a channel group, so the A operand of tap (dy, dx) -- the 128
// pixels shifted by (dy, dx) -- is the same halo read through a descriptor
// whose start moves by ((r + dy) * P + dx) * 16 bytes for tile r (K-major, no
// swizzle: core matrices of 8 pixels x 8 channels, 8-pixel stride SBO = 128
// B, channel-group stride LBO = rows * P * 16 B).  For a narrower layer (W
// dividing 128) a tile is MR = 128 / W whole image rows, which a single
// descriptor covers only if consecutive rows are W pixels apart; so the halo
// comes as NC = 3 copies of RT * MR + 2 rows x W pixels (P = W), taken at x =
// -1, 0, +1 (zero-filled at the image edge), and the shift dx selects the
// copy instead of moving by a pixel.  The nine taps of a chunk read one
// halo, where an im2col tile holds every input value nine times.  The chunk's
// weights (Co x 9 x CK) arrive by TMA as [g][tap][co][8 channels]: B of tap t
// and channel groups 2j, 2j + 1 at ((2 j) * 9 + t) * Co * 16, LBO = 9 * Co *
// 16, SBO = 128.  One thread issues the copies (one mbarrier per stage counts
// their bytes) and the MMAs (committed to the stage's second mbarrier, which
// frees the stage for the chunk S later).  Every wait is bounded; on timeout
// the CTA records the failure in *err, waits (bounded) for the copies it
// issued, and frees its TMEM.

constexpr int HX = 130; // halo pixels per row

struct HaloArgs {
	const float *bias;
	bf16 *y; // (N,H,W,Co)
	int N, H, W, Ci, Co, CK;
	int RT;        // accumulators (M tiles of 128 pixels) per CTA
	int NC, P, MR; // halo copies (1, or 3 shifted by dx), pixels per copy row, image rows per M tile
	int CoT;       // output channels per CTA (Co / CoT CTAs share a pixel tile)
	int relu, use_bias;
	int stages;
	uint32_t copy_bytes;       // one halo copy of a chunk
	uint32_t a_bytes, b_bytes; // bytes of the TMA boxes of a chunk (NC copies; the weights)
	uint32_t a_span, stage_bytes; // B's offset in a stage and the stage size (1024-byte multiples)
	uint32_t tmem_cols;
	int *err;
};

__device__ __forceinline__ void mbar_expect_tx(uint32_t addr, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(addr), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *map, uint32_t mbar, int c0, int c1, int c2,
											int c3, int c4) {
	asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, "
				 "%6, %7}], [%2];\n" ::"r"(dst),
				 "l"(map), "r"(mbar), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
				 : "memory");
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, uint32_t mbar, int c0, int c1, int c2,
											int c3) {
	asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, "
				 "%6}], [%2];\n" ::"r"(dst),
				 "l"(map), "r"(mbar), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
				 : "memory");
}

__global__ void __launch_bounds__(128) conv_halo(const __grid_constant__ CUtensorMap tx,
												 const __grid_constant__ CUtensorMap tw, HaloArgs a) {
	extern __shared__ __align__(1024) uint8_t sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int S = a.stages;
	uint64_t *full = reinterpret_cast<uint64_t *>(sm + (size_t)S * a.stage_bytes);
	uint64_t *done = full + S;
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + S);

	const int tpr = a.W >= 128 ? a.W / 128 : 1; // tiles per row
	const int cot = a.Co / a.CoT;
	const int co0 = (int)(blockIdx.x % cot) * a.CoT;
	const int tile = (int)(blockIdx.x / cot);
	const int x0 = (tile % tpr) * 128;
	const int row = (tile / tpr) * a.RT * a.MR; // n * H + y0
	const int n = row / a.H, yy = row - n * a.H;
	const int RT = a.RT;
	const int nch = a.Ci / a.CK;
	const uint32_t tx_bytes = a.a_bytes + a.b_bytes;

	if (tid == 0) {
		for (int s = 0; s < S; ++s) {
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(full + s)));
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(done + s)));
		}
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
					 "r"(a.tmem_cols));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	const uint32_t tmem = *tmem_slot;

	// instruction descriptor: D f32, A bf16, B bf16, both K-major, N = Co, M = 128
	const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(a.CoT >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
	const uint32_t lbo_a = (uint32_t)(RT * a.MR + 2) * (uint32_t)a.P * 16u, lbo_b = 9u * (uint32_t)a.CoT * 16u;
	// the shift dx: a pixel (one copy) or a copy (three)
	const uint64_t dx_step = a.NC == 3 ? (uint64_t)(a.copy_bytes >> 4) : 1u;
	int fail = 0, loaded = 0, issued = -1;
	if (tid == 0) {
		auto load = [&](int c) {
			const int s = c % S;
			const uint32_t base = smem_u32(sm + (size_t)s * a.stage_bytes);
			mbar_expect_tx(smem_u32(full + s), tx_bytes);
			for (int cp = 0; cp < a.NC; ++cp)
				tma_load_5d(base + (uint32_t)cp * a.copy_bytes, &tx, smem_u32(full + s), 0, x0 - 1 + (a.NC == 3 ? cp : 0),
							yy - 1, c * (a.CK / 8), n);
			tma_load_4d(base + a.a_span, &tw, smem_u32(full + s), 0, co0, 0, c * (a.CK / 8));
		};
		for (int c = 0; c < S && c < nch; ++c) load(c);
		loaded = S < nch ? S : nch;
		for (int c = 0; c < nch; ++c) {
			const int s = c % S;
			if (!mbar_wait(smem_u32(full + s), (uint32_t)((c / S) & 1))) {
				fail = 1;
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
			const uint32_t abase = smem_u32(sm + (size_t)s * a.stage_bytes);
			const uint32_t bbase = abase + a.a_span;
			// descriptors stepped by constant adds (16-byte units)
			const uint64_t ad0 = umma_desc(abase, lbo_a, 128u), bd0 = umma_desc(bbase, lbo_b, 128u);
			for (int j = 0; j < a.CK / 16; ++j)
				for (int t = 0; t < 9; ++t) {
					const int dy = t / 3, dx = t % 3;
					const uint64_t bd = bd0 + (uint64_t)((2 * j * 9 + t) * a.CoT);
					const uint32_t acc = (c > 0 || j > 0 || t > 0) ? 1u : 0u;
					uint64_t ad = ad0 + (uint64_t)(2 * j) * (lbo_a >> 4) + (uint64_t)(dy * a.P) + (uint64_t)dx * dx_step;
					for (int r = 0; r < RT; ++r) {
						umma_f16(tmem + (uint32_t)(r * a.CoT), ad, bd, idesc, acc);
						ad += (uint64_t)(a.MR * a.P);
					}
				}
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
				smem_u32(done + s)));
			issued = c;
			// refill the stage chunk c - 1 used with chunk c - 1 + S once its
			// MMAs are done (chunk c's are queued behind them meanwhile)
			if (c >= 1 && c - 1 + S < nch) {
				const int cp = c - 1;
				if (!mbar_wait(smem_u32(done + cp % S), (uint32_t)((cp / S) & 1))) {
					fail = 1;
					break;
				}
				load(cp + S);
				++loaded;
			}
		}
		// the last commit covers every MMA issued before it
		if (issued >= 0 && !mbar_wait(smem_u32(done + issued % S), (uint32_t)((issued / S) & 1))) fail = 1;
		// copies issued but not consumed (after a failure): wait for them
		// (bounded) before the CTA's shared memory can be reused
		for (int c = issued + 1; c < loaded; ++c) mbar_wait(smem_u32(full + c % S), (uint32_t)((c / S) & 1));
		if (fail || issued != nch - 1) atomicExch(a.err, 1);
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	const int failed = __syncthreads_or(tid == 0 && (fail || issued != nch - 1));
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	if (!failed) {
		// epilogue: warp w owns TMEM lanes (= tile pixels) 32 w .. 32 w + 31
		const int px = warp * 32 + lane;
		for (int rr = 0; rr < RT; ++rr) {
			for (int c0 = 0; c0 < a.CoT; c0 += 16) {
				const int64_t m = ((int64_t)(row + rr * a.MR) * a.W) + x0 + px;
				uint32_t r[16];
				const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(rr * a.CoT + c0);
				asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
							 "[%16];\n"
							 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
							   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
							   "=r"(r[14]), "=r"(r[15])
							 : "r"(taddr));
				asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
				__align__(16) __nv_bfloat162 o[8];
#pragma unroll
				for (int q = 0; q < 8; ++q) {
					float v0 = __uint_as_float(r[2 * q]), v1 = __uint_as_float(r[2 * q + 1]);
					if (a.use_bias) {
						v0 += a.bias[co0 + c0 + 2 * q];
						v1 += a.bias[co0 + c0 + 2 * q + 1];
					}
					if (a.relu) {
						v0 = fmaxf(v0, 0.f);
						v1 = fmaxf(v1, 0.f);
					}
					o[q] = __floats2bfloat162_rn(v0, v1);
				}
				uint4 *dst = reinterpret_cast<uint4 *>(a.y + m * a.Co + co0 + c0);
				dst[0] = *reinterpret_cast<const uint4 *>(&o[0]);
				dst[1] = *reinterpret_cast<const uint4 *>(&o[4]);
			}
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	if (warp == 0) {
		asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tmem_cols));
	}
}

// ---- row-run convolution: resident weights, input-row stationary ----------------
//
// For layers whose weights and four input rows fit shared memory: one CTA
// computes RL consecutive output rows of one 128-pixel column tile (n, x0).
// The weights (Co x 9 x Ci) arrive once, by TMA, as [g][kx][ky][co][8
// channels]: for a column shift dx the three kernel rows' Co x 8 blocks are
// consecutive, so B rows (ky, co) form one operand of up to 3 Co rows (8-row
// stride 128 B, channel-group stride 9 * Co * 16 B).  Input rows y0 - 1 ..
// y0 + RL stream once each through a ring of NR slots, each row a TMA box of
// 130 pixels x Ci channels, zero-filled outside the image, laid out (channel
// group, pixel, 8 channels): the A operand of input row X and shift dx is
// the slot read from pixel dx (K-major, no swizzle: 8-pixel stride 128 B,
// channel-group stride 130 * 16 B).  Input row X feeds output rows X + 1, X,
// X - 1 through kernel rows ky = 0, 1, 2; the accumulators of consecutive
// output rows sit in TMEM in decreasing row order (Co columns each), so one
// MMA with N = (number of kernel rows) x Co adds X's contribution to up to
// three output rows at once: the A operand is read once per input row
// instead of three times.  Accumulators come in blocks of RB output rows,
// double-buffered (2 RB Co columns); an MMA whose output rows fall in two
// blocks is split in two.  The epilogue warps zero a block's columns after
// draining it (and both blocks at the start), so every MMA accumulates.
// Warp roles: warp 0 issues the copies, warp 1 the MMAs, warps 2-5 drain the
// accumulators (bias, ReLU, bf16, NHWC stores) row by row as each output
// row completes.  mbarriers: row_full / row_empty per ring slot (TMA bytes;
// the MMAs that read the row), w_full, row_done per accumulator row slot
// (MMA commit) and acc_empty per block buffer (the four epilogue warps, once
// the block's rows are drained and zeroed).  Every wait is bounded; on timeout the thread records the failure
// in *err and stops, the producer waits (bounded) for the copies it issued,
// and the MMA thread for its MMAs before TMEM is freed.

struct RowsArgs {
	const float *bias;
	bf16 *y; // (N,H,W,Co)
	int N, H, W, Ci, Co;
	int relu, use_bias;
	int RL, NR, runs; // output rows per CTA, ring slots, CTAs per column tile
	int RB, KY;       // output rows per accumulator block, kernel rows per MMA (N = KY Co <= 256)
	uint32_t row_bytes, row_span, w_bytes, w_off, mbar_off;
	uint32_t tmem_cols;
	int *err;
};

__global__ void __launch_bounds__(192) conv_rows(const __grid_constant__ CUtensorMap tx,
												 const __grid_constant__ CUtensorMap tw, RowsArgs a) {
	extern __shared__ __align__(1024) uint8_t sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int NR = a.NR, RB = a.RB;
	uint64_t *row_full = reinterpret_cast<uint64_t *>(sm + a.mbar_off);
	uint64_t *row_empty = row_full + NR;
	uint64_t *w_full = row_empty + NR;
	uint64_t *acc_empty = w_full + 1;  // [2]: a block buffer drained and zeroed
	uint64_t *row_done = acc_empty + 2; // [2 RB]: an output row's accumulator complete
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(row_done + 2 * RB);

	const int tpr = a.W / 128;
	const int colt = (int)(blockIdx.x / (unsigned)a.runs), run = (int)(blockIdx.x % (unsigned)a.runs);
	const int n = colt / tpr, x0 = (colt % tpr) * 128;
	const int y0 = run * a.RL;
	const int rows = a.H - y0 < a.RL ? a.H - y0 : a.RL;
	const int nx = rows + 2;
	constexpr uint32_t R = HX * 16u;
	// TMEM column of output row r (0 .. rows - 1): block r / RB in buffer
	// (r / RB) & 1, rows of a block in decreasing order; slot_of(r) numbers
	// the 2 RB row slots, used by rows r, r + 2 RB, ...
	auto slot_of = [&](int r) -> int { return ((r / RB) & 1) * RB + (RB - 1 - r % RB); };
	auto col_of = [&](int r) -> uint32_t { return (uint32_t)(slot_of(r) * a.Co); };

	if (tid == 0) {
		for (int s = 0; s < NR; ++s) {
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(row_full + s)));
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(row_empty + s)));
		}
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(w_full)));
		for (int b = 0; b < 2; ++b)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(smem_u32(acc_empty + b)));
		for (int k = 0; k < 2 * RB; ++k)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(row_done + k)));
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
	}
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
					 "r"(a.tmem_cols));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	const uint32_t tmem = *tmem_slot;

	if (warp == 0) {
		if (lane == 0) { // producer
			int fail = 0, issued = 0;
			mbar_expect_tx(smem_u32(w_full), a.w_bytes);
			tma_load_5d(smem_u32(sm + a.w_off), &tw, smem_u32(w_full), 0, 0, 0, 0, 0);
			for (int j = 0; j < nx; ++j) {
				const int s = j % NR;
				if (j >= NR && !mbar_wait(smem_u32(row_empty + s), (uint32_t)(((j / NR) - 1) & 1))) {
					fail = 1;
					break;
				}
				mbar_expect_tx(smem_u32(row_full + s), a.row_bytes);
				tma_load_5d(smem_u32(sm + (size_t)s * a.row_span), &tx, smem_u32(row_full + s), 0, x0 - 1, 0,
							y0 - 1 + j, n);
				issued = j + 1;
			}
			// the last copy of each slot has landed before the CTA can end
			for (int j = issued > NR ? issued - NR : 0; j < issued; ++j)
				mbar_wait(smem_u32(row_full + j % NR), (uint32_t)((j / NR) & 1));
			mbar_wait(smem_u32(w_full), 0u);
			if (fail) atomicExch(a.err, 1);
		}
	} else if (warp == 1) {
		if (lane == 0) { // MMA issuer: input row j feeds output rows j - ky, ky = 0, 1, 2
			// D f32, A bf16, B bf16, both K-major, M = 128, N = nky * Co
			const uint32_t idesc0 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 4) << 24);
			const uint32_t lbo_b = 9u * (uint32_t)a.Co * 16u;
			const uint64_t bd0 = umma_desc(smem_u32(sm + a.w_off), lbo_b, 128u);
			const uint64_t a_k = (2u * R) >> 4, b_k = 18u * (uint64_t)a.Co;
			const int nk = a.Ci / 16;
			int fail = !mbar_wait(smem_u32(w_full), 0u), done = 0; // output rows committed
			for (int j = 0; j < nx && !fail; ++j) {
				if (!mbar_wait(smem_u32(row_full + j % NR), (uint32_t)((j / NR) & 1))) {
					fail = 1;
					break;
				}
				// the first output row of a block: its buffer must be drained
				// (and zeroed) by the epilogue
				if (j < rows && j % RB == 0) {
					const int blk = j / RB;
					if (!mbar_wait(smem_u32(acc_empty + (blk & 1)), (uint32_t)((blk >> 1) & 1))) {
						fail = 1;
						break;
					}
				}
				asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
				const int kmin = j - rows + 1 > 0 ? j - rows + 1 : 0, kmax = j < 2 ? j : 2;
				const uint64_t ad_row = umma_desc(smem_u32(sm + (size_t)(j % NR) * a.row_span), R, 128u);
				// groups of kernel rows [k0, k1] whose output rows share a block
				for (int k0 = kmin; k0 <= kmax;) {
					int k1 = k0;
					while (k1 + 1 <= kmax && k1 + 1 - k0 < a.KY && (j - k1 - 1) / RB == (j - k0) / RB) ++k1;
					const int nky = k1 - k0 + 1;
					const uint32_t idesc = idesc0 | ((uint32_t)((nky * a.Co) >> 3) << 17);
					const uint32_t d_tmem = tmem + col_of(j - k0);
					for (int dx = 0; dx < 3; ++dx) {
						uint64_t ad = ad_row + (uint64_t)dx;
						uint64_t bd = bd0 + (uint64_t)((dx * 3 + k0) * a.Co);
#pragma unroll 2
						for (int k = 0; k < nk; ++k) {
							umma_f16(d_tmem, ad, bd, idesc, 1u);
							ad += a_k;
							bd += b_k;
						}
					}
					k0 = k1 + 1;
				}
				// input row j is read by no later MMA
				asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
					smem_u32(row_empty + j % NR)));
				// output row j - 2 is complete
				const int rl = j - 2;
				if (rl >= 0 && rl < rows) {
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
						smem_u32(row_done + slot_of(rl))));
					done = rl + 1;
				}
			}
			// the MMAs and their arrivals have finished before TMEM is freed
			if (done > 0)
				mbar_wait(smem_u32(row_done + slot_of(done - 1)), (uint32_t)(((done - 1) / (2 * RB)) & 1));
			if (fail) atomicExch(a.err, 1);
		}
	} else { // epilogue: warp w reads TMEM lanes (pixels) 32 (w % 4) .. + 31
		const int q = warp & 3;
		const int px = q * 32 + lane;
		const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
		uint32_t zero[16];
#pragma unroll
		for (int k = 0; k < 16; ++k) zero[k] = 0u;
		auto zero_cols = [&](uint32_t c_begin, uint32_t c_end) {
			for (uint32_t c = c_begin; c < c_end; c += 16)
				asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(
								 lane_base + c),
							 "r"(zero[0]), "r"(zero[1]), "r"(zero[2]), "r"(zero[3]), "r"(zero[4]), "r"(zero[5]),
							 "r"(zero[6]), "r"(zero[7]), "r"(zero[8]), "r"(zero[9]), "r"(zero[10]), "r"(zero[11]),
							 "r"(zero[12]), "r"(zero[13]), "r"(zero[14]), "r"(zero[15]));
			asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
		};
		// both buffers start zeroed and free
		zero_cols(0u, 2u * (uint32_t)(RB * a.Co));
		asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
		__syncwarp();
		if (lane == 0)
			for (int b = 0; b < 2; ++b)
				asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(acc_empty + b)) : "memory");
		int fail = 0;
		for (int r = 0; r < rows; ++r) {
			if (!mbar_wait(smem_u32(row_done + slot_of(r)), (uint32_t)((r / (2 * RB)) & 1))) {
				fail = 1;
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
			{
				const int64_t m = ((int64_t)n * a.H + y0 + r) * a.W + x0 + px;
				for (int c0 = 0; c0 < a.Co; c0 += 16) {
					uint32_t v[16];
					asm volatile(
						"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
						"[%16];\n"
						: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
						  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
						  "=r"(v[15])
						: "r"(lane_base + col_of(r) + (uint32_t)c0));
					asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
					__align__(16) __nv_bfloat162 o[8];
#pragma unroll
					for (int k = 0; k < 8; ++k) {
						float v0 = __uint_as_float(v[2 * k]), v1 = __uint_as_float(v[2 * k + 1]);
						if (a.use_bias) {
							v0 += a.bias[c0 + 2 * k];
							v1 += a.bias[c0 + 2 * k + 1];
						}
						if (a.relu) {
							v0 = fmaxf(v0, 0.f);
							v1 = fmaxf(v1, 0.f);
						}
						o[k] = __floats2bfloat162_rn(v0, v1);
					}
					uint4 *dst = reinterpret_cast<uint4 *>(a.y + m * a.Co + c0);
					dst[0] = *reinterpret_cast<const uint4 *>(&o[0]);
					dst[1] = *reinterpret_cast<const uint4 *>(&o[4]);
				}
			}
			// zero the row's columns for the slot's next use; after the
			// block's last row, free the block buffer
			zero_cols(col_of(r), col_of(r) + (uint32_t)a.Co);
			if (r % RB == RB - 1 || r == rows - 1) {
				asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
				__syncwarp();
				if (lane == 0)
					asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(acc_empty + ((r / RB) & 1)))
								 : "memory");
			}
		}
		if (fail && lane == 0) atomicExch(a.err, 1);
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	if (warp == 1) {
		asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tmem_cols));
	}
}

// ---- weight gradient on the tensor cores -----------------------------------------
//
// D[kcol][co] = sum over a chunk of pixels m of im2col(X)[m][kcol] dY[m][co]:
// M = 128 columns kcol = tap * Ci + ci of the weight, N = Co, K = pixels.  In
// NHWC memory both operands run along M/N (8 consecutive kcol of one pixel,
// or 8 consecutive co, are 16 contiguous bytes), so they are staged
// MN-major: core matrices of 8 pixels (16-byte rows) x 8 elements; element
// (r, m) of a stage at (r / 8) * 1024 + (m / 8) * 128 + (m % 8) * 16 +
// (r % 8) * 2.  For the no-swizzle MN-major layout the descriptor's leading
// byte offset is the K-direction stride (128 B between 8-pixel groups) and
// its stride byte offset the M/N-direction stride (1024 B).  Pipeline, bounded waits
// and TMEM handling as conv_tc; the epilogue writes this chunk's FP32
// partial sums partial[chunk][co][kcol], reduced later in fixed chunk order.

struct TcWgradArgs {
	const bf16 *x;  // (N,H,W,Ci) forward input
	const bf16 *dy; // (N,H,W,Co) gradient at the pre-activation
	float *partial; // (chunks, Co, 9 Ci)
	int N, H, W, Ci, Co;
	int64_t chunk;  // pixels per chunk (multiple of 64)
	int stages;
	uint32_t tmem_cols;
	int *err;
};

__global__ void __launch_bounds__(128) conv_wgrad_tc(TcWgradArgs a) {
	extern __shared__ __align__(1024) uint8_t sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int S = a.stages;
	const uint32_t b_bytes = (uint32_t)a.Co * 128u;
	const uint32_t a_bytes = TC_M * 128u;
	uint8_t *Bs = sm;
	uint8_t *As = sm + (size_t)S * b_bytes;
	uint64_t *mbar = reinterpret_cast<uint64_t *>(As + (size_t)S * a_bytes);
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + S);

	const int64_t M = (int64_t)a.N * a.H * a.W;
	const int K = 9 * a.Ci;
	const int kc0 = blockIdx.x * TC_M;
	const int64_t p_begin = (int64_t)blockIdx.y * a.chunk;
	const int64_t p_end = p_begin + a.chunk < M ? p_begin + a.chunk : M;
	const int nk = (int)((p_end - p_begin + TC_K - 1) / TC_K);
	const int HW = a.H * a.W;

	if (tid == 0) {
		for (int s = 0; s < S; ++s)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar + s)));
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
					 "r"(a.tmem_cols));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	const uint32_t tmem = *tmem_slot;

	const int cog = a.Co >> 3; // 16-byte groups of dY per pixel
	// This thread's A vectors: kcol group g = tid % 16 (the same in every
	// chunk, so its tap and channel are fixed) and pixels tid / 16 + 8 i.
	const int ga = tid & 15, pa = tid >> 4;
	const int ka = kc0 + ga * 8;
	const int tap_a = ka < K ? ka / a.Ci : 0, ci_a = ka - tap_a * a.Ci;
	const int dy_a = tap_a / 3 - 1, dx_a = tap_a % 3 - 1;
	auto load_chunk = [&](int c, int s) {
		const uint32_t abase = smem_u32(As + (size_t)s * a_bytes);
		const uint32_t bbase = smem_u32(Bs + (size_t)s * b_bytes);
		const int64_t q0 = p_begin + (int64_t)c * TC_K;
		// A: 64 pixels x 16 groups of 8 kcol; (n, y, x) of the first pixel by
		// one division, then stepped by 8 pixels with carries
		int64_t m = q0 + pa;
		int64_t n = m / HW;
		int r = (int)(m - n * HW);
		int y = r / a.W, x = r - (r / a.W) * a.W;
#pragma unroll
		for (int i = 0; i < 8; ++i) {
			const int pp = pa + 8 * i;
			const int yy = y + dy_a, xx = x + dx_a;
			const bool ok = m < p_end && ka < K && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
			const bf16 *src = ok ? a.x + ((n * a.H + yy) * (int64_t)a.W + xx) * a.Ci + ci_a : a.x;
			cp_async16(abase + ga * 1024 + (pp >> 3) * 128 + (pp & 7) * 16, src, ok);
			m += 8;
			x += 8;
			while (x >= a.W) {
				x -= a.W;
				if (++y == a.H) {
					y = 0;
					++n;
				}
			}
		}
		// B: 64 pixels x Co / 8 groups of dY
		for (int v = tid; v < TC_K * cog; v += 128) {
			const int g = v % cog, pp = v / cog;
			const int64_t mb = q0 + pp;
			const bool ok = mb < p_end;
			cp_async16(bbase + g * 1024 + (pp >> 3) * 128 + (pp & 7) * 16, ok ? a.dy + mb * a.Co + g * 8 : a.dy, ok);
		}
	};

	// D f32, A bf16, B bf16, A and B MN-major, N = Co, M = 128
	const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
						   ((uint32_t)(a.Co >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

	for (int c = 0; c < S - 1; ++c) {
		if (c < nk) load_chunk(c, c);
		cp_async_commit();
	}
	int issued = -1;
	int my_fail = 0;
	for (int c = 0; c < nk; ++c) {
		const int s = c % S;
		if (S == 2) cp_async_wait<0>();
		else if (S == 3) cp_async_wait<1>();
		else cp_async_wait<2>();
		asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
		if (__syncthreads_or(my_fail)) break;
		issued = c;
		if (tid == 0) {
			asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
			const uint32_t abase = smem_u32(As + (size_t)s * a_bytes);
			const uint32_t bbase = smem_u32(Bs + (size_t)s * b_bytes);
			for (int j = 0; j < TC_K / 16; ++j) {
				const uint64_t ad = umma_desc(abase + j * 256, 128u, 1024u);
				const uint64_t bd = umma_desc(bbase + j * 256, 128u, 1024u);
				const uint32_t acc = (c > 0 || j > 0) ? 1u : 0u;
				asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
							 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
							 "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
			}
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
				smem_u32(mbar + s)));
		}
		const int cn = c + S - 1;
		if (cn < nk) {
			if (c >= 1 && !mbar_wait(smem_u32(mbar + (c - 1) % S), (uint32_t)(((c - 1) / S) & 1))) my_fail = 1;
			else load_chunk(cn, cn % S);
		}
		cp_async_commit();
	}
	cp_async_wait<0>();
	if (issued >= 0 && !mbar_wait(smem_u32(mbar + issued % S), (uint32_t)((issued / S) & 1))) my_fail = 1;
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	const int failed = __syncthreads_or(my_fail || issued != nk - 1);
	if (failed) {
		if (tid == 0) atomicExch(a.err, 1);
	} else {
		const int kcol = kc0 + warp * 32 + lane;
		float *out = a.partial + (int64_t)blockIdx.y * a.Co * K;
		for (int c0 = 0; c0 < a.Co; c0 += 16) {
			uint32_t r[16];
			const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
			asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
						 "[%16];\n"
						 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
						   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
						   "=r"(r[14]), "=r"(r[15])
						 : "r"(taddr));
			asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
			if (kcol < K)
#pragma unroll
				for (int q = 0; q < 16; ++q) out[(int64_t)(c0 + q) * K + kcol] = __uint_as_float(r[q]);
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	if (warp == 0) {
		asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tmem_cols));
	}
}

// ---- weight gradient from TMA-loaded halo rows ----------------------------------
//
// For each column shift dx of the 3x3 stencil one accumulator
// D[(r, ci)][co] = sum over the pixels p of the CTA's row tiles of
// x[y - 1 + r][p - 1 + dx][ci] dY[y][p][co]: M = 128 rows of (halo row r,
// input channel ci) pairs, N = Co, K = the WT pixels of a row tile (WT = W,
// at most 128).  Per row tile the input arrives as one TMA box of rows_box
// halo rows x (WT + 2) pixels x CT channels, zero-filled outside the image,
// laid out halo row major: element (row r, channel group g, pixel p, channel
// e) at ((r * CT / 8 + g) * (WT + 2) + p) * 16 + 2 e.  The 8-row groups of M
// (channel groups, then halo rows) are then R = (WT + 2) * 16 bytes apart --
// the descriptor's stride byte offset -- and pixels 16 bytes apart, so the
// shift dx only moves the descriptor's start by 16 dx bytes (MN-major, no
// swizzle: core matrices of 8 pixels x 8 channels, K-direction stride 128 B).
// dY arrives as (channel group, pixel, 8 channels), N-direction stride WT * 16.
// With CT <= 32 channels per tile one accumulator holds all three halo rows
// (RPM = 3 rows per MMA, 3 CT of its 128 rows used); with CT = 128 each halo
// row is a row group of its own (RPM = 1), and when 9 Co columns do not fit
// TMEM the three row groups go to three CTAs (rows_box = 1).  M rows past the
// loaded halo read other shared memory of the CTA; their accumulator lanes
// are never stored.  A CTA sums the row tiles of its chunk (consecutive tiles
// in (n, y, x tile) order) and writes partial[chunk][co][tap * Ci + ci],
// reduced later in chunk order.  One thread issues the copies and the MMAs;
// waits are bounded and handled as in conv_halo.

struct WhaloArgs {
	float *partial; // (chunks, Co, 9 Ci)
	int N, H, W, Ci, Co;
	int WT, CT, RPM, RG;    // row tile width, channels per tile, halo rows per MMA, row groups
	int rg_cta, rows_box;   // row groups per CTA, halo rows per TMA box
	int ci_tiles, cta_groups;
	int64_t tiles, per_chunk; // row tiles in all and per chunk
	int stages;
	uint32_t x_bytes, dy_bytes;  // TMA box bytes
	uint32_t x_span, dy_span;    // shared-memory bytes per stage of each
	uint32_t dy_off, mbar_off;   // offsets of the dY stages and the mbarriers
	uint32_t tmem_cols;
	int *err;
};

__global__ void __launch_bounds__(128) conv_wgrad_halo(const __grid_constant__ CUtensorMap tx,
													   const __grid_constant__ CUtensorMap tdy, WhaloArgs a) {
	extern __shared__ __align__(1024) uint8_t sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int S = a.stages;
	uint64_t *full = reinterpret_cast<uint64_t *>(sm + a.mbar_off);
	uint64_t *done = full + S;
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + S);

	const int grp = (int)(blockIdx.x % (unsigned)a.cta_groups);
	const int rest = (int)(blockIdx.x / (unsigned)a.cta_groups);
	const int ct = rest % a.ci_tiles;
	const int64_t chunk = rest / a.ci_tiles;
	const int64_t t0 = chunk * a.per_chunk;
	const int64_t t1 = t0 + a.per_chunk < a.tiles ? t0 + a.per_chunk : a.tiles;
	const int nsteps = (int)(t1 - t0);
	const int tpr = a.W / a.WT;
	const int row0 = grp * a.rg_cta * a.RPM; // first halo row of this CTA (0: y - 1)
	const int cg = a.CT / 8;
	const uint32_t R = (uint32_t)(a.WT + 2) * 16u;
	const uint32_t grp_bytes = (uint32_t)(a.RPM * cg) * R;
	const int nk = a.WT / 16;

	if (tid == 0) {
		for (int s = 0; s < S; ++s) {
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(full + s)));
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(done + s)));
		}
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
					 "r"(a.tmem_cols));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	const uint32_t tmem = *tmem_slot;

	// D f32, A bf16, B bf16, A and B MN-major, N = Co, M = 128
	const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
						   ((uint32_t)(a.Co >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
	int fail = 0, loaded = 0, issued = -1;
	if (tid == 0) {
		auto load = [&](int i) {
			const int s = i % S;
			const int64_t t = t0 + i;
			const int xt = (int)(t % tpr);
			const int64_t rw = t / tpr; // n * H + y
			const int n = (int)(rw / a.H), y = (int)(rw - (int64_t)n * a.H);
			const uint32_t xb = smem_u32(sm + (size_t)s * a.x_span);
			const uint32_t db = smem_u32(sm + a.dy_off + (size_t)s * a.dy_span);
			mbar_expect_tx(smem_u32(full + s), a.x_bytes + a.dy_bytes);
			tma_load_5d(xb, &tx, smem_u32(full + s), 0, xt * a.WT - 1, ct * cg, y - 1 + row0, n);
			tma_load_5d(db, &tdy, smem_u32(full + s), 0, xt * a.WT, 0, y, n);
		};
		for (int i = 0; i < S && i < nsteps; ++i) load(i);
		loaded = S < nsteps ? S : nsteps;
		for (int i = 0; i < nsteps; ++i) {
			const int s = i % S;
			if (!mbar_wait(smem_u32(full + s), (uint32_t)((i / S) & 1))) {
				fail = 1;
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
			const uint32_t xb = smem_u32(sm + (size_t)s * a.x_span);
			const uint32_t db = smem_u32(sm + a.dy_off + (size_t)s * a.dy_span);
			// descriptors stepped by constant adds (16-byte units): a k-step
			// moves both operands by 16 pixels
			const uint64_t ad0 = umma_desc(xb, 128u, R), bd0 = umma_desc(db, 128u, (uint32_t)a.WT * 16u);
			for (int k = 0; k < nk; ++k) {
				const uint64_t bd = bd0 + (uint64_t)(16 * k);
				const uint32_t acc = (i > 0 || k > 0) ? 1u : 0u;
				for (int g = 0; g < a.rg_cta; ++g) {
					const uint64_t ad = ad0 + (uint64_t)g * (grp_bytes >> 4) + (uint64_t)(16 * k);
					for (int dx = 0; dx < 3; ++dx)
						umma_f16(tmem + (uint32_t)((g * 3 + dx) * a.Co), ad + (uint64_t)dx, bd, idesc, acc);
				}
			}
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
				smem_u32(done + s)));
			issued = i;
			// refill the stage tile i - 1 used once its MMAs are done (tile
			// i's are queued behind them meanwhile)
			if (i >= 1 && i - 1 + S < nsteps) {
				const int ip = i - 1;
				if (!mbar_wait(smem_u32(done + ip % S), (uint32_t)((ip / S) & 1))) {
					fail = 1;
					break;
				}
				load(ip + S);
				++loaded;
			}
		}
		if (issued >= 0 && !mbar_wait(smem_u32(done + issued % S), (uint32_t)((issued / S) & 1))) fail = 1;
		for (int i = issued + 1; i < loaded; ++i) mbar_wait(smem_u32(full + i % S), (uint32_t)((i / S) & 1));
		if (fail || issued != nsteps - 1) atomicExch(a.err, 1);
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	const int failed = __syncthreads_or(tid == 0 && (fail || issued != nsteps - 1));
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
	if (!failed && warp * 32 < a.RPM * a.CT) {
		// warp w owns TMEM lanes 32 w .. 32 w + 31: lane L = (halo row r, channel ci)
		const int L = warp * 32 + lane;
		const int r = L / a.CT, ci = L - (L / a.CT) * a.CT;
		const int K = 9 * a.Ci;
		float *out = a.partial + chunk * (int64_t)a.Co * K;
		for (int g = 0; g < a.rg_cta; ++g) {
			const int hrow = row0 + g * a.RPM + r;
			const bool ok = r < a.RPM && hrow < 3;
			for (int dx = 0; dx < 3; ++dx) {
				const int col = (hrow * 3 + dx) * a.Ci + ct * a.CT + ci;
				for (int c0 = 0; c0 < a.Co; c0 += 16) {
					uint32_t v[16];
					const uint32_t taddr =
						tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)((g * 3 + dx) * a.Co + c0);
					asm volatile(
						"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
						"[%16];\n"
						: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
						  "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
						  "=r"(v[14]), "=r"(v[15])
						: "r"(taddr));
					asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
					if (ok)
#pragma unroll
						for (int q = 0; q < 16; ++q) out[(int64_t)(c0 + q) * K + col] = __uint_as_float(v[q]);
				}
			}
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
	__syncthreads();
	if (warp == 0) {
		asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tmem_cols));
	}
}

// ---- weight gradient: dW[co][k] = sum_m dY[m][co] * im2col(X)[m][k] -------------

struct WgradArgs {
	const bf16 *x;  // (N,H,W,Ci) forward input
	const bf16 *dy; // (N,H,W,Co) gradient at the pre-activation
	float *partial; // (chunks, Co, 9 Ci)
	int N, H, W, Ci, Co;
	int64_t chunk; // pixels per chunk (multiple of 16)
};

__global__ void __launch_bounds__(128) conv_wgrad(WgradArgs a) {
	__shared__ __align__(16) bf16 As[CB_M][CPAD]; // [co][pixel]
	__shared__ __align__(16) bf16 Bs[CB_N][CPAD]; // [kcol][pixel]
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int wm = warp >> 1, wn = warp & 1;
	const int g = lane >> 2, t = lane & 3;
	const int64_t M = (int64_t)a.N * a.H * a.W;
	const int K = 9 * a.Ci;
	const int co0 = blockIdx.x * CB_M, k0 = blockIdx.y * CB_N;
	const int64_t p_begin = (int64_t)blockIdx.z * a.chunk;
	const int64_t p_end = p_begin + a.chunk < M ? p_begin + a.chunk : M;
	float acc[2][4][4];
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j)
#pragma unroll
			for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
	// per k-step of 16 pixels: thread -> (pixel = tid / 8, vector v = tid % 8 of 8 bf16)
	const int lp = tid >> 3, lv = tid & 7;
	for (int64_t pb = p_begin; pb < p_end; pb += 16) {
		const int64_t m = pb + lp;
		int n = 0, yy = 0, xx = 0;
		const bool mv = m < p_end;
		if (mv) {
			n = (int)(m / ((int64_t)a.H * a.W));
			const int r = (int)(m - (int64_t)n * a.H * a.W);
			yy = r / a.W;
			xx = r - yy * a.W;
		}
		// A: dY[m][co0 + 8 lv .. +7]
		{
			uint4 v = make_uint4(0, 0, 0, 0);
			const int co = co0 + lv * 8;
			if (mv && co < a.Co) v = *reinterpret_cast<const uint4 *>(a.dy + m * a.Co + co);
			const bf16 *e = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
			for (int q = 0; q < 8; ++q) As[lv * 8 + q][lp] = e[q];
		}
		// B: im2col(X)[m][k0 + 8 lv .. +7]
		{
			uint4 v = make_uint4(0, 0, 0, 0);
			const int k = k0 + lv * 8;
			if (mv && k < K) {
				const int tap = k / a.Ci, ci = k - tap * a.Ci;
				const int sy = yy + tap / 3 - 1, sx = xx + tap % 3 - 1;
				if (sy >= 0 && sy < a.H && sx >= 0 && sx < a.W)
					v = *reinterpret_cast<const uint4 *>(a.x + (((int64_t)n * a.H + sy) * a.W + sx) * a.Ci + ci);
			}
			const bf16 *e = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
			for (int q = 0; q < 8; ++q) Bs[lv * 8 + q][lp] = e[q];
		}
		__syncthreads();
		uint32_t af[2][4], bfr[4][2];
#pragma unroll
		for (int i = 0; i < 2; ++i) {
			const int r = wm * 32 + i * 16 + g;
			af[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][2 * t]);
			af[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][2 * t]);
			af[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][2 * t + 8]);
			af[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][2 * t + 8]);
		}
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const int c = wn * 32 + j * 8 + g;
			bfr[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][2 * t]);
			bfr[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][2 * t + 8]);
		}
#pragma unroll
		for (int i = 0; i < 2; ++i)
#pragma unroll
			for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
		__syncthreads();
	}
	float *out = a.partial + (int64_t)blockIdx.z * a.Co * K;
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j)
#pragma unroll
			for (int h = 0; h < 2; ++h) {
				const int co = co0 + wm * 32 + i * 16 + g + h * 8;
				const int k = k0 + wn * 32 + j * 8 + 2 * t;
				if (co < a.Co && k < K) {
					out[(int64_t)co * K + k] = acc[i][j][2 * h];
					if (k + 1 < K) out[(int64_t)co * K + k + 1] = acc[i][j][2 * h + 1];
				}
			}
}

// grad[j] += sum over the chunks of partial[c][j], in a fixed order: block
// (32, SL) takes 32 consecutive j; thread row y sums the chunks of its slice
// [c0, c1) in order, then the SL sums are added in order of y.  SL = 8, or 32
// when there are few j (a long chain of loads per thread otherwise).
__global__ void reduce_partials(const float *partial, int64_t per, int chunks, float *grad) {
	__shared__ float sh[32][33];
	const int64_t j = (int64_t)blockIdx.x * 32 + threadIdx.x;
	const int y = threadIdx.y, SL = blockDim.y;
	const int c0 = (int)((int64_t)chunks * y / SL), c1 = (int)((int64_t)chunks * (y + 1) / SL);
	float s = 0.f;
	if (j < per)
#pragma unroll 8
		for (int c = c0; c < c1; ++c) s += partial[(int64_t)c * per + j];
	sh[y][threadIdx.x] = s;
	__syncthreads();
	if (y == 0 && j < per) {
		float t = 0.f;
		for (int k = 0; k < SL; ++k) t += sh[k][threadIdx.x];
		grad[j] += t;
	}
}

void launch_reduce_partials(const float *partial, int64_t per, int chunks, float *grad, cudaStream_t st) {
	reduce_partials<<<(unsigned)((per + 31) / 32), dim3(32, per < 4096 ? 32 : 8), 0, st>>>(partial, per, chunks, grad);
}

// db[co] += sum over pixels of dY[m][co] (one block per channel, fixed order)
__global__ void bias_grad(const bf16 *dy, int64_t M, int Co, float *db) {
	__shared__ float sh[256];
	const int co = blockIdx.x;
	float s = 0.f;
	for (int64_t m = threadIdx.x; m < M; m += blockDim.x) s += __bfloat162float(dy[m * Co + co]);
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) db[co] += sh[0];
}

// Per-channel sums over pixels, in parallel over pixel chunks: block b sums
// pixels [b * chunk, (b + 1) * chunk) of dY (M x Co, bf16); thread t owns
// channel t % Co and every (blockDim / Co)-th pixel of the chunk (coalesced
// rows), then the threads of one channel are added in thread order.
// partial[b][co] is reduced over blocks in order by reduce_partials.
// 8 bf16 values (16 bytes) to and from floats
__device__ __forceinline__ void unpack8(const uint4 &q, float (&f)[8]) {
	const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&q);
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		const float2 t = __bfloat1622float2(h[k]);
		f[2 * k] = t.x;
		f[2 * k + 1] = t.y;
	}
}

__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
	uint4 q;
	__nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&q);
#pragma unroll
	for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
	return q;
}

// partial[block][c] = sum over the block's pixel chunk of dY[m][c]: thread
// (g, r) takes channels 8g .. 8g + 7 (one 16-byte load) of the pixels r, r +
// per, ... of the chunk; the per sums of a channel are then added in order of r
__global__ void __launch_bounds__(256) channel_sums_partial(const bf16 *dy, int64_t M, int Co, int64_t chunk,
															 float *partial) {
	__shared__ float sh[256 * 8];
	const int G = Co / 8, per = (int)blockDim.x / G; // pixels in flight per block (Co / 8 divides 256)
	const int g = threadIdx.x % G, r = threadIdx.x / G;
	const int64_t m0 = (int64_t)blockIdx.x * chunk;
	const int64_t m1 = m0 + chunk < M ? m0 + chunk : M;
	float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	if (r < per)
		for (int64_t m = m0 + r; m < m1; m += per) {
			float v[8];
			unpack8(reinterpret_cast<const uint4 *>(dy + m * Co)[g], v);
#pragma unroll
			for (int e = 0; e < 8; ++e) acc[e] += v[e];
		}
#pragma unroll
	for (int e = 0; e < 8; ++e) sh[threadIdx.x * 8 + e] = acc[e];
	__syncthreads();
	for (int c = threadIdx.x; c < Co; c += blockDim.x) {
		float t = 0.f;
		for (int k = 0; k < per; ++k) t += sh[(k * G + c / 8) * 8 + c % 8];
		partial[(int64_t)blockIdx.x * Co + c] = t;
	}
}

// db[co] += sum over pixels of dY[m][co], deterministic (fixed chunks and order)
void bias_grads(const bf16 *dy, int64_t M, int Co, float *scratch, float *db, cudaStream_t st) {
	if (Co > 256) {
		bias_grad<<<Co, 256, 0, st>>>(dy, M, Co, db);
		return;
	}
	const int blocks = 1216;
	const int64_t chunk = (M + blocks - 1) / blocks;
	const int nb = (int)((M + chunk - 1) / chunk);
	channel_sums_partial<<<nb, 256, 0, st>>>(dy, M, Co, chunk, scratch);
	launch_reduce_partials(scratch, Co, nb, db, st);
}

// ---- element-wise pieces -----------------------------------------------------------
//
// One thread per pixel and group of 8 channels (channel counts are
// multiples of 16): 16-byte loads and stores, index arithmetic once per 8
// values; the per-value arithmetic and its rounding are those of one value
// at a time.

// dy = 0 where !(y > 0); n values (a multiple of 8)
__global__ void relu_backward(bf16 *dy, const bf16 *y, int64_t n) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n / 8; i += (int64_t)gridDim.x * blockDim.x) {
		float yv[8];
		unpack8(reinterpret_cast<const uint4 *>(y)[i], yv);
		uint4 q = reinterpret_cast<const uint4 *>(dy)[i];
		uint16_t *d = reinterpret_cast<uint16_t *>(&q);
#pragma unroll
		for (int k = 0; k < 8; ++k)
			if (!(yv[k] > 0.f)) d[k] = 0; // bf16 +0
		reinterpret_cast<uint4 *>(dy)[i] = q;
	}
}

__global__ void pool_forward(const bf16 *x, bf16 *y, int N, int H, int W, int C) {
	const int G = C / 8;
	const int64_t n = (int64_t)N * (H / 2) * (W / 2) * G;
	const uint4 *xv = reinterpret_cast<const uint4 *>(x);
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int g = (int)(i % G);
		int64_t r = i / G;
		const int xo = (int)(r % (W / 2));
		r /= (W / 2);
		const int yo = (int)(r % (H / 2));
		const int b = (int)(r / (H / 2));
		const int64_t base = (((int64_t)b * H + 2 * yo) * W + 2 * xo) * G + g;
		float a[8], c[8], d[8], e[8], o[8];
		unpack8(xv[base], a);
		unpack8(xv[base + G], c);
		unpack8(xv[base + (int64_t)W * G], d);
		unpack8(xv[base + (int64_t)W * G + G], e);
#pragma unroll
		for (int k = 0; k < 8; ++k) o[k] = 0.25f * (a[k] + c[k] + d[k] + e[k]);
		reinterpret_cast<uint4 *>(y)[i] = pack8(o);
	}
}

// dx (N,H,W,C) = pool_backward(dy (N,H/2,W/2,C)) + skip_grad (skip may be dx)
__global__ void pool_backward_add(const bf16 *dy, const bf16 *skip, bf16 *dx, int N, int H, int W, int C) {
	const int G = C / 8;
	const int64_t n = (int64_t)N * H * W * G;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int g = (int)(i % G);
		int64_t r = i / G;
		const int x = (int)(r % W);
		r /= W;
		const int y = (int)(r % H);
		const int b = (int)(r / H);
		float p[8], s[8], o[8];
		unpack8(reinterpret_cast<const uint4 *>(dy)[(((int64_t)b * (H / 2) + y / 2) * (W / 2) + x / 2) * G + g], p);
		unpack8(reinterpret_cast<const uint4 *>(skip)[i], s);
#pragma unroll
		for (int k = 0; k < 8; ++k) o[k] = 0.25f * p[k] + s[k];
		reinterpret_cast<uint4 *>(dx)[i] = pack8(o);
	}
}

// cat (N,H,W,Cu+Cs) = [upsample2(u (N,H/2,W/2,Cu)), s (N,H,W,Cs)]
__global__ void upcat_forward(const bf16 *u, const bf16 *s, bf16 *cat, int N, int H, int W, int Cu, int Cs) {
	const int Gu = Cu / 8, Gs = Cs / 8, G = Gu + Gs;
	const int64_t n = (int64_t)N * H * W * G;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int g = (int)(i % G);
		const int64_t p = i / G;
		uint4 q;
		if (g < Gu) {
			const int x = (int)(p % W);
			const int64_t r = p / W;
			const int y = (int)(r % H);
			const int b = (int)(r / H);
			q = reinterpret_cast<const uint4 *>(u)[(((int64_t)b * (H / 2) + y / 2) * (W / 2) + x / 2) * Gu + g];
		} else {
			q = reinterpret_cast<const uint4 *>(s)[p * Gs + (g - Gu)];
		}
		reinterpret_cast<uint4 *>(cat)[i] = q;
	}
}

// split d(cat): d_up (N,H/2,W/2,Cu) = upsample_backward(first Cu), d_skip = last Cs
__global__ void upcat_backward(const bf16 *dcat, bf16 *du, bf16 *ds, int N, int H, int W, int Cu, int Cs) {
	const int Gu = Cu / 8, Gs = Cs / 8, G = Gu + Gs;
	const int64_t nu = (int64_t)N * (H / 2) * (W / 2) * Gu;
	const int64_t ns = (int64_t)N * H * W * Gs;
	const uint4 *dv = reinterpret_cast<const uint4 *>(dcat);
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nu + ns; i += (int64_t)gridDim.x * blockDim.x) {
		if (i < nu) {
			const int g = (int)(i % Gu);
			int64_t r = i / Gu;
			const int xo = (int)(r % (W / 2));
			r /= (W / 2);
			const int yo = (int)(r % (H / 2));
			const int b = (int)(r / (H / 2));
			const int64_t base = (((int64_t)b * H + 2 * yo) * W + 2 * xo) * G + g;
			float a[8], c[8], d[8], e[8], o[8];
			unpack8(dv[base], a);
			unpack8(dv[base + G], c);
			unpack8(dv[base + (int64_t)W * G], d);
			unpack8(dv[base + (int64_t)W * G + G], e);
#pragma unroll
			for (int k = 0; k < 8; ++k) o[k] = a[k] + c[k] + d[k] + e[k];
			reinterpret_cast<uint4 *>(du)[i] = pack8(o);
		} else {
			const int64_t j = i - nu;
			const int g = (int)(j % Gs);
			const int64_t p = j / Gs;
			reinterpret_cast<uint4 *>(ds)[j] = dv[p * G + Gu + g];
		}
	}
}

// Residual inputs of the head, per output channel: in[co] < 0 for none.
constexpr int MAX_RES = 8;
struct HeadRes {
	int in[MAX_RES];
	float scale[MAX_RES];
};

// 1x1 head: y (N,H,W,3) fp32 = x (.., Ci) * Wh^T + b, plus, on an output
// channel co with r.in[co] >= 0, r.scale[co] times input plane r.in[co] of the
// network input `in` (Cin planes): the network then learns the correction to
// that plane (a residual target).
// 1x1 head, one thread per pixel: the pixel's channels in 16-byte loads, the
// weights (Co x Ci, Co <= 8) in shared memory; each output sums its inputs
// in channel order from the bias
__global__ void head_forward(const bf16 *x, const float *w, const float *b, float *y, int64_t M, int Ci, int Co,
							 const bf16 *in, int Cin, HeadRes r) {
	extern __shared__ float hw[];
	for (int k = threadIdx.x; k < Co * Ci; k += blockDim.x) hw[k] = w[k];
	__syncthreads();
	for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
		float acc[MAX_RES];
#pragma unroll
		for (int co = 0; co < MAX_RES; ++co) acc[co] = co < Co ? b[co] : 0.f;
		const uint4 *xr = reinterpret_cast<const uint4 *>(x + m * Ci);
		for (int v = 0; v < Ci / 8; ++v) {
			float xv[8];
			unpack8(xr[v], xv);
#pragma unroll
			for (int e = 0; e < 8; ++e)
#pragma unroll
				for (int co = 0; co < MAX_RES; ++co)
					if (co < Co) acc[co] += hw[co * Ci + 8 * v + e] * xv[e];
		}
#pragma unroll
		for (int co = 0; co < MAX_RES; ++co) {
			if (co >= Co) break;
			float s = acc[co];
			if (r.in[co] >= 0) s += r.scale[co] * __bfloat162float(in[m * Cin + r.in[co]]);
			y[m * Co + co] = s;
		}
	}
}

// masked-free MSE: loss = mean (y - t)^2, dy = 2 (y - t) / n; partial loss per block
__global__ void mse_loss(const float *y, const float *tgt, float *dy, int64_t n, double *partial) {
	__shared__ double sh[256];
	double s = 0.0;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const float d = y[i] - tgt[i];
		dy[i] = 2.f * d / (float)n;
		s += (double)d * d;
	}
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// head backward: dx (bf16) = dy * Wh, dW/db accumulated per block then reduced
// dx = W^T dy per pixel (Co <= 8): each input channel sums over the outputs
// in order from 0; 8 channels per 16-byte store
__global__ void head_backward_dx(const float *dy, const float *w, bf16 *dx, int64_t M, int Ci, int Co) {
	extern __shared__ float hw[];
	for (int k = threadIdx.x; k < Co * Ci; k += blockDim.x) hw[k] = w[k];
	__syncthreads();
	for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
		float d[MAX_RES];
#pragma unroll
		for (int co = 0; co < MAX_RES; ++co) d[co] = co < Co ? dy[m * Co + co] : 0.f;
		uint4 *xr = reinterpret_cast<uint4 *>(dx + m * Ci);
		for (int v = 0; v < Ci / 8; ++v) {
			float o[8];
#pragma unroll
			for (int e = 0; e < 8; ++e) {
				float s = 0.f;
#pragma unroll
				for (int co = 0; co < MAX_RES; ++co)
					if (co < Co) s += d[co] * hw[co * Ci + 8 * v + e];
				o[e] = s;
			}
			xr[v] = pack8(o);
		}
	}
}

__global__ void head_backward_dw(const float *dy, const bf16 *x, int64_t M, int Ci, int Co, float *partial) {
	// one block per (co, ci) pair plus one per co for the bias; fixed-order reduction
	__shared__ float sh[256];
	const int j = blockIdx.x; // j < Co*Ci: weight, else bias
	const int co = j < Co * Ci ? j / Ci : j - Co * Ci;
	const int ci = j < Co * Ci ? j % Ci : -1;
	float s = 0.f;
	for (int64_t m = threadIdx.x; m < M; m += blockDim.x)
		s += dy[m * Co + co] * (ci >= 0 ? __bfloat162float(x[m * Ci + ci]) : 1.f);
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) partial[j] += sh[0];
}

// The same sums in parallel over pixel chunks (Ci divides 256, Co <= 8):
// block b covers pixels [b * chunk, ...); thread t owns input channel t % Ci
// and every (256 / Ci)-th pixel; partial[b][co * Ci + ci] and, for the bias,
// partial[b][Co * Ci + co]; reduced over blocks in order by reduce_partials.
// Head weight and bias gradient partials over a chunk of pixels per block
// (Co <= 8): thread (g, r) takes input channels 8g .. 8g + 7 (one 16-byte
// load) of the pixels r, r + per, ...; per output channel the per sums are
// then added in order of r (threads g = 0 also sum dy for the bias).
__global__ void __launch_bounds__(256) head_dw_partial(const float *dy, const bf16 *x, int64_t M, int Ci, int Co,
														int64_t chunk, float *partial) {
	__shared__ float sh[256 * 8];
	__shared__ float shb[256];
	const int G = Ci / 8, per = (int)blockDim.x / G;
	const int g = threadIdx.x % G, r = threadIdx.x / G;
	const int64_t m0 = (int64_t)blockIdx.x * chunk;
	const int64_t m1 = m0 + chunk < M ? m0 + chunk : M;
	float acc[MAX_RES][8], bacc[MAX_RES];
#pragma unroll
	for (int co = 0; co < MAX_RES; ++co) {
		bacc[co] = 0.f;
#pragma unroll
		for (int e = 0; e < 8; ++e) acc[co][e] = 0.f;
	}
	if (r < per)
		for (int64_t m = m0 + r; m < m1; m += per) {
			float xv[8];
			unpack8(reinterpret_cast<const uint4 *>(x + m * Ci)[g], xv);
#pragma unroll
			for (int co = 0; co < MAX_RES; ++co) {
				if (co >= Co) break;
				const float d = dy[m * Co + co];
				bacc[co] += d;
#pragma unroll
				for (int e = 0; e < 8; ++e) acc[co][e] += d * xv[e];
			}
		}
	const int64_t base = (int64_t)blockIdx.x * (Co * Ci + Co);
#pragma unroll
	for (int co = 0; co < MAX_RES; ++co) {
		if (co >= Co) break;
#pragma unroll
		for (int e = 0; e < 8; ++e) sh[threadIdx.x * 8 + e] = acc[co][e];
		shb[threadIdx.x] = bacc[co];
		__syncthreads();
		for (int c = threadIdx.x; c < Ci; c += blockDim.x) {
			float t = 0.f;
			for (int k = 0; k < per; ++k) t += sh[(k * G + c / 8) * 8 + c % 8];
			partial[base + co * Ci + c] = t;
		}
		if (threadIdx.x == 0) { // the g = 0 threads saw every pixel once
			float tb = 0.f;
			for (int k = 0; k < per; ++k) tb += shb[k * G];
			partial[base + Co * Ci + co] = tb;
		}
		__syncthreads();
	}
}

// Adam on the FP32 master copy, then the bf16 copies: w (co,3,3,ci) and the
// flipped/transposed wf (ci,3,3,co) used by the data gradient.
__global__ void adam_update(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
							float eps, float c1, float c2) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const float gi = g[i];
		const float mi = b1 * m[i] + (1.f - b1) * gi;
		const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
	}
}

// Adam with lr and the bias corrections read from the device (c = lr, c1, c2):
// the same arithmetic as adam_update, for a step replayed from a graph
__global__ void adam_update_dev(float *p, const float *g, float *m, float *v, int64_t n, const float *c, float b1,
								float b2, float eps) {
	const float lr = c[0], c1 = c[1], c2 = c[2];
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const float gi = g[i];
		const float mi = b1 * m[i] + (1.f - b1) * gi;
		const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
	}
}

__global__ void adam_consts(float *c, float lr, float c1, float c2) {
	c[0] = lr;
	c[1] = c1;
	c[2] = c2;
}

// the mean loss from the blocks' partial sums, in block order (as the host adds them)
// loss = (sum of the nb block partials) / n in a fixed order that the host
// path repeats: thread t of 64 sums partials t, t + 64, ... in order, then a
// pairwise tree over the 64 sums (a single thread's chain of nb dependent
// FP64 additions is slow on this GPU's FP64 pipe)
__global__ void loss_finish(const double *partial, int nb, int64_t n, double *loss) {
	__shared__ double sh[64];
	const int t = threadIdx.x;
	double s = 0.0;
	for (int k = t; k < nb; k += 64) s += partial[k];
	sh[t] = s;
	__syncthreads();
	for (int o = 32; o > 0; o >>= 1) {
		if (t < o) sh[t] += sh[t + o];
		__syncthreads();
	}
	if (t == 0) *loss = sh[0] / (double)n;
}

// bf16 copies of the 3x3 conv weights: w = [co][ky][kx][ci] and the flipped,
// transposed wf = [ci][2-ky][2-kx][co] of the data gradient.  One launch for
// every layer: blockIdx.y picks the layer from the table.
constexpr int MAX_CONV = 16;
struct ConvTable {
	int nl;
	int64_t off[MAX_CONV]; // FP32 weights in the parameter vector
	int co[MAX_CONV], ci[MAX_CONV];
	bf16 *w[MAX_CONV], *wf[MAX_CONV];
};

__global__ void refresh_conv_weights(const float *p, const __grid_constant__ ConvTable t) {
	const int l = blockIdx.y;
	const int Co = t.co[l], Ci = t.ci[l], k = 3;
	const float *w32 = p + t.off[l];
	bf16 *w = t.w[l], *wf = t.wf[l];
	const int64_t n = (int64_t)Co * k * k * Ci;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int ci = (int)(i % Ci);
		int64_t r = i / Ci;
		const int kx = (int)(r % k);
		r /= k;
		const int ky = (int)(r % k);
		const int co = (int)(r / k);
		const bf16 v = __float2bfloat16(w32[i]);
		w[i] = v;
		if (wf) wf[(((int64_t)ci * k + (k - 1 - ky)) * k + (k - 1 - kx)) * Co + co] = v;
	}
}

// Network input (16 channels, bf16).  From the obstacle mask (1 = solid) and
// the two flow parameters:
//   0 mask, 1 u_max / 0.08, 2 (tau - 0.55) / 0.45, 3 y / (H - 1), 4 x / (W - 1),
//   5 open fraction of the column (fluid cells / (H - 2)),
//   6 downstream resistance: sum over columns x' >= x of 1 / open^3, / W,
//   7 height of the vertical gap holding the cell / (H - 2),
//   8 4 s (1 - s), s the cell's position across that gap,
//   9 lubrication estimate of u_x / u_max, halved: with the inlet flux
//     Q = 2/3 u_max (H - 2) split over a column's gaps as h^3, the gap's
//     Poiseuille profile gives u_x / u_max = (H - 2) h^2 / sum h^3 4 s (1 - s),
//   10 lubrication pressure, normalised: each column's Poiseuille pressure
//     gradient is 12 nu Q / sum h^3, so the pressure above the outlet is
//     proportional to the suffix sum S(x) of 1 / sum h^3 over columns
//     x' >= x; the plane holds S(x) / S(0) (1 at the inlet),
//   11-15 zero.
// Solid cells carry only channels 0-4.

// per (sample, column): fluid-cell count and sum of the cubes of its gap heights
__global__ void column_features(const uint8_t *mask, int N, int H, int W, float *open, float *h3) {
	const int idx = blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= N * W) return;
	const int b = idx / W, x = idx - b * W;
	const uint8_t *m = mask + (int64_t)b * H * W;
	int cnt = 0, run = 0;
	float s3 = 0.f;
	for (int y = 0; y < H; ++y) {
		if (!m[(int64_t)y * W + x]) {
			++cnt;
			++run;
		} else {
			s3 += (float)run * run * run;
			run = 0;
		}
	}
	s3 += (float)run * run * run;
	open[idx] = fminf((float)cnt / (float)(H > 2 ? H - 2 : H), 1.f);
	h3[idx] = s3;
}

// per sample (one block): suffix sums over the columns of the column
// resistance 1 / max(open, 1/8)^3, and of the lubrication resistance
// 1 / max(sum h^3, 1) normalised by its total; a Hillis-Steele scan in shared
// memory (fixed order).  Dynamic shared memory: 4 W floats.
__global__ void column_resistance(const float *open, const float *h3, int N, int W, float *R, float *PL) {
	extern __shared__ float cs[];
	float *a0 = cs, *b0 = cs + W, *a1 = cs + 2 * W, *b1 = cs + 3 * W;
	const int b = blockIdx.x;
	for (int x = threadIdx.x; x < W; x += blockDim.x) {
		const float o = fmaxf(open[(int64_t)b * W + x], 0.125f);
		a0[x] = 1.f / (o * o * o);
		b0[x] = 1.f / fmaxf(h3[(int64_t)b * W + x], 1.f);
	}
	__syncthreads();
	for (int off = 1; off < W; off <<= 1) {
		for (int x = threadIdx.x; x < W; x += blockDim.x) {
			a1[x] = x + off < W ? a0[x] + a0[x + off] : a0[x];
			b1[x] = x + off < W ? b0[x] + b0[x + off] : b0[x];
		}
		__syncthreads();
		float *t = a0;
		a0 = a1;
		a1 = t;
		t = b0;
		b0 = b1;
		b1 = t;
	}
	const float inv = 1.f / b0[0];
	for (int x = threadIdx.x; x < W; x += blockDim.x) {
		R[(int64_t)b * W + x] = a0[x] / (float)W;
		PL[(int64_t)b * W + x] = b0[x] * inv;
	}
}

// The 16 input channels of pixel (yy, xx) of a sample, mv its mask value;
// solid(y) reads the mask of the pixel's column at row y (to find the
// vertical gap holding the pixel).
template <typename Solid>
__device__ __forceinline__ void input_pixel(float (&v)[16], uint8_t mv, const Solid &solid, int yy, int H, int64_t col,
											float c1, float c2, float c4, const float *open, const float *h3,
											const float *R, const float *PL) {
#pragma unroll
	for (int k = 0; k < 16; ++k) v[k] = 0.f;
	v[0] = (float)mv;
	v[1] = c1;
	v[2] = c2;
	v[3] = (float)yy / (float)(H - 1);
	v[4] = c4;
	if (!mv) {
		const float hin = (float)(H > 2 ? H - 2 : H);
		int lo = yy, hi = yy;
		while (lo > 0 && !solid(lo - 1)) --lo;
		while (hi + 1 < H && !solid(hi + 1)) ++hi;
		const float h = (float)(hi - lo + 1);
		const float sp = ((float)(yy - lo) + 0.5f) / h;
		const float shape = 4.f * sp * (1.f - sp);
		v[5] = open[col];
		v[6] = R[col];
		v[7] = h / hin;
		v[8] = shape;
		v[9] = 0.5f * fminf(hin * h * h / fmaxf(h3[col], 1.f) * shape, 8.f);
		v[10] = PL[col];
	}
}

__device__ __forceinline__ void store_input16(bf16 *o, const float (&v)[16]) {
	__align__(16) __nv_bfloat162 q[8];
#pragma unroll
	for (int k = 0; k < 8; ++k) q[k] = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
	uint4 *d = reinterpret_cast<uint4 *>(o);
	d[0] = *reinterpret_cast<const uint4 *>(&q[0]);
	d[1] = *reinterpret_cast<const uint4 *>(&q[4]);
}

// One block per (sample, 32 columns): the block's mask columns are staged in
// shared memory (H x 32 bytes), then thread (column c, row r) finds its
// vertical gap's ends there and writes the pixel's 16 channels as two
// 16-byte stores (a warp's stores cover 32 consecutive pixels of a row).
// Dynamic shared memory: 32 H bytes.
__global__ void make_input(const uint8_t *mask, const float *umax, const float *tau, const float *open,
						   const float *h3, const float *R, const float *PL, bf16 *x, int N, int H, int W) {
	extern __shared__ uint8_t mt[]; // [H][32]
	const int tpb = (W + 31) / 32;
	const int b = blockIdx.x / tpb, x0 = (blockIdx.x % tpb) * 32;
	const uint8_t *m = mask + (int64_t)b * H * W;
	for (int i = threadIdx.x; i < H * 32; i += blockDim.x) {
		const int yy = i >> 5, c = i & 31;
		mt[i] = x0 + c < W ? m[(int64_t)yy * W + x0 + c] : (uint8_t)1;
	}
	__syncthreads();
	const int c = threadIdx.x & 31, xx = x0 + c;
	if (xx >= W) return;
	const int64_t col = (int64_t)b * W + xx;
	const float c1 = umax[b] / 0.08f, c2 = (tau[b] - 0.55f) / 0.45f, c4 = (float)xx / (float)(W - 1);
	const auto solid = [&](int y) { return mt[y * 32 + c] != 0; };
	for (int yy = threadIdx.x >> 5; yy < H; yy += blockDim.x >> 5) {
		float v[16];
		input_pixel(v, mt[yy * 32 + c], solid, yy, H, col, c1, c2, c4, open, h3, R, PL);
		store_input16(x + (((int64_t)b * H + yy) * W + xx) * 16, v);
	}
}

// The same for grids too tall for the shared-memory tile: one thread per
// pixel, the gap found in global memory.
__global__ void make_input_tall(const uint8_t *mask, const float *umax, const float *tau, const float *open,
								const float *h3, const float *R, const float *PL, bf16 *x, int N, int H, int W) {
	const int64_t n = (int64_t)N * H * W;
	for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
		const int b = (int)(p / ((int64_t)H * W));
		const int r = (int)(p - (int64_t)b * H * W);
		const int yy = r / W, xx = r - yy * W;
		const uint8_t *m = mask + (int64_t)b * H * W;
		const auto solid = [&](int y) { return m[(int64_t)y * W + xx] != 0; };
		float v[16];
		input_pixel(v, m[r], solid, yy, H, (int64_t)b * W + xx, umax[b] / 0.08f, (tau[b] - 0.55f) / 0.45f,
					(float)xx / (float)(W - 1), open, h3, R, PL);
		store_input16(x + p * 16, v);
	}
}

int grid_of(int64_t n) { return grid_for(n); }

} // namespace

// ----------------------------------------------------------------------------------
// network object

struct UnetLayer {
	int co, ci, k;  // conv shape
	int64_t woff;   // offset of the weights in the flat parameter vector (bias follows)
	bf16 *w = nullptr, *wf = nullptr;
	int level;      // spatial level (0 = full resolution)
};

struct kel_unet {
	kel_unet_desc d;
	std::vector<UnetLayer> L; // enc0a enc0b enc1a enc1b enc2a enc2b botta bottb dec2a dec2b dec1a dec1b dec0a dec0b head
	int64_t nparam = 0;
	float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
	float *partial = nullptr;
	int64_t partial_len = 0;
	double *loss_partial = nullptr;
	cudaStream_t stream = nullptr;
	// activations / gradients, one per named tensor
	std::vector<bf16 *> act, grad;
	bf16 *input = nullptr;
	float *out = nullptr, *dout = nullptr;
	int batch = 0;
	int conv_kernel = KEL_UNET_CONV_TCGEN05;
	int *d_err = nullptr; // set by a tensor-core kernel whose bounded wait ran out
	float *col_open = nullptr, *col_h3 = nullptr, *col_res = nullptr, *col_pl = nullptr; // input-feature scratch (max_batch x W)
	HeadRes res; // residual head per output channel (kel_unet_set_residual)
	cudaStream_t own_stream = nullptr; // the stream the net created (stream may be a caller's)
	int sms = 0;                       // the device's SM count (grid sizing)
	// kel_unet_train_step: the target copy, Adam's lr and bias corrections on
	// the device, the last loss, and the captured step (forward, backward,
	// Adam, weight refresh) for batch train_n and these Adam constants
	float *tgt = nullptr, *adam_c = nullptr;
	double *dev_loss = nullptr;
	cudaGraphExec_t train_graph = nullptr;
	int train_n = 0;
	float train_b1 = 0.f, train_b2 = 0.f, train_eps = 0.f;
	bool train_warm = false;
};

namespace {

// tensor ids
enum { T_E0A, T_E0B, T_P0, T_E1A, T_E1B, T_P1, T_E2A, T_E2B, T_P2, T_BA, T_BB, T_C2, T_D2A, T_D2B, T_C1, T_D1A,
	   T_D1B, T_C0, T_D0A, T_D0B, T_COUNT };

struct TShape {
	int level, ch;
};

TShape tshape(const kel_unet *U, int t) {
	const int *w = U->d.widths;
	switch (t) {
	case T_E0A: case T_E0B: return {0, w[0]};
	case T_P0: return {1, w[0]};
	case T_E1A: case T_E1B: return {1, w[1]};
	case T_P1: return {2, w[1]};
	case T_E2A: case T_E2B: return {2, w[2]};
	case T_P2: return {3, w[2]};
	case T_BA: case T_BB: return {3, w[3]};
	case T_C2: return {2, w[3] + w[2]};
	case T_D2A: case T_D2B: return {2, w[2]};
	case T_C1: return {1, w[2] + w[1]};
	case T_D1A: case T_D1B: return {1, w[1]};
	case T_C0: return {0, w[1] + w[0]};
	default: return {0, w[0]};
	}
}

int64_t telems(const kel_unet *U, int t, int n) {
	const TShape s = tshape(U, t);
	return (int64_t)n * (U->d.height >> s.level) * (U->d.width >> s.level) * s.ch;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
								  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
								  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (null if
// the driver does not provide it)
EncodeTiledFn encode_tiled() {
	static const EncodeTiledFn fn = []() -> EncodeTiledFn {
		void *p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
			q != cudaDriverEntryPointSuccess)
			return nullptr;
		return reinterpret_cast<EncodeTiledFn>(p);
	}();
	return fn;
}

uint32_t align1k(uint64_t v) { return (uint32_t)((v + 1023) / 1024 * 1024); }

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per kernel and
// device: the attribute belongs to the device's context, so a flag per
// process would leave a second device's launches without it.  One
// instantiation (and flag array) per kernel.
template <auto Kernel>
cudaError_t allow_dynamic_smem(int bytes) {
	static bool done[64] = {};
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
	e = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
	return e;
}

// Channel chunk and stage count of conv_halo: the largest chunk (64, 48, 32 or
// 16 channels dividing Ci) whose stages (up to three, at least two when there
// are two chunks or more) fit 110 KB (two CTAs per SM), else 200 KB; 0: none.
int halo_plan(int Ci, int Co, int RT, HaloArgs &a) {
	for (const uint32_t cap : {110u * 1024u, 200u * 1024u})
		for (const int ck : {64, 48, 32, 16}) {
			if (Ci % ck) continue;
			const int nch = Ci / ck;
			const uint32_t cb = (uint32_t)(RT * a.MR + 2) * (uint32_t)a.P * (uint32_t)ck * 2u;
			const uint32_t ab = (uint32_t)a.NC * cb, bb = 18u * (uint32_t)a.CoT * (uint32_t)ck;
			const uint32_t stage = align1k(ab) + align1k(bb);
			int S = nch < 3 ? nch : 3;
			while (S > 1 && (uint64_t)S * stage + 1024 > cap) --S;
			if ((nch > 1 && S < 2) || (uint64_t)S * stage + 1024 > cap) continue;
			a.CK = ck;
			a.stages = S;
			a.copy_bytes = cb;
			a.a_bytes = ab;
			a.b_bytes = bb;
			a.a_span = align1k(ab);
			a.stage_bytes = stage;
			return 1;
		}
	return 0;
}

// The halo convolution (conv_halo); returns 0 without
// launching when the layer does not fit it.
int conv_halo_launch(kel_unet *U, const bf16 *x, const bf16 *w, const float *b, bf16 *y, int n, int H, int W, int ci,
					 int co, bool relu, bool bias, int *launched) {
	*launched = 0;
	const EncodeTiledFn enc = encode_tiled();
	HaloArgs a;
	memset(&a, 0, sizeof(a));
	if (!enc || ci % 16 || co % 16 || co < 16 || co > 256) return KEL_OK;
	if (W % 128 == 0) {
		a.NC = 1;
		a.P = HX;
		a.MR = 1;
	} else if (W >= 8 && W % 8 == 0 && 128 % W == 0 && H % (128 / W) == 0) {
		a.NC = 3;
		a.P = W;
		a.MR = 128 / W;
	} else {
		return KEL_OK;
	}
	const int tpr = W >= 128 ? W / 128 : 1;
	const int sms = U->sms > 0 ? U->sms : 148;
	// M tiles per CTA: the most (4, 2, 1) whose accumulators fit TMEM and
	// that still leave a CTA per SM; with fewer tiles than SMs, the output
	// channels split over two CTAs (at least 32 channels each)
	a.RT = 0;
	a.CoT = co;
	for (const int rt : {4, 2, 1})
		if (!a.RT && rt * co <= 512 && H % (rt * a.MR) == 0 && (int64_t)n * (H / (rt * a.MR)) * tpr >= sms &&
			halo_plan(ci, co, rt, a))
			a.RT = rt;
	if (!a.RT && H % a.MR == 0) {
		const int64_t tiles = (int64_t)n * (H / a.MR) * tpr;
		if (tiles < sms && co % 32 == 0 && co / 2 >= 32) a.CoT = co / 2;
		if (halo_plan(ci, co, 1, a)) a.RT = 1;
	}
	if (!a.RT) return KEL_OK;
	CUtensorMap tx, tw;
	{ // x (N,H,W,Ci) as (8 channels, x, y, channel group, n)
		const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)(ci / 8), (cuuint64_t)n};
		const cuuint64_t strides[4] = {(cuuint64_t)ci * 2, (cuuint64_t)W * ci * 2, 16, (cuuint64_t)H * W * ci * 2};
		const cuuint32_t box[5] = {8, (cuuint32_t)a.P, (cuuint32_t)(a.RT * a.MR + 2), (cuuint32_t)(a.CK / 8), 1};
		const cuuint32_t es[5] = {1, 1, 1, 1, 1};
		if (enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(x), dims, strides, box, es,
				CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
				CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
			return KEL_OK;
	}
	{ // w (Co, 9, Ci) as (8 channels, co, tap, channel group)
		const cuuint64_t dims[4] = {8, (cuuint64_t)co, 9, (cuuint64_t)(ci / 8)};
		const cuuint64_t strides[3] = {(cuuint64_t)9 * ci * 2, (cuuint64_t)ci * 2, 16};
		const cuuint32_t box[4] = {8, (cuuint32_t)a.CoT, 9, (cuuint32_t)(a.CK / 8)};
		const cuuint32_t es[4] = {1, 1, 1, 1};
		if (enc(&tw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(w), dims, strides, box, es,
				CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
				CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
			return KEL_OK;
	}
	a.bias = b;
	a.y = y;
	a.N = n;
	a.H = H;
	a.W = W;
	a.Ci = ci;
	a.Co = co;
	a.relu = relu;
	a.use_bias = bias;
	a.tmem_cols = 32;
	while (a.tmem_cols < (uint32_t)(a.RT * a.CoT)) a.tmem_cols <<= 1;
	a.err = U->d_err;
	const size_t smem = (size_t)a.stages * a.stage_bytes + (size_t)a.stages * 16 + 16;
	KEL_CUDA(allow_dynamic_smem<conv_halo>(210 * 1024));
	conv_halo<<<(unsigned)((int64_t)n * (H / (a.RT * a.MR)) * tpr * (co / a.CoT)), 128, smem, U->stream>>>(tx, tw, a);
	KEL_CUDA(cudaGetLastError());
	*launched = 1;
	return KEL_OK;
}

// Plan of conv_rows for a layer (W a multiple of 128; the weights and four
// input rows within 200 KB of shared memory); 0 when the layer does not fit
// it.  Rows per CTA: the run length that minimises (waves of CTAs) x (rows +
// 3), the three being the two extra input rows and the weight load of a run.
int rows_plan(const kel_unet *U, int n, int H, int W, int Ci, int Co, RowsArgs &a) {
	if (W % 128 || Ci % 16 || Co % 16 || Co < 16 || Co > 256 || H < 1) return 0;
	a.NR = 4;
	a.row_bytes = (uint32_t)HX * (uint32_t)Ci * 2u;
	a.row_span = (a.row_bytes + 127u) / 128u * 128u;
	a.w_bytes = (uint32_t)Co * 9u * (uint32_t)Ci * 2u;
	a.w_off = (uint32_t)a.NR * a.row_span;
	a.mbar_off = a.w_off + (a.w_bytes + 127u) / 128u * 128u;
	const uint32_t smem = a.mbar_off + (2u * (uint32_t)a.NR + 3u + 16u) * 8u + 16u;
	if (smem > 200u * 1024u) return 0;
	const int smem_per_sm = (int)((227u * 1024u) / (smem + 1024u));
	// accumulator blocks of RB output rows, up to three kernel rows per MMA:
	// RB as large as the TMEM share of the CTAs that shared memory lets onto
	// an SM allows (up to four CTAs, at most 8 rows).  RB >= 2: the three
	// output rows an input row feeds must lie in the two buffered blocks, or
	// the MMAs would wait for a block that they have yet to complete.
	const int share = 512 / (smem_per_sm < 1 ? 1 : (smem_per_sm > 4 ? 4 : smem_per_sm));
	a.RB = share / (2 * Co) > 8 ? 8 : share / (2 * Co);
	if (a.RB < 2) a.RB = 2;
	if (2 * a.RB * Co > 512) return 0;
	a.KY = 256 / Co < 3 ? 256 / Co : 3;
	a.tmem_cols = 32;
	while (a.tmem_cols < 2u * (uint32_t)(a.RB * Co)) a.tmem_cols <<= 1;
	int per_sm = smem_per_sm;
	if (per_sm > (int)(512u / a.tmem_cols)) per_sm = (int)(512u / a.tmem_cols);
	if (per_sm > 10) per_sm = 10;
	if (per_sm < 1) per_sm = 1;
	const int64_t cols = (int64_t)n * (W / 128), slots = (int64_t)per_sm * (U->sms > 0 ? U->sms : 148);
	int64_t best = -1;
	for (int k = 1; k <= H; ++k) {
		const int RL = (H + k - 1) / k, runs = (H + RL - 1) / RL;
		const int64_t waves = (cols * runs + slots - 1) / slots, cost = waves * (RL + 3);
		if (best < 0 || cost < best) {
			best = cost;
			a.RL = RL;
			a.runs = runs;
		}
	}
	return 1;
}

// conv_rows for one layer; returns 0 without launching when it does not fit.
int conv_rows_launch(kel_unet *U, const bf16 *x, const bf16 *w, const float *b, bf16 *y, int n, int H, int W, int ci,
					 int co, bool relu, bool bias, int *launched) {
	*launched = 0;
	const EncodeTiledFn enc = encode_tiled();
	RowsArgs a;
	memset(&a, 0, sizeof(a));
	if (!enc || !rows_plan(U, n, H, W, ci, co, a)) return KEL_OK;
	CUtensorMap tx, tw;
	{ // x (N,H,W,Ci) as (8 channels, x, channel group, y, n): one row per box
		const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)(ci / 8), (cuuint64_t)H, (cuuint64_t)n};
		const cuuint64_t strides[4] = {(cuuint64_t)ci * 2, 16, (cuuint64_t)W * ci * 2, (cuuint64_t)H * W * ci * 2};
		const cuuint32_t box[5] = {8, HX, (cuuint32_t)(ci / 8), 1, 1};
		const cuuint32_t es[5] = {1, 1, 1, 1, 1};
		if (enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(x), dims, strides, box, es,
				CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
				CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
			return KEL_OK;
	}
	{ // w (Co, 3, 3, Ci) as (8 channels, co, ky, kx, channel group): the whole
	  // tensor, in shared memory as [g][kx][ky][co][8]
		const cuuint64_t dims[5] = {8, (cuuint64_t)co, 3, 3, (cuuint64_t)(ci / 8)};
		const cuuint64_t strides[4] = {(cuuint64_t)9 * ci * 2, (cuuint64_t)3 * ci * 2, (cuuint64_t)ci * 2, 16};
		const cuuint32_t box[5] = {8, (cuuint32_t)co, 3, 3, (cuuint32_t)(ci / 8)};
		const cuuint32_t es[5] = {1, 1, 1, 1, 1};
		if (enc(&tw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(w), dims, strides, box, es,
				CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
				CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
			return KEL_OK;
	}
	a.bias = b;
	a.y = y;
	a.N = n;
	a.H = H;
	a.W = W;
	a.Ci = ci;
	a.Co = co;
	a.relu = relu;
	a.use_bias = bias;
	a.err = U->d_err;
	const size_t smem = (size_t)a.mbar_off + (2u * (size_t)a.NR + 3u + 16u) * 8u + 16u;
	KEL_CUDA(allow_dynamic_smem<conv_rows>(210 * 1024));
	conv_rows<<<(unsigned)((int64_t)n * (W / 128) * a.runs), 192, smem, U->stream>>>(tx, tw, a);
	KEL_CUDA(cudaGetLastError());
	*launched = 1;
	return KEL_OK;
}

int conv_fwd(kel_unet *U, const bf16 *x, const bf16 *w, const float *b, bf16 *y, int n, int level, int ci, int co,
			 bool relu, bool bias) {
	ConvArgs a;
	a.x = x;
	a.w = w;
	a.bias = b;
	a.y = y;
	a.N = n;
	a.H = U->d.height >> level;
	a.W = U->d.width >> level;
	a.Ci = ci;
	a.Co = co;
	a.relu = relu;
	a.use_bias = bias;
	const int64_t M = (int64_t)n * a.H * a.W;
	if (U->conv_kernel == KEL_UNET_CONV_TCGEN05) {
		if (ci % 16 || co % 16 || co < 16 || co > 256)
			return fail(KEL_ERR_UNSUPPORTED, "conv: tensor-core path needs c_in, c_out multiples of 16, c_out <= 256");
		int launched = 0, rc;
		if ((rc = conv_rows_launch(U, x, w, b, y, n, a.H, a.W, ci, co, relu, bias, &launched))) return rc;
		if (launched) return KEL_OK;
		if ((rc = conv_halo_launch(U, x, w, b, y, n, a.H, a.W, ci, co, relu, bias, &launched))) return rc;
		if (launched) return KEL_OK;
		TcArgs t;
		t.x = x;
		t.w = w;
		t.bias = b;
		t.y = y;
		t.N = n;
		t.H = a.H;
		t.W = a.W;
		t.Ci = ci;
		t.Co = co;
		t.relu = relu;
		t.use_bias = bias;
		t.stages = co <= 128 ? 3 : 2; // 2-3 CTAs per SM by shared memory
		t.tmem_cols = 32;
		while (t.tmem_cols < (uint32_t)co) t.tmem_cols <<= 1;
		t.err = U->d_err;
		const size_t smem = (size_t)t.stages * ((size_t)co * 128 + (size_t)TC_M * 128) + (size_t)t.stages * 8 + 16;
		KEL_CUDA(allow_dynamic_smem<conv_tc>(200 * 1024));
		conv_tc<<<(unsigned)((M + TC_M - 1) / TC_M), 128, smem, U->stream>>>(t);
		KEL_CUDA(cudaGetLastError());
		return KEL_OK;
	}
	dim3 grid((unsigned)((M + CB_M - 1) / CB_M), (unsigned)((co + CB_N - 1) / CB_N));
	conv_igemm<<<grid, 128, 0, U->stream>>>(a);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

// Plan of conv_wgrad_halo for a layer; 0 when the layer does not fit it.
// Channels per tile: 128 when Ci allows (one halo row per MMA, all 128 M rows
// used), else 32 or 16 (three halo rows per MMA).  Stages: up to four within
// 110 KB when the CTA's TMEM columns leave room for a second CTA on the SM,
// else up to six within 220 KB (one CTA per SM).
int whalo_plan(int Ci, int Co, int W, WhaloArgs &a) {
	if (Co % 16 || Co < 16 || Co > 256 || Ci % 16) return 0;
	a.WT = W >= 128 ? 128 : W;
	if (a.WT % 16 || W % a.WT) return 0;
	if (Ci % 128 == 0) {
		a.CT = 128;
		a.RPM = 1;
		a.RG = 3;
	} else {
		a.CT = Ci % 32 == 0 ? 32 : 16;
		a.RPM = 3;
		a.RG = 1;
	}
	a.rg_cta = a.RG * 3 * Co <= 512 ? a.RG : 1;
	if (a.rg_cta * 3 * Co > 512) return 0;
	a.cta_groups = a.RG / a.rg_cta;
	a.ci_tiles = Ci / a.CT;
	a.rows_box = a.rg_cta * a.RPM;
	const uint32_t R = (uint32_t)(a.WT + 2) * 16u, cg = (uint32_t)a.CT / 8u;
	a.x_bytes = (uint32_t)a.rows_box * cg * R;
	a.dy_bytes = (uint32_t)a.WT * (uint32_t)Co * 2u;
	a.x_span = align1k(a.x_bytes);
	a.dy_span = align1k(a.dy_bytes);
	// the last row group's MMAs read 16 channel groups of 8 rows from its start
	const uint64_t need = ((uint64_t)(a.rg_cta - 1) * a.RPM * cg + 16u) * R;
	a.tmem_cols = 32;
	while (a.tmem_cols < (uint32_t)(a.rg_cta * 3 * Co)) a.tmem_cols <<= 1;
	auto operand_bytes = [&](int S) -> uint64_t {
		uint64_t t = (uint64_t)S * (a.x_span + a.dy_span), r = (uint64_t)(S - 1) * a.x_span + need;
		return align1k(t > r ? t : r);
	};
	a.stages = 0;
	if (a.tmem_cols <= 256)
		for (int S = 4; S >= 2 && !a.stages; --S)
			if (operand_bytes(S) + 1024 <= 110u * 1024u) a.stages = S;
	if (!a.stages)
		for (int S = 6; S >= 2 && !a.stages; --S)
			if (operand_bytes(S) + 1024 <= 220u * 1024u) a.stages = S;
	if (!a.stages) return 0;
	a.dy_off = (uint32_t)a.stages * a.x_span;
	a.mbar_off = (uint32_t)operand_bytes(a.stages);
	return 1;
}

// conv_wgrad_halo for one layer (weight gradient into U->partial, reduced into
// the layer's gradient); returns 0 without launching when the layer does not
// fit it.
int wgrad_halo_launch(kel_unet *U, const UnetLayer &l, const bf16 *x, const bf16 *dy, int n, int *launched) {
	*launched = 0;
	const EncodeTiledFn enc = encode_tiled();
	WhaloArgs a;
	memset(&a, 0, sizeof(a));
	const int H = U->d.height >> l.level, W = U->d.width >> l.level;
	if (!enc || !whalo_plan(l.ci, l.co, W, a)) return KEL_OK;
	CUtensorMap tx, tdy;
	{ // x (N,H,W,Ci) as (8 channels, x, channel group, y, n)
		const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)(l.ci / 8), (cuuint64_t)H, (cuuint64_t)n};
		const cuuint64_t strides[4] = {(cuuint64_t)l.ci * 2, 16, (cuuint64_t)W * l.ci * 2, (cuuint64_t)H * W * l.ci * 2};
		const cuuint32_t box[5] = {8, (cuuint32_t)(a.WT + 2), (cuuint32_t)(a.CT / 8), (cuuint32_t)a.rows_box, 1};
		const cuuint32_t es[5] = {1, 1, 1, 1, 1};
		if (enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(x), dims, strides, box, es,
				CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
				CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
			return KEL_OK;
	}
	{ // dY (N,H,W,Co) as (8 channels, x, channel group, y, n)
		const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)(l.co / 8), (cuuint64_t)H, (cuuint64_t)n};
		const cuuint64_t strides[4] = {(cuuint64_t)l.co * 2, 16, (cuuint64_t)W * l.co * 2, (cuuint64_t)H * W * l.co * 2};
		const cuuint32_t box[5] = {8, (cuuint32_t)a.WT, (cuuint32_t)(l.co / 8), 1, 1};
		const cuuint32_t es[5] = {1, 1, 1, 1, 1};
		if (enc(&tdy, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(dy), dims, strides, box, es,
				CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
				CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
			return KEL_OK;
	}
	a.partial = U->partial;
	a.N = n;
	a.H = H;
	a.W = W;
	a.Ci = l.ci;
	a.Co = l.co;
	a.err = U->d_err;
	a.tiles = (int64_t)n * H * (W / a.WT);
	// one wave: two CTAs per SM when TMEM and shared memory allow it
	const size_t smem = (size_t)a.mbar_off + (size_t)a.stages * 16 + 16;
	const int per_sm = (a.tmem_cols <= 256 && smem <= 110u * 1024u) ? 2 : 1;
	const int per_chunk_ctas = a.ci_tiles * a.cta_groups;
	const int64_t per = (int64_t)l.co * 9 * l.ci;
	int64_t chunks = ((int64_t)per_sm * (U->sms > 0 ? U->sms : 148) + per_chunk_ctas / 2) / per_chunk_ctas;
	if (chunks > U->partial_len / per) chunks = U->partial_len / per;
	if (chunks > a.tiles) chunks = a.tiles;
	if (chunks < 1) chunks = 1;
	a.per_chunk = (a.tiles + chunks - 1) / chunks;
	chunks = (a.tiles + a.per_chunk - 1) / a.per_chunk;
	KEL_CUDA(allow_dynamic_smem<conv_wgrad_halo>(222 * 1024));
	// one CTA per SM when its TMEM columns would not leave room for a second
	const size_t smem_launch = per_sm == 1 && smem < 116u * 1024u ? 116u * 1024u : smem;
	conv_wgrad_halo<<<(unsigned)(chunks * per_chunk_ctas), 128, smem_launch, U->stream>>>(tx, tdy, a);
	KEL_CUDA(cudaGetLastError());
	launch_reduce_partials(U->partial, per, (int)chunks, U->g + l.woff, U->stream);
	*launched = 1;
	return KEL_OK;
}

int conv_grads_tc(kel_unet *U, const UnetLayer &l, const bf16 *x, const bf16 *dy, int n) {
	if (l.ci % 16 || l.co % 16 || l.co > 256)
		return fail(KEL_ERR_UNSUPPORTED, "wgrad: tensor-core path needs c_in, c_out multiples of 16, c_out <= 256");
	{
		int launched = 0, rc;
		if ((rc = wgrad_halo_launch(U, l, x, dy, n, &launched))) return rc;
		if (launched) {
			const int64_t M = (int64_t)n * (U->d.height >> l.level) * (U->d.width >> l.level);
			bias_grads(dy, M, l.co, U->partial, U->g + l.woff + (int64_t)l.co * 9 * l.ci, U->stream);
			KEL_CUDA(cudaGetLastError());
			return KEL_OK;
		}
	}
	TcWgradArgs a;
	a.x = x;
	a.dy = dy;
	a.partial = U->partial;
	a.N = n;
	a.H = U->d.height >> l.level;
	a.W = U->d.width >> l.level;
	a.Ci = l.ci;
	a.Co = l.co;
	const int64_t M = (int64_t)n * a.H * a.W;
	const int K = 9 * l.ci;
	const int tiles = (K + TC_M - 1) / TC_M;
	int64_t chunks = (608 + tiles - 1) / tiles;
	const int64_t max_chunks = U->partial_len / ((int64_t)l.co * K);
	if (chunks > max_chunks) chunks = max_chunks;
	if (chunks > (M + 255) / 256) chunks = (M + 255) / 256;
	if (chunks < 1) chunks = 1;
	a.chunk = ((M + chunks - 1) / chunks + TC_K - 1) / TC_K * TC_K;
	chunks = (M + a.chunk - 1) / a.chunk;
	a.stages = l.co <= 128 ? 3 : 2;
	a.tmem_cols = 32;
	while (a.tmem_cols < (uint32_t)l.co) a.tmem_cols <<= 1;
	a.err = U->d_err;
	const size_t smem = (size_t)a.stages * ((size_t)l.co * 128 + (size_t)TC_M * 128) + (size_t)a.stages * 8 + 16;
	KEL_CUDA(allow_dynamic_smem<conv_wgrad_tc>(200 * 1024));
	conv_wgrad_tc<<<dim3((unsigned)tiles, (unsigned)chunks), 128, smem, U->stream>>>(a);
	const int64_t per = (int64_t)l.co * K;
	launch_reduce_partials(U->partial, per, (int)chunks, U->g + l.woff, U->stream);
	bias_grads(dy, M, l.co, U->partial, U->g + l.woff + per, U->stream);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

int conv_grads(kel_unet *U, const UnetLayer &l, const bf16 *x, const bf16 *dy, int n) {
	if (U->conv_kernel == KEL_UNET_CONV_TCGEN05) return conv_grads_tc(U, l, x, dy, n);
	WgradArgs a;
	a.x = x;
	a.dy = dy;
	a.partial = U->partial;
	a.N = n;
	a.H = U->d.height >> l.level;
	a.W = U->d.width >> l.level;
	a.Ci = l.ci;
	a.Co = l.co;
	const int64_t M = (int64_t)n * a.H * a.W;
	const int K = 9 * l.ci;
	const int tiles = ((l.co + CB_M - 1) / CB_M) * ((K + CB_N - 1) / CB_N);
	int64_t chunks = (600 + tiles - 1) / tiles;
	const int64_t max_chunks = U->partial_len / ((int64_t)l.co * K);
	if (chunks > max_chunks) chunks = max_chunks;
	if (chunks > (M + 255) / 256) chunks = (M + 255) / 256;
	if (chunks < 1) chunks = 1;
	a.chunk = ((M + chunks - 1) / chunks + 15) / 16 * 16;
	chunks = (M + a.chunk - 1) / a.chunk;
	dim3 grid((unsigned)((l.co + CB_M - 1) / CB_M), (unsigned)((K + CB_N - 1) / CB_N), (unsigned)chunks);
	conv_wgrad<<<grid, 128, 0, U->stream>>>(a);
	const int64_t per = (int64_t)l.co * K;
	launch_reduce_partials(U->partial, per, (int)chunks, U->g + l.woff, U->stream);
	bias_grads(dy, M, l.co, U->partial, U->g + l.woff + per, U->stream);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

void init_params(kel_unet *U, uint64_t seed, std::vector<float> &h) {
	h.assign(U->nparam, 0.f);
	uint64_t s = seed * 6364136223846793005ull + 1442695040888963407ull;
	auto next = [&]() {
		s = s * 6364136223846793005ull + 1442695040888963407ull;
		return (double)((s >> 11) & ((1ull << 53) - 1)) / (double)(1ull << 53);
	};
	for (const auto &l : U->L) {
		const int64_t fan_in = (int64_t)l.k * l.k * l.ci;
		const double bound = std::sqrt(6.0 / (double)fan_in); // He-uniform
		const int64_t nw = (int64_t)l.co * fan_in;
		for (int64_t i = 0; i < nw; ++i) h[l.woff + i] = (float)((2.0 * next() - 1.0) * bound);
	}
}

int refresh(kel_unet *U) {
	ConvTable t;
	memset(&t, 0, sizeof(t));
	int64_t most = 0;
	for (auto &l : U->L) {
		if (l.k != 3) continue;
		if (t.nl == MAX_CONV) return fail(KEL_ERR_INVALID_ARGUMENT, "refresh: more than %d conv layers", MAX_CONV);
		t.off[t.nl] = l.woff;
		t.co[t.nl] = l.co;
		t.ci[t.nl] = l.ci;
		t.w[t.nl] = l.w;
		t.wf[t.nl] = l.wf;
		++t.nl;
		if ((int64_t)l.co * 9 * l.ci > most) most = (int64_t)l.co * 9 * l.ci;
	}
	if (t.nl) {
		const unsigned bx = (unsigned)((most + 255) / 256 < 296 ? (most + 255) / 256 : 296);
		refresh_conv_weights<<<dim3(bx, (unsigned)t.nl), 256, 0, U->stream>>>(U->p, t);
	}
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

} // namespace

// After a stream synchronisation: KEL_ERR_TIMEOUT if a tensor-core kernel
// gave up on a bounded wait since the last check (its output is not valid).
static int check_device_error(kel_unet *U, const char *who) {
	int e = 0;
	KEL_CUDA(cudaMemcpyAsync(&e, U->d_err, sizeof(int), cudaMemcpyDeviceToHost, U->stream));
	KEL_CUDA(cudaStreamSynchronize(U->stream));
	if (e) {
		KEL_CUDA(cudaMemsetAsync(U->d_err, 0, sizeof(int), U->stream));
		return fail(KEL_ERR_TIMEOUT, "%s: a tensor-core pipeline wait timed out", who);
	}
	return KEL_OK;
}

extern "C" int kel_unet_create(const kel_unet_desc *desc, uint64_t seed, kel_unet **out) {
	if (!desc || !out) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_create: null argument");
	*out = nullptr;
	if (desc->height % 8 || desc->width % 8 || desc->height < 8 || desc->width < 8)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_create: height and width must be multiples of 8");
	if (desc->in_channels != 16 || desc->out_channels < 1 || desc->out_channels > 8 || desc->max_batch < 1)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_create: in_channels must be 16, out_channels 1..8");
	for (int i = 0; i < 4; ++i)
		if (desc->widths[i] < 16 || desc->widths[i] % 16)
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_create: widths must be multiples of 16");
	kel_unet *U = new kel_unet();
	U->d = *desc;
	for (int k = 0; k < MAX_RES; ++k) {
		U->res.in[k] = -1;
		U->res.scale[k] = 0.f;
	}
	const int *w = desc->widths;
	struct Spec {
		int co, ci, k, level;
	};
	const Spec specs[15] = {{w[0], 16, 3, 0},		 {w[0], w[0], 3, 0}, {w[1], w[0], 3, 1},		{w[1], w[1], 3, 1},
							{w[2], w[1], 3, 2},		 {w[2], w[2], 3, 2}, {w[3], w[2], 3, 3},		{w[3], w[3], 3, 3},
							{w[2], w[3] + w[2], 3, 2}, {w[2], w[2], 3, 2}, {w[1], w[2] + w[1], 3, 1}, {w[1], w[1], 3, 1},
							{w[0], w[1] + w[0], 3, 0}, {w[0], w[0], 3, 0}, {desc->out_channels, w[0], 1, 0}};
	int64_t off = 0;
	int64_t max_w = 0;
	for (const auto &s : specs) {
		UnetLayer l;
		l.co = s.co;
		l.ci = s.ci;
		l.k = s.k;
		l.level = s.level;
		l.woff = off;
		off += (int64_t)s.co * s.k * s.k * s.ci + s.co;
		if ((int64_t)s.co * 9 * s.ci > max_w) max_w = (int64_t)s.co * 9 * s.ci;
		U->L.push_back(l);
	}
	U->nparam = off;
	{
		int dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&U->sms, cudaDevAttrMultiProcessorCount, dev);
	}
	cudaStreamCreateWithFlags(&U->stream, cudaStreamNonBlocking);
	U->own_stream = U->stream;
	auto fail_out = [&](cudaError_t e) {
		kel_unet_destroy(U);
		return fail(e == cudaErrorMemoryAllocation ? KEL_ERR_OUT_OF_MEMORY : KEL_ERR_CUDA, "kel_unet_create: %s",
					cudaGetErrorString(e));
	};
	cudaError_t e;
	if ((e = cudaMalloc(&U->p, sizeof(float) * off)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->g, sizeof(float) * off)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->m, sizeof(float) * off)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->v, sizeof(float) * off)) != cudaSuccess) return fail_out(e);
	cudaMemsetAsync(U->m, 0, sizeof(float) * off, U->stream);
	cudaMemsetAsync(U->v, 0, sizeof(float) * off, U->stream);
	cudaMemsetAsync(U->g, 0, sizeof(float) * off, U->stream);
	for (auto &l : U->L) {
		if (l.k != 3) continue;
		const int64_t nw = (int64_t)l.co * 9 * l.ci;
		if ((e = cudaMalloc(&l.w, sizeof(bf16) * nw)) != cudaSuccess) return fail_out(e);
		if ((e = cudaMalloc(&l.wf, sizeof(bf16) * nw)) != cudaSuccess) return fail_out(e);
	}
	U->partial_len = max_w * 64;
	if ((e = cudaMalloc(&U->partial, sizeof(float) * U->partial_len)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->loss_partial, sizeof(double) * 1024)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->d_err, sizeof(int))) != cudaSuccess) return fail_out(e);
	if ((e = cudaMemsetAsync(U->d_err, 0, sizeof(int), U->stream)) != cudaSuccess) return fail_out(e);
	const int n = desc->max_batch;
	U->batch = n;
	U->act.assign(T_COUNT, nullptr);
	U->grad.assign(T_COUNT, nullptr);
	for (int t = 0; t < T_COUNT; ++t) {
		if ((e = cudaMalloc(&U->act[t], sizeof(bf16) * telems(U, t, n))) != cudaSuccess) return fail_out(e);
		if ((e = cudaMalloc(&U->grad[t], sizeof(bf16) * telems(U, t, n))) != cudaSuccess) return fail_out(e);
	}
	const int64_t pix = (int64_t)n * desc->height * desc->width;
	if ((e = cudaMalloc(&U->input, sizeof(bf16) * pix * 16)) != cudaSuccess) return fail_out(e);
	const size_t colb = sizeof(float) * (size_t)desc->max_batch * desc->width;
	if ((e = cudaMalloc(&U->col_open, colb)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->col_h3, colb)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->col_res, colb)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->col_pl, colb)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->out, sizeof(float) * pix * desc->out_channels)) != cudaSuccess) return fail_out(e);
	if ((e = cudaMalloc(&U->dout, sizeof(float) * pix * desc->out_channels)) != cudaSuccess) return fail_out(e);
	std::vector<float> h;
	init_params(U, seed, h);
	if ((e = cudaMemcpyAsync(U->p, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice, U->stream)) != cudaSuccess)
		return fail_out(e);
	int rc = refresh(U);
	if (rc) {
		kel_unet_destroy(U);
		return rc;
	}
	cudaStreamSynchronize(U->stream);
	*out = U;
	return KEL_OK;
}

extern "C" int kel_unet_destroy(kel_unet *U) {
	if (!U) return KEL_OK;
	if (U->stream) cudaStreamSynchronize(U->stream);
	for (auto &l : U->L) {
		cudaFree(l.w);
		cudaFree(l.wf);
	}
	for (auto *p : U->act) cudaFree(p);
	for (auto *p : U->grad) cudaFree(p);
	cudaFree(U->p);
	cudaFree(U->g);
	cudaFree(U->m);
	cudaFree(U->v);
	cudaFree(U->partial);
	cudaFree(U->loss_partial);
	cudaFree(U->input);
	cudaFree(U->out);
	cudaFree(U->dout);
	cudaFree(U->d_err);
	cudaFree(U->col_open);
	cudaFree(U->col_h3);
	cudaFree(U->col_res);
	cudaFree(U->col_pl);
	cudaFree(U->tgt);
	cudaFree(U->adam_c);
	cudaFree(U->dev_loss);
	if (U->train_graph) cudaGraphExecDestroy(U->train_graph);
	if (U->own_stream) {
		cudaStreamSynchronize(U->own_stream);
		cudaStreamDestroy(U->own_stream);
	}
	delete U;
	return KEL_OK;
}

extern "C" int kel_unet_param_count(const kel_unet *U, int64_t *n) {
	if (!U || !n) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_param_count: null argument");
	*n = U->nparam;
	return KEL_OK;
}

extern "C" int kel_unet_get_params(kel_unet *U, float *host) {
	if (!U || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_get_params: null argument");
	KEL_CUDA(cudaMemcpyAsync(host, U->p, sizeof(float) * U->nparam, cudaMemcpyDeviceToHost, U->stream));
	KEL_CUDA(cudaStreamSynchronize(U->stream));
	return KEL_OK;
}

extern "C" int kel_unet_set_params(kel_unet *U, const float *host) {
	if (!U || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_set_params: null argument");
	KEL_CUDA(cudaMemcpyAsync(U->p, host, sizeof(float) * U->nparam, cudaMemcpyHostToDevice, U->stream));
	int rc = refresh(U);
	if (rc) return rc;
	KEL_CUDA(cudaStreamSynchronize(U->stream));
	return KEL_OK;
}

extern "C" int kel_unet_get_grads(kel_unet *U, float *host) {
	if (!U || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_get_grads: null argument");
	KEL_CUDA(cudaMemcpyAsync(host, U->g, sizeof(float) * U->nparam, cudaMemcpyDeviceToHost, U->stream));
	KEL_CUDA(cudaStreamSynchronize(U->stream));
	return KEL_OK;
}

static int check_batch(const kel_unet *U, int32_t n, const char *who) {
	if (!U || n < 1 || n > U->batch) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: batch must be 1..max_batch", who);
	return KEL_OK;
}

extern "C" int kel_unet_make_input(kel_unet *U, const uint8_t *d_mask, const float *d_umax, const float *d_tau,
								   int32_t n) {
	int rc = check_batch(U, n, "kel_unet_make_input");
	if (rc) return rc;
	const int H = U->d.height, W = U->d.width;
	column_features<<<(n * W + 127) / 128, 128, 0, U->stream>>>(d_mask, n, H, W, U->col_open, U->col_h3);
	column_resistance<<<n, 256, sizeof(float) * 4 * W, U->stream>>>(U->col_open, U->col_h3, n, W, U->col_res,
																	 U->col_pl);
	if ((size_t)H * 32 <= 48 * 1024)
		make_input<<<n * ((W + 31) / 32), 256, (size_t)H * 32, U->stream>>>(d_mask, d_umax, d_tau, U->col_open, U->col_h3,
																			  U->col_res, U->col_pl, U->input, n, H, W);
	else
		make_input_tall<<<grid_of((int64_t)n * H * W), 256, 0, U->stream>>>(d_mask, d_umax, d_tau, U->col_open, U->col_h3,
																			 U->col_res, U->col_pl, U->input, n, H, W);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

extern "C" int kel_unet_forward(kel_unet *U, int32_t n, float *d_out) {
	int rc = check_batch(U, n, "kel_unet_forward");
	if (rc) return rc;
	auto &A = U->act;
	const auto &L = U->L;
	const int *w = U->d.widths;
	const int H = U->d.height, W = U->d.width;
	auto cv = [&](int li, const bf16 *x, bf16 *y) {
		const UnetLayer &l = L[li];
		return conv_fwd(U, x, l.w, U->p + l.woff + (int64_t)l.co * 9 * l.ci, y, n, l.level, l.ci, l.co, true, true);
	};
	if ((rc = cv(0, U->input, A[T_E0A])) || (rc = cv(1, A[T_E0A], A[T_E0B]))) return rc;
	pool_forward<<<grid_of(telems(U, T_P0, n) / 8), 256, 0, U->stream>>>(A[T_E0B], A[T_P0], n, H, W, w[0]);
	if ((rc = cv(2, A[T_P0], A[T_E1A])) || (rc = cv(3, A[T_E1A], A[T_E1B]))) return rc;
	pool_forward<<<grid_of(telems(U, T_P1, n) / 8), 256, 0, U->stream>>>(A[T_E1B], A[T_P1], n, H / 2, W / 2, w[1]);
	if ((rc = cv(4, A[T_P1], A[T_E2A])) || (rc = cv(5, A[T_E2A], A[T_E2B]))) return rc;
	pool_forward<<<grid_of(telems(U, T_P2, n) / 8), 256, 0, U->stream>>>(A[T_E2B], A[T_P2], n, H / 4, W / 4, w[2]);
	if ((rc = cv(6, A[T_P2], A[T_BA])) || (rc = cv(7, A[T_BA], A[T_BB]))) return rc;
	upcat_forward<<<grid_of(telems(U, T_C2, n) / 8), 256, 0, U->stream>>>(A[T_BB], A[T_E2B], A[T_C2], n, H / 4, W / 4, w[3],
																	   w[2]);
	if ((rc = cv(8, A[T_C2], A[T_D2A])) || (rc = cv(9, A[T_D2A], A[T_D2B]))) return rc;
	upcat_forward<<<grid_of(telems(U, T_C1, n) / 8), 256, 0, U->stream>>>(A[T_D2B], A[T_E1B], A[T_C1], n, H / 2, W / 2, w[2],
																	   w[1]);
	if ((rc = cv(10, A[T_C1], A[T_D1A])) || (rc = cv(11, A[T_D1A], A[T_D1B]))) return rc;
	upcat_forward<<<grid_of(telems(U, T_C0, n) / 8), 256, 0, U->stream>>>(A[T_D1B], A[T_E0B], A[T_C0], n, H, W, w[1], w[0]);
	if ((rc = cv(12, A[T_C0], A[T_D0A])) || (rc = cv(13, A[T_D0A], A[T_D0B]))) return rc;
	const UnetLayer &hd = L[14];
	const int64_t M = (int64_t)n * H * W;
	head_forward<<<grid_of(M), 256, sizeof(float) * hd.co * hd.ci, U->stream>>>(A[T_D0B], U->p + hd.woff, U->p + hd.woff + (int64_t)hd.co * hd.ci,
													U->out, M, hd.ci, hd.co, U->input, U->d.in_channels, U->res);
	KEL_CUDA(cudaGetLastError());
	if (d_out && d_out != U->out)
		KEL_CUDA(cudaMemcpyAsync(d_out, U->out, sizeof(float) * M * hd.co, cudaMemcpyDeviceToDevice, U->stream));
	return KEL_OK;
}

// After kel_unet_forward with the same n: masked-free MSE against d_target
// (N,H,W,out_channels), all gradients into the FP32 gradient vector
// (overwritten).  *loss receives the loss (host).
static int unet_backward(kel_unet *U, const float *d_target, int32_t n, double *loss, double *dev_loss);

extern "C" int kel_unet_backward(kel_unet *U, const float *d_target, int32_t n, double *loss) {
	int rc = check_batch(U, n, "kel_unet_backward");
	if (rc) return rc;
	if (!d_target) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_backward: null target");
	return unet_backward(U, d_target, n, loss, nullptr);
}

// backward with the loss to the host (loss, synchronising) and/or to the
// device (dev_loss, on the net's stream)
static int unet_backward(kel_unet *U, const float *d_target, int32_t n, double *loss, double *dev_loss) {
	int rc;
	auto &A = U->act;
	auto &G = U->grad;
	const auto &L = U->L;
	const int *w = U->d.widths;
	const int H = U->d.height, W = U->d.width;
	const UnetLayer &hd = L[14];
	const int64_t M = (int64_t)n * H * W;
	const int64_t nout = M * hd.co;
	KEL_CUDA(cudaMemsetAsync(U->g, 0, sizeof(float) * U->nparam, U->stream));
	const int lb = 512;
	mse_loss<<<lb, 256, 0, U->stream>>>(U->out, d_target, U->dout, nout, U->loss_partial);
	// head
	head_backward_dx<<<grid_of(M), 256, sizeof(float) * hd.co * hd.ci, U->stream>>>(U->dout, U->p + hd.woff, G[T_D0B],
																						 M, hd.ci, hd.co);
	if (hd.co <= 8 && hd.ci % 8 == 0 && hd.ci <= 2048) {
		// enough blocks to keep every SM's loads in flight (each block's loop is
		// a chain of dependent accumulations)
		const int64_t chunk = (M + 1215) / 1216;
		const int nb = (int)((M + chunk - 1) / chunk);
		const int64_t per = (int64_t)hd.co * hd.ci + hd.co;
		head_dw_partial<<<nb, 256, 0, U->stream>>>(U->dout, A[T_D0B], M, hd.ci, hd.co, chunk, U->partial);
		launch_reduce_partials(U->partial, per, nb, U->g + hd.woff, U->stream);
	} else {
		head_backward_dw<<<hd.co * hd.ci + hd.co, 256, 0, U->stream>>>(U->dout, A[T_D0B], M, hd.ci, hd.co,
																	   U->g + hd.woff);
	}
	// one conv layer: relu backward on dy, weight/bias grads, data grad into dx
	auto back = [&](int li, int t_in, const bf16 *x_in, int t_out, bf16 *dx) -> int {
		const UnetLayer &l = L[li];
		relu_backward<<<grid_of(telems(U, t_out, n) / 8), 256, 0, U->stream>>>(G[t_out], A[t_out], telems(U, t_out, n));
		int r = conv_grads(U, l, x_in, G[t_out], n);
		if (r) return r;
		if (dx) r = conv_fwd(U, G[t_out], l.wf, nullptr, dx, n, l.level, l.co, l.ci, false, false);
		(void)t_in;
		return r;
	};
	if ((rc = back(13, T_D0A, A[T_D0A], T_D0B, G[T_D0A])) || (rc = back(12, T_C0, A[T_C0], T_D0A, G[T_C0]))) return rc;
	upcat_backward<<<grid_of(telems(U, T_C0, n) / 8), 256, 0, U->stream>>>(G[T_C0], G[T_D1B], G[T_E0B], n, H, W, w[1], w[0]);
	if ((rc = back(11, T_D1A, A[T_D1A], T_D1B, G[T_D1A])) || (rc = back(10, T_C1, A[T_C1], T_D1A, G[T_C1]))) return rc;
	upcat_backward<<<grid_of(telems(U, T_C1, n) / 8), 256, 0, U->stream>>>(G[T_C1], G[T_D2B], G[T_E1B], n, H / 2, W / 2, w[2],
																		w[1]);
	if ((rc = back(9, T_D2A, A[T_D2A], T_D2B, G[T_D2A])) || (rc = back(8, T_C2, A[T_C2], T_D2A, G[T_C2]))) return rc;
	upcat_backward<<<grid_of(telems(U, T_C2, n) / 8), 256, 0, U->stream>>>(G[T_C2], G[T_BB], G[T_E2B], n, H / 4, W / 4, w[3],
																		w[2]);
	if ((rc = back(7, T_BA, A[T_BA], T_BB, G[T_BA])) || (rc = back(6, T_P2, A[T_P2], T_BA, G[T_P2]))) return rc;
	// encoder level 2: d(e2b) = pool_backward(d p2) + d skip2 (kept in G[T_E2B])
	pool_backward_add<<<grid_of(telems(U, T_E2B, n) / 8), 256, 0, U->stream>>>(G[T_P2], G[T_E2B], G[T_E2B], n, H / 4,
																			 W / 4, w[2]);
	if ((rc = back(5, T_E2A, A[T_E2A], T_E2B, G[T_E2A])) || (rc = back(4, T_P1, A[T_P1], T_E2A, G[T_P1]))) return rc;
	pool_backward_add<<<grid_of(telems(U, T_E1B, n) / 8), 256, 0, U->stream>>>(G[T_P1], G[T_E1B], G[T_E1B], n, H / 2,
																			 W / 2, w[1]);
	if ((rc = back(3, T_E1A, A[T_E1A], T_E1B, G[T_E1A])) || (rc = back(2, T_P0, A[T_P0], T_E1A, G[T_P0]))) return rc;
	pool_backward_add<<<grid_of(telems(U, T_E0B, n) / 8), 256, 0, U->stream>>>(G[T_P0], G[T_E0B], G[T_E0B], n, H, W, w[0]);
	if ((rc = back(1, T_E0A, A[T_E0A], T_E0B, G[T_E0A])) || (rc = back(0, -1, U->input, T_E0A, nullptr))) return rc;
	KEL_CUDA(cudaGetLastError());
	if (dev_loss) {
		loss_finish<<<1, 64, 0, U->stream>>>(U->loss_partial, lb, nout, dev_loss);
		KEL_CUDA(cudaGetLastError());
	}
	if (loss) {
		std::vector<double> part(lb);
		KEL_CUDA(cudaMemcpyAsync(part.data(), U->loss_partial, sizeof(double) * lb, cudaMemcpyDeviceToHost, U->stream));
		KEL_CUDA(cudaStreamSynchronize(U->stream));
		if ((rc = check_device_error(U, "kel_unet_backward"))) return rc;
		// loss_finish's order: 64 strided sums, then a pairwise tree
		double s64[64];
		for (int t = 0; t < 64; ++t) {
			double s = 0.0;
			for (int k = t; k < lb; k += 64) s += part[k];
			s64[t] = s;
		}
		for (int o = 32; o > 0; o >>= 1)
			for (int t = 0; t < o; ++t) s64[t] += s64[t + o];
		*loss = s64[0] / (double)nout;
	}
	return KEL_OK;
}

extern "C" int kel_unet_adam_step(kel_unet *U, float lr, float beta1, float beta2, float eps, int32_t step) {
	if (!U || step < 1) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_adam_step: bad arguments");
	const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
	adam_update<<<grid_of(U->nparam), 256, 0, U->stream>>>(U->p, U->g, U->m, U->v, U->nparam, lr, beta1, beta2, eps, c1,
														   c2);
	KEL_CUDA(cudaGetLastError());
	return refresh(U);
}

// forward, backward (device loss), Adam from the device constants, refresh
static int train_body(kel_unet *U, int32_t n, float b1, float b2, float eps) {
	int rc;
	if ((rc = kel_unet_forward(U, n, nullptr))) return rc;
	if ((rc = unet_backward(U, U->tgt, n, nullptr, U->dev_loss))) return rc;
	adam_update_dev<<<grid_of(U->nparam), 256, 0, U->stream>>>(U->p, U->g, U->m, U->v, U->nparam, U->adam_c, b1, b2, eps);
	KEL_CUDA(cudaGetLastError());
	return refresh(U);
}

extern "C" int kel_unet_train_step(kel_unet *U, const float *d_target, int32_t n, float lr, float beta1, float beta2,
								   float eps, int32_t step, double *d_loss) {
	int rc = check_batch(U, n, "kel_unet_train_step");
	if (rc) return rc;
	if (!d_target || step < 1) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_train_step: bad arguments");
	const int64_t tcount = (int64_t)U->d.max_batch * U->d.height * U->d.width * U->d.out_channels;
	if (!U->tgt) {
		KEL_CUDA(cudaMalloc(&U->tgt, sizeof(float) * tcount));
		KEL_CUDA(cudaMalloc(&U->adam_c, sizeof(float) * 4));
		KEL_CUDA(cudaMalloc(&U->dev_loss, sizeof(double)));
	}
	const int64_t bytes = sizeof(float) * (int64_t)n * U->d.height * U->d.width * U->d.out_channels;
	KEL_CUDA(cudaMemcpyAsync(U->tgt, d_target, bytes, cudaMemcpyDeviceToDevice, U->stream));
	const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
	adam_consts<<<1, 1, 0, U->stream>>>(U->adam_c, lr, c1, c2);
	KEL_CUDA(cudaGetLastError());
	const bool same = U->train_graph && U->train_n == n && U->train_b1 == beta1 && U->train_b2 == beta2 &&
					  U->train_eps == eps;
	if (!same) {
		if (U->train_graph) cudaGraphExecDestroy(U->train_graph);
		U->train_graph = nullptr;
		if (!U->train_warm) {
			// the first step runs its launches one by one (one-time set-up of
			// the kernels happens outside any capture)
			if ((rc = train_body(U, n, beta1, beta2, eps))) return rc;
			U->train_warm = true;
		} else {
			cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
			KEL_CUDA(cudaStreamIsCapturing(U->stream, &cap));
			cudaGraph_t g = nullptr;
			bool ok = cap == cudaStreamCaptureStatusNone &&
					  cudaStreamBeginCapture(U->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
			if (ok) {
				rc = train_body(U, n, beta1, beta2, eps);
				const cudaError_t e = cudaStreamEndCapture(U->stream, &g);
				ok = rc == KEL_OK && e == cudaSuccess && g && cudaGraphInstantiate(&U->train_graph, g, 0) == cudaSuccess;
				if (g) cudaGraphDestroy(g);
				if (rc) return rc;
			}
			if (!ok) { // no graph: launches one by one
				cudaGetLastError();
				U->train_graph = nullptr;
				if ((rc = train_body(U, n, beta1, beta2, eps))) return rc;
			} else {
				U->train_n = n;
				U->train_b1 = beta1;
				U->train_b2 = beta2;
				U->train_eps = eps;
			}
		}
	}
	// replay (a graph captured just now has not run yet either)
	if (U->train_graph) KEL_CUDA(cudaGraphLaunch(U->train_graph, U->stream));
	if (d_loss) KEL_CUDA(cudaMemcpyAsync(d_loss, U->dev_loss, sizeof(double), cudaMemcpyDeviceToDevice, U->stream));
	return KEL_OK;
}

extern "C" int kel_unet_last_loss(kel_unet *U, double *loss) {
	if (!U || !loss) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_last_loss: null argument");
	if (!U->dev_loss) return fail(KEL_ERR_STATE, "kel_unet_last_loss: no training step yet");
	KEL_CUDA(cudaMemcpyAsync(loss, U->dev_loss, sizeof(double), cudaMemcpyDeviceToHost, U->stream));
	KEL_CUDA(cudaStreamSynchronize(U->stream));
	return check_device_error(U, "kel_unet_last_loss");
}

extern "C" int kel_unet_set_stream(kel_unet *U, void *stream) {
	if (!U) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_set_stream: null net");
	U->stream = static_cast<cudaStream_t>(stream);
	return KEL_OK;
}

extern "C" int kel_unet_synchronize(kel_unet *U) {
	if (!U) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_synchronize: null net");
	KEL_CUDA(cudaStreamSynchronize(U->stream));
	return check_device_error(U, "kel_unet_synchronize");
}

extern "C" int kel_unet_set_residual(kel_unet *U, int32_t out_channel, int32_t in_channel, float scale) {
	if (!U) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_set_residual: null net");
	if (out_channel >= U->d.out_channels || out_channel >= MAX_RES ||
		(out_channel >= 0 && (in_channel < 0 || in_channel >= U->d.in_channels)))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_set_residual: channels %d <- %d out of range", out_channel,
					in_channel);
	if (out_channel < 0) {
		for (int k = 0; k < MAX_RES; ++k) U->res.in[k] = -1;
		return KEL_OK;
	}
	U->res.in[out_channel] = in_channel;
	U->res.scale[out_channel] = scale;
	return KEL_OK;
}

extern "C" int kel_unet_set_conv_kernel(kel_unet *U, int32_t kind) {
	if (!U) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_set_conv_kernel: null net");
	if (kind != KEL_UNET_CONV_TCGEN05 && kind != KEL_UNET_CONV_MMA_SYNC)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_set_conv_kernel: unknown kind %d", kind);
	U->conv_kernel = kind;
	return KEL_OK;
}

// Direct input (bf16 NHWC, 16 channels) for tests: copies into the net's input.
extern "C" int kel_unet_get_input(kel_unet *U, uint16_t *d_out_bf16, int32_t n) {
	int rc = check_batch(U, n, "kel_unet_get_input");
	if (rc) return rc;
	if (!d_out_bf16) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_unet_get_input: null output");
	KEL_CUDA(cudaMemcpyAsync(d_out_bf16, U->input, sizeof(bf16) * (int64_t)n * U->d.height * U->d.width * 16,
							 cudaMemcpyDeviceToDevice, U->stream));
	KEL_CUDA(cudaStreamSynchronize(U->stream));
	return KEL_OK;
}

extern "C" int kel_unet_set_input(kel_unet *U, const uint16_t *d_input_bf16, int32_t n) {
	int rc = check_batch(U, n, "kel_unet_set_input");
	if (rc) return rc;
	KEL_CUDA(cudaMemcpyAsync(U->input, d_input_bf16, sizeof(bf16) * (int64_t)n * U->d.height * U->d.width * 16,
							 cudaMemcpyDeviceToDevice, U->stream));
	return KEL_OK;
}
