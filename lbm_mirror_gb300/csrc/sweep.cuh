// Fused collide + boundary + stream sweep (AA pattern, in place) for sm_103a.
//
// One kernel launch is one time step of keldu/lbm_mirror's driver loop: the
// collide+BC parallel_for and the pull-Stream parallel_for of
// examples/poiseulle_2d_gpu/poiseulle_2d_gpu.cpp:169-224,384-399 fused into a
// single pass over HBM.
//
// Memory: one lattice of populations, structure of arrays.  Direction plane i
// holds f_i of every cell; a plane is nz*ny rows of nxp cells (nxp = nx padded
// to a multiple of 4; padding cells carry flag 0).  The AA pattern keeps the
// reference's two-lattice semantics with one array:
//   even t: cell x reads f_i from A[i][x] and writes f*_i to A[opp i][x];
//   odd  t: cell x reads f_i from A[opp i][x - c_i] and writes f*_i to
//           A[i][x + c_i].
// Every location touched in a step is read and written by the same cell, so
// the step is race free.  The reference's zero ghost ring is reproduced by
// substituting zero for reads whose source lies outside the lattice and by
// dropping writes whose destination does; a flag-0 cell emits zero
// populations, which is what the ghost ring supplies.
//
// Threads: each thread owns 4 consecutive cells of a row (128-bit accesses for
// FP32, 64-bit for FP16S).  Warps never straddle rows, so the x-shifted
// accesses of odd steps are realigned with warp shuffles; only the first and
// last lane of a warp touch a neighbouring warp's cells with scalar accesses.
#pragma once

#include <cuda_fp16.h>
#include <cstdint>

#include "descriptors.cuh"

namespace kel {
namespace gb {

enum : int { STORE_FP32 = 0, STORE_FP16S = 1 };
enum : int { COLL_BGK = 0, COLL_BGK_GUO = 1, COLL_PSM = 2, COLL_PSM_GUO = 3, COLL_HLBM = 4 };
enum : int {
	BC_NONE = 0,
	BC_BOUNCE_BACK = 1,
	BC_FLUID = 2,
	BC_ZOUHE_VELOCITY_X = 3,
	BC_ZOUHE_PRESSURE_X = 4,
	BC_MOVING_WALL = 5,
	BC_ANTI_BOUNCE_BACK = 6,
	BC_EQUILIBRIUM = 7,
	BC_HALFWAY_WALL = 8
};
constexpr int MAX_FLAGS = 8;
constexpr int CPT_ROWS = -1; // launch shape of the row pipeline (KEL_LAUNCH_ROWS)

// Per-flag operation, resident in device memory (read through the read-only path).
struct OpEntry {
	int32_t bc, collide, east, use_profile;
	// FPLBM programs (swept with the Guo-forcing kernels): bgk_only -- this
	// op's cells collide with plain BGK (a boundary step precedes); no_macros
	// -- its cells leave the density / momentum macros as the FPLBM reset
	// wrote them
	int32_t bgk_only, no_macros;
	float rho;
	float u[3];
	float lid[27]; // moving-wall additive term 2 w_i (c_i.u_w)/cs^2, rounded like the reference
	float eq[27];  // equilibrium(rho, u) for the Equilibrium boundary
};

struct SweepParams {
	void *f;          // populations (float or __half), plane-major
	int64_t plane;    // cells per direction plane (nz*ny*nxp)
	const uint8_t *flags;
	float *rho;       // macros "density" (plane layout)
	float *u;         // macros "velocity", D planes
	const float *por; // macros "porosity"
	const float *force; // macros "force", D planes
	const float *hN;    // HLBM "particle_N", D planes
	const float *hD;    // HLBM "particle_D"
	const float *profile; // inlet u_x per y
	const OpEntry *ops;
	int nxp, ny, nz;
	int nq;  // quads per row (nxp / 4)
	int wpr; // warps per row
	int periodic;
	int write_macros;
	float omega;      // 1/tau in float, as the reference divides
	float guo_scale;  // 1 - 0.5 * omega
	float g[3];       // global force
	float wshift[27]; // FP16S: stored value is f - wshift[i]
	int cpt;          // cells per thread: 1 (sweep1_kernel), 2 (sweep2_kernel), 4 (sweep_kernel), CPT_ROWS (sweep_rows_kernel)
	int idx32;        // Q * plane < 2^31: offsets from a cell fit 32-bit arithmetic
	int block;        // threads per block
	int wpr2;         // sweep2_kernel: warps per row (32 cell pairs per warp)
	const uint32_t *hw_mask; // half-way walls: per cell, bit i = the neighbour x + c_i is one (null: none)
	int stages;       // sweep_rows_kernel: row stages in shared memory
	int sms;          // multiprocessors of the device (persistent grid of sweep_rows_kernel)
	unsigned *err;    // sweep_rows_kernel: set to 1 when a bounded wait gave up
	// bit f: flag value f (1 .. MAX_FLAGS-1) has no boundary step and collides,
	// so its cells skip the operation-table dispatch (same result)
	uint32_t plain;
	// sweep1_kernel: blocks ahead whose rows a block prefetches into L2 (0: none)
	int pf_ahead;
};

// What the per-cell physics needs from a launch: the flag -> operation table,
// the inlet profile and the collision constants.
struct CellCtx {
	const OpEntry *ops;
	const float *profile;
	float omega;
	float guo_scale;
	float g[3];
};

__device__ __forceinline__ CellCtx cell_ctx(const SweepParams &p) {
	CellCtx c;
	c.ops = p.ops;
	c.profile = p.profile;
	c.omega = p.omega;
	c.guo_scale = p.guo_scale;
	c.g[0] = p.g[0];
	c.g[1] = p.g[1];
	c.g[2] = p.g[2];
	return c;
}

// ---------------------------------------------------------------------------
// Arithmetic policy.  EXACT: the reference's rounding sequence (no fused
// multiply-add, equilibrium bracket in double); otherwise plain float math.
template <bool EXACT>
struct Ar;

template <>
struct Ar<true> {
	__device__ static __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
	__device__ static __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
	__device__ static __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
	__device__ static __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};

template <>
struct Ar<false> {
	__device__ static __forceinline__ float add(float a, float b) { return a + b; }
	__device__ static __forceinline__ float sub(float a, float b) { return a - b; }
	__device__ static __forceinline__ float mul(float a, float b) { return a * b; }
	__device__ static __forceinline__ float div(float a, float b) { return a / b; }
};

// ---------------------------------------------------------------------------
// Storage policy.
template <int STORE>
struct Store;

template <>
struct Store<STORE_FP32> {
	using T = float;
	__device__ static __forceinline__ float4 ld4(const void *base, int64_t idx, float) {
		return __ldcs(reinterpret_cast<const float4 *>(static_cast<const float *>(base) + idx));
	}
	__device__ static __forceinline__ float ld1(const void *base, int64_t idx, float) {
		return __ldcs(static_cast<const float *>(base) + idx);
	}
	__device__ static __forceinline__ void st4(void *base, int64_t idx, float4 v, float) {
		__stcs(reinterpret_cast<float4 *>(static_cast<float *>(base) + idx), v);
	}
	__device__ static __forceinline__ void st1(void *base, int64_t idx, float v, float) {
		__stcs(static_cast<float *>(base) + idx, v);
	}
	__device__ static __forceinline__ float2 ld2(const void *base, int64_t idx, float) {
		return __ldcs(reinterpret_cast<const float2 *>(static_cast<const float *>(base) + idx));
	}
	__device__ static __forceinline__ void st2(void *base, int64_t idx, float2 v, float) {
		__stcs(reinterpret_cast<float2 *>(static_cast<float *>(base) + idx), v);
	}
};

template <>
struct Store<STORE_FP16S> {
	using T = __half;
	__device__ static __forceinline__ float4 ld4(const void *base, int64_t idx, float s) {
		uint2 r = __ldcs(reinterpret_cast<const uint2 *>(static_cast<const __half *>(base) + idx));
		__half2 a = *reinterpret_cast<__half2 *>(&r.x);
		__half2 b = *reinterpret_cast<__half2 *>(&r.y);
		float2 fa = __half22float2(a), fb = __half22float2(b);
		return make_float4(fa.x + s, fa.y + s, fb.x + s, fb.y + s);
	}
	// f = float(h) + s with one rounding, as one mixed-precision add (the
	// exact conversion of h, then the float add: the same bits as
	// __half2float(h) + s)
	__device__ static __forceinline__ float ld1(const void *base, int64_t idx, float s) {
		const unsigned short h = __half_as_ushort(static_cast<const __half *>(base)[idx]);
		float r;
		asm("add.rn.f32.f16 %0, %1, %2;" : "=f"(r) : "h"(h), "f"(s));
		return r;
	}
	__device__ static __forceinline__ void st4(void *base, int64_t idx, float4 v, float s) {
		__half2 a = __floats2half2_rn(v.x - s, v.y - s);
		__half2 b = __floats2half2_rn(v.z - s, v.w - s);
		uint2 r;
		r.x = *reinterpret_cast<uint32_t *>(&a);
		r.y = *reinterpret_cast<uint32_t *>(&b);
		__stcs(reinterpret_cast<uint2 *>(static_cast<__half *>(base) + idx), r);
	}
	__device__ static __forceinline__ void st1(void *base, int64_t idx, float v, float s) {
		static_cast<__half *>(base)[idx] = __float2half_rn(v - s);
	}
	__device__ static __forceinline__ float2 ld2(const void *base, int64_t idx, float s) {
		unsigned r = __ldcs(reinterpret_cast<const unsigned *>(static_cast<const __half *>(base) + idx));
		const float2 v = __half22float2(*reinterpret_cast<__half2 *>(&r));
		return make_float2(v.x + s, v.y + s);
	}
	__device__ static __forceinline__ void st2(void *base, int64_t idx, float2 v, float s) {
		__half2 h = __floats2half2_rn(v.x - s, v.y - s);
		__stcs(reinterpret_cast<unsigned *>(static_cast<__half *>(base) + idx), *reinterpret_cast<unsigned *>(&h));
	}
};

// ---------------------------------------------------------------------------
// Cell physics (one cell, populations in registers).

// compute_rho_u, modules/core/c++/macroscopic.hpp:10-35: the reference's
// summation order; EXACT divides each component by rho, the fast arithmetic
// multiplies by the correctly rounded reciprocal of rho (one rounding more).
template <class L, bool EXACT>
__device__ __forceinline__ void moments(const float (&f)[L::Q], float &rho, float (&u)[3]) {
	using A = Ar<true>;
	float r = 0.f, v0 = 0.f, v1 = 0.f, v2 = 0.f;
#pragma unroll
	for (int j = 0; j < L::Q; ++j) {
		r = A::add(r, f[j]);
		if (L::cx(j) > 0) v0 = A::add(v0, f[j]);
		if (L::cx(j) < 0) v0 = A::sub(v0, f[j]);
		if (L::cy(j) > 0) v1 = A::add(v1, f[j]);
		if (L::cy(j) < 0) v1 = A::sub(v1, f[j]);
		if (L::D == 3) {
			if (L::cz(j) > 0) v2 = A::add(v2, f[j]);
			if (L::cz(j) < 0) v2 = A::sub(v2, f[j]);
		}
	}
	rho = r;
	if (EXACT) {
		u[0] = A::div(v0, r);
		u[1] = A::div(v1, r);
		u[2] = L::D == 3 ? A::div(v2, r) : 0.f;
	} else {
		const float ir = __frcp_rn(r);
		u[0] = v0 * ir;
		u[1] = v1 * ir;
		u[2] = L::D == 3 ? v2 * ir : 0.f;
	}
}

// c_i . u with the reference's summation order (0 + u_0 c_0 + u_1 c_1 ...)
template <class L, bool EXACT>
__device__ __forceinline__ float cdot(int i, const float (&u)[3]) {
	using A = Ar<EXACT>;
	float s = 0.f;
	if (L::cx(i) > 0) s = A::add(s, u[0]);
	if (L::cx(i) < 0) s = A::sub(s, u[0]);
	if (L::cy(i) > 0) s = A::add(s, u[1]);
	if (L::cy(i) < 0) s = A::sub(s, u[1]);
	if (L::D == 3) {
		if (L::cz(i) > 0) s = A::add(s, u[2]);
		if (L::cz(i) < 0) s = A::sub(s, u[2]);
	}
	return s;
}

// equilibrium, modules/core/c++/equilibrium.hpp:7-48
template <class L, bool EXACT>
__device__ __forceinline__ void equilibrium(float rho, const float (&u)[3], float (&eq)[L::Q]) {
	using A = Ar<true>;
	float vv = A::mul(u[0], u[0]);
	vv = A::add(vv, A::mul(u[1], u[1]));
	if (L::D == 3) vv = A::add(vv, A::mul(u[2], u[2]));
	if (EXACT) {
		const double h = __dmul_rn(1.5, (double)vv);
#pragma unroll
		for (int i = 0; i < L::Q; ++i) {
			const float vcc = A::mul(cdot<L, true>(i, u), 3.0f);
			const float wr = A::mul((float)L::w(i), rho);
			double br = __dsub_rn(__dadd_rn(1.0, (double)vcc), h);
			br = __dadd_rn(br, __dmul_rn((double)A::mul(vcc, vcc), 0.5));
			eq[i] = __double2float_rn(__dmul_rn((double)wr, br));
		}
	} else {
		// w rho (1 + d), d = vcc + (vcc^2/2 - 1.5 vv), with the reference's float
		// sub-terms and one fused rounding at the end.  Opposite directions
		// share w, and their c.u and vcc are exact negatives (IEEE rounding is
		// sign-symmetric), so vcc, the symmetric part and w rho are computed
		// once per pair: the same bits as computing each direction alone.
		const float h = __fmul_rn(1.5f, vv);
#pragma unroll
		for (int i = 0; i < L::Q; ++i) {
			if (L::opp(i) < i) continue; // done with its partner
			const float vcc = __fmul_rn(3.0f, cdot<L, true>(i, u));
			const float sym = __fmaf_rn(0.5f * vcc, vcc, -h);
			const float wr = __fmul_rn((float)L::w(i), rho);
			eq[i] = __fmaf_rn(wr, vcc + sym, wr);
			if (L::opp(i) != i) eq[L::opp(i)] = __fmaf_rn(wr, sym - vcc, wr);
		}
	}
}

// Guo forcing term F_i, modules/core/c++/collision.hpp:170-196
template <class L, bool EXACT>
__device__ __forceinline__ float guo_term(int i, const float (&u)[3], const float (&F)[3]) {
	using A = Ar<true>;
	const float s = A::mul(A::mul(cdot<L, true>(i, u), 3.0f), 3.0f);
	float proj = 0.f;
#pragma unroll
	for (int k = 0; k < L::D; ++k) {
		const float ck = (float)cdir<L>(i, k);
		const float t1 = A::mul(A::sub(ck, u[k]), 3.0f);
		const float t2 = A::mul(ck, s);
		proj = A::add(proj, A::mul(A::add(t1, t2), F[k]));
	}
	return A::mul((float)L::w(i), proj);
}

// D2Q9 ZouHePressureX<Dir>, modules/core/c++/boundary.hpp:186-226
template <bool EXACT>
__device__ __forceinline__ void zouhe_pressure_d2q9(float (&f)[9], bool east, float rs) {
	using A = Ar<true>;
	const float c23 = (float)(2.0 / 3.0), c16 = (float)(1.0 / 6.0);
	if (east) {
		const float S = A::add(A::add(A::add(f[0], f[3]), f[4]), A::mul(A::add(A::add(f[1], f[5]), f[7]), 2.f));
		const float r = A::sub(rs, S);
		f[2] = A::add(f[1], A::mul(c23, r));
		f[6] = A::add(A::add(f[5], A::mul(c16, r)), A::mul(0.5f, A::sub(f[3], f[4])));
		f[8] = A::add(A::add(f[7], A::mul(c16, r)), A::mul(0.5f, A::sub(f[4], f[3])));
	} else {
		const float S = A::add(A::add(A::add(f[0], f[3]), f[4]), A::mul(A::add(A::add(f[2], f[6]), f[8]), 2.f));
		const float r = A::sub(S, rs);
		f[1] = A::sub(f[2], A::mul(c23, r));
		f[5] = A::add(A::sub(f[6], A::mul(c16, r)), A::mul(0.5f, A::sub(f[4], f[3])));
		f[7] = A::add(A::sub(f[8], A::mul(c16, r)), A::mul(0.5f, A::sub(f[3], f[4])));
	}
}

// D2Q9 ZouHeVelocityX<East>, modules/core/c++/boundary.hpp:775-802
template <bool EXACT>
__device__ __forceinline__ void zouhe_velocity_d2q9(float (&f)[9], bool east, float ux, float uy) {
	using A = Ar<true>;
	const float c23 = (float)(2.0 / 3.0), c16 = (float)(1.0 / 6.0);
	const float ds = east ? A::add(A::add(f[1], f[5]), f[7]) : A::add(A::add(f[2], f[6]), f[8]);
	const float rho = A::div(A::add(A::add(A::add(f[0], f[4]), f[3]), A::mul(ds, 2.f)), A::add(ux, 1.0f));
	const float rux = A::mul(A::mul(c16, rho), ux);
	const float ruy = A::mul(rho, uy);
	if (east) {
		f[2] = A::add(f[1], A::mul(A::mul(c23, rho), ux));
		f[6] = A::add(A::add(f[5], rux), A::mul(A::add(A::sub(f[3], f[4]), ruy), 0.5f));
		f[8] = A::add(A::add(f[7], rux), A::mul(A::add(A::sub(f[4], f[3]), ruy), 0.5f));
	} else {
		f[1] = A::add(f[2], A::mul(A::mul(c23, rho), ux));
		f[5] = A::add(A::add(f[6], rux), A::mul(A::add(A::sub(f[4], f[3]), ruy), 0.5f));
		f[7] = A::add(A::add(f[8], rux), A::mul(A::add(A::sub(f[3], f[4]), ruy), 0.5f));
	}
}

// D3Q27 ZouHePressureX<East>, modules/core/c++/boundary.hpp:229-756.  The
// side is a template argument: a run-time side would index f with a run-time
// offset and move the whole population array to local memory.
template <bool EXACT, bool east>
__device__ __forceinline__ void zouhe_pressure_d3q27(float (&f)[27], float rs) {
	using A = Ar<true>;
	const float a = (float)(4.0 / 9.0), b = (float)(1.0 / 9.0), e = (float)(1.0 / 36.0);
	float S = f[0];
	S = A::add(S, f[3]);
	S = A::add(S, f[6]);
	S = A::add(S, f[9]);
	S = A::add(S, f[12]);
	S = A::add(S, f[15]);
	S = A::add(S, f[18]);
	S = A::add(S, f[21]);
	S = A::add(S, f[24]);
	// known side: cx = +1 at x = max (east = false), cx = -1 at x = 0 (east = true)
	constexpr int k0 = east ? 1 : 2;
	float K = f[k0];
#pragma unroll
	for (int j = 1; j < 9; ++j) K = A::add(K, f[k0 + 3 * j]);
	S = A::add(S, A::mul(2.f, K));
	const float rux = east ? A::sub(rs, S) : A::sub(S, rs);
	// tangential momenta
	float ruy = A::add(-f[3], f[6]);
	ruy = A::sub(ruy, f[12]);
	ruy = A::add(ruy, f[15]);
	ruy = A::sub(ruy, f[21]);
	ruy = A::add(ruy, f[24]);
	float ty = A::add(-f[k0 + 3], f[k0 + 6]);
	ty = A::sub(ty, f[k0 + 12]);
	ty = A::add(ty, f[k0 + 15]);
	ty = A::sub(ty, f[k0 + 21]);
	ty = A::add(ty, f[k0 + 24]);
	ruy = A::add(ruy, A::mul(2.f, ty));
	float ruz = A::sub(-f[9], f[12]);
	ruz = A::sub(ruz, f[15]);
	ruz = A::add(ruz, f[18]);
	ruz = A::add(ruz, f[21]);
	ruz = A::add(ruz, f[24]);
	float tz = A::sub(-f[k0 + 9], f[k0 + 12]);
	tz = A::sub(tz, f[k0 + 15]);
	tz = A::add(tz, f[k0 + 18]);
	tz = A::add(tz, f[k0 + 21]);
	tz = A::add(tz, f[k0 + 24]);
	ruz = A::add(ruz, A::mul(2.f, tz));
	if constexpr (!east) {
		f[1] = A::sub(f[2], A::mul(a, rux));
		f[4] = A::sub(f[5], A::mul(b, A::add(rux, ruy)));
		f[7] = A::add(f[8], A::mul(b, A::add(-rux, ruy)));
		f[10] = A::sub(f[11], A::mul(b, A::add(rux, ruz)));
		f[13] = A::sub(f[14], A::mul(e, A::add(A::add(rux, ruy), ruz)));
		f[16] = A::add(f[17], A::mul(e, A::add(A::add(-rux, ruy), ruz)));
		f[19] = A::add(f[20], A::mul(b, A::add(-rux, ruz)));
		f[22] = A::add(f[23], A::mul(e, A::add(A::sub(-rux, ruy), ruz)));
		f[25] = A::add(f[26], A::mul(e, A::add(A::add(-rux, ruy), ruz)));
	} else {
		f[2] = A::add(f[1], A::mul(a, rux));
		f[5] = A::add(f[4], A::mul(b, A::sub(rux, ruy)));
		f[8] = A::add(f[7], A::mul(b, A::add(rux, ruy)));
		f[11] = A::add(f[10], A::mul(b, A::sub(rux, ruz)));
		f[14] = A::add(f[13], A::mul(e, A::sub(A::sub(rux, ruy), ruz)));
		f[17] = A::add(f[16], A::mul(e, A::sub(A::add(rux, ruy), ruz)));
		f[20] = A::add(f[19], A::mul(b, A::add(rux, ruz)));
		f[23] = A::add(f[22], A::mul(e, A::add(A::sub(rux, ruy), ruz)));
		f[26] = A::add(f[25], A::mul(e, A::add(A::add(rux, ruy), ruz)));
	}
}

// The collision chosen by the program (BGK / BGKGuo / Psm / Psm + Guo).
// For COLL_HLBM the force argument carries the cell's HLBM accumulators
// (N_x, N_y, D) and por its porosity.
template <class L, int COLL, bool EXACT>
__device__ __forceinline__ void collide(float (&f)[L::Q], const CellCtx &p, float por, const float (&Fc)[3],
										float &rho, float (&u)[3]) {
	using A = Ar<true>;
	moments<L, EXACT>(f, rho, u);
	if (COLL == COLL_HLBM) {
		// hlbm.hpp:86-96: u <- u por + (D > 0 ? N (1 - por) / D : N)
		const float flip = A::sub(1.0f, por), Dv = Fc[2];
#pragma unroll
		for (int k = 0; k < 2; ++k) {
			const float add = Dv > 0.f ? A::div(A::mul(Fc[k], flip), Dv) : Fc[k];
			u[k] = A::add(A::mul(u[k], por), add);
		}
	}
	float eq[L::Q];
	equilibrium<L, EXACT>(rho, u, eq);
	float F[3] = {0.f, 0.f, 0.f};
	if (COLL == COLL_BGK_GUO || COLL == COLL_PSM_GUO) {
#pragma unroll
		for (int k = 0; k < L::D; ++k) F[k] = A::add(Fc[k], p.g[k]);
	}
	if (COLL == COLL_BGK || COLL == COLL_HLBM) {
#pragma unroll
		for (int i = 0; i < L::Q; ++i)
			f[i] = EXACT ? A::add(f[i], A::mul(p.omega, A::sub(eq[i], f[i]))) : __fmaf_rn(p.omega, A::sub(eq[i], f[i]), f[i]);
	} else if (COLL == COLL_BGK_GUO) {
#pragma unroll
		for (int i = 0; i < L::Q; ++i) {
			const float Fi = guo_term<L, EXACT>(i, u, F);
			f[i] = A::add(A::add(f[i], A::mul(p.omega, A::sub(eq[i], f[i]))), A::mul(Fi, p.guo_scale));
		}
	} else { // PSM, psm.hpp:79-88
		const float flip = A::sub(1.0f, por);
		float pre[L::Q];
#pragma unroll
		for (int i = 0; i < L::Q; ++i) pre[i] = f[i];
#pragma unroll
		for (int i = 0; i < L::Q; ++i) {
			float v = A::add(pre[i], A::mul(A::mul(p.omega, A::sub(eq[i], pre[i])), por));
			v = A::add(v, A::mul(A::sub(pre[L::opp(i)], pre[i]), flip));
			if (COLL == COLL_PSM_GUO) v = A::add(v, A::mul(guo_term<L, EXACT>(i, u, F), p.guo_scale));
			f[i] = v;
		}
	}
}

// Boundary step + collision of one cell (the body of a driver's switch(info)).
// Returns true when the cell collided (its moments go to the macro fields).
template <class L, int COLL, bool EXACT>
__device__ __forceinline__ bool cell_update(float (&f)[L::Q], int flag, int y, const CellCtx &p, float por,
											const float (&Fc)[3], float &rho, float (&u)[3]) {
	using A = Ar<true>;
	if (flag == 0) { // outside the lattice: what the zero ghost ring supplies
#pragma unroll
		for (int i = 0; i < L::Q; ++i) f[i] = 0.f;
		return false;
	}
	if (flag >= MAX_FLAGS) return false; // the drivers' `default: break;`
	const OpEntry *op = p.ops + flag;
	const int bc = __ldg(&op->bc); // BC_HALFWAY_WALL: no boundary step and collide = 0 (lower_program)
	float cpy[L::Q];
	switch (bc) {
	case BC_BOUNCE_BACK: // boundary.hpp:58-75 (full-way)
#pragma unroll
		for (int i = 0; i < L::Q; ++i) cpy[i] = f[i];
#pragma unroll
		for (int i = 0; i < L::Q; ++i) f[i] = cpy[L::opp(i)];
		break;
	case BC_MOVING_WALL: // examples/cavity_2d_gpu/cavity_2d_gpu.cpp:222-234
#pragma unroll
		for (int i = 0; i < L::Q; ++i) cpy[i] = f[i];
#pragma unroll
		for (int i = 0; i < L::Q; ++i) f[i] = A::add(cpy[L::opp(i)], __ldg(&op->lid[i]));
		break;
	case BC_EQUILIBRIUM: // boundary.hpp:147-160
#pragma unroll
		for (int i = 0; i < L::Q; ++i) f[i] = __ldg(&op->eq[i]);
		break;
	case BC_ANTI_BOUNCE_BACK: // boundary.hpp:119-132 (D2Q9 only)
		if constexpr (L::Q == 9) {
			float t;
			t = f[3]; f[3] = f[4]; f[4] = t;
			t = f[5]; f[5] = f[7]; f[7] = t;
			t = f[6]; f[6] = f[8]; f[8] = t;
		}
		break;
	case BC_ZOUHE_PRESSURE_X:
		if constexpr (L::Q == 9) zouhe_pressure_d2q9<EXACT>(f, __ldg(&op->east) != 0, __ldg(&op->rho));
		if constexpr (L::Q == 27) {
			if (__ldg(&op->east) != 0) zouhe_pressure_d3q27<EXACT, true>(f, __ldg(&op->rho));
			else zouhe_pressure_d3q27<EXACT, false>(f, __ldg(&op->rho));
		}
		break;
	case BC_ZOUHE_VELOCITY_X:
		if constexpr (L::Q == 9) {
			const float ux = __ldg(&op->use_profile) ? __ldg(p.profile + y) : __ldg(&op->u[0]);
			zouhe_velocity_d2q9<EXACT>(f, __ldg(&op->east) != 0, ux, __ldg(&op->u[1]));
		}
		break;
	default:
		break;
	}
	if (__ldg(&op->collide)) {
		if (COLL == COLL_BGK_GUO) {
			if (__ldg(&op->bgk_only)) {
				collide<L, COLL_BGK, EXACT>(f, p, por, Fc, rho, u);
				return true;
			}
			collide<L, COLL, EXACT>(f, p, por, Fc, rho, u);
			return !__ldg(&op->no_macros);
		}
		collide<L, COLL, EXACT>(f, p, por, Fc, rho, u);
		return true;
	}
	return false;
}

// ---------------------------------------------------------------------------
// The sweep kernel.

__device__ __forceinline__ float f4get(const float4 &v, int k) {
	return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

template <class L, int STORE, bool ODD, int COLL, bool EXACT>
__global__ void __launch_bounds__(256) sweep_kernel(const __grid_constant__ SweepParams p) {
	using S = Store<STORE>;
	constexpr int Q = L::Q;
	const int lane = threadIdx.x & 31;
	const int64_t gwarp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
	const int64_t row = gwarp / p.wpr;
	const int64_t nrows = static_cast<int64_t>(p.ny) * p.nz;
	if (row >= nrows) return; // warp-uniform: a warp never spans rows
	const int qd = static_cast<int>(gwarp % p.wpr) * 32 + lane;
	const bool active = qd < p.nq;
	const int x0 = qd * 4;
	const int y = static_cast<int>(row % p.ny);
	const int z = static_cast<int>(row / p.ny);
	const int nxp = p.nxp;
	const int64_t rbase = row * nxp; // first cell of this row
	const unsigned FULL = 0xffffffffu;

	float f[Q][4];

	// ---- gather the post-stream populations f_i of the 4 cells -------------
#pragma unroll
	for (int i = 0; i < Q; ++i) {
		const float s = p.wshift[i];
		if (!ODD) {
			float4 v = active ? S::ld4(p.f, i * p.plane + rbase + x0, s) : make_float4(0.f, 0.f, 0.f, 0.f);
			f[i][0] = v.x; f[i][1] = v.y; f[i][2] = v.z; f[i][3] = v.w;
		} else {
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int sy = y - cy, sz = z - cz;
			const bool row_in = (sy >= 0) && (sy < p.ny) && (sz >= 0) && (sz < p.nz);
			const int64_t sb = static_cast<int64_t>(L::opp(i)) * p.plane + (static_cast<int64_t>(sz) * p.ny + sy) * nxp;
			float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
			if (row_in && active) v = S::ld4(p.f, sb + x0, s);
			if (cx == 0) {
				f[i][0] = v.x; f[i][1] = v.y; f[i][2] = v.z; f[i][3] = v.w;
			} else if (cx > 0) { // source x - 1
				float prev = __shfl_up_sync(FULL, v.w, 1);
				if (lane == 0 || x0 == 0) {
					prev = 0.f;
					if (row_in && active) {
						if (x0 > 0) prev = S::ld1(p.f, sb + x0 - 1, s);
						else if (p.periodic) prev = S::ld1(p.f, sb + nxp - 1, s);
					}
				}
				f[i][0] = prev; f[i][1] = v.x; f[i][2] = v.y; f[i][3] = v.z;
			} else { // source x + 1
				float next = __shfl_down_sync(FULL, v.x, 1);
				if (lane == 31 || x0 + 4 >= nxp) {
					next = 0.f;
					if (row_in && active) {
						if (x0 + 4 < nxp) next = S::ld1(p.f, sb + x0 + 4, s);
						else if (p.periodic) next = S::ld1(p.f, sb, s);
					}
				}
				f[i][0] = v.y; f[i][1] = v.z; f[i][2] = v.w; f[i][3] = next;
			}
		}
	}

	// ---- boundary step + collision per cell ---------------------------------
	uchar4 fl = make_uchar4(0, 0, 0, 0);
	if (active) fl = *reinterpret_cast<const uchar4 *>(p.flags + rbase + x0);
	float4 porv = make_float4(1.f, 1.f, 1.f, 1.f);
	if ((COLL == COLL_PSM || COLL == COLL_PSM_GUO) && active)
		porv = *reinterpret_cast<const float4 *>(p.por + rbase + x0);
	float4 fcv[3] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
	if ((COLL == COLL_BGK_GUO || COLL == COLL_PSM_GUO) && active) {
#pragma unroll
		for (int k = 0; k < L::D; ++k) fcv[k] = *reinterpret_cast<const float4 *>(p.force + k * p.plane + rbase + x0);
	}
	const CellCtx ctx = cell_ctx(p);
	float4 rho4 = make_float4(0.f, 0.f, 0.f, 0.f);
	float4 u4[3] = {rho4, rho4, rho4};
	int collided = 0;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		const int flag = k == 0 ? fl.x : (k == 1 ? fl.y : (k == 2 ? fl.z : fl.w));
		float c[Q];
#pragma unroll
		for (int i = 0; i < Q; ++i) c[i] = f[i][k];
		float Fc[3] = {f4get(fcv[0], k), f4get(fcv[1], k), f4get(fcv[2], k)};
		float rho = 1.f, u[3] = {0.f, 0.f, 0.f};
		const bool col = cell_update<L, COLL, EXACT>(c, flag, y, ctx, f4get(porv, k), Fc, rho, u);
		collided |= (col ? 1 : 0) << k;
		if (k == 0) { rho4.x = rho; u4[0].x = u[0]; u4[1].x = u[1]; u4[2].x = u[2]; }
		if (k == 1) { rho4.y = rho; u4[0].y = u[0]; u4[1].y = u[1]; u4[2].y = u[2]; }
		if (k == 2) { rho4.z = rho; u4[0].z = u[0]; u4[1].z = u[1]; u4[2].z = u[2]; }
		if (k == 3) { rho4.w = rho; u4[0].w = u[0]; u4[1].w = u[1]; u4[2].w = u[2]; }
#pragma unroll
		for (int i = 0; i < Q; ++i) f[i][k] = c[i];
	}

	// ---- macros of collided cells (collision.hpp:83-89) ---------------------
	if (p.write_macros && active && collided) {
		if (collided == 0xF) {
			*reinterpret_cast<float4 *>(p.rho + rbase + x0) = rho4;
#pragma unroll
			for (int k = 0; k < L::D; ++k) *reinterpret_cast<float4 *>(p.u + k * p.plane + rbase + x0) = u4[k];
		} else {
#pragma unroll
			for (int k = 0; k < 4; ++k) {
				if (collided & (1 << k)) {
					p.rho[rbase + x0 + k] = f4get(rho4, k);
#pragma unroll
					for (int d = 0; d < L::D; ++d) p.u[d * p.plane + rbase + x0 + k] = f4get(u4[d], k);
				}
			}
		}
	}

	// ---- scatter the post-collision populations -----------------------------
#pragma unroll
	for (int i = 0; i < Q; ++i) {
		const float s = p.wshift[i];
		if (!ODD) {
			if (active)
				S::st4(p.f, static_cast<int64_t>(L::opp(i)) * p.plane + rbase + x0,
					   make_float4(f[i][0], f[i][1], f[i][2], f[i][3]), s);
		} else {
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int64_t pb = static_cast<int64_t>(i) * p.plane;
			// slots of this row whose source lies outside: the ghost ring's zero
			{
				const int sy = y - cy, sz = z - cz;
				const bool src_row_in = (sy >= 0) && (sy < p.ny) && (sz >= 0) && (sz < p.nz);
				if (!src_row_in) {
					if (active) S::st4(p.f, pb + rbase + x0, make_float4(0.f, 0.f, 0.f, 0.f), s);
				} else if (!p.periodic && active) {
					if (cx > 0 && x0 == 0) S::st1(p.f, pb + rbase, 0.f, s);
					if (cx < 0 && x0 + 4 == nxp) S::st1(p.f, pb + rbase + nxp - 1, 0.f, s);
				}
			}
			const int dy = y + cy, dz = z + cz;
			const bool row_in = (dy >= 0) && (dy < p.ny) && (dz >= 0) && (dz < p.nz);
			const int64_t db = pb + (static_cast<int64_t>(dz) * p.ny + dy) * nxp;
			if (cx == 0) {
				if (row_in && active) S::st4(p.f, db + x0, make_float4(f[i][0], f[i][1], f[i][2], f[i][3]), s);
			} else if (cx > 0) { // destination x + 1
				const float q = __shfl_up_sync(FULL, f[i][3], 1);
				if (row_in && active) {
					if (lane > 0) {
						S::st4(p.f, db + x0, make_float4(q, f[i][0], f[i][1], f[i][2]), s);
					} else { // element x0 belongs to the previous warp (or is a ghost slot zeroed above)
						S::st1(p.f, db + x0 + 1, f[i][0], s);
						S::st1(p.f, db + x0 + 2, f[i][1], s);
						S::st1(p.f, db + x0 + 3, f[i][2], s);
					}
					if (x0 + 4 < nxp) {
						if (lane == 31) S::st1(p.f, db + x0 + 4, f[i][3], s);
					} else if (p.periodic) {
						S::st1(p.f, db, f[i][3], s);
					}
				}
			} else { // destination x - 1
				const float r = __shfl_down_sync(FULL, f[i][0], 1);
				if (row_in && active) {
					if (lane < 31 && x0 + 4 < nxp) {
						S::st4(p.f, db + x0, make_float4(f[i][1], f[i][2], f[i][3], r), s);
					} else { // element x0+3 belongs to the next warp (or is a ghost slot zeroed above)
						S::st1(p.f, db + x0, f[i][1], s);
						S::st1(p.f, db + x0 + 1, f[i][2], s);
						S::st1(p.f, db + x0 + 2, f[i][3], s);
					}
					if (x0 > 0) {
						if (lane == 0) S::st1(p.f, db + x0 - 1, f[i][0], s);
					} else if (p.periodic) {
						S::st1(p.f, db + nxp - 1, f[i][0], s);
					}
				}
			}
		}
	}
}


// Two consecutive cells per thread (x0 = 2 * pair), 64-bit FP32 / 32-bit
// FP16S accesses: half the load/store instructions of the one-cell sweep and,
// in FP16S, one register per population pair in flight.  A warp covers 32
// pairs of one row; the x-shifted accesses of odd steps are realigned with
// one warp shuffle per direction, and only the lanes at a warp's or row's end
// touch the neighbouring pair with a scalar access (as sweep_kernel does
// with four cells).
template <class L, int STORE, bool ODD, int COLL, bool EXACT>
__global__ void __launch_bounds__(256) sweep2_kernel(const __grid_constant__ SweepParams p) {
	using S = Store<STORE>;
	constexpr int Q = L::Q;
	const int lane = threadIdx.x & 31;
	const int64_t gwarp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
	const int64_t row = gwarp / p.wpr2;
	const int64_t nrows = static_cast<int64_t>(p.ny) * p.nz;
	if (row >= nrows) return; // warp-uniform: a warp never spans rows
	const int nxp = p.nxp;
	const int pr = static_cast<int>(gwarp % p.wpr2) * 32 + lane;
	const bool active = 2 * pr < nxp;
	const int x0 = 2 * pr;
	const int y = static_cast<int>(row % p.ny);
	const int z = static_cast<int>(row / p.ny);
	const int64_t rbase = row * nxp; // first cell of this row
	const unsigned FULL = 0xffffffffu;

	float f[Q][2];

	// ---- gather the post-stream populations f_i of the 2 cells -------------
#pragma unroll
	for (int i = 0; i < Q; ++i) {
		const float s = p.wshift[i];
		if (!ODD) {
			const float2 v = active ? S::ld2(p.f, i * p.plane + rbase + x0, s) : make_float2(0.f, 0.f);
			f[i][0] = v.x;
			f[i][1] = v.y;
		} else {
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int sy = y - cy, sz = z - cz;
			const bool row_in = (sy >= 0) && (sy < p.ny) && (sz >= 0) && (sz < p.nz);
			const int64_t sb = static_cast<int64_t>(L::opp(i)) * p.plane + (static_cast<int64_t>(sz) * p.ny + sy) * nxp;
			float2 v = make_float2(0.f, 0.f);
			if (row_in && active) v = S::ld2(p.f, sb + x0, s);
			if (cx == 0) {
				f[i][0] = v.x;
				f[i][1] = v.y;
			} else if (cx > 0) { // source x - 1
				float prev = __shfl_up_sync(FULL, v.y, 1);
				if (lane == 0 || x0 == 0) {
					prev = 0.f;
					if (row_in && active) {
						if (x0 > 0) prev = S::ld1(p.f, sb + x0 - 1, s);
						else if (p.periodic) prev = S::ld1(p.f, sb + nxp - 1, s);
					}
				}
				f[i][0] = prev;
				f[i][1] = v.x;
			} else { // source x + 1
				float next = __shfl_down_sync(FULL, v.x, 1);
				if (lane == 31 || x0 + 2 >= nxp) {
					next = 0.f;
					if (row_in && active) {
						if (x0 + 2 < nxp) next = S::ld1(p.f, sb + x0 + 2, s);
						else if (p.periodic) next = S::ld1(p.f, sb, s);
					}
				}
				f[i][0] = v.y;
				f[i][1] = next;
			}
		}
	}

	// ---- boundary step + collision per cell ---------------------------------
	uchar2 fl = make_uchar2(0, 0);
	if (active) fl = *reinterpret_cast<const uchar2 *>(p.flags + rbase + x0);
	float2 porv = make_float2(1.f, 1.f);
	if ((COLL == COLL_PSM || COLL == COLL_PSM_GUO || COLL == COLL_HLBM) && active)
		porv = *reinterpret_cast<const float2 *>(p.por + rbase + x0);
	float2 fcv[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
	if ((COLL == COLL_BGK_GUO || COLL == COLL_PSM_GUO) && active) {
#pragma unroll
		for (int k = 0; k < L::D; ++k) fcv[k] = *reinterpret_cast<const float2 *>(p.force + k * p.plane + rbase + x0);
	}
	if (COLL == COLL_HLBM && active) {
		fcv[0] = *reinterpret_cast<const float2 *>(p.hN + rbase + x0);
		fcv[1] = *reinterpret_cast<const float2 *>(p.hN + p.plane + rbase + x0);
		fcv[2] = *reinterpret_cast<const float2 *>(p.hD + rbase + x0);
	}
	const CellCtx ctx = cell_ctx(p);
	float2 rho2 = make_float2(0.f, 0.f);
	float2 u2[3] = {rho2, rho2, rho2};
	int collided = 0;
#pragma unroll
	for (int k = 0; k < 2; ++k) {
		const int flag = k == 0 ? fl.x : fl.y;
		float c[Q];
#pragma unroll
		for (int i = 0; i < Q; ++i) c[i] = f[i][k];
		float Fc[3] = {k ? fcv[0].y : fcv[0].x, k ? fcv[1].y : fcv[1].x, k ? fcv[2].y : fcv[2].x};
		float rho = 1.f, u[3] = {0.f, 0.f, 0.f};
		const bool col = cell_update<L, COLL, EXACT>(c, flag, y, ctx, k ? porv.y : porv.x, Fc, rho, u);
		collided |= (col ? 1 : 0) << k;
		if (k == 0) { rho2.x = rho; u2[0].x = u[0]; u2[1].x = u[1]; u2[2].x = u[2]; }
		else { rho2.y = rho; u2[0].y = u[0]; u2[1].y = u[1]; u2[2].y = u[2]; }
#pragma unroll
		for (int i = 0; i < Q; ++i) f[i][k] = c[i];
	}

	// ---- macros of collided cells (collision.hpp:83-89) ---------------------
	if (p.write_macros && active && collided) {
		if (collided == 3) {
			*reinterpret_cast<float2 *>(p.rho + rbase + x0) = rho2;
#pragma unroll
			for (int k = 0; k < L::D; ++k) *reinterpret_cast<float2 *>(p.u + k * p.plane + rbase + x0) = u2[k];
		} else {
			const int k = collided == 1 ? 0 : 1;
			p.rho[rbase + x0 + k] = k ? rho2.y : rho2.x;
#pragma unroll
			for (int d = 0; d < L::D; ++d) p.u[d * p.plane + rbase + x0 + k] = k ? u2[d].y : u2[d].x;
		}
	}

	// ---- scatter the post-collision populations -----------------------------
#pragma unroll
	for (int i = 0; i < Q; ++i) {
		const float s = p.wshift[i];
		if (!ODD) {
			if (active) S::st2(p.f, static_cast<int64_t>(L::opp(i)) * p.plane + rbase + x0, make_float2(f[i][0], f[i][1]), s);
		} else {
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int64_t pb = static_cast<int64_t>(i) * p.plane;
			// slots of this row whose source lies outside: the ghost ring's zero
			{
				const int sy = y - cy, sz = z - cz;
				const bool src_row_in = (sy >= 0) && (sy < p.ny) && (sz >= 0) && (sz < p.nz);
				if (!src_row_in) {
					if (active) S::st2(p.f, pb + rbase + x0, make_float2(0.f, 0.f), s);
				} else if (!p.periodic && active) {
					if (cx > 0 && x0 == 0) S::st1(p.f, pb + rbase, 0.f, s);
					if (cx < 0 && x0 + 2 == nxp) S::st1(p.f, pb + rbase + nxp - 1, 0.f, s);
				}
			}
			const int dy = y + cy, dz = z + cz;
			const bool row_in = (dy >= 0) && (dy < p.ny) && (dz >= 0) && (dz < p.nz);
			const int64_t db = pb + (static_cast<int64_t>(dz) * p.ny + dy) * nxp;
			if (cx == 0) {
				if (row_in && active) S::st2(p.f, db + x0, make_float2(f[i][0], f[i][1]), s);
			} else if (cx > 0) { // destination x + 1
				const float q = __shfl_up_sync(FULL, f[i][1], 1);
				if (row_in && active) {
					if (lane > 0) S::st2(p.f, db + x0, make_float2(q, f[i][0]), s);
					else S::st1(p.f, db + x0 + 1, f[i][0], s); // element x0: previous warp, or the ghost slot
					if (x0 + 2 < nxp) {
						if (lane == 31) S::st1(p.f, db + x0 + 2, f[i][1], s);
					} else if (p.periodic) {
						S::st1(p.f, db, f[i][1], s);
					}
				}
			} else { // destination x - 1
				const float r = __shfl_down_sync(FULL, f[i][0], 1);
				if (row_in && active) {
					if (lane < 31 && x0 + 2 < nxp) S::st2(p.f, db + x0, make_float2(f[i][1], r), s);
					else S::st1(p.f, db + x0, f[i][1], s); // element x0 + 1: next warp, or the ghost slot
					if (x0 > 0) {
						if (lane == 0) S::st1(p.f, db + x0 - 1, f[i][0], s);
					} else if (p.periodic) {
						S::st1(p.f, db + nxp - 1, f[i][0], s);
					}
				}
			}
		}
	}
}


// Two consecutive cells per thread in FP16S storage, the pair held as raw
// halves: one 32-bit register per population (cell x0 in the low half, x0 + 1
// in the high half) from the load to the store, so each 32-bit access moves
// two cells' populations and the pair costs what one cell of sweep1_kernel
// costs in registers.  The two cells are collided one after the other (the
// loop over them is not unrolled): one cell's FP32 populations are live at a
// time.  A warp covers 32 pairs of one row (nxp is even in FP16S storage);
// x-shifted odd-step accesses are realigned with one warp shuffle per
// direction, and the lanes at a warp's or row's end touch the neighbouring
// pair with a 16-bit access.  Per cell the arithmetic is that of
// sweep1_kernel: f_i = half(A) + w_i on load (0 for the ghost ring),
// A = half_rn(f_i - w_i) on store.
template <class L, bool ODD, int COLL, bool EXACT>
__global__ void __launch_bounds__(256, 4) sweep2h_kernel(const __grid_constant__ SweepParams p) {
	constexpr int Q = L::Q;
	static_assert(Q <= 32, "one zero bit per population");
	const int lane = threadIdx.x & 31;
	const int64_t gwarp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
	const int64_t row = gwarp / p.wpr2;
	const int64_t nrows = static_cast<int64_t>(p.ny) * p.nz;
	if (row >= nrows) return; // warp-uniform: a warp never spans rows
	const int nxp = p.nxp;
	const int x0 = 2 * (static_cast<int>(gwarp % p.wpr2) * 32 + lane);
	const bool active = x0 < nxp; // nxp even: x0 + 1 < nxp too
	const int y = static_cast<int>(row % p.ny);
	const int z = static_cast<int>(row / p.ny);
	const int64_t rbase = row * nxp;
	const int64_t oy = nxp, oz = static_cast<int64_t>(nxp) * p.ny;
	const unsigned FULL = 0xffffffffu;
	unsigned short *const A = static_cast<unsigned short *>(p.f);
	auto ld2h = [&](int64_t idx) { return __ldcs(reinterpret_cast<const unsigned *>(A + idx)); };
	auto st2h = [&](int64_t idx, unsigned v) { __stcs(reinterpret_cast<unsigned *>(A + idx), v); };
	auto ld1h = [&](int64_t idx) { return static_cast<unsigned>(__ldcs(A + idx)); };
	auto st1h = [&](int64_t idx, unsigned v) { __stcs(A + idx, static_cast<unsigned short>(v)); };

	uint32_t h[Q];
	uint32_t zero0 = 0u, zero1 = 0u; // bit i: f_i of cell x0 / x0 + 1 is the ghost ring's zero

	// ---- gather the post-stream populations of the pair ---------------------
#pragma unroll
	for (int i = 0; i < Q; ++i) {
		if (!ODD) {
			h[i] = active ? ld2h(static_cast<int64_t>(i) * p.plane + rbase + x0) : 0u;
		} else {
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int sy = y - cy, sz = z - cz;
			const bool row_in = (sy >= 0) && (sy < p.ny) && (sz >= 0) && (sz < p.nz);
			const int64_t sb = static_cast<int64_t>(L::opp(i)) * p.plane + rbase - cy * oy - cz * oz;
			const unsigned w = (row_in && active) ? ld2h(sb + x0) : 0u;
			if (!row_in) {
				zero0 |= 1u << i;
				zero1 |= 1u << i;
			}
			if (cx == 0) {
				h[i] = w;
			} else if (cx > 0) { // sources x0 - 1, x0
				unsigned lo = __shfl_up_sync(FULL, w, 1) >> 16;
				if (lane == 0 || x0 == 0) {
					lo = 0u;
					if (row_in && active) {
						if (x0 > 0) lo = ld1h(sb + x0 - 1);
						else if (p.periodic) lo = ld1h(sb + nxp - 1);
						else zero0 |= 1u << i;
					}
				}
				h[i] = lo | (w << 16);
			} else { // sources x0 + 1, x0 + 2
				unsigned hi = __shfl_down_sync(FULL, w, 1) & 0xffffu;
				if (lane == 31 || x0 + 2 >= nxp) {
					hi = 0u;
					if (row_in && active) {
						if (x0 + 2 < nxp) hi = ld1h(sb + x0 + 2);
						else if (p.periodic) hi = ld1h(sb);
						else zero1 |= 1u << i;
					}
				}
				h[i] = (w >> 16) | (hi << 16);
			}
		}
	}

	// ---- boundary step + collision, one cell after the other ----------------
	uchar2 fl = make_uchar2(0, 0);
	if (active) fl = *reinterpret_cast<const uchar2 *>(p.flags + rbase + x0);
	float2 porv = make_float2(1.f, 1.f);
	if ((COLL == COLL_PSM || COLL == COLL_PSM_GUO || COLL == COLL_HLBM) && active)
		porv = *reinterpret_cast<const float2 *>(p.por + rbase + x0);
	float2 fcv[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
	if ((COLL == COLL_BGK_GUO || COLL == COLL_PSM_GUO) && active) {
#pragma unroll
		for (int k = 0; k < L::D; ++k) fcv[k] = *reinterpret_cast<const float2 *>(p.force + k * p.plane + rbase + x0);
	}
	if (COLL == COLL_HLBM && active) {
		fcv[0] = *reinterpret_cast<const float2 *>(p.hN + rbase + x0);
		fcv[1] = *reinterpret_cast<const float2 *>(p.hN + p.plane + rbase + x0);
		fcv[2] = *reinterpret_cast<const float2 *>(p.hD + rbase + x0);
	}
	const CellCtx ctx = cell_ctx(p);
#pragma unroll 1
	for (int k = 0; k < 2; ++k) {
		const int sh = 16 * k;
		const uint32_t zm = k ? zero1 : zero0;
		float c[Q];
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			const float v = __half2float(__ushort_as_half(static_cast<unsigned short>(h[i] >> sh)));
			c[i] = ((zm >> i) & 1u) ? 0.f : v + p.wshift[i];
		}
		const float Fc[3] = {k ? fcv[0].y : fcv[0].x, k ? fcv[1].y : fcv[1].x, k ? fcv[2].y : fcv[2].x};
		float rho = 1.f, u[3] = {0.f, 0.f, 0.f};
		const bool col = cell_update<L, COLL, EXACT>(c, k ? fl.y : fl.x, y, ctx, k ? porv.y : porv.x, Fc, rho, u);
		if (p.write_macros && col && active) {
			p.rho[rbase + x0 + k] = rho;
#pragma unroll
			for (int d = 0; d < L::D; ++d) p.u[d * p.plane + rbase + x0 + k] = u[d];
		}
		const uint32_t keep = k ? 0x0000ffffu : 0xffff0000u;
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			const uint32_t b = __half_as_ushort(__float2half_rn(c[i] - p.wshift[i]));
			h[i] = (h[i] & keep) | (b << sh);
		}
	}

	// ---- scatter the post-collision populations -----------------------------
#pragma unroll
	for (int i = 0; i < Q; ++i) {
		if (!ODD) {
			if (active) st2h(static_cast<int64_t>(L::opp(i)) * p.plane + rbase + x0, h[i]);
		} else {
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int64_t pb = static_cast<int64_t>(i) * p.plane;
			// slots of this row whose source lies outside: the ghost ring's zero
			{
				const uint32_t zh = __half_as_ushort(__float2half_rn(0.f - p.wshift[i]));
				const int sy = y - cy, sz = z - cz;
				const bool src_row_in = (sy >= 0) && (sy < p.ny) && (sz >= 0) && (sz < p.nz);
				if (!src_row_in) {
					if (active) st2h(pb + rbase + x0, zh | (zh << 16));
				} else if (!p.periodic && active) {
					if (cx > 0 && x0 == 0) st1h(pb + rbase, zh);
					if (cx < 0 && x0 + 2 == nxp) st1h(pb + rbase + nxp - 1, zh);
				}
			}
			const int dy = y + cy, dz = z + cz;
			const bool row_in = (dy >= 0) && (dy < p.ny) && (dz >= 0) && (dz < p.nz);
			const int64_t db = pb + rbase + cy * oy + cz * oz;
			if (cx == 0) {
				if (row_in && active) st2h(db + x0, h[i]);
			} else if (cx > 0) { // destinations x0 + 1, x0 + 2
				const unsigned q = __shfl_up_sync(FULL, h[i], 1);
				if (row_in && active) {
					if (lane > 0) st2h(db + x0, (q >> 16) | (h[i] << 16));
					else st1h(db + x0 + 1, h[i] & 0xffffu); // element x0: previous warp, or the ghost slot
					if (x0 + 2 < nxp) {
						if (lane == 31) st1h(db + x0 + 2, h[i] >> 16);
					} else if (p.periodic) {
						st1h(db, h[i] >> 16);
					}
				}
			} else { // destinations x0 - 1, x0
				const unsigned r = __shfl_down_sync(FULL, h[i], 1);
				if (row_in && active) {
					if (lane < 31 && x0 + 2 < nxp) st2h(db + x0, (h[i] >> 16) | (r << 16));
					else st1h(db + x0, h[i] >> 16); // element x0 + 1: next warp, or the ghost slot
					if (x0 > 0) {
						if (lane == 0) st1h(db + x0 - 1, h[i] & 0xffffu);
					} else if (p.periodic) {
						st1h(db + nxp - 1, h[i] & 0xffffu);
					}
				}
			}
		}
	}
}

// One cell per thread.  Same physics and the same AA addressing as
// sweep_kernel, with 32-bit accesses: the x-shifted loads/stores of odd steps
// are plain unit offsets, coalesced across the warp, and the register budget
// (~70) leaves room for four times as many resident warps.
// Grid: (ceil(nxp / blockDim.x), ny, nz) -- a block never leaves its row, so
// "the row and its y/z neighbours exist" is uniform over the block and
// interior rows take a path with no per-direction bounds arithmetic: each
// neighbour is the cell index plus a row offset, and only the first and last
// cell of a row carry an x predicate.
// At most 64 registers (four 256-thread blocks per SM): the sweep waits on
// global-load latency, and 32 resident warps per SM keep more loads in
// flight than 24 at 80 registers (measured +3 % FP32, +6 % FP16S at 256^3;
// the few spilled words stay in L1).
// HW: the lattice has half-way walls (p.hw_mask set); a separate
// instantiation, so that the stores' redirection costs the common case
// nothing.
template <class L, int STORE, bool ODD, int COLL, bool EXACT, bool HW = false>
__global__ void __launch_bounds__(256, 4) sweep1_kernel(const __grid_constant__ SweepParams p) {
	using S = Store<STORE>;
	constexpr int Q = L::Q;
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	if (x >= p.nxp) return;
	const int y = blockIdx.y, z = blockIdx.z;
	const int nxp = p.nxp;
	const int64_t cell = (static_cast<int64_t>(z) * p.ny + y) * nxp + x;
	const int64_t oy = nxp, oz = static_cast<int64_t>(nxp) * p.ny;
	// the lanes still running (a row's last warp may be partial); the fast
	// paths below are chosen per warp, so that no warp runs two variants
	const unsigned lanes = __activemask();
	// neighbour x offsets (periodic rows wrap; nxp == nx then)
	const bool has_xm = x > 0, has_xp = x + 1 < nxp;
	const bool x_inner = __all_sync(lanes, has_xm && has_xp); // no lane at the row's ends
	const int xm = has_xm ? -1 : nxp - 1;     // offset of x - 1
	const int xp = has_xp ? 1 : -(nxp - 1);   // offset of x + 1
	const bool ok_xm = has_xm || p.periodic;  // x - 1 exists
	const bool ok_xp = has_xp || p.periodic;  // x + 1 exists
	const bool row_interior = y > 0 && y + 1 < p.ny && (L::D == 2 || (z > 0 && z + 1 < p.nz));
	// 32-bit offsets from this cell's slot in plane 0 (when they fit): one
	// 32-bit multiply-add per population instead of 64-bit index arithmetic
	using ST = typename S::T;
	ST *const fc = static_cast<ST *>(p.f) + cell;
	const int pl32 = (int)p.plane, oy32 = nxp, oz32 = nxp * p.ny;
	// L2 prefetch of the rows the block p.pf_ahead places later in launch
	// order will read (its x range in every direction plane; in odd steps its
	// neighbours' rows are prefetched by their own predecessors): requests in
	// flight that hold no registers, one 128-byte line per thread.
	if (p.pf_ahead > 0) {
		const unsigned gx = gridDim.x;
		const int64_t nblk = (int64_t)gx * gridDim.y * gridDim.z;
		const int64_t b = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gx + blockIdx.x + p.pf_ahead;
		if (b < nblk) {
			const int x0 = (int)(b % gx) * (int)blockDim.x;
			const int64_t row = b / gx;
			const int n = min((int)blockDim.x, nxp - x0);
			constexpr int per = 128 / (int)sizeof(ST); // cells per line
			const int lines = (n + per - 1) / per;
			const int t = threadIdx.x;
			if (t < Q * lines) {
				const int i = t / lines, l = t - i * lines;
				const ST *a = static_cast<const ST *>(p.f) + i * p.plane + row * nxp + x0 + l * per;
				asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
			}
		}
	}

	float f[Q];
	if (!ODD && p.idx32) {
#pragma unroll
		for (int i = 0; i < Q; ++i) f[i] = S::ld1(fc, i * pl32, p.wshift[i]);
	} else if (!ODD) {
#pragma unroll
		for (int i = 0; i < Q; ++i) f[i] = S::ld1(p.f, i * p.plane + cell, p.wshift[i]);
	} else if (row_interior && p.idx32 && x_inner) {
		// every neighbour exists: unit x offsets, no predicates
#pragma unroll
		for (int i = 0; i < Q; ++i)
			f[i] = S::ld1(fc, L::opp(i) * pl32 - L::cx(i) - L::cy(i) * oy32 - L::cz(i) * oz32, p.wshift[i]);
	} else if (row_interior && p.idx32) {
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int off = L::opp(i) * pl32 + (cx > 0 ? xm : (cx < 0 ? xp : 0)) - cy * oy32 - cz * oz32;
			const bool ok = cx > 0 ? ok_xm : (cx < 0 ? ok_xp : true);
			f[i] = ok ? S::ld1(fc, off, p.wshift[i]) : 0.f;
		}
	} else if (row_interior) {
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			// f_i(x) = A[opp i][x - c_i]
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int64_t off = (cx > 0 ? xm : (cx < 0 ? xp : 0)) - cy * oy - cz * oz;
			const bool ok = cx > 0 ? ok_xm : (cx < 0 ? ok_xp : true);
			f[i] = ok ? S::ld1(p.f, static_cast<int64_t>(L::opp(i)) * p.plane + cell + off, p.wshift[i]) : 0.f;
		}
	} else {
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			int sx = x - L::cx(i);
			const int sy = y - L::cy(i), sz = z - L::cz(i);
			if (p.periodic) sx = sx < 0 ? sx + nxp : (sx >= nxp ? sx - nxp : sx);
			const bool in = sx >= 0 && sx < nxp && sy >= 0 && sy < p.ny && sz >= 0 && sz < p.nz;
			f[i] = in ? S::ld1(p.f, static_cast<int64_t>(L::opp(i)) * p.plane +
										(static_cast<int64_t>(sz) * p.ny + sy) * nxp + sx, p.wshift[i])
					  : 0.f;
		}
	}
	const int flag = p.flags[cell];
	const float por = (COLL == COLL_PSM || COLL == COLL_PSM_GUO || COLL == COLL_HLBM) ? p.por[cell] : 1.f;
	float Fc[3] = {0.f, 0.f, 0.f};
	if (COLL == COLL_BGK_GUO || COLL == COLL_PSM_GUO) {
#pragma unroll
		for (int k = 0; k < L::D; ++k) Fc[k] = p.force[k * p.plane + cell];
	}
	if (COLL == COLL_HLBM) {
		Fc[0] = p.hN[cell];
		Fc[1] = p.hN[p.plane + cell];
		Fc[2] = p.hD[cell];
	}
	float rho = 1.f, u[3] = {0.f, 0.f, 0.f};
	bool col;
	if (__all_sync(lanes, flag < MAX_FLAGS && ((p.plain >> flag) & 1u))) { // no boundary step: straight to the collision
		collide<L, COLL, EXACT>(f, cell_ctx(p), por, Fc, rho, u);
		col = true;
	} else {
		col = cell_update<L, COLL, EXACT>(f, flag, y, cell_ctx(p), por, Fc, rho, u);
	}
	if (p.write_macros && col) {
		p.rho[cell] = rho;
#pragma unroll
		for (int k = 0; k < L::D; ++k) p.u[k * p.plane + cell] = u[k];
	}
	if (HW) {
		// half-way bounce-back: a wall cell writes nothing; a population sent
		// towards a wall goes to the slot this cell reads f_opp(i) from next
		// step (even: A[i][x + c_i], which the odd step reads as
		// A[opp(opp i)][x - c_opp i]; odd: A[opp i][x], read by the even step)
		if (flag > 0 && flag < MAX_FLAGS && __ldg(&p.ops[flag].bc) == BC_HALFWAY_WALL) return;
		const uint32_t hw = p.hw_mask[cell];
		if (hw) {
#pragma unroll
			for (int i = 0; i < Q; ++i) {
				const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
				const int64_t pb = static_cast<int64_t>(i) * p.plane;
				const int64_t po = static_cast<int64_t>(L::opp(i)) * p.plane;
				int dx = x + cx;
				if (p.periodic) dx = dx < 0 ? dx + nxp : (dx >= nxp ? dx - nxp : dx);
				const int dy = y + cy, dz = z + cz;
				const int64_t dcell = (static_cast<int64_t>(dz) * p.ny + dy) * nxp + dx;
				const bool wall = (hw >> i) & 1u;
				if (!ODD) {
					S::st1(p.f, wall ? pb + dcell : po + cell, f[i], p.wshift[i]);
				} else {
					int sx = x - cx;
					const int sy = y - cy, sz = z - cz;
					if (p.periodic) sx = sx < 0 ? sx + nxp : (sx >= nxp ? sx - nxp : sx);
					if (sx < 0 || sx >= nxp || sy < 0 || sy >= p.ny || sz < 0 || sz >= p.nz)
						S::st1(p.f, pb + cell, 0.f, p.wshift[i]); // ghost ring's zero
					if (wall) S::st1(p.f, po + cell, f[i], p.wshift[i]);
					else if (dx >= 0 && dx < nxp && dy >= 0 && dy < p.ny && dz >= 0 && dz < p.nz)
						S::st1(p.f, pb + dcell, f[i], p.wshift[i]);
				}
			}
			return;
		}
	}
	if (!ODD) {
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			if (p.idx32) S::st1(fc, L::opp(i) * pl32, f[i], p.wshift[i]);
			else S::st1(p.f, static_cast<int64_t>(L::opp(i)) * p.plane + cell, f[i], p.wshift[i]);
		}
	} else if (row_interior && p.idx32 && x_inner) {
		// every destination exists and no source lies outside: no predicates
#pragma unroll
		for (int i = 0; i < Q; ++i)
			S::st1(fc, i * pl32 + L::cx(i) + L::cy(i) * oy32 + L::cz(i) * oz32, f[i], p.wshift[i]);
	} else if (row_interior && p.idx32) {
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int pb = i * pl32;
			if (cx > 0 && !ok_xm) S::st1(fc, pb, 0.f, p.wshift[i]);
			if (cx < 0 && !ok_xp) S::st1(fc, pb, 0.f, p.wshift[i]);
			const int off = (cx > 0 ? xp : (cx < 0 ? xm : 0)) + cy * oy32 + cz * oz32;
			const bool ok = cx > 0 ? ok_xp : (cx < 0 ? ok_xm : true);
			if (ok) S::st1(fc, pb + off, f[i], p.wshift[i]);
		}
	} else if (row_interior) {
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			// f*_i(x) -> A[i][x + c_i]; the slot A[i][x] whose source x - c_i
			// lies outside gets the ghost ring's zero
			const int cx = L::cx(i), cy = L::cy(i), cz = L::cz(i);
			const int64_t pb = static_cast<int64_t>(i) * p.plane + cell;
			if (cx > 0 && !ok_xm) S::st1(p.f, pb, 0.f, p.wshift[i]);
			if (cx < 0 && !ok_xp) S::st1(p.f, pb, 0.f, p.wshift[i]);
			const int64_t off = (cx > 0 ? xp : (cx < 0 ? xm : 0)) + cy * oy + cz * oz;
			const bool ok = cx > 0 ? ok_xp : (cx < 0 ? ok_xm : true);
			if (ok) S::st1(p.f, pb + off, f[i], p.wshift[i]);
		}
	} else {
#pragma unroll
		for (int i = 0; i < Q; ++i) {
			const int64_t pb = static_cast<int64_t>(i) * p.plane;
			{
				const int sx = x - L::cx(i), sy = y - L::cy(i), sz = z - L::cz(i);
				const bool out_x = !p.periodic && (sx < 0 || sx >= nxp);
				if (out_x || sy < 0 || sy >= p.ny || sz < 0 || sz >= p.nz) S::st1(p.f, pb + cell, 0.f, p.wshift[i]);
			}
			int dx = x + L::cx(i);
			const int dy = y + L::cy(i), dz = z + L::cz(i);
			if (p.periodic) dx = dx < 0 ? dx + nxp : (dx >= nxp ? dx - nxp : dx);
			if (dx >= 0 && dx < nxp && dy >= 0 && dy < p.ny && dz >= 0 && dz < p.nz)
				S::st1(p.f, pb + (static_cast<int64_t>(dz) * p.ny + dy) * nxp + dx, f[i], p.wshift[i]);
		}
	}
}

} // namespace gb
} // namespace kel
