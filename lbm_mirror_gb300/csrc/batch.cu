// Many independent D2Q9 channels of uneven size in one launch (C ABI
// kel_batch_*).
//
// The reference runs one compile-time-sized Chunk per process
// (modules/core/c++/chunk.hpp:25-39; SuperChunk "Not needed for now"), so a
// parameter sweep over many channels is many separate runs.  Here all channels
// share one allocation:
//   - populations: 9 planes over the packed cells of every channel; channel c
//     owns [off_c, off_c + nxp_c * ny_c), padded up to whole tiles;
//   - one tile (= one thread block, `tile` cells, one cell per thread) never
//     spans two channels: a launched block reads its (tile, channel) pair
//     from the launch list;
//   - per-channel relaxation rate and parabolic inlet profile come from the
//     channel table; the flag -> operation table is shared.
// Steps run as a captured CUDA graph of `check_every` sweeps followed by the
// FP64 convergence residual per channel; converged channels drop out (their
// blocks return at once) and the graph is replayed until none is left.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "lattice_internal.cuh"

using namespace kel::gb;

namespace {

struct ChannelRec {
	int64_t off;     // first packed cell
	int nx, nxp, ny; // extents (nxp = nx padded to 4)
	int first_block; // first tile
	int nblocks;     // tiles
	int prof_off;    // offset into the packed inlet profiles
	float omega;     // 1 / tau in float
	float guo_scale; // 1 - omega / 2
};

// What one launched block of the sweep needs, in one 32-byte record read at
// the block's start (the block's tile and its channel's extents, relaxation
// rate and inlet profile), so that its population loads follow a single
// load instead of a chain (launch list -> channel record).  `live` drops to
// 0 when the channel converges (k_batch_residual_final).
struct __align__(16) TileRec {
	int64_t cell0; // packed index of the tile's first cell
	int l0;        // index of that cell within its channel
	int nxp, ny;   // channel extents
	float omega;   // channel relaxation rate
	int prof_off;  // channel inlet profile offset
	int live;      // channel still running
};

struct BatchParams {
	TileRec *trec;   // per launched block
	int *lfirst;     // per channel: index of its first tile in the launch list (-1: not launched)
	float *f;
	int64_t plane;
	const uint8_t *flags;
	float *rho, *u, *u_prev;
	const OpEntry *ops;
	const float *profiles;
	const ChannelRec *ch;
	const int *block_ch;
	const int2 *blist; // launched block -> (tile, channel): all tiles, or those of active channels
	int *active;
	double2 *partial; // per-tile residual partial sums (scratch)
	int tile;
	int write_macros;
	int shifted; // populations hold g = f - w_i (MODE_SHIFTED)
	int idx32;   // 9 * plane < 2^31: population offsets from a cell fit 32-bit arithmetic
	int pf_ahead; // launched blocks ahead whose tiles a block prefetches into L2 (0: none)
};

// Arithmetic of a batch: the library's two (fast, reference rounding) on
// populations f, or SHIFTED on g = f - w_i (FP32 storage of the deviation
// from rest, "DDF shifting").  The rest populations (w_0 = 4/9 ...) dominate
// the rounding error of f in FP32; g is of the order of the flow's own
// deviation, so its rounding noise, which sets the floor of the relative
// velocity change a run can reach, is one to two orders of magnitude lower.
enum { MODE_FAST = 0, MODE_EXACT = 1, MODE_SHIFTED = 2 };

// One D2Q9 cell in shifted form: the same operations as cell_update for the
// boundaries a batch accepts, written on g.  Bounce-back and anti-bounce-back
// permute directions of equal weight, so they act on g unchanged; Zou-He
// keeps its linear updates (pairs of equal weight cancel) with the closure
// sums taken on g (the weights of the summed populations add up to 1); BGK
// relaxes g towards g_eq = w (rho - 1) + w rho (3 c.u + 4.5 (c.u)^2 - 1.5 u^2).
__device__ __forceinline__ bool cell_update_shifted(float (&g)[9], int flag, int y, const CellCtx &p, float &rho,
													float (&u)[3]) {
	using L = D2Q9;
	if (flag == 0) {
#pragma unroll
		for (int i = 0; i < 9; ++i) g[i] = 0.f;
		return false;
	}
	if (flag >= MAX_FLAGS) return false;
	const OpEntry *op = p.ops + flag;
	const int bc = __ldg(&op->bc);
	const float c23 = (float)(2.0 / 3.0), c16 = (float)(1.0 / 6.0);
	float t;
	switch (bc) {
	case BC_BOUNCE_BACK: {
		float cpy[9];
#pragma unroll
		for (int i = 0; i < 9; ++i) cpy[i] = g[i];
#pragma unroll
		for (int i = 0; i < 9; ++i) g[i] = cpy[L::opp(i)];
		break;
	}
	case BC_ANTI_BOUNCE_BACK:
		t = g[3]; g[3] = g[4]; g[4] = t;
		t = g[5]; g[5] = g[7]; g[7] = t;
		t = g[6]; g[6] = g[8]; g[8] = t;
		break;
	case BC_ZOUHE_PRESSURE_X: {
		const bool east = __ldg(&op->east) != 0;
		const float drs = __ldg(&op->rho) - 1.0f;
		if (east) {
			const float Sg = (g[0] + g[3] + g[4]) + 2.f * (g[1] + g[5] + g[7]);
			const float r = drs - Sg;
			g[2] = g[1] + c23 * r;
			g[6] = g[5] + c16 * r + 0.5f * (g[3] - g[4]);
			g[8] = g[7] + c16 * r + 0.5f * (g[4] - g[3]);
		} else {
			const float Sg = (g[0] + g[3] + g[4]) + 2.f * (g[2] + g[6] + g[8]);
			const float r = Sg - drs;
			g[1] = g[2] - c23 * r;
			g[5] = g[6] - c16 * r + 0.5f * (g[4] - g[3]);
			g[7] = g[8] - c16 * r + 0.5f * (g[3] - g[4]);
		}
		break;
	}
	case BC_ZOUHE_VELOCITY_X: {
		const bool east = __ldg(&op->east) != 0;
		const float ux = __ldg(&op->use_profile) ? __ldg(p.profile + y) : __ldg(&op->u[0]);
		const float uy = __ldg(&op->u[1]);
		const float dg = east ? (g[1] + g[5] + g[7]) : (g[2] + g[6] + g[8]);
		// rho = (f0 + f4 + f3 + 2 ds) / (u_x + 1) as the library's Zou-He inlet
		const float r0 = (1.0f + ((g[0] + g[4] + g[3]) + 2.f * dg)) / (ux + 1.0f);
		const float rux = c16 * r0 * ux, ruy = r0 * uy;
		if (east) {
			g[2] = g[1] + c23 * r0 * ux;
			g[6] = g[5] + rux + 0.5f * (g[3] - g[4] + ruy);
			g[8] = g[7] + rux + 0.5f * (g[4] - g[3] + ruy);
		} else {
			g[1] = g[2] + c23 * r0 * ux;
			g[5] = g[6] + rux + 0.5f * (g[4] - g[3] + ruy);
			g[7] = g[8] + rux + 0.5f * (g[3] - g[4] + ruy);
		}
		break;
	}
	default:
		break;
	}
	if (!__ldg(&op->collide)) return false;
	// moments on g: rho - 1 = sum g, rho u = sum c g
	float drho = 0.f, jx = 0.f, jy = 0.f;
#pragma unroll
	for (int i = 0; i < 9; ++i) {
		drho += g[i];
		if (L::cx(i) > 0) jx += g[i];
		if (L::cx(i) < 0) jx -= g[i];
		if (L::cy(i) > 0) jy += g[i];
		if (L::cy(i) < 0) jy -= g[i];
	}
	rho = 1.0f + drho;
	const float ir = 1.0f / rho;
	u[0] = jx * ir;
	u[1] = jy * ir;
	u[2] = 0.f;
	const float h = 1.5f * (u[0] * u[0] + u[1] * u[1]);
#pragma unroll
	for (int i = 0; i < 9; ++i) {
		const float w = (float)L::w(i);
		const float vcc = 3.f * ((float)L::cx(i) * u[0] + (float)L::cy(i) * u[1]);
		const float geq = __fmaf_rn(w * rho, vcc + __fmaf_rn(0.5f * vcc, vcc, -h), w * drho);
		g[i] = __fmaf_rn(p.omega, geq - g[i], g[i]);
	}
	return true;
}

template <bool ODD, int MODE>
__global__ void __launch_bounds__(512, MODE == MODE_EXACT ? 1 : 4) k_batch_sweep(const __grid_constant__ BatchParams p) {
	using L = D2Q9;
	const int4 *tr = reinterpret_cast<const int4 *>(p.trec + blockIdx.x);
	const int4 r0 = __ldg(tr), r1 = __ldg(tr + 1);
	TileRec ch;
	ch.cell0 = (int64_t)(((uint64_t)(uint32_t)r0.y << 32) | (uint32_t)r0.x);
	ch.l0 = r0.z;
	ch.nxp = r0.w;
	ch.ny = r1.x;
	ch.omega = __int_as_float(r1.y);
	ch.prof_off = r1.z;
	if (!r1.w) return; // converged channel
	const int l = ch.l0 + (int)threadIdx.x;
	if (l >= ch.nxp * ch.ny) return;
	const int y = l / ch.nxp, x = l - y * ch.nxp;
	const int64_t cell = ch.cell0 + threadIdx.x;
	const int64_t ch_off = ch.cell0 - ch.l0; // the channel's first cell
	// interior cells: every neighbour inside the channel, offsets from the
	// cell in 32-bit arithmetic
	const bool fast = p.idx32 && x > 0 && x + 1 < ch.nxp && y > 0 && y + 1 < ch.ny;
	const float *const fc = p.f + cell;
	const int pl32 = static_cast<int>(p.plane), nxp = ch.nxp;
	float f[9];
	if (fast) {
#pragma unroll
		for (int i = 0; i < 9; ++i)
			f[i] = ODD ? __ldcs(fc + (L::opp(i) * pl32 - L::cx(i) - L::cy(i) * nxp)) : __ldcs(fc + i * pl32);
	} else {
#pragma unroll
		for (int i = 0; i < 9; ++i) {
			if (!ODD) {
				f[i] = __ldcs(p.f + i * p.plane + cell);
			} else {
				const int sx = x - L::cx(i), sy = y - L::cy(i);
				const bool in = sx >= 0 && sx < ch.nxp && sy >= 0 && sy < ch.ny;
				f[i] = in ? __ldcs(p.f + L::opp(i) * p.plane + ch_off + sy * ch.nxp + sx) : 0.f;
			}
		}
	}
	CellCtx ctx;
	ctx.ops = p.ops;
	ctx.profile = p.profiles + ch.prof_off;
	ctx.omega = ch.omega;
	ctx.guo_scale = 1.0f - 0.5f * ch.omega; // unused by BGK
	ctx.g[0] = ctx.g[1] = ctx.g[2] = 0.f;
	const float Fc[3] = {0.f, 0.f, 0.f};
	float rho = 1.f, u[3] = {0.f, 0.f, 0.f};
	// L2 prefetch of the tile p.pf_ahead launched blocks later (every
	// direction plane, one 128-byte line per thread), issued after this
	// block's own loads: requests in flight that hold no registers
	if (p.pf_ahead > 0) {
		const int64_t bt = (int64_t)blockIdx.x + p.pf_ahead;
		const int lines = (int)blockDim.x / 32;
		if (bt < (int64_t)gridDim.x && (int)threadIdx.x < 9 * lines) {
			const int4 *tt = reinterpret_cast<const int4 *>(p.trec + bt);
			const int4 q0 = __ldg(tt), q1 = __ldg(tt + 1);
			if (q1.w) {
				const int64_t c0 = (int64_t)(((uint64_t)(uint32_t)q0.y << 32) | (uint32_t)q0.x);
				const int i = (int)threadIdx.x / lines, k = (int)threadIdx.x - i * lines;
				asm volatile("prefetch.global.L2 [%0];" ::"l"(p.f + i * p.plane + c0 + k * 32));
			}
		}
	}
	const bool col = MODE == MODE_SHIFTED
						 ? cell_update_shifted(f, p.flags[cell], y, ctx, rho, u)
						 : cell_update<L, COLL_BGK, MODE == MODE_EXACT>(f, p.flags[cell], y, ctx, 1.f, Fc, rho, u);
	if (p.write_macros && col) {
		p.rho[cell] = rho;
		p.u[cell] = u[0];
		p.u[p.plane + cell] = u[1];
	}
	float *const fw = p.f + cell;
	if (fast) {
#pragma unroll
		for (int i = 0; i < 9; ++i)
			__stcs(fw + (ODD ? i * pl32 + L::cx(i) + L::cy(i) * nxp : L::opp(i) * pl32), f[i]);
		return;
	}
#pragma unroll
	for (int i = 0; i < 9; ++i) {
		if (!ODD) {
			__stcs(p.f + L::opp(i) * p.plane + cell, f[i]);
		} else {
			const int64_t pb = static_cast<int64_t>(i) * p.plane;
			const int sx = x - L::cx(i), sy = y - L::cy(i);
			if (sx < 0 || sx >= ch.nxp || sy < 0 || sy >= ch.ny) __stcs(p.f + pb + cell, 0.f);
			const int dx = x + L::cx(i), dy = y + L::cy(i);
			if (dx >= 0 && dx < ch.nxp && dy >= 0 && dy < ch.ny) __stcs(p.f + pb + ch_off + dy * ch.nxp + dx, f[i]);
		}
	}
}

// Per tile: sum over its cells of |u - u_prev|^2 and |u|^2 in FP64, then
// u_prev = u.  Fixed reduction order (warp shuffle, then warps in order).
__global__ void __launch_bounds__(512) k_batch_residual_partial(BatchParams p) {
	__shared__ double sh[2][16];
	const int2 tc = p.blist[blockIdx.x];
	const int ob = tc.x, c = tc.y;
	double num = 0.0, den = 0.0;
	if (p.active[c]) {
		const ChannelRec ch = p.ch[c];
		const int l = (ob - ch.first_block) * blockDim.x + threadIdx.x;
		if (l < ch.nxp * ch.ny) {
			const int64_t cell = ch.off + l;
			for (int d = 0; d < 2; ++d) {
				const double a = p.u[d * p.plane + cell], b = p.u_prev[d * p.plane + cell];
				num += (a - b) * (a - b);
				den += a * a;
				p.u_prev[d * p.plane + cell] = (float)a;
			}
			// a density that overflowed (u may still read 0) marks the run diverged
			if (!isfinite(p.rho[cell])) num = CUDART_NAN;
		}
	}
	for (int o = 16; o > 0; o >>= 1) {
		num += __shfl_down_sync(0xffffffffu, num, o);
		den += __shfl_down_sync(0xffffffffu, den, o);
	}
	if ((threadIdx.x & 31) == 0) {
		sh[0][threadIdx.x >> 5] = num;
		sh[1][threadIdx.x >> 5] = den;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		double a = 0.0, b = 0.0;
		for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
			a += sh[0][w];
			b += sh[1][w];
		}
		p.partial[ob] = make_double2(a, b);
	}
}

// Per channel: relative L2 change sqrt(sum|du|^2 / sum|u|^2) over its tiles
// (in tile order); a channel below `tol` is deactivated, and so is one whose
// residual is not finite (a diverged run; its residual stays NaN / inf).
__global__ void k_batch_residual_final(BatchParams p, int n_channels, double tol, double *residual) {
	const int c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c >= n_channels || !p.active[c]) return;
	const ChannelRec ch = p.ch[c];
	double a = 0.0, b = 0.0;
	for (int k = 0; k < ch.nblocks; ++k) {
		const double2 v = p.partial[ch.first_block + k];
		a += v.x;
		b += v.y;
	}
	// NaN sums (a NaN or overflowed field) give a NaN residual: diverged
	const double r = (isnan(a) || isnan(b)) ? (double)NAN : (b > 0.0 ? sqrt(a / b) : (a > 0.0 ? INFINITY : 0.0));
	residual[c] = r;
	if (r < tol || !isfinite(r)) {
		p.active[c] = 0;
		const int lf = p.lfirst[c];
		if (lf >= 0)
			for (int k = 0; k < ch.nblocks; ++k) p.trec[lf + k].live = 0;
	}
}

__global__ void k_batch_init(BatchParams p, int64_t n) {
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
		for (int i = 0; i < 9; ++i) p.f[i * p.plane + k] = p.shifted ? 0.f : (float)D2Q9::w(i);
		p.rho[k] = 1.f;
		p.u[k] = p.u[p.plane + k] = 0.f;
		p.u_prev[k] = p.u_prev[p.plane + k] = 0.f;
	}
}

// packed host flags (nx*ny per channel, concatenated) -> padded device tiles
__global__ void k_batch_flags(BatchParams p, const uint8_t *packed, const int64_t *src_off, int n_channels) {
	const int c = blockIdx.y;
	if (c >= n_channels) return;
	const ChannelRec ch = p.ch[c];
	const int64_t cells = (int64_t)ch.nxp * ch.ny;
	uint8_t *dst = const_cast<uint8_t *>(p.flags);
	for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < cells; l += (int64_t)gridDim.x * blockDim.x) {
		const int y = (int)(l / ch.nxp), x = (int)(l - (int64_t)y * ch.nxp);
		dst[ch.off + l] = x < ch.nx ? packed[src_off[c] + (int64_t)y * ch.nx + x] : 0;
	}
}

// channel c -> host layouts (AoS populations, or rho / u)
__global__ void k_batch_download(BatchParams p, ChannelRec ch, int odd, int what, float *out) {
	const int64_t n = (int64_t)ch.nx * ch.ny;
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
		const int y = (int)(k / ch.nx), x = (int)(k - (int64_t)y * ch.nx);
		const int64_t cell = ch.off + (int64_t)y * ch.nxp + x;
		if (what == 0) {
			for (int i = 0; i < 9; ++i) {
				float v;
				const float wi = p.shifted ? (float)D2Q9::w(i) : 0.f;
				if (!odd) {
					v = p.f[i * p.plane + cell] + wi;
				} else {
					const int sx = x - D2Q9::cx(i), sy = y - D2Q9::cy(i);
					v = (sx >= 0 && sx < ch.nxp && sy >= 0 && sy < ch.ny)
							? p.f[D2Q9::opp(i) * p.plane + ch.off + (int64_t)sy * ch.nxp + sx] + wi
							: 0.f;
				}
				out[k * 9 + i] = v;
			}
		} else {
			out[k * 3 + 0] = p.rho[cell];
			out[k * 3 + 1] = p.u[cell];
			out[k * 3 + 2] = p.u[p.plane + cell];
		}
	}
}

// Warm start of channels [first, first + gridDim.y) at an even time step.
// Channel first + j reads its predicted field at pred + j * pred_stride: three
// values v per cell (x fastest), physical (u_x, u_y, rho) = v * scale + offset
// with scale / offset = sc[3j..3j+2] / of[3j..3j+2].  A fluid cell gets
//   f_i = f_eq(rho, u) - (tau w_i rho / cs^2) Q_i : grad u   (with_neq)
// with Q_i = c_i c_i - cs^2 I and grad u by central differences (one-sided at
// the channel ends; u = 0 in wall cells): the first-order Chapman-Enskog
// population of the predicted field.  A wall cell (flag 1) holds, in each
// slot i whose source x - c_i is fluid, that neighbour's post-collision
// population f_eq + (1 - omega) f_neq (what the last stream step would have
// brought), and the rest state at the mean predicted density of its fluid
// neighbours in the other slots; u_prev takes the predicted u, so the first
// residual measures the change from the prediction.
__global__ void k_batch_warm_start(BatchParams p, int first, const float *pred, int64_t pred_stride, const float *sc,
								   const float *of, int with_neq) {
	const int j = blockIdx.y;
	const ChannelRec ch = p.ch[first + j];
	const float *pr = pred + (int64_t)j * pred_stride;
	const float s0 = sc[3 * j], s1 = sc[3 * j + 1], s2 = sc[3 * j + 2];
	const float o0 = of[3 * j], o1 = of[3 * j + 1], o2 = of[3 * j + 2];
	const float tau = 1.f / ch.omega;
	const float post = 1.f - ch.omega; // f_neq factor after a BGK collision
	const int64_t n = (int64_t)ch.nx * ch.ny;
	auto is_fluid = [&](int xx, int yy) {
		const uint8_t f2 = p.flags[ch.off + (int64_t)yy * ch.nxp + xx];
		return f2 != 1 && f2 != 0;
	};
	auto ux_at = [&](int xx, int yy) {
		return is_fluid(xx, yy) ? pr[((int64_t)yy * ch.nx + xx) * 3 + 0] * s0 + o0 : 0.f;
	};
	auto uy_at = [&](int xx, int yy) {
		return is_fluid(xx, yy) ? pr[((int64_t)yy * ch.nx + xx) * 3 + 1] * s1 + o1 : 0.f;
	};
	// population i of fluid cell (xx, yy): f_eq + fac f_neq (fac = 1: before,
	// 1 - omega: after its collision)
	auto pop = [&](int xx, int yy, int i, float fac) {
		float u[3] = {ux_at(xx, yy), uy_at(xx, yy), 0.f};
		const float rho = pr[((int64_t)yy * ch.nx + xx) * 3 + 2] * s2 + o2;
		float eq[9];
		equilibrium<D2Q9, true>(rho, u, eq);
		float v = eq[i];
		if (with_neq) {
			const int xm = xx > 0 ? xx - 1 : xx, xp = xx + 1 < ch.nx ? xx + 1 : xx;
			const int ym = yy > 0 ? yy - 1 : yy, yp = yy + 1 < ch.ny ? yy + 1 : yy;
			const float ix = 1.f / (float)(xp - xm), iy = 1.f / (float)(yp - ym);
			const float dxu = (ux_at(xp, yy) - ux_at(xm, yy)) * ix, dxv = (uy_at(xp, yy) - uy_at(xm, yy)) * ix;
			const float dyu = (ux_at(xx, yp) - ux_at(xx, ym)) * iy, dyv = (uy_at(xx, yp) - uy_at(xx, ym)) * iy;
			const float cx = (float)D2Q9::cx(i), cy = (float)D2Q9::cy(i);
			const float qs = (cx * cx - 1.f / 3.f) * dxu + (cy * cy - 1.f / 3.f) * dyv + cx * cy * (dxv + dyu);
			v -= fac * tau * (float)D2Q9::w(i) * rho * 3.f * qs;
		}
		return v;
	};
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
		const int y = (int)(k / ch.nx), x = (int)(k - (int64_t)y * ch.nx);
		const int64_t cell = ch.off + (int64_t)y * ch.nxp + x;
		float f[9];
		if (!is_fluid(x, y)) {
			// what streamed in from fluid neighbours: their post-collision
			// populations; the rest of the slots at the mean neighbour density
			float rs = 0.f;
			int cnt = 0;
			for (int i = 1; i < 9; ++i) {
				const int xx = x + D2Q9::cx(i), yy = y + D2Q9::cy(i);
				if (xx >= 0 && xx < ch.nx && yy >= 0 && yy < ch.ny && is_fluid(xx, yy)) {
					rs += pr[((int64_t)yy * ch.nx + xx) * 3 + 2] * s2 + o2;
					++cnt;
				}
			}
			const float rho = cnt ? rs / (float)cnt : 1.f;
			for (int i = 0; i < 9; ++i) {
				const int xs = x - D2Q9::cx(i), ys = y - D2Q9::cy(i);
				const bool from_fluid = i > 0 && xs >= 0 && xs < ch.nx && ys >= 0 && ys < ch.ny && is_fluid(xs, ys);
				f[i] = from_fluid ? pop(xs, ys, i, post) : (float)D2Q9::w(i) * rho;
			}
		} else {
			for (int i = 0; i < 9; ++i) f[i] = pop(x, y, i, 1.f);
			p.u_prev[cell] = ux_at(x, y);
			p.u_prev[p.plane + cell] = uy_at(x, y);
		}
		for (int i = 0; i < 9; ++i) p.f[i * p.plane + cell] = f[i] - (p.shifted ? (float)D2Q9::w(i) : 0.f);
	}
}

// Refinement of a warm start, channels [first, first + gridDim.y) at an even
// time step, same prediction arguments as k_batch_warm_start: every fluid cell
// keeps the non-equilibrium part of its current populations and gets the
// predicted macroscopic field back,
//   f_i <- f_i - f_eq(rho_f, u_f) + f_eq(rho_p, u_p),
// rho_f, u_f the moments of f and (rho_p, u_p) the prediction (rho_p = rho_f
// with keep_rho).  After a few sweeps from the first-order reconstruction,
// the non-equilibrium part is the one the lattice dynamics and its boundary
// rules produce for this field, not a finite-difference estimate.
__global__ void k_batch_reimpose(BatchParams p, int first, const float *pred, int64_t pred_stride, const float *sc,
								 const float *of, int keep_rho) {
	const int j = blockIdx.y;
	const ChannelRec ch = p.ch[first + j];
	const float *pr = pred + (int64_t)j * pred_stride;
	const float s0 = sc[3 * j], s1 = sc[3 * j + 1], s2 = sc[3 * j + 2];
	const float o0 = of[3 * j], o1 = of[3 * j + 1], o2 = of[3 * j + 2];
	const int64_t n = (int64_t)ch.nx * ch.ny;
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
		const int y = (int)(k / ch.nx), x = (int)(k - (int64_t)y * ch.nx);
		const int64_t cell = ch.off + (int64_t)y * ch.nxp + x;
		const uint8_t fl = p.flags[cell];
		if (fl == 1 || fl == 0) continue;
		float f[9];
		for (int i = 0; i < 9; ++i) f[i] = p.f[i * p.plane + cell] + (p.shifted ? (float)D2Q9::w(i) : 0.f);
		float rho_f, u_f[3];
		moments<D2Q9, true>(f, rho_f, u_f);
		const float *v = pr + k * 3;
		float u_p[3] = {v[0] * s0 + o0, v[1] * s1 + o1, 0.f};
		const float rho_p = keep_rho ? rho_f : v[2] * s2 + o2;
		float eq_f[9], eq_p[9];
		equilibrium<D2Q9, true>(rho_f, u_f, eq_f);
		equilibrium<D2Q9, true>(rho_p, u_p, eq_p);
		for (int i = 0; i < 9; ++i)
			p.f[i * p.plane + cell] = f[i] - eq_f[i] + eq_p[i] - (p.shifted ? (float)D2Q9::w(i) : 0.f);
	}
}

// f <-> g = f - w_i on every slot (sign -1: to shifted, +1: back), when a
// program switches between shifted and unshifted arithmetic
__global__ void k_batch_shift(BatchParams p, float sign) {
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < p.plane; k += (int64_t)gridDim.x * blockDim.x)
		for (int i = 0; i < 9; ++i) p.f[i * p.plane + k] += sign * (float)D2Q9::w(i);
}

} // namespace

struct kel_batch {
	int n = 0;
	int tile = 256;
	int sms = 1; // multiprocessors of the batch's device
	std::vector<kel_channel_desc> desc;
	std::vector<ChannelRec> rec;
	std::vector<int> block_ch;
	std::vector<int2> blist; // launched (tile, channel) pairs (host copy of d_blist)
	int nlaunch = 0;        // tiles launched per sweep
	std::vector<uint64_t> t;          // per-channel time step
	std::vector<uint8_t> host_flags;  // packed copy (kept for re-layout)
	std::vector<float> host_profiles; // packed inlet profiles
	int64_t plane = 0;
	int nblocks = 0;
	int64_t profile_len = 0;
	// device
	float *f = nullptr, *rho = nullptr, *u = nullptr, *u_prev = nullptr, *profiles = nullptr;
	uint8_t *flags = nullptr;
	ChannelRec *d_rec = nullptr;
	int *d_block_ch = nullptr, *d_active = nullptr;
	int2 *d_blist = nullptr;
	TileRec *d_trec = nullptr; // per launched block (same order as d_blist)
	int *d_lfirst = nullptr;   // per channel: first launch index of its tiles, -1 if not launched
	double2 *partial = nullptr;
	double *d_residual = nullptr;
	OpEntry *ops = nullptr;
	bool have_ops = false;
	kel_step_program prog;
	int mode = MODE_FAST; // arithmetic of the sweep
	bool shifted = false; // populations stored as g = f - w_i
	cudaStream_t stream = nullptr;
	bool own_stream = false;
	cudaGraphExec_t graph = nullptr;
	int graph_check = 0;
	double graph_tol = 0.0;
};

namespace {

void free_device(kel_batch *B) {
	cudaFree(B->f);
	cudaFree(B->rho);
	cudaFree(B->u);
	cudaFree(B->u_prev);
	cudaFree(B->profiles);
	cudaFree(B->flags);
	cudaFree(B->d_rec);
	cudaFree(B->d_block_ch);
	cudaFree(B->d_blist);
	cudaFree(B->d_trec);
	cudaFree(B->d_lfirst);
	B->d_trec = nullptr;
	B->d_lfirst = nullptr;
	cudaFree(B->d_active);
	cudaFree(B->partial);
	cudaFree(B->d_residual);
	B->f = B->rho = B->u = B->u_prev = B->profiles = nullptr;
	B->flags = nullptr;
	B->d_rec = nullptr;
	B->d_block_ch = B->d_active = nullptr;
	B->d_blist = nullptr;
	B->partial = nullptr;
	B->d_residual = nullptr;
	if (B->graph) cudaGraphExecDestroy(B->graph);
	B->graph = nullptr;
}

BatchParams params(const kel_batch *B, int write_macros) {
	BatchParams p;
	memset(&p, 0, sizeof(p));
	p.trec = B->d_trec;
	p.lfirst = B->d_lfirst;
	p.f = B->f;
	p.plane = B->plane;
	p.flags = B->flags;
	p.rho = B->rho;
	p.u = B->u;
	p.u_prev = B->u_prev;
	p.ops = B->ops;
	p.profiles = B->profiles;
	p.ch = B->d_rec;
	p.block_ch = B->d_block_ch;
	p.blist = B->d_blist;
	p.active = B->d_active;
	p.partial = B->partial;
	p.tile = B->tile;
	p.write_macros = write_macros;
	p.shifted = B->shifted ? 1 : 0;
	p.idx32 = 9 * B->plane < ((int64_t)1 << 31) ? 1 : 0;
	// prefetch the tiles one resident wave later (2048 threads per SM):
	// measured with 1024 channels 0.82 -> 0.85 of HBM; two waves gained less
	p.pf_ahead = B->sms * (2048 / (B->tile > 0 ? B->tile : 256));
	return p;
}

// Tile records and per-channel launch offsets for the current launch list
// (B->blist, B->nlaunch; every listed channel is running).
int upload_tile_records(kel_batch *B) {
	std::vector<TileRec> tr(B->nlaunch);
	std::vector<int> lf(B->n, -1);
	for (int k = 0; k < B->nlaunch; ++k) {
		const int tile = B->blist[k].x, c = B->blist[k].y;
		const ChannelRec &r = B->rec[c];
		if (lf[c] < 0) lf[c] = k;
		TileRec &t = tr[k];
		t.l0 = (tile - r.first_block) * B->tile;
		t.cell0 = r.off + t.l0;
		t.nxp = r.nxp;
		t.ny = r.ny;
		t.omega = r.omega;
		t.prof_off = r.prof_off;
		t.live = 1;
	}
	KEL_CUDA(cudaMemcpyAsync(B->d_trec, tr.data(), sizeof(TileRec) * B->nlaunch, cudaMemcpyHostToDevice, B->stream));
	KEL_CUDA(cudaMemcpyAsync(B->d_lfirst, lf.data(), sizeof(int) * B->n, cudaMemcpyHostToDevice, B->stream));
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	return KEL_OK;
}

// Lay the channels out in tiles of `tile` cells and allocate the device side.
int layout(kel_batch *B, int tile) {
	free_device(B);
	B->tile = tile;
	B->rec.assign(B->n, ChannelRec{});
	B->block_ch.clear();
	int64_t off = 0;
	int64_t poff = 0;
	for (int c = 0; c < B->n; ++c) {
		const kel_channel_desc &d = B->desc[c];
		ChannelRec &r = B->rec[c];
		r.nx = (int)d.nx;
		r.nxp = (int)((d.nx + 3) / 4 * 4);
		r.ny = (int)d.ny;
		r.off = off;
		r.first_block = (int)B->block_ch.size();
		const int64_t cells = (int64_t)r.nxp * r.ny;
		r.nblocks = (int)((cells + tile - 1) / tile);
		for (int k = 0; k < r.nblocks; ++k) B->block_ch.push_back(c);
		off += (int64_t)r.nblocks * tile;
		r.prof_off = (int)poff;
		poff += r.ny;
		r.omega = 1.0f / (float)d.tau;
		r.guo_scale = 1.0f - 0.5f * r.omega;
	}
	B->plane = off;
	B->nblocks = (int)B->block_ch.size();
	B->profile_len = poff;
	KEL_CUDA(cudaMalloc(&B->f, sizeof(float) * 9 * B->plane));
	KEL_CUDA(cudaMalloc(&B->rho, sizeof(float) * B->plane));
	KEL_CUDA(cudaMalloc(&B->u, sizeof(float) * 2 * B->plane));
	KEL_CUDA(cudaMalloc(&B->u_prev, sizeof(float) * 2 * B->plane));
	KEL_CUDA(cudaMalloc(&B->profiles, sizeof(float) * (B->profile_len + 1)));
	KEL_CUDA(cudaMalloc(&B->flags, B->plane));
	KEL_CUDA(cudaMalloc(&B->d_rec, sizeof(ChannelRec) * B->n));
	KEL_CUDA(cudaMalloc(&B->d_block_ch, sizeof(int) * B->nblocks));
	KEL_CUDA(cudaMalloc(&B->d_blist, sizeof(int2) * B->nblocks));
	KEL_CUDA(cudaMalloc(&B->d_trec, sizeof(TileRec) * B->nblocks));
	KEL_CUDA(cudaMalloc(&B->d_lfirst, sizeof(int) * B->n));
	B->blist.resize(B->nblocks);
	for (int b = 0; b < B->nblocks; ++b) B->blist[b] = make_int2(b, B->block_ch[b]);
	B->nlaunch = B->nblocks;
	KEL_CUDA(cudaMemcpyAsync(B->d_blist, B->blist.data(), sizeof(int2) * B->nblocks, cudaMemcpyHostToDevice,
							 B->stream));
	{
		int rc2 = upload_tile_records(B);
		if (rc2) return rc2;
	}
	KEL_CUDA(cudaMalloc(&B->d_active, sizeof(int) * B->n));
	KEL_CUDA(cudaMalloc(&B->partial, sizeof(double2) * B->nblocks));
	KEL_CUDA(cudaMalloc(&B->d_residual, sizeof(double) * B->n));
	KEL_CUDA(cudaMemcpyAsync(B->d_rec, B->rec.data(), sizeof(ChannelRec) * B->n, cudaMemcpyHostToDevice, B->stream));
	KEL_CUDA(cudaMemcpyAsync(B->d_block_ch, B->block_ch.data(), sizeof(int) * B->nblocks, cudaMemcpyHostToDevice,
							 B->stream));
	KEL_CUDA(cudaMemcpyAsync(B->profiles, B->host_profiles.data(), sizeof(float) * B->profile_len,
							 cudaMemcpyHostToDevice, B->stream));
	std::vector<int> ones(B->n, 1);
	KEL_CUDA(cudaMemcpyAsync(B->d_active, ones.data(), sizeof(int) * B->n, cudaMemcpyHostToDevice, B->stream));
	KEL_CUDA(cudaMemsetAsync(B->d_residual, 0, sizeof(double) * B->n, B->stream));
	KEL_CUDA(cudaMemsetAsync(B->flags, 0, B->plane, B->stream));
	BatchParams p = params(B, 0);
	k_batch_init<<<grid_for(B->plane), 256, 0, B->stream>>>(p, B->plane);
	KEL_CUDA(cudaGetLastError());
	if (!B->host_flags.empty()) {
		uint8_t *dpk = nullptr;
		int64_t *doff = nullptr;
		std::vector<int64_t> soff(B->n);
		int64_t s = 0;
		for (int c = 0; c < B->n; ++c) {
			soff[c] = s;
			s += B->desc[c].nx * B->desc[c].ny;
		}
		KEL_CUDA(cudaMalloc(&dpk, B->host_flags.size()));
		KEL_CUDA(cudaMalloc(&doff, sizeof(int64_t) * B->n));
		KEL_CUDA(cudaMemcpyAsync(dpk, B->host_flags.data(), B->host_flags.size(), cudaMemcpyHostToDevice, B->stream));
		KEL_CUDA(cudaMemcpyAsync(doff, soff.data(), sizeof(int64_t) * B->n, cudaMemcpyHostToDevice, B->stream));
		k_batch_flags<<<dim3(64, B->n), 256, 0, B->stream>>>(p, dpk, doff, B->n);
		KEL_CUDA(cudaGetLastError());
		KEL_CUDA(cudaStreamSynchronize(B->stream));
		cudaFree(dpk);
		cudaFree(doff);
	}
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	for (auto &tc : B->t) tc = 0;
	return KEL_OK;
}

cudaError_t launch_sweep_batch(const kel_batch *B, bool odd, int write_macros) {
	BatchParams p = params(B, write_macros);
	const dim3 g(B->nlaunch), b(B->tile);
	switch (B->mode) {
	case MODE_EXACT:
		if (odd) k_batch_sweep<true, MODE_EXACT><<<g, b, 0, B->stream>>>(p);
		else k_batch_sweep<false, MODE_EXACT><<<g, b, 0, B->stream>>>(p);
		break;
	case MODE_SHIFTED:
		if (odd) k_batch_sweep<true, MODE_SHIFTED><<<g, b, 0, B->stream>>>(p);
		else k_batch_sweep<false, MODE_SHIFTED><<<g, b, 0, B->stream>>>(p);
		break;
	default:
		if (odd) k_batch_sweep<true, MODE_FAST><<<g, b, 0, B->stream>>>(p);
		else k_batch_sweep<false, MODE_FAST><<<g, b, 0, B->stream>>>(p);
	}
	return cudaGetLastError();
}

cudaError_t launch_residual(const kel_batch *B, double tol) {
	BatchParams p = params(B, 0);
	k_batch_residual_partial<<<B->nlaunch, B->tile, 0, B->stream>>>(p);
	k_batch_residual_final<<<(B->n + 127) / 128, 128, 0, B->stream>>>(p, B->n, tol, B->d_residual);
	return cudaGetLastError();
}

} // namespace

extern "C" int kel_batch_create(int32_t n_channels, const kel_channel_desc *ch, int32_t tile, kel_batch **out) {
	if (!out || !ch || n_channels < 1) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_create: bad arguments");
	*out = nullptr;
	if (tile == 0) tile = 256;
	if (tile != 128 && tile != 256 && tile != 512)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_create: tile must be 128, 256 or 512");
	for (int c = 0; c < n_channels; ++c) {
		if (ch[c].nx < 3 || ch[c].ny < 3 || ch[c].nx > (1 << 20) || ch[c].ny > (1 << 20))
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_create: channel %d has bad extents", c);
		if (!(ch[c].tau > 0.0)) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_create: channel %d tau", c);
	}
	kel_batch *B = new kel_batch();
	B->n = n_channels;
	{
		int dev = 0;
		if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&B->sms, cudaDevAttrMultiProcessorCount, dev);
		if (B->sms < 1) B->sms = 1;
	}
	B->desc.assign(ch, ch + n_channels);
	B->t.assign(n_channels, 0);
	// parabolic inlet per channel, as the single-lattice inlet profile (float)
	for (int c = 0; c < n_channels; ++c) {
		const int ny = (int)ch[c].ny;
		for (int y = 0; y < ny; ++y) {
			double eta = (y - 0.5) / (double)(ny - 2);
			double u = (y == 0 || y == ny - 1) ? 0.0 : 4.0 * ch[c].u_max * eta * (1.0 - eta);
			B->host_profiles.push_back((float)u);
		}
	}
	if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess) {
		delete B;
		return fail(KEL_ERR_CUDA, "kel_batch_create: stream creation failed");
	}
	B->own_stream = true;
	if (cudaMalloc(&B->ops, sizeof(OpEntry) * MAX_FLAGS) != cudaSuccess) {
		cudaStreamDestroy(B->stream);
		delete B;
		return fail(KEL_ERR_OUT_OF_MEMORY, "kel_batch_create: allocation failed");
	}
	int rc = layout(B, tile);
	if (rc) {
		kel_batch_destroy(B);
		return rc;
	}
	*out = B;
	return KEL_OK;
}

extern "C" int kel_batch_destroy(kel_batch *B) {
	if (!B) return KEL_OK;
	cudaStreamSynchronize(B->stream);
	free_device(B);
	cudaFree(B->ops);
	if (B->own_stream) cudaStreamDestroy(B->stream);
	delete B;
	return KEL_OK;
}

extern "C" int kel_batch_upload_flags(kel_batch *B, const uint8_t *packed) {
	if (!B || !packed) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_upload_flags: null argument");
	int64_t total = 0;
	for (int c = 0; c < B->n; ++c) total += B->desc[c].nx * B->desc[c].ny;
	B->host_flags.assign(packed, packed + total);
	return layout(B, B->tile);
}

extern "C" int kel_batch_set_program(kel_batch *B, const kel_step_program *P) {
	if (!B || !P) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_set_program: null argument");
	if (P->collision != KEL_COLL_BGK)
		return fail(KEL_ERR_UNSUPPORTED, "kel_batch_set_program: channels run BGK (one tau per channel)");
	OpEntry ops[MAX_FLAGS];
	memset(ops, 0, sizeof(ops));
	for (int fl = 0; fl < MAX_FLAGS; ++fl) {
		const kel_flag_op &o = P->ops[fl];
		if (o.bc == KEL_BC_MOVING_WALL || o.bc == KEL_BC_EQUILIBRIUM)
			return fail(KEL_ERR_UNSUPPORTED, "kel_batch_set_program: flag %d: boundary %d not batched", fl, o.bc);
		if (o.bc < KEL_BC_NONE || o.bc > KEL_BC_ANTI_BOUNCE_BACK)
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_set_program: flag %d: unknown boundary %d", fl, o.bc);
		ops[fl].bc = o.bc;
		ops[fl].collide = o.collide ? 1 : 0;
		ops[fl].east = o.east ? 1 : 0;
		ops[fl].use_profile = o.use_profile ? 1 : 0;
		ops[fl].rho = (float)o.rho;
		for (int k = 0; k < 3; ++k) ops[fl].u[k] = (float)o.u[k];
	}
	if (P->arithmetic != KEL_ARITH_FAST && P->arithmetic != KEL_ARITH_REFERENCE && P->arithmetic != KEL_ARITH_SHIFTED)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_set_program: unknown arithmetic");
	B->mode = P->arithmetic == KEL_ARITH_REFERENCE ? MODE_EXACT
			  : (P->arithmetic == KEL_ARITH_SHIFTED ? MODE_SHIFTED : MODE_FAST);
	const bool shifted = B->mode == MODE_SHIFTED;
	if (shifted != B->shifted) { // re-express the stored populations
		B->shifted = shifted;
		k_batch_shift<<<grid_for(B->plane), 256, 0, B->stream>>>(params(B, 0), shifted ? -1.f : 1.f);
		KEL_CUDA(cudaGetLastError());
	}
	KEL_CUDA(cudaMemcpyAsync(B->ops, ops, sizeof(ops), cudaMemcpyHostToDevice, B->stream));
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	B->prog = *P;
	B->have_ops = true;
	if (B->graph) {
		cudaGraphExecDestroy(B->graph);
		B->graph = nullptr;
	}
	return KEL_OK;
}

static uint64_t global_t(const kel_batch *B) {
	uint64_t t = 0;
	for (auto v : B->t) t = v > t ? v : t;
	return t;
}

extern "C" int kel_batch_step(kel_batch *B, uint64_t n_steps) {
	if (!B) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_step: null batch");
	if (!B->have_ops) return fail(KEL_ERR_STATE, "kel_batch_step: no program set");
	std::vector<int> act(B->n);
	KEL_CUDA(cudaMemcpyAsync(act.data(), B->d_active, sizeof(int) * B->n, cudaMemcpyDeviceToHost, B->stream));
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	uint64_t t = global_t(B);
	for (int c = 0; c < B->n; ++c)
		if (act[c] && B->t[c] != t) return fail(KEL_ERR_STATE, "kel_batch_step: channel time steps diverged");
	for (uint64_t s = 0; s < n_steps; ++s) {
		cudaError_t e = launch_sweep_batch(B, ((t + s) & 1u) != 0, s + 1 == n_steps);
		if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_batch_step: %s", cudaGetErrorString(e));
	}
	for (int c = 0; c < B->n; ++c)
		if (act[c]) B->t[c] += n_steps;
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	return KEL_OK;
}

// Launch only the tiles of active channels once they are at most half of
// the tiles launched so far (a converged channel's tiles otherwise still
// cost a block launch each per sweep).  Any captured graph is dropped.
static int compact(kel_batch *B, const std::vector<int> &act) {
	int keep = 0;
	for (int c = 0; c < B->n; ++c)
		if (act[c]) keep += B->rec[c].nblocks;
	if (keep == 0 || 2 * keep > B->nlaunch) return KEL_OK;
	B->blist.clear();
	for (int c = 0; c < B->n; ++c)
		if (act[c])
			for (int k = 0; k < B->rec[c].nblocks; ++k) B->blist.push_back(make_int2(B->rec[c].first_block + k, c));
	KEL_CUDA(cudaMemcpyAsync(B->d_blist, B->blist.data(), sizeof(int2) * keep, cudaMemcpyHostToDevice, B->stream));
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	B->nlaunch = keep;
	int rc = upload_tile_records(B);
	if (rc) return rc;
	if (B->graph) cudaGraphExecDestroy(B->graph);
	B->graph = nullptr;
	return KEL_OK;
}

// Capture `check` sweeps + the residual as one graph.
static int build_graph(kel_batch *B, int check, double tol) {
	if (B->graph && B->graph_check == check && B->graph_tol == tol) return KEL_OK;
	if (B->graph) cudaGraphExecDestroy(B->graph);
	B->graph = nullptr;
	cudaGraph_t g;
	KEL_CUDA(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
	cudaError_t e = cudaSuccess;
	for (int s = 0; s < check && e == cudaSuccess; ++s) e = launch_sweep_batch(B, (s & 1) != 0, s + 1 == check);
	if (e == cudaSuccess) e = launch_residual(B, tol);
	cudaError_t e2 = cudaStreamEndCapture(B->stream, &g);
	if (e != cudaSuccess || e2 != cudaSuccess)
		return fail(KEL_ERR_CUDA, "kel_batch_run_until: graph capture failed: %s",
					cudaGetErrorString(e != cudaSuccess ? e : e2));
	e = cudaGraphInstantiate(&B->graph, g, 0);
	cudaGraphDestroy(g);
	if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_batch_run_until: instantiate: %s", cudaGetErrorString(e));
	B->graph_check = check;
	B->graph_tol = tol;
	return KEL_OK;
}

extern "C" int kel_batch_run_until(kel_batch *B, double tol, uint64_t check_every, uint64_t max_steps,
								   int32_t use_graph, uint64_t *steps_out, double *residual_out) {
	if (!B) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_run_until: null batch");
	if (!B->have_ops) return fail(KEL_ERR_STATE, "kel_batch_run_until: no program set");
	if (check_every < 2 || (check_every & 1u) || check_every > 100000)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_run_until: check_every must be even, 2..100000");
	uint64_t t0 = global_t(B);
	if (t0 & 1u) return fail(KEL_ERR_STATE, "kel_batch_run_until: needs an even time step");
	std::vector<int> act(B->n);
	KEL_CUDA(cudaMemcpyAsync(act.data(), B->d_active, sizeof(int) * B->n, cudaMemcpyDeviceToHost, B->stream));
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	int rc;
	uint64_t done = 0;
	int n_active = 0;
	for (int c = 0; c < B->n; ++c) n_active += act[c] != 0;
	while (n_active > 0 && done < max_steps) {
		if ((rc = compact(B, act))) return rc;
		if (use_graph && (rc = build_graph(B, (int)check_every, tol))) return rc;
		if (use_graph) {
			KEL_CUDA(cudaGraphLaunch(B->graph, B->stream));
		} else {
			for (uint64_t s = 0; s < check_every; ++s) {
				cudaError_t e = launch_sweep_batch(B, (s & 1u) != 0, s + 1 == check_every);
				if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_batch_run_until: %s", cudaGetErrorString(e));
			}
			cudaError_t e = launch_residual(B, tol);
			if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_batch_run_until: %s", cudaGetErrorString(e));
		}
		done += check_every;
		for (int c = 0; c < B->n; ++c)
			if (act[c]) B->t[c] += check_every;
		KEL_CUDA(cudaMemcpyAsync(act.data(), B->d_active, sizeof(int) * B->n, cudaMemcpyDeviceToHost, B->stream));
		KEL_CUDA(cudaStreamSynchronize(B->stream));
		n_active = 0;
		for (int c = 0; c < B->n; ++c) n_active += act[c] != 0;
	}
	if (steps_out)
		for (int c = 0; c < B->n; ++c) steps_out[c] = B->t[c];
	if (residual_out) {
		KEL_CUDA(cudaMemcpyAsync(residual_out, B->d_residual, sizeof(double) * B->n, cudaMemcpyDeviceToHost, B->stream));
		KEL_CUDA(cudaStreamSynchronize(B->stream));
	}
	return KEL_OK;
}

extern "C" int kel_batch_active_count(kel_batch *B, int32_t *count) {
	if (!B || !count) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_active_count: null argument");
	std::vector<int> act(B->n);
	KEL_CUDA(cudaMemcpyAsync(act.data(), B->d_active, sizeof(int) * B->n, cudaMemcpyDeviceToHost, B->stream));
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	int n = 0;
	for (int c = 0; c < B->n; ++c) n += act[c] != 0;
	*count = n;
	return KEL_OK;
}

static int batch_download(kel_batch *B, int32_t channel, int what, float *host) {
	if (!B || !host || channel < 0 || channel >= B->n)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_download: bad arguments");
	const ChannelRec ch = B->rec[channel];
	const int64_t n = (int64_t)ch.nx * ch.ny * (what == 0 ? 9 : 3);
	float *d = nullptr;
	KEL_CUDA(cudaMalloc(&d, sizeof(float) * n));
	k_batch_download<<<grid_for((int64_t)ch.nx * ch.ny), 256, 0, B->stream>>>(params(B, 0), ch, (int)(B->t[channel] & 1u),
																			  what, d);
	cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaMemcpyAsync(host, d, sizeof(float) * n, cudaMemcpyDeviceToHost, B->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
	cudaFree(d);
	if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_batch_download: %s", cudaGetErrorString(e));
	return KEL_OK;
}

extern "C" int kel_batch_warm_start(kel_batch *B, int32_t first, int32_t count, const float *d_pred,
									int64_t pred_stride, const float *d_scale, const float *d_offset,
									int32_t with_neq) {
	if (!B || !d_pred || !d_scale || !d_offset)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_warm_start: null argument");
	if (first < 0 || count < 1 || count > 65535 || first > B->n - count)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_warm_start: channels [%d, %d) outside [0, %d)", first,
					first + count, B->n);
	int64_t most = 0;
	for (int c = first; c < first + count; ++c) {
		if (B->t[c] & 1u)
			return fail(KEL_ERR_STATE, "kel_batch_warm_start: channel %d is at an odd time step", c);
		const int64_t cells = (int64_t)B->rec[c].nx * B->rec[c].ny;
		if (cells * 3 > pred_stride)
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_warm_start: channel %d needs %lld floats > stride %lld", c,
						(long long)(cells * 3), (long long)pred_stride);
		most = cells > most ? cells : most;
	}
	const int bx = (int)((most + 255) / 256 < 1024 ? (most + 255) / 256 : 1024);
	k_batch_warm_start<<<dim3(bx, count), 256, 0, B->stream>>>(params(B, 0), first, d_pred, pred_stride, d_scale,
															   d_offset, with_neq);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

extern "C" int kel_batch_warm_refine(kel_batch *B, int32_t first, int32_t count, const float *d_pred,
									 int64_t pred_stride, const float *d_scale, const float *d_offset,
									 int32_t iterations, int32_t keep_rho) {
	if (!B || !d_pred || !d_scale || !d_offset)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_warm_refine: null argument");
	if (first < 0 || count < 1 || count > 65535 || first > B->n - count || iterations < 0)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_warm_refine: channels [%d, %d) outside [0, %d)", first,
					first + count, B->n);
	int64_t most = 0;
	for (int c = first; c < first + count; ++c) {
		if (B->t[c] & 1u) return fail(KEL_ERR_STATE, "kel_batch_warm_refine: channel %d is at an odd time step", c);
		const int64_t cells = (int64_t)B->rec[c].nx * B->rec[c].ny;
		if (cells * 3 > pred_stride)
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_warm_refine: channel %d needs %lld floats > stride %lld",
						c, (long long)(cells * 3), (long long)pred_stride);
		most = cells > most ? cells : most;
	}
	const int bx = (int)((most + 255) / 256 < 1024 ? (most + 255) / 256 : 1024);
	int rc;
	for (int it = 0; it < iterations; ++it) {
		if ((rc = kel_batch_step(B, 2))) return rc;
		k_batch_reimpose<<<dim3(bx, count), 256, 0, B->stream>>>(params(B, 0), first, d_pred, pred_stride, d_scale,
																 d_offset, keep_rho);
		KEL_CUDA(cudaGetLastError());
	}
	return KEL_OK;
}

extern "C" int kel_batch_synchronize(kel_batch *B) {
	if (!B) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_synchronize: null batch");
	KEL_CUDA(cudaStreamSynchronize(B->stream));
	return KEL_OK;
}

extern "C" int kel_batch_download_populations(kel_batch *B, int32_t channel, float *host_aos) {
	return batch_download(B, channel, 0, host_aos);
}

extern "C" int kel_batch_download_macros(kel_batch *B, int32_t channel, float *host_rho_u) {
	return batch_download(B, channel, 1, host_rho_u);
}

extern "C" int kel_batch_channel_time_step(const kel_batch *B, int32_t channel, uint64_t *t) {
	if (!B || !t || channel < 0 || channel >= B->n) return fail(KEL_ERR_INVALID_ARGUMENT, "bad arguments");
	*t = B->t[channel];
	return KEL_OK;
}

extern "C" int kel_batch_info(const kel_batch *B, int64_t *cells, int64_t *padded_cells, int32_t *tile) {
	if (!B) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_info: null batch");
	int64_t s = 0;
	for (auto &d : B->desc) s += d.nx * d.ny;
	if (cells) *cells = s;
	if (padded_cells) *padded_cells = B->plane;
	if (tile) *tile = B->tile;
	return KEL_OK;
}

// Time `steps` sweeps for each candidate tile on the current flags and keep the
// fastest; the state returns to rest equilibrium (call before stepping).
extern "C" int kel_batch_autotune(kel_batch *B, int32_t steps, int32_t *chosen_tile, float *ms_per_step) {
	if (!B || steps < 2) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_batch_autotune: bad arguments");
	if (!B->have_ops) return fail(KEL_ERR_STATE, "kel_batch_autotune: set a program first");
	for (auto t : B->t)
		if (t != 0) return fail(KEL_ERR_STATE, "kel_batch_autotune: only before the first step");
	const int cand[3] = {128, 256, 512};
	float best = 1e30f;
	int best_tile = B->tile;
	cudaEvent_t e0, e1;
	KEL_CUDA(cudaEventCreate(&e0));
	KEL_CUDA(cudaEventCreate(&e1));
	for (int k = 0; k < 3; ++k) {
		int rc = layout(B, cand[k]);
		if (rc) return rc;
		launch_sweep_batch(B, false, 0);
		launch_sweep_batch(B, true, 0);
		KEL_CUDA(cudaEventRecord(e0, B->stream));
		for (int s = 0; s < steps; ++s) launch_sweep_batch(B, (s & 1) != 0, 0);
		KEL_CUDA(cudaEventRecord(e1, B->stream));
		KEL_CUDA(cudaEventSynchronize(e1));
		float ms = 0.f;
		KEL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
		ms /= steps;
		if (ms < best) {
			best = ms;
			best_tile = cand[k];
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	int rc = layout(B, best_tile);
	if (rc) return rc;
	if (chosen_tile) *chosen_tile = best_tile;
	if (ms_per_step) *ms_per_step = best;
	return KEL_OK;
}
