// C ABI of the sweep (include/kel_lbm_cuda.h): lattice ownership, host
// uploads/downloads with the AA-parity conversion, program lowering and the
// per-step launch.
//
// Replaces, for the hot path, the reference's SYCL device layer
// (modules/sycl/c++/data.hpp:23-61 ownership, :557-819 copies, :932-965
// device) and the per-driver step()/stream loops.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lattice_internal.cuh"
#include "sweep_dispatch.cuh"
#include "sweep_rows.cuh"

using namespace kel::gb;


// ---------------------------------------------------------------------------
// errors

static thread_local std::string g_err;

namespace kel {
namespace gb {
int fail(int code, const char *fmt, ...) {
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_err = buf;
	return code;
}
} // namespace gb
} // namespace kel

extern "C" const char *kel_last_error_string(void) { return g_err.c_str(); }
extern "C" const char *kel_version(void) { return "kel-lbm-gb300 0.1 (sm_103a)"; }

// ---------------------------------------------------------------------------
// descriptor tables on the host

template <class L>
static HostDesc host_desc() {
	HostDesc h;
	h.D = L::D;
	h.Q = L::Q;
	for (int i = 0; i < L::Q; ++i) {
		h.c[i][0] = L::cx(i);
		h.c[i][1] = L::cy(i);
		h.c[i][2] = L::cz(i);
		h.opp[i] = L::opp(i);
		h.w[i] = L::w(i);
	}
	return h;
}

static bool desc_for(int q, HostDesc &h) {
	if (q == KEL_D2Q9) h = host_desc<D2Q9>();
	else if (q == KEL_D3Q19) h = host_desc<D3Q19>();
	else if (q == KEL_D3Q27) h = host_desc<D3Q27>();
	else return false;
	return true;
}

// equilibrium.hpp:7-48 on the host with the reference's rounding (this file
// is compiled without floating-point contraction).
static void host_equilibrium(const HostDesc &d, float rho, const float *u, float *eq) {
	float vv = 0.f;
	for (int k = 0; k < d.D; ++k) vv = vv + u[k] * u[k];
	for (int i = 0; i < d.Q; ++i) {
		float vc = 0.f;
		for (int k = 0; k < d.D; ++k) vc = vc + u[k] * (float)d.c[i][k];
		float vcc = vc * 3.0f;
		float wr = (float)d.w[i] * rho;
		double br = 1.0 + (double)vcc - (double)3.0f * 0.5 * (double)vv + (double)(vcc * vcc) * 0.5;
		eq[i] = (float)((double)wr * br);
	}
}

__global__ void k_fill_f32(float *p, int64_t n, float v) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

__global__ void k_fill_pop(void *f, int64_t plane, int storage, float v, float s) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < plane; i += (int64_t)gridDim.x * blockDim.x) {
		if (storage == STORE_FP32) static_cast<float *>(f)[i] = v;
		else static_cast<__half *>(f)[i] = __float2half_rn(v - s);
	}
}

int kel::gb::grid_for(int64_t n) {
	int64_t b = (n + 255) / 256;
	if (b > 152 * 64) b = 152 * 64;
	if (b < 1) b = 1;
	return (int)b;
}

static int ensure_staging(kel_lattice *L, size_t bytes) {
	if (L->staging_bytes >= bytes) return KEL_OK;
	if (L->staging) cudaFree(L->staging);
	L->staging = nullptr;
	L->staging_bytes = 0;
	KEL_CUDA(cudaMalloc(&L->staging, bytes));
	L->staging_bytes = bytes;
	return KEL_OK;
}

int kel::gb::ensure_field(kel_lattice *L, float **ptr, int64_t count, float init) {
	if (*ptr) return KEL_OK;
	KEL_CUDA(cudaMalloc(ptr, count * sizeof(float)));
	k_fill_f32<<<grid_for(count), 256, 0, L->stream>>>(*ptr, count, init);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

extern "C" int kel_lattice_create(const kel_lattice_desc *desc, kel_lattice **out) {
	if (!desc || !out) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_create: null argument");
	*out = nullptr;
	HostDesc d;
	if (!desc_for(desc->descriptor, d))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_create: unknown descriptor %d", desc->descriptor);
	if (desc->storage != KEL_STORAGE_FP32 && desc->storage != KEL_STORAGE_FP16S)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_create: unknown storage %d", desc->storage);
	if (desc->nx < 1 || desc->ny < 1 || desc->nz < 1 || desc->nx > (1 << 30) || desc->ny > (1 << 30) ||
		desc->nz > (1 << 30))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_create: bad extents %lld x %lld x %lld",
					(long long)desc->nx, (long long)desc->ny, (long long)desc->nz);
	if (d.D == 2 && desc->nz != 1) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_create: D2Q9 needs nz = 1");
	if ((desc->flags & KEL_LATTICE_PERIODIC_X) && (desc->nx % 4) != 0)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_create: periodic x needs nx %% 4 == 0");
	if (desc->flags & ~KEL_LATTICE_PERIODIC_X) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_create: unknown flags");

	kel_lattice *L = new kel_lattice();
	L->desc = *desc;
	L->d = d;
	// rows padded to 16 bytes (FP32: 4 cells, FP16S: 8 cells) so that every row
	// starts on a bulk-copy boundary; periodic rows are not padded (nxp == nx)
	const bool periodic = (desc->flags & KEL_LATTICE_PERIODIC_X) != 0;
	const int64_t pad = (desc->storage == KEL_STORAGE_FP16S && !periodic) ? 8 : 4;
	L->nxp = (int)((desc->nx + pad - 1) / pad * pad);
	L->nq = L->nxp / 4;
	L->wpr = (L->nq + 31) / 32;
	L->ncell = desc->nx * desc->ny * desc->nz;
	L->plane = (int64_t)L->nxp * desc->ny * desc->nz;
	L->elem = desc->storage == KEL_STORAGE_FP32 ? 4 : 2;
	cudaGetDevice(&L->device);
	cudaDeviceGetAttribute(&L->sms, cudaDevAttrMultiProcessorCount, L->device);
	if (L->sms < 1) L->sms = 1;
	for (int i = 0; i < 27; ++i) L->wshift[i] = 0.f;
	if (desc->storage == KEL_STORAGE_FP16S)
		for (int i = 0; i < d.Q; ++i) L->wshift[i] = __half2float(__float2half_rn((float)d.w[i]));

	auto cleanup = [&](int rc) {
		kel_lattice_destroy(L);
		return rc;
	};
	cudaError_t e;
	if ((e = cudaMalloc(&L->f, (size_t)d.Q * L->plane * L->elem)) != cudaSuccess ||
		// 64 bytes past the last row: the row pipeline widens its flag copies
		// to 16-byte boundaries
		(e = cudaMalloc(&L->flags, (size_t)L->plane + 64)) != cudaSuccess ||
		(e = cudaMalloc(&L->d_err, sizeof(unsigned))) != cudaSuccess ||
		(e = cudaMalloc(&L->rho, (size_t)L->plane * sizeof(float))) != cudaSuccess ||
		(e = cudaMalloc(&L->u, (size_t)d.D * L->plane * sizeof(float))) != cudaSuccess ||
		(e = cudaMalloc(&L->profile, (size_t)desc->ny * sizeof(float))) != cudaSuccess ||
		(e = cudaMalloc(&L->ops, sizeof(OpEntry) * MAX_FLAGS)) != cudaSuccess) {
		int rc = fail(e == cudaErrorMemoryAllocation ? KEL_ERR_OUT_OF_MEMORY : KEL_ERR_CUDA,
					  "kel_lattice_create: %s", cudaGetErrorString(e));
		return cleanup(rc);
	}
	// rest equilibrium f = w_i everywhere, flags 0, rho = 1, u = 0
	for (int i = 0; i < d.Q; ++i) {
		void *pl = static_cast<char *>(L->f) + (size_t)i * L->plane * L->elem;
		k_fill_pop<<<grid_for(L->plane), 256, 0, L->stream>>>(pl, L->plane, desc->storage, (float)d.w[i], L->wshift[i]);
	}
	k_fill_f32<<<grid_for(L->plane), 256, 0, L->stream>>>(L->rho, L->plane, 1.0f);
	k_fill_f32<<<grid_for(d.D * L->plane), 256, 0, L->stream>>>(L->u, d.D * L->plane, 0.0f);
	k_fill_f32<<<grid_for(desc->ny), 256, 0, L->stream>>>(L->profile, desc->ny, 0.0f);
	if ((e = cudaMemsetAsync(L->flags, 0, (size_t)L->plane + 64, L->stream)) != cudaSuccess ||
		(e = cudaMemsetAsync(L->d_err, 0, sizeof(unsigned), L->stream)) != cudaSuccess ||
		(e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(L->stream)) != cudaSuccess) {
		int rc = fail(KEL_ERR_CUDA, "kel_lattice_create: %s", cudaGetErrorString(e));
		return cleanup(rc);
	}
	*out = L;
	return KEL_OK;
}

extern "C" int kel_lattice_destroy(kel_lattice *L) {
	if (!L) return KEL_OK;
	if (L->stream) cudaStreamSynchronize(L->stream);
	else cudaDeviceSynchronize();
	cudaFree(L->f);
	cudaFree(L->flags);
	cudaFree(L->d_seen);
	cudaFree(L->d_err);
	cudaFree(L->hw_mask);
	if (L->graph) cudaGraphExecDestroy(L->graph);
	cudaFree(L->rho);
	cudaFree(L->u);
	cudaFree(L->por);
	cudaFree(L->force);
	cudaFree(L->hN);
	cudaFree(L->hD);
	cudaFree(L->profile);
	cudaFree(L->ops);
	cudaFree(L->staging);
	delete L;
	return KEL_OK;
}

extern "C" int kel_lattice_set_stream(kel_lattice *L, void *stream) {
	if (!L) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_set_stream: null lattice");
	L->stream = static_cast<cudaStream_t>(stream);
	return KEL_OK;
}

extern "C" int kel_lattice_time_step(const kel_lattice *L, uint64_t *t) {
	if (!L || !t) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_time_step: null argument");
	*t = L->t;
	return KEL_OK;
}

// After the lattice's stream has drained: did a row-pipeline sweep give up on
// a bounded wait?  The flag is cleared when reported.
static int check_sweep_error(kel_lattice *L, const char *who) {
	if (!L->rows_used) return KEL_OK;
	unsigned err = 0;
	KEL_CUDA(cudaMemcpyAsync(&err, L->d_err, sizeof(err), cudaMemcpyDeviceToHost, L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	if (err == 0) return KEL_OK;
	KEL_CUDA(cudaMemsetAsync(L->d_err, 0, sizeof(unsigned), L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	return fail(KEL_ERR_TIMEOUT, "%s: a row-pipeline sweep gave up waiting for its row copies; the populations are invalid",
				who);
}

extern "C" int kel_lattice_synchronize(kel_lattice *L) {
	if (!L) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_synchronize: null lattice");
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	return check_sweep_error(L, "kel_lattice_synchronize");
}

// ---------------------------------------------------------------------------
// flags

// Which flag values occur in the lattice's own cells (the row padding x >= nx
// is skipped): one bit per value, OR-ed per block in shared memory, then
// into `seen`.
__global__ void k_flag_presence(const uint8_t *flags, int64_t n, int nx, int nxp, unsigned *seen) {
	__shared__ unsigned blk[8];
	if (threadIdx.x < 8) blk[threadIdx.x] = 0u;
	__syncthreads();
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
		if ((int)(k % nxp) >= nx) continue;
		const unsigned v = flags[k];
		atomicOr(&blk[v >> 5], 1u << (v & 31));
	}
	__syncthreads();
	if (threadIdx.x < 8 && blk[threadIdx.x]) atomicOr(&seen[threadIdx.x], blk[threadIdx.x]);
}

extern "C" int kel_upload_flags(kel_lattice *L, const uint8_t *host) {
	if (!L || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_upload_flags: null argument");
	const auto &D = L->desc;
	KEL_CUDA(cudaMemcpy2DAsync(L->flags, (size_t)L->nxp, host, (size_t)D.nx, (size_t)D.nx, (size_t)(D.ny * D.nz),
							   cudaMemcpyHostToDevice, L->stream));
	if (!L->d_seen) KEL_CUDA(cudaMalloc(&L->d_seen, 8 * sizeof(unsigned)));
	KEL_CUDA(cudaMemsetAsync(L->d_seen, 0, 8 * sizeof(unsigned), L->stream));
	k_flag_presence<<<grid_for(L->plane), 256, 0, L->stream>>>(L->flags, L->plane, (int)D.nx, L->nxp, L->d_seen);
	KEL_CUDA(cudaGetLastError());
	unsigned seen[8];
	KEL_CUDA(cudaMemcpyAsync(seen, L->d_seen, sizeof(seen), cudaMemcpyDeviceToHost, L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	for (int fl = 0; fl < MAX_FLAGS; ++fl) L->present[fl] = (seen[fl >> 5] >> (fl & 31)) & 1u;
	L->have_ops = false; // re-validate the program against the new flag set
	return KEL_OK;
}

// ---------------------------------------------------------------------------
// populations: host AoS/SoA <-> AA lattice, parity aware

struct ConvArgs {
	void *f;
	void *buf;
	int64_t plane, ncell;
	int nx, ny, nz, nxp;
	int Q, D;
	int storage, dtype, layout;
	int odd, periodic;
	int c[27][3];
	int opp[27];
	float wshift[27];
};

__device__ __forceinline__ float ldpop(const ConvArgs &a, int64_t idx, int i) {
	if (a.storage == STORE_FP32) return static_cast<const float *>(a.f)[idx];
	return __half2float(static_cast<const __half *>(a.f)[idx]) + a.wshift[i];
}

__device__ __forceinline__ void stpop(const ConvArgs &a, int64_t idx, int i, float v) {
	if (a.storage == STORE_FP32) static_cast<float *>(a.f)[idx] = v;
	else static_cast<__half *>(a.f)[idx] = __float2half_rn(v - a.wshift[i]);
}

// Location in the AA lattice of the post-stream population f_i(x):
// even t: A[i][x]; odd t: A[opp i][x - c_i] (or nothing if that is outside).
__device__ __forceinline__ bool pop_slot(const ConvArgs &a, int x, int y, int z, int i, int64_t &idx) {
	if (!a.odd) {
		idx = (int64_t)i * a.plane + ((int64_t)z * a.ny + y) * a.nxp + x;
		return true;
	}
	int sx = x - a.c[i][0], sy = y - a.c[i][1], sz = z - a.c[i][2];
	if (a.periodic) sx = (sx + a.nx) % a.nx;
	if (sx < 0 || sx >= a.nxp || sy < 0 || sy >= a.ny || sz < 0 || sz >= a.nz) return false;
	idx = (int64_t)a.opp[i] * a.plane + ((int64_t)sz * a.ny + sy) * a.nxp + sx;
	return true;
}

__global__ void k_pop_convert(ConvArgs a, int upload) {
	const int64_t total = a.ncell * a.Q;
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
		int64_t c, i;
		if (a.layout == KEL_LAYOUT_AOS) {
			c = k / a.Q;
			i = k % a.Q;
		} else {
			i = k / a.ncell;
			c = k % a.ncell;
		}
		const int x = (int)(c % a.nx);
		const int y = (int)((c / a.nx) % a.ny);
		const int z = (int)(c / ((int64_t)a.nx * a.ny));
		int64_t idx;
		const bool ok = pop_slot(a, x, y, z, (int)i, idx);
		if (upload) {
			if (!ok) continue;
			float v = a.dtype == KEL_DTYPE_F32 ? static_cast<const float *>(a.buf)[k]
											   : (float)static_cast<const double *>(a.buf)[k];
			stpop(a, idx, (int)i, v);
		} else {
			float v = ok ? ldpop(a, idx, (int)i) : 0.f;
			if (a.dtype == KEL_DTYPE_F32) static_cast<float *>(a.buf)[k] = v;
			else static_cast<double *>(a.buf)[k] = (double)v;
		}
	}
}

// Host AoS (Q values per cell, cells x fastest) <-> lattice, one tile of
// CONV_TILE consecutive cells per block staged in shared memory as [cell][i]
// (Q odd: a stride-Q walk is free of bank conflicts), so that the host-side
// reads / writes and the per-plane lattice writes / reads are both coalesced.
constexpr int CONV_TILE = 256;

template <typename H>
__global__ void __launch_bounds__(CONV_TILE) k_pop_aos(ConvArgs a, int upload) {
	extern __shared__ float tile[];
	const int64_t c0 = (int64_t)blockIdx.x * CONV_TILE;
	const int n = (int)(a.ncell - c0 < CONV_TILE ? a.ncell - c0 : CONV_TILE);
	const int Q = a.Q;
	H *hb = static_cast<H *>(a.buf) + c0 * Q;
	const int64_t c = c0 + threadIdx.x;
	const int64_t row = c / a.nx;
	const int x = (int)(c - row * a.nx);
	const int y = (int)(row % a.ny);
	const int z = (int)(row / a.ny);
	if (upload) {
		for (int k = threadIdx.x; k < n * Q; k += CONV_TILE) tile[k] = (float)hb[k];
		__syncthreads();
		if (threadIdx.x < n)
			for (int i = 0; i < Q; ++i) {
				int64_t idx;
				if (pop_slot(a, x, y, z, i, idx)) stpop(a, idx, i, tile[threadIdx.x * Q + i]);
			}
	} else {
		if (threadIdx.x < n)
			for (int i = 0; i < Q; ++i) {
				int64_t idx;
				tile[threadIdx.x * Q + i] = pop_slot(a, x, y, z, i, idx) ? ldpop(a, idx, i) : 0.f;
			}
		__syncthreads();
		for (int k = threadIdx.x; k < n * Q; k += CONV_TILE) hb[k] = (H)tile[k];
	}
}

static void launch_pop_convert(const kel_lattice *L, const ConvArgs &a, int upload) {
	if (a.layout == KEL_LAYOUT_AOS) {
		const unsigned blocks = (unsigned)((a.ncell + CONV_TILE - 1) / CONV_TILE);
		const size_t sm = sizeof(float) * CONV_TILE * a.Q;
		if (a.dtype == KEL_DTYPE_F32) k_pop_aos<float><<<blocks, CONV_TILE, sm, L->stream>>>(a, upload);
		else k_pop_aos<double><<<blocks, CONV_TILE, sm, L->stream>>>(a, upload);
	} else {
		k_pop_convert<<<grid_for(a.ncell * a.Q), 256, 0, L->stream>>>(a, upload);
	}
}

// ---------------------------------------------------------------------------
// geometry and initial state on the device

// Flag painting: each op writes `flag` into the cells of its box (lo <= x < hi
// per axis) -- for a sphere only those with sum (x - c)^2 <= r^2, cell centres
// at integer coordinates -- applied in order, one cell per thread.
__global__ void k_paint(uint8_t *flags, int nx, int ny, int nz, int nxp, const kel_paint_op *ops, int n_ops) {
	const int64_t n = (int64_t)nx * ny * nz;
	for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
		const int x = (int)(c % nx);
		const int64_t r = c / nx;
		const int y = (int)(r % ny), z = (int)(r / ny);
		const int64_t pos[3] = {x, y, z};
		const int64_t at = r * nxp + x;
		uint8_t v = flags[at];
		for (int k = 0; k < n_ops; ++k) {
			const kel_paint_op &o = ops[k];
			bool in = true;
			for (int d = 0; d < 3; ++d) in = in && pos[d] >= o.lo[d] && pos[d] < o.hi[d];
			if (in && o.shape == KEL_PAINT_SPHERE) {
				double s2 = 0.0;
				for (int d = 0; d < 3; ++d) {
					const double dd = (double)pos[d] - o.center[d];
					s2 = s2 + dd * dd;
				}
				in = s2 <= o.radius * o.radius;
			}
			if (in) v = (uint8_t)o.flag;
		}
		flags[at] = v;
	}
}

// Populations f_i(x) = equilibrium(rho, u) with the reference's rounding
// (equilibrium.hpp:7-48), placed for the lattice's current time step; rho and
// u per cell from the fields (cells x fastest; u one plane per component) or
// the constants.
template <class L>
__global__ void k_init_equilibrium(ConvArgs a, const float *rho_f, const float *u_f, float rho0, float u0x, float u0y,
								   float u0z) {
	for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.ncell; c += (int64_t)gridDim.x * blockDim.x) {
		const int x = (int)(c % a.nx);
		const int64_t r = c / a.nx;
		const int y = (int)(r % a.ny), z = (int)(r / a.ny);
		const float rho = rho_f ? rho_f[c] : rho0;
		float u[3] = {u0x, u0y, u0z};
		if (u_f)
			for (int d = 0; d < L::D; ++d) u[d] = u_f[(int64_t)d * a.ncell + c];
		if (L::D == 2) u[2] = 0.f;
		float eq[L::Q];
		equilibrium<L, true>(rho, u, eq);
		for (int i = 0; i < L::Q; ++i) {
			int64_t idx;
			if (pop_slot(a, x, y, z, i, idx)) stpop(a, idx, i, eq[i]);
		}
	}
}

static ConvArgs conv_args(const kel_lattice *L, int dtype, int layout) {
	ConvArgs a;
	memset(&a, 0, sizeof(a));
	a.f = L->f;
	a.buf = L->staging;
	a.plane = L->plane;
	a.ncell = L->ncell;
	a.nx = (int)L->desc.nx;
	a.ny = (int)L->desc.ny;
	a.nz = (int)L->desc.nz;
	a.nxp = L->nxp;
	a.Q = L->d.Q;
	a.D = L->d.D;
	a.storage = L->desc.storage;
	a.dtype = dtype;
	a.layout = layout;
	a.odd = (int)(L->t & 1u);
	a.periodic = (L->desc.flags & KEL_LATTICE_PERIODIC_X) ? 1 : 0;
	for (int i = 0; i < L->d.Q; ++i) {
		for (int k = 0; k < 3; ++k) a.c[i][k] = L->d.c[i][k];
		a.opp[i] = L->d.opp[i];
		a.wshift[i] = L->wshift[i];
	}
	return a;
}

static int check_io(kel_lattice *L, const void *host, int32_t dtype, int32_t layout, const char *who) {
	if (!L || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: null argument", who);
	if (dtype != KEL_DTYPE_F32 && dtype != KEL_DTYPE_F64) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: bad dtype", who);
	if (layout != KEL_LAYOUT_AOS && layout != KEL_LAYOUT_SOA) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: bad layout", who);
	return KEL_OK;
}

// A page-locked host buffer the device can address directly (cudaHostAlloc /
// cudaHostRegister; with NVLink-C2C the GPU reads and writes it at several
// hundred GB/s): the conversion kernels then read or write it in place, with
// no staging copy.  Other host memory (pageable) goes through the staging
// buffer and one cudaMemcpyAsync.
static void *mapped_host(const void *host) {
	cudaPointerAttributes at;
	if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
		cudaGetLastError(); // an unregistered pointer is not an error here
		return nullptr;
	}
	return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

extern "C" int kel_upload_populations(kel_lattice *L, const void *host, int32_t dtype, int32_t layout) {
	int rc = check_io(L, host, dtype, layout, "kel_upload_populations");
	if (rc) return rc;
	const size_t bytes = (size_t)L->ncell * L->d.Q * (dtype == KEL_DTYPE_F32 ? 4 : 8);
	ConvArgs a = conv_args(L, dtype, layout);
	if (void *m = mapped_host(host)) {
		a.buf = m;
	} else {
		if ((rc = ensure_staging(L, bytes))) return rc;
		a.buf = L->staging;
		KEL_CUDA(cudaMemcpyAsync(L->staging, host, bytes, cudaMemcpyHostToDevice, L->stream));
	}
	launch_pop_convert(L, a, 1);
	KEL_CUDA(cudaGetLastError());
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	return KEL_OK;
}

extern "C" int kel_download_populations(kel_lattice *L, void *host, int32_t dtype, int32_t layout) {
	int rc = check_io(L, host, dtype, layout, "kel_download_populations");
	if (rc) return rc;
	const size_t bytes = (size_t)L->ncell * L->d.Q * (dtype == KEL_DTYPE_F32 ? 4 : 8);
	ConvArgs a = conv_args(L, dtype, layout);
	void *m = mapped_host(host);
	if (m) {
		a.buf = m;
	} else {
		if ((rc = ensure_staging(L, bytes))) return rc;
		a.buf = L->staging;
	}
	launch_pop_convert(L, a, 0);
	KEL_CUDA(cudaGetLastError());
	if (!m) KEL_CUDA(cudaMemcpyAsync(host, L->staging, bytes, cudaMemcpyDeviceToHost, L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	return check_sweep_error(L, "kel_download_populations");
}

extern "C" int kel_lattice_paint(kel_lattice *L, const kel_paint_op *ops, int32_t n_ops) {
	if (!L || !ops || n_ops < 1 || n_ops > 4096)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_paint: bad arguments");
	for (int k = 0; k < n_ops; ++k) {
		if (ops[k].shape != KEL_PAINT_BOX && ops[k].shape != KEL_PAINT_SPHERE)
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_paint: op %d: unknown shape %d", k, ops[k].shape);
		if (ops[k].flag < 0 || ops[k].flag > 255)
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_paint: op %d: flag %d outside 0..255", k, ops[k].flag);
	}
	kel_paint_op *d_ops = nullptr;
	KEL_CUDA(cudaMalloc(&d_ops, sizeof(kel_paint_op) * n_ops));
	cudaError_t e = cudaMemcpyAsync(d_ops, ops, sizeof(kel_paint_op) * n_ops, cudaMemcpyHostToDevice, L->stream);
	if (e == cudaSuccess) {
		k_paint<<<grid_for(L->ncell), 256, 0, L->stream>>>(L->flags, (int)L->desc.nx, (int)L->desc.ny,
														   (int)L->desc.nz, L->nxp, d_ops, n_ops);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
	cudaFree(d_ops);
	if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_lattice_paint: %s", cudaGetErrorString(e));
	// the program is validated against the flags present: rescan them
	if (!L->d_seen) KEL_CUDA(cudaMalloc(&L->d_seen, 8 * sizeof(unsigned)));
	KEL_CUDA(cudaMemsetAsync(L->d_seen, 0, 8 * sizeof(unsigned), L->stream));
	k_flag_presence<<<grid_for(L->plane), 256, 0, L->stream>>>(L->flags, L->plane, (int)L->desc.nx, L->nxp, L->d_seen);
	KEL_CUDA(cudaGetLastError());
	unsigned seen[8];
	KEL_CUDA(cudaMemcpyAsync(seen, L->d_seen, sizeof(seen), cudaMemcpyDeviceToHost, L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	for (int fl = 0; fl < MAX_FLAGS; ++fl) L->present[fl] = (seen[fl >> 5] >> (fl & 31)) & 1u;
	L->have_ops = false;
	return KEL_OK;
}

extern "C" int kel_download_flags(kel_lattice *L, uint8_t *host) {
	if (!L || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_download_flags: null argument");
	const auto &D = L->desc;
	KEL_CUDA(cudaMemcpy2DAsync(host, (size_t)D.nx, L->flags, (size_t)L->nxp, (size_t)D.nx, (size_t)(D.ny * D.nz),
							   cudaMemcpyDeviceToHost, L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	return KEL_OK;
}

extern "C" int kel_lattice_init_equilibrium(kel_lattice *L, const float *d_rho, const float *d_u, double rho0,
											const double *u0) {
	if (!L) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_init_equilibrium: null lattice");
	const double z[3] = {0.0, 0.0, 0.0};
	const double *u = u0 ? u0 : z;
	const ConvArgs a = conv_args(L, KEL_DTYPE_F32, KEL_LAYOUT_AOS);
	const unsigned g = grid_for(L->ncell);
	switch (L->d.Q) {
	case 9:
		k_init_equilibrium<D2Q9><<<g, 256, 0, L->stream>>>(a, d_rho, d_u, (float)rho0, (float)u[0], (float)u[1], 0.f);
		break;
	case 19:
		k_init_equilibrium<D3Q19><<<g, 256, 0, L->stream>>>(a, d_rho, d_u, (float)rho0, (float)u[0], (float)u[1],
															(float)u[2]);
		break;
	default:
		k_init_equilibrium<D3Q27><<<g, 256, 0, L->stream>>>(a, d_rho, d_u, (float)rho0, (float)u[0], (float)u[1],
															(float)u[2]);
		break;
	}
	KEL_CUDA(cudaGetLastError());
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	return KEL_OK;
}

// ---------------------------------------------------------------------------
// macros and per-cell fields: padded plane layout <-> host AoS

// Padded planes (comps of them) <-> host AoS (comps values per cell), one
// tile of CONV_TILE cells per block staged in shared memory as [cell][d].
__global__ void __launch_bounds__(CONV_TILE) k_field_io(float *dev, float *buf, int64_t plane, int64_t ncell, int nx,
														 int nxp, int comps, int upload) {
	__shared__ float tile[CONV_TILE * 3];
	const int64_t c0 = (int64_t)blockIdx.x * CONV_TILE;
	const int n = (int)(ncell - c0 < CONV_TILE ? ncell - c0 : CONV_TILE);
	float *hb = buf + c0 * comps;
	const int64_t c = c0 + threadIdx.x;
	const int64_t row = c / nx;
	const int64_t idx = row * nxp + (c - row * nx);
	if (upload) {
		for (int k = threadIdx.x; k < n * comps; k += CONV_TILE) tile[k] = hb[k];
		__syncthreads();
		if (threadIdx.x < n)
			for (int d = 0; d < comps; ++d) dev[d * plane + idx] = tile[threadIdx.x * comps + d];
	} else {
		if (threadIdx.x < n)
			for (int d = 0; d < comps; ++d) tile[threadIdx.x * comps + d] = dev[d * plane + idx];
		__syncthreads();
		for (int k = threadIdx.x; k < n * comps; k += CONV_TILE) hb[k] = tile[k];
	}
}

static int field_io(kel_lattice *L, float *dev, float *host_out, const float *host_in, int comps) {
	const size_t bytes = (size_t)L->ncell * comps * sizeof(float);
	if (comps < 1 || comps > 3) return fail(KEL_ERR_INVALID_ARGUMENT, "field_io: %d components", comps);
	// page-locked host buffers are read / written in place (mapped_host)
	float *buf = static_cast<float *>(mapped_host(host_in ? static_cast<const void *>(host_in) : host_out));
	const bool staged = buf == nullptr;
	if (staged) {
		int rc = ensure_staging(L, bytes);
		if (rc) return rc;
		buf = static_cast<float *>(L->staging);
		if (host_in) KEL_CUDA(cudaMemcpyAsync(buf, host_in, bytes, cudaMemcpyHostToDevice, L->stream));
	}
	k_field_io<<<(unsigned)((L->ncell + CONV_TILE - 1) / CONV_TILE), CONV_TILE, 0, L->stream>>>(
		dev, buf, L->plane, L->ncell, (int)L->desc.nx, L->nxp, comps, host_in ? 1 : 0);
	KEL_CUDA(cudaGetLastError());
	if (host_out && staged) KEL_CUDA(cudaMemcpyAsync(host_out, buf, bytes, cudaMemcpyDeviceToHost, L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	return KEL_OK;
}

int kel::gb::field_to_host(kel_lattice *L, const float *dev, float *host, int comps) {
	return field_io(L, const_cast<float *>(dev), host, nullptr, comps);
}

extern "C" int kel_download_macros(kel_lattice *L, float *host_rho, float *host_u) {
	if (!L || (!host_rho && !host_u)) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_download_macros: null argument");
	int rc;
	if (host_rho && (rc = field_io(L, L->rho, host_rho, nullptr, 1))) return rc;
	if (host_u && (rc = field_io(L, L->u, host_u, nullptr, L->d.D))) return rc;
	return check_sweep_error(L, "kel_download_macros");
}

extern "C" int kel_upload_field(kel_lattice *L, int32_t field, const float *host) {
	if (!L || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_upload_field: null argument");
	int rc;
	if (field == KEL_FIELD_POROSITY) {
		if ((rc = ensure_field(L, &L->por, L->plane, 1.0f))) return rc;
		++L->por_epoch;
		return field_io(L, L->por, nullptr, host, 1);
	}
	if (field == KEL_FIELD_FORCE) {
		if ((rc = ensure_field(L, &L->force, L->plane * L->d.D, 0.0f))) return rc;
		return field_io(L, L->force, nullptr, host, L->d.D);
	}
	if (field == KEL_FIELD_HLBM_N) {
		if ((rc = ensure_field(L, &L->hN, L->plane * L->d.D, 0.0f))) return rc;
		return field_io(L, L->hN, nullptr, host, L->d.D);
	}
	if (field == KEL_FIELD_HLBM_D) {
		if ((rc = ensure_field(L, &L->hD, L->plane, 0.0f))) return rc;
		return field_io(L, L->hD, nullptr, host, 1);
	}
	return fail(KEL_ERR_INVALID_ARGUMENT, "kel_upload_field: unknown field %d", field);
}

extern "C" int kel_download_field(kel_lattice *L, int32_t field, float *host) {
	if (!L || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_download_field: null argument");
	int rc;
	if (field == KEL_FIELD_POROSITY) {
		if ((rc = ensure_field(L, &L->por, L->plane, 1.0f))) return rc;
		return field_io(L, L->por, host, nullptr, 1);
	}
	if (field == KEL_FIELD_FORCE) {
		if ((rc = ensure_field(L, &L->force, L->plane * L->d.D, 0.0f))) return rc;
		return field_io(L, L->force, host, nullptr, L->d.D);
	}
	if (field == KEL_FIELD_HLBM_N) {
		if ((rc = ensure_field(L, &L->hN, L->plane * L->d.D, 0.0f))) return rc;
		return field_io(L, L->hN, host, nullptr, L->d.D);
	}
	if (field == KEL_FIELD_HLBM_D) {
		if ((rc = ensure_field(L, &L->hD, L->plane, 0.0f))) return rc;
		return field_io(L, L->hD, host, nullptr, 1);
	}
	return fail(KEL_ERR_INVALID_ARGUMENT, "kel_download_field: unknown field %d", field);
}

extern "C" int kel_upload_inlet_profile(kel_lattice *L, const double *host_ux, int64_t n) {
	if (!L || !host_ux) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_upload_inlet_profile: null argument");
	if (n != L->desc.ny) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_upload_inlet_profile: need ny = %lld values",
									 (long long)L->desc.ny);
	std::vector<float> v(n);
	for (int64_t i = 0; i < n; ++i) v[i] = (float)host_ux[i];
	KEL_CUDA(cudaMemcpyAsync(L->profile, v.data(), n * sizeof(float), cudaMemcpyHostToDevice, L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	return KEL_OK;
}

// ---------------------------------------------------------------------------
// program lowering and stepping

static int lower_program(kel_lattice *L, const kel_step_program *P, OpEntry *ops) {
	const HostDesc &d = L->d;
	if (P->collision < KEL_COLL_BGK || P->collision > KEL_COLL_FPLBM)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_step: unknown collision %d", P->collision);
	if (P->collision == KEL_COLL_FPLBM) {
		if (d.Q != 9) return fail(KEL_ERR_UNSUPPORTED, "kel_step: the FPLBM collision is D2Q9 only");
		if (P->global_force[0] != 0.0 || P->global_force[1] != 0.0 || P->global_force[2] != 0.0)
			return fail(KEL_ERR_INVALID_ARGUMENT,
						"kel_step: the FPLBM collision takes no global force (fplbm.hpp:57-128; gravity acts on "
						"the bodies)");
	}
	if (P->collision == KEL_COLL_HLBM && d.Q != 9)
		return fail(KEL_ERR_UNSUPPORTED, "kel_step: the HLBM collision is D2Q9 only");
	if (P->arithmetic == KEL_ARITH_SHIFTED)
		return fail(KEL_ERR_UNSUPPORTED, "kel_step: shifted arithmetic is implemented for batches only");
	if (P->arithmetic != KEL_ARITH_FAST && P->arithmetic != KEL_ARITH_REFERENCE)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_step: unknown arithmetic mode %d", P->arithmetic);
	if (P->arithmetic == KEL_ARITH_REFERENCE && L->desc.storage != KEL_STORAGE_FP32)
		return fail(KEL_ERR_UNSUPPORTED, "kel_step: reference arithmetic needs FP32 storage");
	if (!(P->tau > 0.0)) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_step: tau must be positive");
	memset(ops, 0, sizeof(OpEntry) * MAX_FLAGS);
	for (int fl = 0; fl < MAX_FLAGS; ++fl) {
		const kel_flag_op &o = P->ops[fl];
		OpEntry &e = ops[fl];
		if (o.bc < KEL_BC_NONE || o.bc > KEL_BC_HALFWAY_WALL)
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_step: flag %d: unknown boundary op %d", fl, o.bc);
		// A boundary the descriptor has no reference specialisation for is an
		// error only where a cell carries that flag.
		const bool used = L->present[fl] != 0;
		if (used && o.bc == KEL_BC_ZOUHE_VELOCITY_X && d.Q != 9)
			return fail(KEL_ERR_UNSUPPORTED, "kel_step: ZouHeVelocityX exists only for D2Q9 (boundary.hpp:759)");
		if (used && o.bc == KEL_BC_ZOUHE_PRESSURE_X && d.Q == 19)
			return fail(KEL_ERR_UNSUPPORTED, "kel_step: ZouHePressureX has no D3Q19 specialisation");
		if (used && o.bc == KEL_BC_ANTI_BOUNCE_BACK && d.Q != 9)
			return fail(KEL_ERR_UNSUPPORTED, "kel_step: AntiBounceBack is D2Q9 only (boundary.hpp:117)");
		e.bc = used ? o.bc : KEL_BC_NONE;
		e.collide = o.collide && o.bc != KEL_BC_HALFWAY_WALL ? 1 : 0; // a half-way wall is solid
		if (P->collision == KEL_COLL_FPLBM && e.collide) { // the FPLBM drivers' cases
			const bool plain_op = e.bc == KEL_BC_NONE || e.bc == KEL_BC_FLUID;
			e.bgk_only = plain_op ? 0 : 1;
			e.no_macros = plain_op ? 1 : 0;
		}
		e.east = o.east ? 1 : 0;
		e.use_profile = o.use_profile ? 1 : 0;
		e.rho = (float)o.rho;
		for (int k = 0; k < 3; ++k) e.u[k] = (float)o.u[k];
		// moving wall, cavity_2d_gpu.cpp:224-233, e.u summed over all axes in double
		for (int i = 0; i < d.Q; ++i) {
			double edu = 0.0;
			for (int k = 0; k < d.D; ++k) edu = edu + (double)(float)d.c[i][k] * o.u[k];
			e.lid[i] = (float)(2.0 * (double)(float)d.w[i] * (double)3.0f * edu);
		}
		float uf[3] = {(float)o.u[0], (float)o.u[1], (float)o.u[2]};
		host_equilibrium(d, (float)o.rho, uf, e.eq);
	}
	return KEL_OK;
}

// Half-way walls: per cell, bit i set where the neighbour x + c_i is a cell
// whose flag has the half-way wall op (periodic rows wrap); zero for wall
// cells, flag-0 cells and cells with no wall neighbour.
template <class Lc>
__global__ void k_hw_mask(const uint8_t *flags, unsigned hw_flags, int nxp, int ny, int nz, int periodic, int64_t plane,
						  uint32_t *mask) {
	for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < plane; c += (int64_t)gridDim.x * blockDim.x) {
		const int x = (int)(c % nxp);
		const int64_t r = c / nxp;
		const int y = (int)(r % ny), z = (int)(r / ny);
		const unsigned f = flags[c];
		uint32_t m = 0;
		if (f != 0u && !(f < MAX_FLAGS && ((hw_flags >> f) & 1u))) {
#pragma unroll
			for (int i = 1; i < Lc::Q; ++i) {
				int nx = x + Lc::cx(i);
				const int ny2 = y + Lc::cy(i), nz2 = z + Lc::cz(i);
				if (periodic) nx = nx < 0 ? nx + nxp : (nx >= nxp ? nx - nxp : nx);
				if (nx < 0 || nx >= nxp || ny2 < 0 || ny2 >= ny || nz2 < 0 || nz2 >= nz) continue;
				const unsigned g = flags[((int64_t)nz2 * ny + ny2) * nxp + nx];
				if (g < MAX_FLAGS && ((hw_flags >> g) & 1u)) m |= 1u << i;
			}
		}
		mask[c] = m;
	}
}

// After a program is lowered: the half-way wall mask, when a flag present in
// the lattice has the op (else the sweeps run without it).
static int update_halfway(kel_lattice *L, const kel_step_program *P) {
	unsigned hw = 0;
	for (int fl = 1; fl < MAX_FLAGS; ++fl)
		if (P->ops[fl].bc == KEL_BC_HALFWAY_WALL && L->present[fl]) hw |= 1u << fl;
	L->hw_active = hw != 0;
	if (!hw) return KEL_OK;
	if (!L->hw_mask) KEL_CUDA(cudaMalloc(&L->hw_mask, sizeof(uint32_t) * (size_t)L->plane));
	const int periodic = (L->desc.flags & KEL_LATTICE_PERIODIC_X) ? 1 : 0;
	const int ny = (int)L->desc.ny, nz = (int)L->desc.nz;
	switch (L->d.Q) {
	case 9: k_hw_mask<D2Q9><<<grid_for(L->plane), 256, 0, L->stream>>>(L->flags, hw, L->nxp, ny, nz, periodic, L->plane, L->hw_mask); break;
	case 19: k_hw_mask<D3Q19><<<grid_for(L->plane), 256, 0, L->stream>>>(L->flags, hw, L->nxp, ny, nz, periodic, L->plane, L->hw_mask); break;
	default: k_hw_mask<D3Q27><<<grid_for(L->plane), 256, 0, L->stream>>>(L->flags, hw, L->nxp, ny, nz, periodic, L->plane, L->hw_mask); break;
	}
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

static cudaError_t launch_one(const kel_lattice *L, const SweepParams &p, int coll, bool exact, bool odd) {
	if (coll == KEL_COLL_FPLBM) coll = COLL_BGK_GUO; // with the per-op FPLBM switches of lower_program
	switch (L->d.Q) {
	case 9: return launch_sweep<D2Q9>(p, L->desc.storage, odd, coll, exact, L->stream);
	case 19: return launch_sweep<D3Q19>(p, L->desc.storage, odd, coll, exact, L->stream);
	default: return launch_sweep<D3Q27>(p, L->desc.storage, odd, coll, exact, L->stream);
	}
}

static bool launch_ok(const kel_lattice *L, int cpt, int block) {
	if (cpt == CPT_ROWS) { // row pipeline: block = row stages
		if (block < 2 || block > ROWS_MAX_STAGES) return false;
		if (L->nxp > ROWS_MAX_NXP || ((int64_t)L->nxp * (int64_t)L->elem) % 16 != 0) return false;
		int optin = 0;
		if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, L->device) != cudaSuccess) return false;
		return rows_smem_bytes(L->d.Q, L->nxp, (int)L->elem, block) <= optin;
	}
	if (cpt != 1 && cpt != 2 && cpt != 4) return false;
	if (block != 64 && block != 128 && block != 256) return false;
	if (cpt == 1 && (L->desc.ny > 65535 || L->desc.nz > 65535)) return false;
	return true;
}

extern "C" int kel_lattice_set_launch(kel_lattice *L, int32_t cells_per_thread, int32_t block_threads) {
	if (!L) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_set_launch: null lattice");
	if (!launch_ok(L, cells_per_thread, block_threads))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_set_launch: unsupported launch %d cells x %d threads",
					cells_per_thread, block_threads);
	L->cpt = cells_per_thread;
	L->block = block_threads;
	L->tuned = true;
	return KEL_OK;
}

extern "C" int kel_lattice_get_launch(const kel_lattice *L, int32_t *cells_per_thread, int32_t *block_threads) {
	if (!L || !cells_per_thread || !block_threads) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_get_launch: null");
	*cells_per_thread = L->cpt;
	*block_threads = L->block;
	return KEL_OK;
}

// The per-cell fields a collision reads, allocated on first use: porosity
// (1 = fluid), force (0), and for HLBM particle_N / particle_D (0).
static int ensure_collision_fields(kel_lattice *L, int coll) {
	int rc;
	const bool por = coll == KEL_COLL_PSM || coll == KEL_COLL_PSM_GUO || coll == KEL_COLL_HLBM || coll == KEL_COLL_FPLBM;
	const bool guo = coll == KEL_COLL_BGK_GUO || coll == KEL_COLL_PSM_GUO || coll == KEL_COLL_FPLBM;
	if (por && (rc = ensure_field(L, &L->por, L->plane, 1.0f))) return rc;
	if (guo && (rc = ensure_field(L, &L->force, L->plane * L->d.D, 0.0f))) return rc;
	if (coll == KEL_COLL_HLBM) {
		if ((rc = ensure_field(L, &L->hN, L->plane * L->d.D, 0.0f))) return rc;
		if ((rc = ensure_field(L, &L->hD, L->plane, 0.0f))) return rc;
	}
	return KEL_OK;
}

static SweepParams make_params(kel_lattice *L, const kel_step_program *P) {
	SweepParams p;
	memset(&p, 0, sizeof(p));
	p.f = L->f;
	p.plane = L->plane;
	p.flags = L->flags;
	p.rho = L->rho;
	p.u = L->u;
	p.por = L->por;
	p.force = L->force;
	p.hN = L->hN;
	p.hD = L->hD;
	p.profile = L->profile;
	p.ops = L->ops;
	p.nxp = L->nxp;
	p.ny = (int)L->desc.ny;
	p.nz = (int)L->desc.nz;
	p.nq = L->nq;
	p.wpr = L->wpr;
	p.wpr2 = (L->nxp / 2 + 31) / 32;
	p.periodic = (L->desc.flags & KEL_LATTICE_PERIODIC_X) ? 1 : 0;
	const float tau = (float)P->tau;
	p.omega = 1.0f / tau;
	p.guo_scale = 1.0f - 0.5f * p.omega;
	for (int k = 0; k < 3; ++k) p.g[k] = (float)P->global_force[k];
	for (int i = 0; i < 27; ++i) p.wshift[i] = L->wshift[i];
	p.cpt = L->cpt;
	p.idx32 = (int64_t)L->d.Q * L->plane < ((int64_t)1 << 31) ? 1 : 0;
	p.block = L->block;
	p.hw_mask = L->hw_active ? L->hw_mask : nullptr;
	p.plain = L->plain_flags;
	p.stages = L->cpt == CPT_ROWS ? L->block : 0;
	p.sms = L->sms;
	p.err = L->d_err;
	if (L->cpt == CPT_ROWS) L->rows_used = true;
	// one-cell sweep: prefetch the rows of the block one resident wave later
	// (32 warps per SM at most: 1024 / block blocks on each SM); measured at
	// 256^3: D3Q19 FP32 0.92 -> 0.97 of HBM, FP16S 0.50 -> 0.55, D3Q27 FP32
	// 0.88 -> 0.95; two or three waves ahead gained less
	p.pf_ahead = L->sms * (1024 / (L->block > 0 ? L->block : 256));
	return p;
}

namespace kel {
namespace gb {
SweepParams sweep_params(kel_lattice *L, const kel_step_program *P) { return make_params(L, P); }
} // namespace gb
} // namespace kel

// Time every supported launch shape on the lattice's own state, then put the
// state back: the populations are saved to a scratch copy first and restored
// after each trial, macros are not written, the time step does not move.
extern "C" int kel_lattice_autotune(kel_lattice *L, const kel_step_program *P, int32_t steps, int32_t *cells_per_thread,
									int32_t *block_threads, float *ms_per_step) {
	if (!L || !P || steps < 2) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_autotune: bad arguments");
	int rc;
	if ((rc = kel_step(L, P, 0, 0))) return rc; // validates and uploads the program
	if ((rc = ensure_collision_fields(L, P->collision))) return rc;
	const size_t bytes = (size_t)L->d.Q * L->plane * L->elem;
	void *save = nullptr;
	KEL_CUDA(cudaMalloc(&save, bytes));
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	const int cands[][2] = {{1, 64},  {1, 128}, {1, 256}, {2, 64},        {2, 128},       {2, 256},
	                        {4, 64},  {4, 128}, {4, 256}, {CPT_ROWS, 3}, {CPT_ROWS, 4}, {CPT_ROWS, 6}};
	const int ncand = (int)(sizeof(cands) / sizeof(cands[0]));
	float best = 1e30f;
	int bc = L->cpt, bb = L->block;
	cudaError_t e = cudaMemcpyAsync(save, L->f, bytes, cudaMemcpyDeviceToDevice, L->stream);
	SweepParams p = make_params(L, P);
	p.write_macros = 0;
	const bool exact = P->arithmetic == KEL_ARITH_REFERENCE;
	for (int k = 0; k < ncand && e == cudaSuccess; ++k) {
		if (!launch_ok(L, cands[k][0], cands[k][1])) continue;
		p.cpt = cands[k][0];
		p.block = cands[k][1];
		p.stages = p.cpt == CPT_ROWS ? p.block : 0;
		if (p.cpt == CPT_ROWS) L->rows_used = true;
		const bool odd0 = (L->t & 1u) != 0;
		for (int s = 0; s < 2 && e == cudaSuccess; ++s) e = launch_one(L, p, P->collision, exact, odd0 != (s & 1));
		cudaEventRecord(e0, L->stream);
		for (int s = 0; s < steps && e == cudaSuccess; ++s) e = launch_one(L, p, P->collision, exact, odd0 != (s & 1));
		cudaEventRecord(e1, L->stream);
		if (e == cudaSuccess) e = cudaEventSynchronize(e1);
		float ms = 0.f;
		cudaEventElapsedTime(&ms, e0, e1);
		ms /= steps;
		if (ms < best) {
			best = ms;
			bc = cands[k][0];
			bb = cands[k][1];
		}
		if (e == cudaSuccess) e = cudaMemcpyAsync(L->f, save, bytes, cudaMemcpyDeviceToDevice, L->stream);
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(save);
	if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_lattice_autotune: %s", cudaGetErrorString(e));
	if ((rc = check_sweep_error(L, "kel_lattice_autotune"))) return rc;
	L->cpt = bc;
	L->block = bb;
	L->tuned = true;
	if (cells_per_thread) *cells_per_thread = bc;
	if (block_threads) *block_threads = bb;
	if (ms_per_step) *ms_per_step = best;
	return KEL_OK;
}

constexpr int GRAPH_STEPS = 64;

// The captured graph of GRAPH_STEPS sweeps from an even step, for launch
// parameters p (compared bit for bit with those of the cached graph; a
// change re-captures).  A failed capture leaves the caller on plain launches.
static int ensure_step_graph(kel_lattice *L, const SweepParams &p, int coll, bool exact) {
	if (L->graph && L->graph_coll == coll && L->graph_exact == exact && memcmp(&L->graph_params, &p, sizeof(p)) == 0)
		return KEL_OK;
	if (L->graph) cudaGraphExecDestroy(L->graph);
	L->graph = nullptr;
	cudaGraph_t g = nullptr;
	if (cudaStreamBeginCapture(L->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
		cudaGetLastError();
		return KEL_ERR_CUDA;
	}
	cudaError_t e = cudaSuccess;
	for (int k = 0; k < GRAPH_STEPS && e == cudaSuccess; ++k) e = launch_one(L, p, coll, exact, (k & 1) != 0);
	cudaError_t e2 = cudaStreamEndCapture(L->stream, &g);
	if (e == cudaSuccess && e2 == cudaSuccess && g) e = cudaGraphInstantiate(&L->graph, g, 0);
	else if (e == cudaSuccess) e = e2;
	if (g) cudaGraphDestroy(g);
	if (e != cudaSuccess || !L->graph) {
		cudaGetLastError();
		L->graph = nullptr;
		return KEL_ERR_CUDA;
	}
	L->graph_params = p;
	L->graph_coll = coll;
	L->graph_exact = exact;
	return KEL_OK;
}

extern "C" int kel_step(kel_lattice *L, const kel_step_program *P, uint64_t n_steps, uint32_t step_flags) {
	if (!L || !P) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_step: null argument");
	if (step_flags & ~(KEL_STEP_WRITE_MACROS | KEL_STEP_ALL_MACROS))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_step: unknown step flags");
	int rc;
	// A caller may capture its own loop of kel_step calls into a graph.  Then
	// kel_step must neither synchronise nor capture a graph of its own (both
	// are illegal on a capturing stream): the launches go into the caller's
	// graph one by one, and the program must have been uploaded before.
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	if (L->stream != nullptr) KEL_CUDA(cudaStreamIsCapturing(L->stream, &cap));
	const bool capturing = cap != cudaStreamCaptureStatusNone;
	if (!L->have_ops || memcmp(&L->last_prog, P, sizeof(*P)) != 0) {
		if (capturing)
			return fail(KEL_ERR_INVALID_ARGUMENT,
						"kel_step: a new step program during stream capture; call kel_step with this program once "
						"before capturing");
		OpEntry ops[MAX_FLAGS];
		if ((rc = lower_program(L, P, ops))) return rc;
		uint32_t plain = 0;
		for (int fl = 1; fl < MAX_FLAGS; ++fl)
			if ((ops[fl].bc == KEL_BC_NONE || ops[fl].bc == KEL_BC_FLUID) && ops[fl].collide && !ops[fl].no_macros)
				plain |= 1u << fl;
		L->plain_flags = plain;
		uint32_t fp = 0;
		for (int fl = 1; fl < MAX_FLAGS; ++fl)
			if ((ops[fl].bc == KEL_BC_NONE || ops[fl].bc == KEL_BC_FLUID) && ops[fl].collide) fp |= 1u << fl;
		L->plain_flags_fplbm = fp;
		KEL_CUDA(cudaMemcpyAsync(L->ops, ops, sizeof(ops), cudaMemcpyHostToDevice, L->stream));
		if ((rc = update_halfway(L, P))) return rc;
		KEL_CUDA(cudaStreamSynchronize(L->stream));
		L->last_prog = *P;
		L->have_ops = true;
	}
	if ((rc = ensure_collision_fields(L, P->collision))) return rc;

	SweepParams p = make_params(L, P);
	const bool exact = P->arithmetic == KEL_ARITH_REFERENCE;
	uint64_t s = 0;
	// Long runs without macro output replay a captured graph of GRAPH_STEPS
	// sweeps (starting at an even step): one launch per block of steps
	// instead of one per step, which is what bounds small lattices.
	const uint64_t plain = (step_flags & KEL_STEP_ALL_MACROS)
							   ? 0
							   : ((step_flags & KEL_STEP_WRITE_MACROS) && n_steps > 0 ? n_steps - 1 : n_steps);
	if (L->stream != nullptr && !capturing && L->cpt != CPT_ROWS && plain >= 2 * GRAPH_STEPS) {
		p.write_macros = 0;
		for (; (L->t & 1u) && s < plain; ++s, ++L->t) {
			cudaError_t e = launch_one(L, p, P->collision, exact, true);
			if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_step: launch failed: %s", cudaGetErrorString(e));
		}
		const uint64_t reps = (plain - s) / GRAPH_STEPS;
		if (reps > 0 && ensure_step_graph(L, p, P->collision, exact) == KEL_OK) {
			for (uint64_t r = 0; r < reps; ++r) {
				cudaError_t e = cudaGraphLaunch(L->graph, L->stream);
				if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_step: graph launch failed: %s", cudaGetErrorString(e));
			}
			s += reps * GRAPH_STEPS;
			L->t += reps * GRAPH_STEPS;
		}
	}
	for (; s < n_steps; ++s) {
		p.write_macros = (step_flags & KEL_STEP_ALL_MACROS) || ((step_flags & KEL_STEP_WRITE_MACROS) && s + 1 == n_steps);
		const bool odd = (L->t & 1u) != 0;
		cudaError_t e = launch_one(L, p, P->collision, exact, odd);
		if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_step: launch failed: %s", cudaGetErrorString(e));
		L->t += 1;
	}
	return KEL_OK;
}
