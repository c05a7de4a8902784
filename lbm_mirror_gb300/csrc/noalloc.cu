// Convergence residual that allocates nothing (kel_velocity_residual_noalloc).
//
// Same computation as the per-channel residual of the batched runner
// (batch.cu: k_batch_residual_partial / k_batch_residual_final): FP64 sums of
// |u - u_prev|^2 and |u|^2 per tile of 256 cells into a scratch array of
// partial sums, then one fixed-order reduction of the partials.  Here the
// scratch is not allocated per call: it is the file-scope device array below,
// which every GPU that loads this library holds until the process exits.
//
// Who needs this: a caller that may not allocate device memory while it runs.
// cudaMalloc/cudaFree synchronise the device and can fail once a pooling
// allocator (a framework's caching allocator, a pre-reserved memory budget)
// has claimed the memory, so a host loop that checks convergence every few
// hundred steps between its own kernels -- or code that manages all device
// memory through its own pool -- cannot afford either.  The caller passes the
// inputs and the output; this entry point adds nothing to the device heap.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "lattice_internal.cuh"

using namespace kel::gb;

namespace {

constexpr int NA_TILE = 256;
constexpr int NA_MAX_TILES = 65536; // => at most 16,777,216 cells per call

// Scratch: one (sum |du|^2, sum |u|^2) pair per tile.  Every call overwrites
// the first ceil(n / 256) entries before reading them, so nothing has to start
// at zero; calls whose kernels overlap on the GPU share these entries and race.
__device__ __align__(256) double2 g_noalloc_partials[NA_MAX_TILES];

__global__ void __launch_bounds__(NA_TILE) na_partial(const float *u, const float *u_prev, int64_t n, int comps,
													  double2 *partial) {
	__shared__ double sh[2][NA_TILE / 32];
	const int64_t c = (int64_t)blockIdx.x * NA_TILE + threadIdx.x;
	double num = 0.0, den = 0.0;
	if (c < n) {
		for (int d = 0; d < comps; ++d) {
			const double a = u[d * n + c], b = u_prev[d * n + c];
			num += (a - b) * (a - b);
			den += a * a;
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
		for (int w = 0; w < NA_TILE / 32; ++w) {
			a += sh[0][w];
			b += sh[1][w];
		}
		partial[blockIdx.x] = make_double2(a, b);
	}
}

// One block: each thread sums a fixed stride of tiles, then a fixed tree.
__global__ void __launch_bounds__(1024) na_final(const double2 *partial, int tiles, double *result) {
	__shared__ double sa[1024], sb[1024];
	double a = 0.0, b = 0.0;
	for (int k = threadIdx.x; k < tiles; k += 1024) {
		a += partial[k].x;
		b += partial[k].y;
	}
	sa[threadIdx.x] = a;
	sb[threadIdx.x] = b;
	__syncthreads();
	for (int o = 512; o > 0; o >>= 1) {
		if (threadIdx.x < o) {
			sa[threadIdx.x] += sa[threadIdx.x + o];
			sb[threadIdx.x] += sb[threadIdx.x + o];
		}
		__syncthreads();
	}
	if (threadIdx.x == 0)
		*result = (isnan(sa[0]) || isnan(sb[0])) ? (double)NAN
											   : (sb[0] > 0.0 ? sqrt(sa[0] / sb[0]) : (sa[0] > 0.0 ? INFINITY : 0.0));
}

// Device address of the scratch array, looked up with the device current (in
// host code the array's name is only a host-side stand-in).  The address is
// cached per device together with the id of the context it was resolved in:
// after a cudaDeviceReset the runtime creates a new context, whose module
// holds the array at another address, and the id tells the two apart.  The
// context id comes from the driver through the runtime's entry-point lookup,
// so the library needs no link against the driver library.
constexpr int NA_MAX_DEVICES = 64;
struct ScratchSlot {
	double2 *ptr = nullptr;
	unsigned long long ctx_id = 0;
};
ScratchSlot g_scratch[NA_MAX_DEVICES];
std::mutex g_scratch_mutex;

typedef CUresult (*PFN_ctx_get_current)(CUcontext *);
typedef CUresult (*PFN_ctx_get_id)(CUcontext, unsigned long long *);
PFN_ctx_get_current g_ctx_get_current = nullptr;
PFN_ctx_get_id g_ctx_get_id = nullptr;
bool g_ctx_lookup_done = false;

// Id of the calling thread's current context, false when it is unknown.
bool current_context_id(unsigned long long *id) {
	if (!g_ctx_lookup_done) {
		g_ctx_lookup_done = true;
		void *a = nullptr, *b = nullptr;
		cudaDriverEntryPointQueryResult qa, qb;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
			qa == cudaDriverEntryPointSuccess &&
			cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
			qb == cudaDriverEntryPointSuccess) {
			g_ctx_get_current = reinterpret_cast<PFN_ctx_get_current>(a);
			g_ctx_get_id = reinterpret_cast<PFN_ctx_get_id>(b);
		}
		cudaGetLastError();
	}
	if (!g_ctx_get_current || !g_ctx_get_id) return false;
	CUcontext c = nullptr;
	if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c) return false;
	return g_ctx_get_id(c, id) == CUDA_SUCCESS;
}

int scratch_for_current_device(double2 **out) {
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_velocity_residual_noalloc: %s", cudaGetErrorString(e));
	if (dev < 0 || dev >= NA_MAX_DEVICES)
		return fail(KEL_ERR_UNSUPPORTED, "kel_velocity_residual_noalloc: device %d beyond %d", dev, NA_MAX_DEVICES);
	std::lock_guard<std::mutex> lock(g_scratch_mutex);
	unsigned long long id = 0;
	const bool known = current_context_id(&id);
	ScratchSlot &slot = g_scratch[dev];
	if (!slot.ptr || !known || slot.ctx_id != id) {
		void *p = nullptr;
		e = cudaGetSymbolAddress(&p, g_noalloc_partials);
		if (e != cudaSuccess || !p)
			return fail(KEL_ERR_CUDA, "kel_velocity_residual_noalloc: cudaGetSymbolAddress failed: %s",
						cudaGetErrorString(e));
		slot.ptr = static_cast<double2 *>(p);
		// the lookup made the device's context current if it was not yet
		slot.ctx_id = current_context_id(&id) ? id : 0;
	}
	*out = slot.ptr;
	return KEL_OK;
}

} // namespace

extern "C" int kel_velocity_residual_noalloc(const float *d_u, const float *d_u_prev, int64_t n, int32_t comps,
											 double *d_result, void *stream) {
	if (!d_u || !d_u_prev || !d_result)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_velocity_residual_noalloc: null device pointer");
	if (comps < 1 || comps > 3)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_velocity_residual_noalloc: comps must be 1, 2 or 3 (got %d)", comps);
	if (n < 1 || n > (int64_t)NA_MAX_TILES * NA_TILE)
		return fail(KEL_ERR_INVALID_ARGUMENT,
					"kel_velocity_residual_noalloc: n = %lld cells is outside 1..%lld (the fixed scratch holds %d "
					"tiles of %d cells)",
					(long long)n, (long long)NA_MAX_TILES * NA_TILE, NA_MAX_TILES, NA_TILE);
	double2 *scratch = nullptr;
	int rc = scratch_for_current_device(&scratch);
	if (rc) return rc;
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	const int tiles = (int)((n + NA_TILE - 1) / NA_TILE);
	na_partial<<<tiles, NA_TILE, 0, st>>>(d_u, d_u_prev, n, comps, scratch);
	na_final<<<1, 1024, 0, st>>>(scratch, tiles, d_result);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_velocity_residual_noalloc: %s", cudaGetErrorString(e));
	return KEL_OK;
}
