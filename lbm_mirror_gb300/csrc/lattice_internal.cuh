// Internal state of the C ABI objects, shared by the translation units that
// implement include/kel_lbm_cuda.h (lattice.cu, particles.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/kel_lbm_cuda.h"
#include "descriptors.cuh"
#include "sweep.cuh"

namespace kel {
namespace gb {

int fail(int code, const char *fmt, ...);

#define KEL_CUDA(call)                                                                             \
	do {                                                                                           \
		cudaError_t e__ = (call);                                                                  \
		if (e__ != cudaSuccess)                                                                    \
			return ::kel::gb::fail(e__ == cudaErrorMemoryAllocation ? KEL_ERR_OUT_OF_MEMORY : KEL_ERR_CUDA, \
								   "%s: %s (%s:%d)", #call, cudaGetErrorString(e__), __FILE__, __LINE__); \
	} while (0)

struct HostDesc {
	int D = 0, Q = 0;
	int c[27][3];
	int opp[27];
	double w[27];
};

int grid_for(int64_t n);
// Launch parameters of the sweep kel_step runs for program P on lattice L.
SweepParams sweep_params(kel_lattice *L, const kel_step_program *P);
int ensure_field(kel_lattice *L, float **ptr, int64_t count, float init);
// Copy `comps` device planes (padded plane layout) to host AoS (N*comps).
int field_to_host(kel_lattice *L, const float *dev, float *host, int comps);

} // namespace gb
} // namespace kel

struct kel_lattice {
	kel_lattice_desc desc;
	kel::gb::HostDesc d;
	int nxp = 0, nq = 0, wpr = 0;
	int64_t plane = 0, ncell = 0;
	size_t elem = 4;
	void *f = nullptr;
	uint8_t *flags = nullptr;
	float *rho = nullptr, *u = nullptr, *por = nullptr, *force = nullptr, *profile = nullptr;
	float *hN = nullptr, *hD = nullptr; // HLBM particle_N (D planes) and particle_D, on first use
	// Counts writes of the porosity field: an uploaded field, an HLBM couple
	// and every PSM couple advance it, so a particle set sees whether the
	// field still is the one its own last couple left.
	uint64_t por_epoch = 1;
	kel::gb::OpEntry *ops = nullptr;
	void *staging = nullptr;
	size_t staging_bytes = 0;
	cudaStream_t stream = nullptr;
	uint64_t t = 0;
	float wshift[27];
	bool have_ops = false;
	uint32_t plain_flags = 0; // SweepParams::plain of the current program
	// flags whose op has no boundary step and collides (the FPLBM drivers'
	// info 2), from the last program passed to kel_step
	uint32_t plain_flags_fplbm = 1u << 2;
	uint8_t present[kel::gb::MAX_FLAGS] = {0}; // flag values present in the uploaded flag field
	unsigned *d_seen = nullptr;                 // device scratch of the flag-presence scan (8 words)
	kel_step_program last_prog;
	int device = 0;
	int cpt = 1;      // sweep launch: cells per thread (1 or 4), or 2 for the row pipeline
	int block = 128;  // threads per block of the sweep launch (row pipeline: row stages)
	int sms = 1;      // multiprocessors of the lattice's device
	unsigned *d_err = nullptr; // set by the row pipeline when a bounded wait gave up
	bool rows_used = false;    // a row-pipeline sweep was launched (d_err worth reading)
	uint32_t *hw_mask = nullptr; // half-way wall neighbour bits per cell (allocated on first use)
	bool hw_active = false;      // the current program has half-way walls present in the lattice
	cudaGraphExec_t graph = nullptr;    // GRAPH_STEPS captured sweeps (kel_step), for graph_params
	kel::gb::SweepParams graph_params;
	int graph_coll = -1;
	bool graph_exact = false;
	bool tuned = false;
};
