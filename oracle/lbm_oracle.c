/*
 * lbm_oracle.c -- CPU restatement of keldu/lbm_mirror's lattice-Boltzmann
 * hot path.  TEST INFRASTRUCTURE: the oracle that the CUDA kernels are checked
 * against (tests/, __graft_entry__.smoke and bench.py's CPU baseline only).
 * The product never links or calls it.
 *
 * Pinned: tests/test_oracle_golden.py compares it bit-for-bit with golden
 * vectors produced by the reference's own components (oracle/ref_harness.cpp,
 * generator tests/golden/make_golden.py).
 *
 * Reference files restated (paths inside keldu/lbm_mirror):
 *   descriptors       modules/core/c++/descriptor/d2q9.hpp:17-57,
 *                     d3q19.hpp:15-67, d3q27.hpp:16-98
 *   equilibrium       modules/core/c++/equilibrium.hpp:7-48
 *   moments           modules/core/c++/macroscopic.hpp:10-35
 *   BGK / BGKGuo      modules/core/c++/collision.hpp:77-96, 135-203
 *   Stream            modules/core/c++/stream.hpp:19-58
 *   boundaries        modules/core/c++/boundary.hpp:32-805
 *   PSM collision     modules/core/c++/psm.hpp:58-89
 *   lid               examples/cavity_2d_gpu/cavity_2d_gpu.cpp:204-235
 *   step order        examples/poiseulle_2d_gpu/poiseulle_2d_gpu.cpp:158-235, 384-399
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/kel_lbm_cuda.h"

typedef struct ko_desc {
	int D, Q;
	int c[27][3];
	int opp[27];
	double w[27];
} ko_desc;

static void ko_make_desc(int q, ko_desc *d) {
	memset(d, 0, sizeof(*d));
	if (q == 9) {
		/* descriptor/d2q9.hpp:17-27 */
		static const int c[9][2] = {{0, 0}, {-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, 1}, {-1, 1}, {1, -1}};
		static const double w[9] = {4. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 36., 1. / 36., 1. / 36., 1. / 36.};
		static const int opp[9] = {0, 2, 1, 4, 3, 6, 5, 8, 7};
		d->D = 2;
		d->Q = 9;
		for (int i = 0; i < 9; ++i) {
			d->c[i][0] = c[i][0];
			d->c[i][1] = c[i][1];
			d->w[i] = w[i];
			d->opp[i] = opp[i];
		}
	} else if (q == 19) {
		/* descriptor/d3q19.hpp:15-67 */
		static const int c[19][3] = {{0, 0, 0},  {-1, 0, 0},  {1, 0, 0},  {0, -1, 0}, {0, 1, 0},  {0, 0, -1}, {0, 0, 1},
									 {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 1, 0},  {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
									 {1, 0, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}, {0, 1, 1}};
		static const int opp[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
		d->D = 3;
		d->Q = 19;
		for (int i = 0; i < 19; ++i) {
			for (int k = 0; k < 3; ++k) d->c[i][k] = c[i][k];
			d->w[i] = i == 0 ? 1. / 3. : (i < 7 ? 1. / 18. : 1. / 36.);
			d->opp[i] = opp[i];
		}
	} else if (q == 27) {
		/* descriptor/d3q27.hpp:16-98: i = a + 3 b + 9 g, axis offsets ordered 0, -1, +1 */
		static const int o3[3] = {0, -1, 1};
		d->D = 3;
		d->Q = 27;
		for (int i = 0; i < 27; ++i) {
			int a = i % 3, b = (i / 3) % 3, g = i / 9;
			d->c[i][0] = o3[a];
			d->c[i][1] = o3[b];
			d->c[i][2] = o3[g];
			int n2 = (a != 0) + (b != 0) + (g != 0);
			d->w[i] = n2 == 0 ? 8. / 27. : n2 == 1 ? 2. / 27. : n2 == 2 ? 1. / 54. : 1. / 216.;
			int oa = a == 0 ? 0 : 3 - a, ob = b == 0 ? 0 : 3 - b, og = g == 0 ? 0 : 3 - g;
			d->opp[i] = oa + 3 * ob + 9 * og;
		}
	}
}

static inline float ko_weight_f32(const ko_desc *d, int i) { return (float)d->w[i]; }
static inline double ko_weight_f64(const ko_desc *d, int i) { return d->w[i]; }

#define REAL float
#define KO_SUFFIX _f32
static inline float weight_f32(const ko_desc *d, int i) { return ko_weight_f32(d, i); }
#include "lbm_oracle_impl.h"
#undef REAL
#undef KO_SUFFIX

#define REAL double
#define KO_SUFFIX _f64
static inline double weight_f64(const ko_desc *d, int i) { return ko_weight_f64(d, i); }
#include "lbm_oracle_impl.h"
#undef REAL
#undef KO_SUFFIX

/* ---------------------------------------------------------------------- */
/* Public (test-only) API, bound by oracle/oracle.py with ctypes.          */

typedef struct ko_lattice {
	int is_f64;
	ko_lat_f32 f32;
	ko_lat_f64 f64;
} ko_lattice;

#define KO_ALLOC_FIELDS(L, REALT)                                                        \
	do {                                                                                 \
		int64_t g = (L)->gx * (L)->gy * (L)->gz * (L)->d.Q;                              \
		(L)->info = (uint8_t *)calloc((size_t)(L)->n, 1);                                \
		(L)->dfs[0] = (REALT *)calloc((size_t)g, sizeof(REALT));                         \
		(L)->dfs[1] = (REALT *)calloc((size_t)g, sizeof(REALT));                         \
		(L)->rho = (REALT *)calloc((size_t)(L)->n, sizeof(REALT));                       \
		(L)->vel = (REALT *)calloc((size_t)((L)->n * (L)->d.D), sizeof(REALT));          \
		(L)->por = (REALT *)calloc((size_t)(L)->n, sizeof(REALT));                       \
		(L)->force = (REALT *)calloc((size_t)((L)->n * (L)->d.D), sizeof(REALT));        \
		(L)->hN = (REALT *)calloc((size_t)((L)->n * (L)->d.D), sizeof(REALT));           \
		(L)->hD = (REALT *)calloc((size_t)(L)->n, sizeof(REALT));                        \
	} while (0)

#define KO_FREE_FIELDS(L)                                                               \
	do {                                                                                \
		free((L)->info);                                                                \
		free((L)->dfs[0]);                                                              \
		free((L)->dfs[1]);                                                              \
		free((L)->rho);                                                                 \
		free((L)->vel);                                                                 \
		free((L)->por);                                                                 \
		free((L)->force);                                                               \
		free((L)->hN);                                                                  \
		free((L)->hD);                                                                  \
	} while (0)

/* Rest-equilibrium initial state as in every reference driver's setup:
 * rho = 1, u = 0 for every cell, dfs_old = equilibrium(rho,u). */
#define KO_INIT_REST(L, SUF, REALT)                                                      \
	do {                                                                                 \
		REALT eq[27], u0[3] = {0, 0, 0};                                                 \
		KO_CAT(equilibrium, SUF)(&(L)->d, (REALT)1, u0, eq);                             \
		for (int64_t c = 0; c < (L)->n; ++c) {                                           \
			int64_t x = c % (L)->nx, y = (c / (L)->nx) % (L)->ny, z = c / ((L)->nx * (L)->ny); \
			REALT *f = (L)->dfs[0] + KO_CAT(gidx, SUF)((L), x, y, z) * (L)->d.Q;           \
			for (int i = 0; i < (L)->d.Q; ++i) f[i] = eq[i];                             \
			(L)->rho[c] = 1;                                                             \
			(L)->por[c] = 1;                                                             \
		}                                                                                \
	} while (0)

ko_lattice *ko_create(int q, int is_f64, int64_t nx, int64_t ny, int64_t nz, int periodic_x) {
	ko_desc d;
	ko_make_desc(q, &d);
	if (d.Q == 0 || nx <= 0 || ny <= 0 || nz <= 0 || (d.D == 2 && nz != 1)) return NULL;
	ko_lattice *h = (ko_lattice *)calloc(1, sizeof(ko_lattice));
	h->is_f64 = is_f64;
#define KO_SETUP(L, SUF, REALT)                       \
	do {                                              \
		(L)->d = d;                                   \
		(L)->nx = nx;                                 \
		(L)->ny = ny;                                 \
		(L)->nz = nz;                                 \
		(L)->n = nx * ny * nz;                        \
		(L)->gx = nx + 2;                             \
		(L)->gy = ny + 2;                             \
		(L)->gz = d.D == 3 ? nz + 2 : 1;              \
		(L)->periodic_x = periodic_x;                 \
		KO_ALLOC_FIELDS(L, REALT);                    \
		KO_INIT_REST(L, SUF, REALT);                  \
	} while (0)
	if (is_f64) KO_SETUP(&h->f64, _f64, double);
	else KO_SETUP(&h->f32, _f32, float);
	return h;
}

void ko_destroy(ko_lattice *h) {
	if (!h) return;
	if (h->is_f64) KO_FREE_FIELDS(&h->f64);
	else KO_FREE_FIELDS(&h->f32);
	free(h);
}

void ko_set_flags(ko_lattice *h, const uint8_t *flags) {
	if (h->is_f64) memcpy(h->f64.info, flags, (size_t)h->f64.n);
	else memcpy(h->f32.info, flags, (size_t)h->f32.n);
}

void ko_set_profile(ko_lattice *h, const double *profile) {
	if (h->is_f64) h->f64.profile = profile;
	else h->f32.profile = profile;
}

void ko_set_populations(ko_lattice *h, const double *aos) {
	if (h->is_f64) set_pops_f64(&h->f64, aos);
	else set_pops_f32(&h->f32, aos);
}

void ko_get_populations(ko_lattice *h, double *aos) {
	if (h->is_f64) get_pops_f64(&h->f64, aos);
	else get_pops_f32(&h->f32, aos);
}

void ko_set_porosity(ko_lattice *h, const double *v) {
	if (h->is_f64) set_vec_f64(h->f64.por, v, h->f64.n);
	else set_vec_f32(h->f32.por, v, h->f32.n);
}

void ko_set_force(ko_lattice *h, const double *v) {
	if (h->is_f64) set_vec_f64(h->f64.force, v, h->f64.n * h->f64.d.D);
	else set_vec_f32(h->f32.force, v, h->f32.n * h->f32.d.D);
}

void ko_get_macros(ko_lattice *h, double *rho, double *vel) {
	if (h->is_f64) {
		get_vec_f64(h->f64.rho, rho, h->f64.n);
		get_vec_f64(h->f64.vel, vel, h->f64.n * h->f64.d.D);
	} else {
		get_vec_f32(h->f32.rho, rho, h->f32.n);
		get_vec_f32(h->f32.vel, vel, h->f32.n * h->f32.d.D);
	}
}

int ko_run(ko_lattice *h, const kel_step_program *prog, uint64_t steps) {
	if (h->is_f64) return run_f64(&h->f64, prog, steps);
	return run_f32(&h->f32, prog, steps);
}

int ko_run_rows(ko_lattice *h, const kel_step_program *prog, int64_t r0, int64_t r1) {
	if (h->is_f64) return run_rows_f64(&h->f64, prog, r0, r1);
	return run_rows_f32(&h->f32, prog, r0, r1);
}

uint64_t ko_time_step(const ko_lattice *h) { return h->is_f64 ? h->f64.t : h->f32.t; }

/* Helper for tests: the reference equilibrium of (rho, u) in float
 * arithmetic (equilibrium.hpp:7-48). */
void ko_equilibrium_f32(int q, float rho, const float *u, float *eq) {
	ko_desc d;
	ko_make_desc(q, &d);
	equilibrium_f32(&d, rho, u, eq);
}

size_t ko_program_size(void) { return sizeof(kel_step_program); }

/* ---- accessors for the particle restatement (particles_oracle.c) ------- */
float ko_lattice_pop_f32(const ko_lattice *h, int64_t x, int64_t y, int64_t z, int i);
int ko_lattice_info(const ko_lattice *h, int *D, int *Q, int64_t *nx, int64_t *ny, int64_t *nz, int *is_f64,
					int *periodic) {
	const ko_desc *d = h->is_f64 ? &h->f64.d : &h->f32.d;
	*D = d->D;
	*Q = d->Q;
	*nx = h->is_f64 ? h->f64.nx : h->f32.nx;
	*ny = h->is_f64 ? h->f64.ny : h->f32.ny;
	*nz = h->is_f64 ? h->f64.nz : h->f32.nz;
	*is_f64 = h->is_f64;
	*periodic = h->is_f64 ? h->f64.periodic_x : h->f32.periodic_x;
	return 0;
}

int ko_lattice_dir(const ko_lattice *h, int i, int k) { return (h->is_f64 ? &h->f64.d : &h->f32.d)->c[i][k]; }
int ko_lattice_opp(const ko_lattice *h, int i) { return (h->is_f64 ? &h->f64.d : &h->f32.d)->opp[i]; }

/* Post-stream population f_i at (x,y,z) of the buffer the next collide reads;
 * outside the lattice: the zero ghost ring. */
double ko_lattice_pop(const ko_lattice *h, int64_t x, int64_t y, int64_t z, int i) {
	if (h->is_f64) {
		const ko_lat_f64 *L = &h->f64;
		if (x < 0 || y < 0 || z < 0 || x >= L->nx || y >= L->ny || z >= L->nz) return 0.0;
		const double *cur = (L->t % 2u == 0u) ? L->dfs[0] : L->dfs[1];
		return cur[gidx_f64(L, x, y, z) * L->d.Q + i];
	}
	return (double)ko_lattice_pop_f32(h, x, y, z, i);
}

float ko_lattice_pop_f32(const ko_lattice *h, int64_t x, int64_t y, int64_t z, int i) {
	const ko_lat_f32 *L = &h->f32;
	if (x < 0 || y < 0 || z < 0 || x >= L->nx || y >= L->ny || z >= L->nz) return 0.0f;
	const float *cur = (L->t % 2u == 0u) ? L->dfs[0] : L->dfs[1];
	return cur[gidx_f32(L, x, y, z) * L->d.Q + i];
}

void ko_lattice_set_porosity_at(ko_lattice *h, int64_t c, double v) {
	if (h->is_f64) h->f64.por[c] = v;
	else h->f32.por[c] = (float)v;
}

double ko_lattice_porosity_at(const ko_lattice *h, int64_t c) {
	return h->is_f64 ? h->f64.por[c] : (double)h->f32.por[c];
}

/* HLBM per-cell accumulators (particle_N: D values, particle_D) */
void ko_lattice_hlbm_add_at(ko_lattice *h, int64_t c, const double *vflip, double flip) {
	if (h->is_f64) {
		for (int k = 0; k < h->f64.d.D; ++k) h->f64.hN[c * h->f64.d.D + k] = h->f64.hN[c * h->f64.d.D + k] + vflip[k];
		h->f64.hD[c] = h->f64.hD[c] + flip;
	} else {
		for (int k = 0; k < h->f32.d.D; ++k)
			h->f32.hN[c * h->f32.d.D + k] = h->f32.hN[c * h->f32.d.D + k] + (float)vflip[k];
		h->f32.hD[c] = h->f32.hD[c] + (float)flip;
	}
}

void ko_lattice_hlbm_reset(ko_lattice *h) {
	if (h->is_f64) {
		for (int64_t c = 0; c < h->f64.n; ++c) h->f64.por[c] = 1.0, h->f64.hD[c] = 0.0;
		memset(h->f64.hN, 0, sizeof(double) * (size_t)(h->f64.n * h->f64.d.D));
	} else {
		for (int64_t c = 0; c < h->f32.n; ++c) h->f32.por[c] = 1.0f, h->f32.hD[c] = 0.0f;
		memset(h->f32.hN, 0, sizeof(float) * (size_t)(h->f32.n * h->f32.d.D));
	}
}

void ko_get_hlbm(ko_lattice *h, double *N, double *Dv) {
	if (h->is_f64) {
		get_vec_f64(h->f64.hN, N, h->f64.n * h->f64.d.D);
		get_vec_f64(h->f64.hD, Dv, h->f64.n);
	} else {
		get_vec_f32(h->f32.hN, N, h->f32.n * h->f32.d.D);
		get_vec_f32(h->f32.hD, Dv, h->f32.n);
	}
}

void ko_set_hlbm(ko_lattice *h, const double *N, const double *Dv) {
	if (h->is_f64) {
		set_vec_f64(h->f64.hN, N, h->f64.n * h->f64.d.D);
		set_vec_f64(h->f64.hD, Dv, h->f64.n);
	} else {
		set_vec_f32(h->f32.hN, N, h->f32.n * h->f32.d.D);
		set_vec_f32(h->f32.hD, Dv, h->f32.n);
	}
}

/* FPLBM (fplbm.hpp): FpLbmReset on every cell, then FpLbmOneParticle for
 * every body (see lbm_oracle_impl.h) */
void ko_fplbm_reset(ko_lattice *h, uint32_t plain_mask) {
	if (h->is_f64) fplbm_reset_f64(&h->f64, plain_mask);
	else fplbm_reset_f32(&h->f32, plain_mask);
}

void ko_fplbm_particles(ko_lattice *h, kel_particle_state *P, int np, const kel_particle_params *prm, int own) {
	if (h->is_f64) fplbm_particles_f64(&h->f64, P, np, prm, own);
	else fplbm_particles_f32(&h->f32, P, np, prm, own);
}

void ko_get_force(ko_lattice *h, double *out) {
	if (h->is_f64) get_vec_f64(h->f64.force, out, h->f64.n * h->f64.d.D);
	else get_vec_f32(h->f32.force, out, h->f32.n * h->f32.d.D);
}

void ko_get_porosity(ko_lattice *h, double *out) {
	if (h->is_f64) get_vec_f64(h->f64.por, out, h->f64.n);
	else get_vec_f32(h->f32.por, out, h->f32.n);
}
