/*
 * particles_oracle.c -- CPU restatement of keldu/lbm_mirror's particle
 * coupling and rigid-body path (spheres / discs).  TEST INFRASTRUCTURE ONLY:
 * the oracle the CUDA particle kernels are checked against.
 *
 * Reference files restated (paths inside keldu/lbm_mirror):
 *   porosity ramp     modules/core/c++/particle/porosity.hpp:56-89
 *   couple (product)  modules/core/c++/particle/couple.hpp:26-58
 *   AABB              modules/core/c++/particle/aabb.hpp:41-84
 *   gather            modules/core/c++/psm.hpp:101-446 (momentum exchange)
 *   torque            modules/core/c++/hlbm.hpp:234,250-251 (r x cell momentum)
 *   reset             modules/core/c++/particle/integrate.hpp:195-212
 *   contact           modules/core/c++/particle/contact.hpp:110-512
 *   integrate         modules/core/c++/particle/integrate.hpp:45-83,
 *                     particle/particle.hpp:171-211 (position Verlet)
 *
 * Lattice values (populations, per-cell momentum, cell force) are computed in
 * the lattice's REAL with the reference's rounding order; particle state and
 * the per-particle sums are double.  With a double lattice this is the
 * reference's T = Float64 path exactly (pinned against the reference's
 * components by tests/test_particles_oracle.py).
 *
 * Restatements beyond the reference (no counterpart there): PSM torque, the
 * 4^D sub-cell solid fraction, periodic x (minimum image, wrapped AABB),
 * DEM walls per axis.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/kel_lbm_cuda.h"

#ifndef KO_PI
#define KO_PI 3.14159265358979323846
#endif

/* The lattice internals live in lbm_oracle.c; these accessors are exported
 * from there. */
typedef struct ko_lattice ko_lattice;
int ko_lattice_info(const ko_lattice *h, int *D, int *Q, int64_t *nx, int64_t *ny, int64_t *nz, int *is_f64,
					int *periodic);
double ko_lattice_pop(const ko_lattice *h, int64_t x, int64_t y, int64_t z, int i); /* post-stream f_i, ghost 0 */
float ko_lattice_pop_f32(const ko_lattice *h, int64_t x, int64_t y, int64_t z, int i);
void ko_lattice_set_porosity_at(ko_lattice *h, int64_t c, double v);
double ko_lattice_porosity_at(const ko_lattice *h, int64_t c);
int ko_lattice_dir(const ko_lattice *h, int i, int k);
int ko_lattice_opp(const ko_lattice *h, int i);

/* ---- porosity ---------------------------------------------------------- */

/* particle_porosity<T,D,1,ParticleSpheroid>::calculate in double */
static double ramp(double s, double rad, double eps) {
	double eps_h = eps / 2;
	double lo = rad - eps_h, hi = rad + eps_h;
	if (s <= lo) return 0.0;
	if (s >= hi) return 1.0;
	double inner = (KO_PI / (2 * eps)) * (s - lo);
	double c = sin(inner);
	return c * c;
}

/* 4^D sub-cell solid fraction (no reference counterpart), in float: the
 * cell's offset from the body is its integer part (x - nearest lattice point
 * of the centre, the nearest periodic image) plus the fraction (that point -
 * the centre); samples at offset + (2 a - 3) / 8 per axis count as inside
 * when their squared distance, summed in axis order, is at most R^2. */
static double subcell(int D, int64_t x, int64_t y, int64_t z, const double *X, double rad, int per, int64_t nx) {
	int total = D == 2 ? 16 : 64, inside = 0;
	int64_t c[3] = {x, y, z};
	float r[3] = {0.f, 0.f, 0.f};
	for (int k = 0; k < D; ++k) {
		const int ic = (int)llround(X[k]);
		const float fr = (float)((double)ic - X[k]);
		int d = (int)(c[k] - ic);
		if (k == 0 && per) {
			if (d > (int)nx / 2) d -= (int)nx;
			else if (d < -((int)nx / 2)) d += (int)nx;
		}
		r[k] = (float)d + fr;
	}
	const float r2 = (float)rad * (float)rad;
	for (int a = 0; a < 4; ++a)
		for (int b = 0; b < 4; ++b)
			for (int g = 0; g < (D == 3 ? 4 : 1); ++g) {
				float px = r[0] + (float)(2 * a - 3) * 0.125f;
				float py = r[1] + (float)(2 * b - 3) * 0.125f;
				float d2 = px * px + py * py;
				if (D == 3) {
					float pz = r[2] + (float)(2 * g - 3) * 0.125f;
					d2 = d2 + pz * pz;
				}
				if (d2 <= r2) ++inside;
			}
	return 1.0 - (double)inside / (double)total;
}

/* Offset of a cell from a particle centre; with periodic x the nearest image. */
static double rel_coord(double cell, double X, int periodic, int64_t n) {
	double r = cell - X;
	if (periodic) {
		double L = (double)n;
		if (r > 0.5 * L) r -= L;
		else if (r < -0.5 * L) r += L;
	}
	return r;
}

/* Growth of the voxel bodies' boxes (KEL_POROSITY_VOXEL): radius R * mul +
 * add, the shape's reach and half the ramp width (set by the caller). */
static double g_voxel_mul = 1.0, g_voxel_add = 0.0;

void ko_particles_set_voxel_box(double mul, double add) {
	g_voxel_mul = mul;
	g_voxel_add = add;
}

/* aabb.hpp:41-84: [a, b) per axis; x unclamped when periodic (cells wrap).
 * subcell_mode: 0 the reference's box, 1 the sub-cell box, 2 the sub-cell
 * box of the grown voxel radius. */
static void aabb(int D, const kel_particle_state *p, const int64_t *ext, int periodic, int subcell_mode,
				 int64_t *a, int64_t *b) {
	for (int k = 0; k < D; ++k) {
		double X = p->position[k], r = subcell_mode == 2 ? p->radius * g_voxel_mul + g_voxel_add : p->radius;
		if (subcell_mode) {
			a[k] = (int64_t)floor(X - r - 0.5);
			b[k] = (int64_t)ceil(X + r + 0.5) + 1;
		} else {
			a[k] = (X >= r) ? (int64_t)(X - r) : 0;
			if (periodic && k == 0 && X < r) a[k] = (int64_t)floor(X - r);
			b[k] = (int64_t)(X + r + 1.0);
		}
		if (!(periodic && k == 0)) {
			if (a[k] < 0) a[k] = 0;
			if (b[k] > ext[k]) b[k] = ext[k];
		}
	}
}


/* Porosity of every cell: product over bodies (couple.hpp:26-58), 1 = fluid.
 * Each body contributes only inside its AABB, which is where the reference's
 * gather stamps it (psm.hpp:198-265); outside every AABB the cell is fluid.
 * A cell counts for a body when the image of the cell nearest the body lies
 * in the body's AABB.  Walked body by body (index order) over the cells of
 * each AABB, with the products kept in double until every body is done: the
 * same factors multiplied in the same order as a loop over the bodies per
 * cell, in time proportional to the AABBs rather than cells x bodies. */
void ko_particles_couple(ko_lattice *h, const kel_particle_state *P, int np, const kel_particle_params *prm) {
	int D, Q, f64, per;
	int64_t nx, ny, nz;
	ko_lattice_info(h, &D, &Q, &nx, &ny, &nz, &f64, &per);
	int64_t ext[3] = {nx, ny, nz};
	int sub = prm->porosity_mode == KEL_POROSITY_SUBCELL;
	int64_t n = nx * ny * nz;
	double *por = (double *)malloc(sizeof(double) * (size_t)n);
	for (int64_t c = 0; c < n; ++c) por[c] = 1.0;
	for (int p = 0; p < np; ++p) {
		int64_t a[3] = {0, 0, 0}, b[3] = {1, 1, 1};
		aabb(D, &P[p], ext, per, sub, a, b);
		for (int64_t iz = a[2]; iz < b[2]; ++iz)
			for (int64_t iy = a[1]; iy < b[1]; ++iy)
				for (int64_t ix = a[0]; ix < b[0]; ++ix) {
					int64_t x = per ? ((ix % nx) + nx) % nx : ix, y = iy, z = D == 3 ? iz : 0;
					double rel[3] = {rel_coord((double)x, P[p].position[0], per, nx), (double)y - P[p].position[1],
									 D == 3 ? (double)z - P[p].position[2] : 0.0};
					double xi = P[p].position[0] + rel[0]; /* the image of x nearest the body */
					int64_t xc = per ? (int64_t)llround(xi) : x;
					if (xc != ix) continue; /* this image is not the nearest one (or lies outside the AABB) */
					double pp;
					if (sub) {
						pp = subcell(D, x, y, z, P[p].position, P[p].radius, per, nx);
					} else {
						double s2 = 0.0;
						for (int k = 0; k < D; ++k) s2 = s2 + rel[k] * rel[k];
						pp = ramp(sqrt(s2), P[p].radius, prm->eps);
					}
					int64_t c = x + nx * (y + ny * z);
					por[c] = por[c] * pp;
				}
	}
	for (int64_t c = 0; c < n; ++c) ko_lattice_set_porosity_at(h, c, por[c]);
	free(por);
}

#define KO_GATHER_BODY(REALT, POP)                                                                           \
	for (int p = 0; p < np; ++p) {                                                                           \
		kel_particle_state *pp = &P[p];                                                                      \
		int64_t a[3] = {0, 0, 0}, b[3] = {1, 1, 1};                                                          \
		aabb(D, pp, ext, per, prm->porosity_mode == KEL_POROSITY_SUBCELL ? 1                                 \
							  : (prm->porosity_mode == KEL_POROSITY_VOXEL ? 2 : 0), a, b);                       \
		double ts = 1.0 / (double)steps;                                                                     \
		double vp[3] = {0, 0, 0};                                                                            \
		for (int k = 0; k < D; ++k) vp[k] = (pp->position[k] - pp->position_old[k]) / ts;                    \
		double fsum[3] = {0, 0, 0}, tsum[3] = {0, 0, 0};                                                     \
		/* iterator<D>::apply: axis 0 is the outermost loop */                                              \
		for (int64_t ix = a[0]; ix < b[0]; ++ix)                                                             \
			for (int64_t iy = a[1]; iy < b[1]; ++iy)                                                         \
				for (int64_t iz = (D == 3 ? a[2] : 0); iz < (D == 3 ? b[2] : 1); ++iz) {                     \
					int64_t x = per ? ((ix % nx) + nx) % nx : ix;                                            \
					int64_t c = x + nx * (iy + ny * iz);                                                     \
					REALT por = (REALT)ko_lattice_porosity_at(h, c);                                         \
					if (por >= (REALT)1.0) continue;                                                         \
					REALT mom[3] = {0, 0, 0};                                                                \
					for (int i = 1; i < Q; ++i) {                                                            \
						int e0 = ko_lattice_dir(h, i, 0), e1 = ko_lattice_dir(h, i, 1), e2 = ko_lattice_dir(h, i, 2); \
						double upe_d = 0.0;                                                                  \
						upe_d = upe_d + (double)e0 * vp[0];                                                  \
						upe_d = upe_d + (double)e1 * vp[1];                                                  \
						if (D == 3) upe_d = upe_d + (double)e2 * vp[2];                                      \
						REALT upe = (REALT)upe_d;                                                            \
						int64_t nx_ = x + e0, ny_ = iy + e1, nz_ = iz + e2;                                  \
						if (per) nx_ = (nx_ + nx) % nx;                                                      \
						REALT fi = POP(h, x, iy, iz, i);                                                     \
						REALT fo = POP(h, nx_, ny_, nz_, ko_lattice_opp(h, i));                              \
						REALT da = fi * ((REALT)1.0 - upe) + fo * ((REALT)1.0 + upe);                        \
						mom[0] = mom[0] + (REALT)e0 * da;                                                    \
						mom[1] = mom[1] + (REALT)e1 * da;                                                    \
						if (D == 3) mom[2] = mom[2] + (REALT)e2 * da;                                        \
					}                                                                                        \
					REALT flip = (REALT)1.0 - por;                                                           \
					double F[3] = {0, 0, 0};                                                                 \
					for (int k = 0; k < D; ++k) F[k] = (double)(mom[k] * flip);                              \
					if (cell_force)                                                                          \
						for (int k = 0; k < D; ++k) cell_force[c * D + k] = F[k];                            \
					for (int k = 0; k < D; ++k) fsum[k] = fsum[k] - F[k];                                    \
					double r[3] = {rel_coord((double)x, pp->position[0], per, nx), (double)iy - pp->position[1], \
								   D == 3 ? (double)iz - pp->position[2] : 0.0};                             \
					if (D == 2) {                                                                            \
						tsum[0] = tsum[0] - (r[0] * F[1] - r[1] * F[0]);                                     \
					} else {                                                                                 \
						tsum[0] = tsum[0] - (r[1] * F[2] - r[2] * F[1]);                                     \
						tsum[1] = tsum[1] - (r[2] * F[0] - r[0] * F[2]);                                     \
						tsum[2] = tsum[2] - (r[0] * F[1] - r[1] * F[0]);                                     \
					}                                                                                        \
				}                                                                                            \
		for (int k = 0; k < D; ++k) pp->force[k] = pp->force[k] + fsum[k];                                   \
		for (int k = 0; k < (D == 2 ? 1 : 3); ++k) pp->torque[k] = pp->torque[k] + tsum[k];                  \
	}

/* PsmOneParticleGather (psm.hpp:101-446) for every particle, reading the
 * porosity field the couple pass wrote.  cell_force (N*D doubles, may be NULL)
 * receives the per-cell force momentum * (1 - porosity). */
void ko_particles_gather(ko_lattice *h, kel_particle_state *P, int np, const kel_particle_params *prm,
						 double *cell_force) {
	int D, Q, f64, per;
	int64_t nx, ny, nz;
	ko_lattice_info(h, &D, &Q, &nx, &ny, &nz, &f64, &per);
	int64_t ext[3] = {nx, ny, nz};
	/* psm.hpp:178-184 divides by the raw sub-step count: 0 gives ts = inf and
	 * a zero particle velocity */
	int steps = prm->sub_steps;
	if (f64) {
		KO_GATHER_BODY(double, ko_lattice_pop)
	} else {
		KO_GATHER_BODY(float, ko_lattice_pop_f32)
	}
}

/* ---- HLBM (hlbm.hpp) ---------------------------------------------------- */

void ko_lattice_hlbm_reset(ko_lattice *h);
void ko_lattice_hlbm_add_at(ko_lattice *h, int64_t c, const double *vflip, double flip);

/* HlbmReset (hlbm.hpp:27-47) on every cell, then the porosity each
 * HlbmOneParticleGather writes over its AABB (hlbm.hpp:178-186, the reference
 * ramp with eps = 1.5), bodies in index order: a cell inside several AABBs
 * keeps the last body's value, 1 included. */
void ko_particles_hlbm_couple(ko_lattice *h, const kel_particle_state *P, int np, const kel_particle_params *prm) {
	int D, Q, f64, per;
	int64_t nx, ny, nz;
	ko_lattice_info(h, &D, &Q, &nx, &ny, &nz, &f64, &per);
	int64_t ext[3] = {nx, ny, nz};
	ko_lattice_hlbm_reset(h);
	for (int p = 0; p < np; ++p) {
		int64_t a[3] = {0, 0, 0}, b[3] = {1, 1, 1};
		aabb(D, &P[p], ext, per, 0, a, b);
		for (int64_t ix = a[0]; ix < b[0]; ++ix)
			for (int64_t iy = a[1]; iy < b[1]; ++iy)
				for (int64_t iz = (D == 3 ? a[2] : 0); iz < (D == 3 ? b[2] : 1); ++iz) {
					int64_t x = per ? ((ix % nx) + nx) % nx : ix;
					double rel[3] = {rel_coord((double)x, P[p].position[0], per, nx), (double)iy - P[p].position[1],
									 D == 3 ? (double)iz - P[p].position[2] : 0.0};
					double s2 = 0.0;
					for (int k = 0; k < D; ++k) s2 = s2 + rel[k] * rel[k];
					ko_lattice_set_porosity_at(h, x + nx * (iy + ny * iz), ramp(sqrt(s2), P[p].radius, prm->eps));
				}
	}
}

/* HlbmOneParticleGather (hlbm.hpp:119-260): momentum exchange with the body's
 * pre-move velocity over the cells of its AABB where its own porosity is
 * below 1, no solid-fraction weight; the cell force (last body wins) is that
 * momentum, the body takes minus the sum and minus the r x momentum torque. */
#define KO_HLBM_GATHER_BODY(REALT, POP)                                                                      \
	for (int p = 0; p < np; ++p) {                                                                           \
		kel_particle_state *pp = &P[p];                                                                      \
		int64_t a[3] = {0, 0, 0}, b[3] = {1, 1, 1};                                                          \
		aabb(D, pp, ext, per, 0, a, b);                                                                      \
		double ts = 1.0 / (double)steps;                                                                     \
		double vp[3] = {0, 0, 0};                                                                            \
		for (int k = 0; k < D; ++k) vp[k] = (pp->position[k] - pp->position_old[k]) / ts;                    \
		double fsum[3] = {0, 0, 0}, tsum[3] = {0, 0, 0};                                                     \
		for (int64_t ix = a[0]; ix < b[0]; ++ix)                                                             \
			for (int64_t iy = a[1]; iy < b[1]; ++iy)                                                         \
				for (int64_t iz = (D == 3 ? a[2] : 0); iz < (D == 3 ? b[2] : 1); ++iz) {                     \
					int64_t x = per ? ((ix % nx) + nx) % nx : ix;                                            \
					int64_t c = x + nx * (iy + ny * iz);                                                     \
					double r[3] = {rel_coord((double)x, pp->position[0], per, nx), (double)iy - pp->position[1], \
								   D == 3 ? (double)iz - pp->position[2] : 0.0};                             \
					double s2 = 0.0;                                                                         \
					for (int k = 0; k < D; ++k) s2 = s2 + r[k] * r[k];                                       \
					REALT por = (REALT)ramp(sqrt(s2), pp->radius, prm->eps);                                 \
					if (por >= (REALT)1.0) continue;                                                         \
					REALT mom[3] = {0, 0, 0};                                                                \
					for (int i = 0; i < Q; ++i) {                                                            \
						int e0 = ko_lattice_dir(h, i, 0), e1 = ko_lattice_dir(h, i, 1), e2 = ko_lattice_dir(h, i, 2); \
						double upe_d = 0.0;                                                                  \
						upe_d = upe_d + (double)e0 * vp[0];                                                  \
						upe_d = upe_d + (double)e1 * vp[1];                                                  \
						if (D == 3) upe_d = upe_d + (double)e2 * vp[2];                                      \
						REALT upe = (REALT)upe_d;                                                            \
						int64_t nx_ = x + e0, ny_ = iy + e1, nz_ = iz + e2;                                  \
						if (per) nx_ = (nx_ + nx) % nx;                                                      \
						REALT fi = POP(h, x, iy, iz, i);                                                     \
						REALT fo = POP(h, nx_, ny_, nz_, ko_lattice_opp(h, i));                              \
						REALT da = fi * ((REALT)1.0 - upe) + fo * ((REALT)1.0 + upe);                        \
						mom[0] = mom[0] + (REALT)e0 * da;                                                    \
						mom[1] = mom[1] + (REALT)e1 * da;                                                    \
						if (D == 3) mom[2] = mom[2] + (REALT)e2 * da;                                        \
					}                                                                                        \
					double F[3] = {0, 0, 0};                                                                 \
					for (int k = 0; k < D; ++k) F[k] = (double)mom[k];                                       \
					if (cell_force)                                                                          \
						for (int k = 0; k < D; ++k) cell_force[c * D + k] = F[k];                            \
					for (int k = 0; k < D; ++k) fsum[k] = fsum[k] - F[k];                                    \
					if (D == 2) {                                                                            \
						tsum[0] = tsum[0] - (r[0] * F[1] - r[1] * F[0]);                                     \
					} else {                                                                                 \
						tsum[0] = tsum[0] - (r[1] * F[2] - r[2] * F[1]);                                     \
						tsum[1] = tsum[1] - (r[2] * F[0] - r[0] * F[2]);                                     \
						tsum[2] = tsum[2] - (r[0] * F[1] - r[1] * F[0]);                                     \
					}                                                                                        \
				}                                                                                            \
		for (int k = 0; k < D; ++k) pp->force[k] = pp->force[k] + fsum[k];                                   \
		for (int k = 0; k < (D == 2 ? 1 : 3); ++k) pp->torque[k] = pp->torque[k] + tsum[k];                  \
	}

void ko_particles_hlbm_gather(ko_lattice *h, kel_particle_state *P, int np, const kel_particle_params *prm,
							  double *cell_force) {
	int D, Q, f64, per;
	int64_t nx, ny, nz;
	ko_lattice_info(h, &D, &Q, &nx, &ny, &nz, &f64, &per);
	int64_t ext[3] = {nx, ny, nz};
	int steps = prm->sub_steps == 0 ? 1 : prm->sub_steps; /* hlbm.hpp:148-151 */
	if (f64) {
		KO_HLBM_GATHER_BODY(double, ko_lattice_pop)
	} else {
		KO_HLBM_GATHER_BODY(float, ko_lattice_pop_f32)
	}
}

/* HlbmOneParticleStamp (hlbm.hpp:269-311), after the integrate: over each
 * body's (post-move) AABB, in body order, D += 1 - por and N += u_p (1 - por)
 * with u_p = (X - X_old) sub_steps and por the porosity field. */
void ko_particles_hlbm_stamp(ko_lattice *h, const kel_particle_state *P, int np, const kel_particle_params *prm) {
	int D, Q, f64, per;
	int64_t nx, ny, nz;
	ko_lattice_info(h, &D, &Q, &nx, &ny, &nz, &f64, &per);
	int64_t ext[3] = {nx, ny, nz};
	int steps = prm->sub_steps == 0 ? 1 : prm->sub_steps;
	double ts = 1.0 / (double)steps;
	for (int p = 0; p < np; ++p) {
		int64_t a[3] = {0, 0, 0}, b[3] = {1, 1, 1};
		aabb(D, &P[p], ext, per, 0, a, b);
		double vp[3] = {0, 0, 0};
		for (int k = 0; k < D; ++k) vp[k] = (P[p].position[k] - P[p].position_old[k]) / ts;
		for (int64_t ix = a[0]; ix < b[0]; ++ix)
			for (int64_t iy = a[1]; iy < b[1]; ++iy)
				for (int64_t iz = (D == 3 ? a[2] : 0); iz < (D == 3 ? b[2] : 1); ++iz) {
					int64_t x = per ? ((ix % nx) + nx) % nx : ix;
					int64_t c = x + nx * (iy + ny * iz);
					double flip;
					double vf[3] = {0, 0, 0};
					if (f64) {
						flip = 1.0 - ko_lattice_porosity_at(h, c);
						for (int k = 0; k < D; ++k) vf[k] = vp[k] * flip;
					} else {
						float fl = 1.0f - (float)ko_lattice_porosity_at(h, c);
						flip = fl;
						for (int k = 0; k < D; ++k) vf[k] = (double)((float)vp[k] * fl);
					}
					ko_lattice_hlbm_add_at(h, c, vf, flip);
				}
	}
}

/* reset_particle_accumulators, integrate.hpp:195-212 */
void ko_particles_reset(kel_particle_state *P, int np) {
	for (int p = 0; p < np; ++p)
		for (int k = 0; k < 3; ++k) {
			P[p].force[k] = 0.0;
			P[p].torque[k] = 0.0;
		}
}

/* ---- DEM contact (contact.hpp) ---------------------------------------- */

static int safe_normalize(int D, const double *in, double *out) {
	double l2 = 0.0;
	for (int k = 0; k < D; ++k) l2 = l2 + in[k] * in[k];
	if (!(l2 > 0)) return 0;
	double inv = 1.0 / sqrt(l2);
	for (int k = 0; k < D; ++k) out[k] = in[k] * inv;
	return 1;
}

static void surface_velocity(int D, const kel_particle_state *p, const double *r, double steps, double *v) {
	for (int k = 0; k < D; ++k) v[k] = (p->position[k] - p->position_old[k]) * steps;
	if (D == 2) {
		double om = (p->rotation[0] - p->rotation_old[0]) * steps;
		double t0 = -(om * r[1]), t1 = om * r[0];
		v[0] = v[0] + t0;
		v[1] = v[1] + t1;
	} else {
		double om[3];
		for (int k = 0; k < 3; ++k) om[k] = (p->rotation[k] - p->rotation_old[k]) * steps;
		double t[3] = {om[1] * r[2] - om[2] * r[1], om[2] * r[0] - om[0] * r[2], om[0] * r[1] - om[1] * r[0]};
		for (int k = 0; k < 3; ++k) v[k] = v[k] + t[k];
	}
}

/* soft_shell_response, contact.hpp:204-264; returns force and torque on self */
static void soft_shell(int D, const double *n, double depth, const double *r_self, const double *v_rel, double m_eff,
					   const kel_particle_params *dem, double *F, double *T) {
	double k_n = dem->k_n, zeta = dem->zeta_n;
	double g_n = 2.0 * zeta * sqrt(m_eff * k_n);
	double v_n = 0.0;
	for (int k = 0; k < D; ++k) v_n = v_n + v_rel[k] * n[k];
	double f_n = k_n * depth - g_n * v_n;
	if (f_n < 0) f_n = 0;
	double v_t[3] = {0, 0, 0}, t_hat[3] = {0, 0, 0};
	for (int k = 0; k < D; ++k) v_t[k] = v_rel[k] - v_n * n[k];
	int have_t = safe_normalize(D, v_t, t_hat);
	double vtt = 0.0;
	for (int k = 0; k < D; ++k) vtt = vtt + v_t[k] * v_t[k];
	double v_t_len = sqrt(vtt);
	double f_t = dem->gamma_t * v_t_len;
	double f_t_cap = dem->mu * f_n;
	if (f_t > f_t_cap) f_t = f_t_cap;
	for (int k = 0; k < D; ++k) {
		double v = f_n * n[k];
		if (have_t) v -= f_t * t_hat[k];
		F[k] = v;
	}
	if (D == 2) {
		T[0] = r_self[0] * F[1] - r_self[1] * F[0];
	} else {
		T[0] = r_self[1] * F[2] - r_self[2] * F[1];
		T[1] = r_self[2] * F[0] - r_self[0] * F[2];
		T[2] = r_self[0] * F[1] - r_self[1] * F[0];
	}
}

/* Difference pos_a - pos_b, nearest image along periodic x. */
static void pdiff(int D, const double *a, const double *b, int per, double Lx, double *d) {
	for (int k = 0; k < D; ++k) d[k] = a[k] - b[k];
	if (per) {
		if (d[0] > 0.5 * Lx) d[0] -= Lx;
		else if (d[0] < -0.5 * Lx) d[0] += Lx;
	}
}

/* accumulate_particle_contacts + accumulate_box_wall_contacts for every
 * particle, all from the same (pre-integration) positions. */
void ko_particles_contact(kel_particle_state *P, int np, int D, const kel_particle_params *prm, const int64_t *ext,
						  int periodic_x) {
	double steps = (double)(prm->sub_steps == 0 ? 1 : prm->sub_steps);
	double Lx = (double)ext[0];
	/* positions and velocities are read from a snapshot, so every particle
	 * sees the same pre-contact state; forces accumulate in place in the
	 * reference's order (pairs by index, then walls) */
	kel_particle_state *S = malloc((size_t)np * sizeof(*S));
	memcpy(S, P, (size_t)np * sizeof(*S));
	for (int s = 0; s < np; ++s) {
		const kel_particle_state *self = &S[s];
		for (int j = 0; j < np; ++j) {
			if (j == s) continue;
			const kel_particle_state *other = &S[j];
			/* broadphase (particle.hpp:248-271), self first */
			double dd[3] = {0, 0, 0};
			pdiff(D, self->position, other->position, periodic_x, Lx, dd);
			double n2 = 0.0;
			for (int k = 0; k < D; ++k) n2 = n2 + dd[k] * dd[k];
			double rl = self->radius, rr = other->radius;
			if (!(n2 < rl * rl + rr * rr + rr * rl * 2.0)) continue;
			int self_is_lo = s < j;
			const kel_particle_state *lo = self_is_lo ? self : other, *hi = self_is_lo ? other : self;
			/* narrow phase (contact.hpp:110-185) */
			double d[3] = {0, 0, 0};
			pdiff(D, lo->position, hi->position, periodic_x, Lx, d);
			double len2 = 0.0;
			for (int k = 0; k < D; ++k) len2 = len2 + d[k] * d[k];
			double sum_r = lo->radius + hi->radius;
			if (!(len2 < sum_r * sum_r)) continue;
			double len = sqrt(len2);
			double depth = sum_r - len;
			double cap = (lo->radius < hi->radius) ? lo->radius : hi->radius;
			if (depth > cap) depth = cap;
			double n[3] = {0, 0, 0};
			if (!safe_normalize(D, d, n)) {
				for (int k = 0; k < D; ++k) n[k] = 0;
				n[0] = 1;
			}
			/* contact point in hi's frame: pos_hi + n (r_hi - depth/2) */
			double off[3];
			for (int k = 0; k < D; ++k) off[k] = n[k] * (hi->radius - depth * 0.5);
			if (!self_is_lo)
				for (int k = 0; k < D; ++k) n[k] = -n[k];
			/* r_s = point - pos_s, r_o = point - pos_o (pos_hi + off relative to each) */
			double r_s[3], r_o[3];
			for (int k = 0; k < D; ++k) {
				double pt = hi->position[k] + off[k];
				r_s[k] = pt - self->position[k];
				r_o[k] = pt - other->position[k];
			}
			if (periodic_x) { /* bring the offsets to the nearest image */
				if (r_s[0] > 0.5 * Lx) r_s[0] -= Lx; else if (r_s[0] < -0.5 * Lx) r_s[0] += Lx;
				if (r_o[0] > 0.5 * Lx) r_o[0] -= Lx; else if (r_o[0] < -0.5 * Lx) r_o[0] += Lx;
			}
			double v_s[3], v_o[3], v_rel[3];
			surface_velocity(D, self, r_s, steps, v_s);
			surface_velocity(D, other, r_o, steps, v_o);
			for (int k = 0; k < D; ++k) v_rel[k] = v_s[k] - v_o[k];
			double m_eff = (self->mass * other->mass) / (self->mass + other->mass);
			double f[3] = {0, 0, 0}, t[3] = {0, 0, 0};
			soft_shell(D, n, depth, r_s, v_rel, m_eff, prm, f, t);
			for (int k = 0; k < D; ++k) P[s].force[k] = P[s].force[k] + f[k];
			if (D == 2) P[s].torque[0] = P[s].torque[0] + t[0];
		}
		/* box walls, contact.hpp:407-456, on the axes selected */
		for (int ax = 0; ax < D; ++ax) {
			if (!(prm->wall_axes & (1u << ax))) continue;
			double x = self->position[ax], r = self->radius, hb = (double)ext[ax];
			for (int side = 0; side < 2; ++side) {
				double depth = side == 0 ? (r - x) : (x - (hb - r));
				if (!(depth > 0)) continue;
				if (depth > r) depth = r;
				double n[3] = {0, 0, 0}, pt[3];
				for (int k = 0; k < D; ++k) pt[k] = self->position[k];
				n[ax] = side == 0 ? 1.0 : -1.0;
				pt[ax] = side == 0 ? 0.0 : hb;
				double r_s[3], v[3];
				for (int k = 0; k < D; ++k) r_s[k] = pt[k] - self->position[k];
				surface_velocity(D, self, r_s, steps, v);
				double f[3] = {0, 0, 0}, t[3] = {0, 0, 0};
				soft_shell(D, n, depth, r_s, v, self->mass, prm, f, t);
				for (int k = 0; k < D; ++k) P[s].force[k] = P[s].force[k] + f[k];
				if (D == 2) P[s].torque[0] = P[s].torque[0] + t[0];
			}
		}
	}
	free(S);
}

/* integrate_particle + verlet_step_lambda (integrate.hpp:45-83,
 * particle.hpp:171-211); periodic x wraps the position pair. */
void ko_particles_integrate(kel_particle_state *P, int np, int D, const kel_particle_params *prm, const int64_t *ext,
							int periodic_x) {
	int steps = prm->sub_steps == 0 ? 1 : prm->sub_steps;
	double ts = 1.0 / (double)steps;
	for (int p = 0; p < np; ++p) {
		kel_particle_state *q = &P[p];
		for (int k = 0; k < D; ++k) q->acceleration[k] = q->force[k] / q->mass + prm->body_acceleration[k];
		if (D == 2) q->angular_acceleration[0] = q->torque[0] / q->inertia;
		for (int s = 0; s < steps; ++s) {
			double t2 = ts * ts;
			for (int k = 0; k < D; ++k) {
				double nw = q->position[k] * 2.0 - q->position_old[k] + q->acceleration[k] * t2;
				q->position_old[k] = q->position[k];
				q->position[k] = nw;
			}
			int nr = D == 2 ? 1 : 3;
			for (int k = 0; k < nr; ++k) {
				double nw = q->rotation[k] * 2.0 - q->rotation_old[k] + q->angular_acceleration[k] * t2;
				q->rotation_old[k] = q->rotation[k];
				q->rotation[k] = nw;
			}
		}
		if (periodic_x) {
			double L = (double)ext[0];
			if (q->position[0] >= L) {
				q->position[0] -= L;
				q->position_old[0] -= L;
			} else if (q->position[0] < 0.0) {
				q->position[0] += L;
				q->position_old[0] += L;
			}
		}
	}
}
