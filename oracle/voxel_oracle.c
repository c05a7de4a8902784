/*
 * voxel_oracle.c -- CPU restatement of keldu/lbm_mirror's voxel signed
 * distance bodies.  TEST INFRASTRUCTURE ONLY: the oracle the CUDA voxel
 * kernels are checked against.
 *
 * Reference files restated (paths inside keldu/lbm_mirror):
 *   mask convention, transforms  modules/core/c++/particle/mask.hpp:11-180
 *   n-linear sample               modules/core/c++/particle/mask.hpp:194-264
 *   signed distance               modules/core/c++/particle/mask.hpp:270-282
 *   cos^2 solid fraction          modules/core/c++/particle/mask.hpp:291-311
 *   sphere / cube SDFs            modules/core/c++/particle/mask.hpp:316-341
 *   mask fill + centroid          modules/core/c++/particle/mask.hpp:351-394
 *   voxel porosity                modules/core/c++/particle/porosity.hpp:24-54
 *   voxel narrow phase            modules/core/c++/particle/voxel_narrow.hpp:45-259
 *   vector dot / cross order      modules/core/c++/abstract/math.hpp:40-49,203-215
 *
 * Masks are R^D doubles with the LAST axis fastest (mask[(k0 R + k1) R + k2]),
 * the order the reference's iterator<D> visits them (axis 0 outermost).
 *
 * Two precisions:
 *   FP64 -- the reference's T = Float64 functions, operation for operation
 *           (pinned against the reference harness's fixtures);
 *   FP32 -- the couple's voxel porosity as the CUDA couple computes it (no
 *           reference counterpart: the reference stamps only analytic spheres
 *           into the lattice): the cell's offset from the body formed as an
 *           exact integer part plus the body's fraction, the inverse rotation
 *           as a matrix rounded to float, then the sample and the ramp in
 *           float with the reference's order of operations.
 * The voxel couple box (no reference counterpart) is the sub-cell style box
 * of radius R * reach + eps / 2, reach the mask's extent (ko_mask_reach).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/kel_lbm_cuda.h"

#ifndef KO_PI
#define KO_PI 3.14159265358979323846
#endif

static int64_t ipow(int64_t r, int d) {
	int64_t n = 1;
	for (int i = 0; i < d; ++i) n *= r;
	return n;
}

/* ---- FP64: the reference's functions ---------------------------------------- */

/* solid_fraction_from_sdf (mask.hpp:291-311) */
double ko_solid_fraction(double sdf, double eps) {
	double half = eps / 2;
	if (sdf <= -half) return 1;
	if (sdf >= half) return 0;
	double t = (sdf + half) / eps;
	double c = cos(KO_PI * t / 2);
	return c * c;
}

/* mask_voxel_to_local (mask.hpp:111-125) for flat voxel index k */
static void voxel_to_local(int D, int R, int64_t k, double *u) {
	double step = 2.0 / (double)R;
	int64_t idx[3] = {0, 0, 0};
	for (int i = D - 1; i >= 0; --i) {
		idx[i] = k % R;
		k /= R;
	}
	for (int i = 0; i < D; ++i) u[i] = -1 + ((double)idx[i] + 0.5) * step;
}

static double sdf_shape(int D, int kind, const double *u) {
	if (kind == KEL_SHAPE_CUBE) { /* sdf::cube: Chebyshev distance - 1 */
		double m = 0;
		for (int i = 0; i < D; ++i) {
			double a = fabs(u[i]);
			if (a > m) m = a;
		}
		return m - 1;
	}
	double d = 0; /* sdf::sphere: sqrt(dot(u, u)) - 1 */
	for (int i = 0; i < D; ++i) d = d + u[i] * u[i];
	return sqrt(d) - 1;
}

/* fill_mask_from_sdf (mask.hpp:351-394): the mask and its solid-fraction
 * weighted centroid (one-voxel ramp), voxels in iteration order. */
void ko_mask_fill(int D, int R, int kind, double *mask, double *com) {
	double step = 2.0 / (double)R, wsum = 0;
	double c[3] = {0, 0, 0};
	int64_t n = ipow(R, D);
	for (int64_t k = 0; k < n; ++k) {
		double u[3] = {0, 0, 0};
		voxel_to_local(D, R, k, u);
		double d = sdf_shape(D, kind, u);
		mask[k] = d;
		double w = ko_solid_fraction(d, step);
		wsum += w;
		for (int i = 0; i < D; ++i) c[i] = c[i] + w * u[i];
	}
	if (wsum > 0)
		for (int i = 0; i < D; ++i) c[i] = c[i] / wsum;
	for (int i = 0; i < 3; ++i) com[i] = i < D ? c[i] : 0.0;
}

/* Normalised extent of the body: the largest |u| over the voxels whose
 * distance is <= 0, plus one voxel diagonal (0 for a mask with no such
 * voxel).  The voxel couple visits the cells within R * reach + eps / 2. */
double ko_mask_reach(int D, int R, const double *mask) {
	double best = -1.0;
	int64_t n = ipow(R, D);
	for (int64_t k = 0; k < n; ++k) {
		if (!(mask[k] <= 0.0)) continue;
		double u[3] = {0, 0, 0};
		voxel_to_local(D, R, k, u);
		double s = 0;
		for (int i = 0; i < D; ++i) s = s + u[i] * u[i];
		s = sqrt(s);
		if (s > best) best = s;
	}
	if (best < 0) return 0.0;
	return best + (2.0 / (double)R) * sqrt((double)D);
}

/* mask_sample_local (mask.hpp:194-264) */
double ko_mask_sample_local(int D, int R, const double *mask, const double *u) {
	double step = 2.0 / (double)R;
	double frac[3];
	int64_t base[3];
	double outside = 0;
	for (int i = 0; i < D; ++i) {
		double g = (u[i] + 1) / step - 0.5;
		if (g < 0) {
			outside += g * g * step * step;
			g = 0;
		} else if (g > (double)(R - 1)) {
			double over = g - (double)(R - 1);
			outside += over * over * step * step;
			g = (double)(R - 1);
		}
		double f = floor(g);
		base[i] = (int64_t)f;
		if (base[i] > (int64_t)R - 2) {
			base[i] = (int64_t)R - 2;
			if (base[i] < 0) base[i] = 0;
		}
		frac[i] = g - (double)base[i];
	}
	int corners = 1 << D;
	double acc = 0;
	for (int c = 0; c < corners; ++c) {
		double w = 1;
		int64_t flat = 0;
		for (int i = 0; i < D; ++i) {
			int hi = (c >> i) & 1;
			int64_t idx = base[i] + (hi ? 1 : 0);
			if (idx < 0) idx = 0;
			if (idx > (int64_t)R - 1) idx = (int64_t)R - 1;
			flat = flat * R + idx;
			w *= hi ? frac[i] : (1 - frac[i]);
		}
		acc += w * mask[flat];
	}
	if (outside > 0) acc += sqrt(outside);
	return acc;
}

/* impl::mask_rotate (mask.hpp:52-105): 2D by the angle rot[0], 3D by the
 * rotation vector rot (Rodrigues); inverse rotates by the negative angle. */
static void mask_rotate(int D, const double *v, const double *rot, int inverse, double *out) {
	if (D == 2) {
		double a = rot[0];
		if (inverse) a = -a;
		double c = cos(a), s = sin(a);
		out[0] = v[0] * c - v[1] * s;
		out[1] = v[0] * s + v[1] * c;
		return;
	}
	double th2 = 0;
	for (int i = 0; i < 3; ++i) th2 = th2 + rot[i] * rot[i];
	if (!(th2 > 0)) {
		for (int i = 0; i < 3; ++i) out[i] = v[i];
		return;
	}
	double th = sqrt(th2);
	if (inverse) th = -th;
	double n[3];
	for (int i = 0; i < 3; ++i) n[i] = rot[i] / sqrt(th2);
	double c = cos(th), s = sin(th);
	double ndv = 0;
	for (int i = 0; i < 3; ++i) ndv = ndv + n[i] * v[i];
	double cr[3] = {n[1] * v[2] - n[2] * v[1], n[2] * v[0] - n[0] * v[2], n[0] * v[1] - n[1] * v[0]};
	for (int i = 0; i < 3; ++i) out[i] = v[i] * c + cr[i] * s + n[i] * ndv * (1 - c);
}

/* mask_global_to_local (mask.hpp:158-180) */
static void global_to_local(int D, const kel_particle_state *p, const double *com, const double *x, double *u) {
	double rel[3] = {0, 0, 0}, un[3] = {0, 0, 0};
	for (int i = 0; i < D; ++i) rel[i] = (x[i] - p->position[i]) / p->radius;
	mask_rotate(D, rel, p->rotation, 1, un);
	for (int i = 0; i < D; ++i) u[i] = un[i] + com[i];
}

/* mask_local_to_global (mask.hpp:130-152) */
void ko_mask_local_to_global(int D, const kel_particle_state *p, const double *com, const double *u, double *x) {
	double rel[3] = {0, 0, 0}, r[3] = {0, 0, 0};
	for (int i = 0; i < D; ++i) rel[i] = u[i] - com[i];
	mask_rotate(D, rel, p->rotation, 0, r);
	for (int i = 0; i < D; ++i) x[i] = p->position[i] + p->radius * r[i];
}

/* mask_signed_distance (mask.hpp:270-282), lattice units */
double ko_mask_signed_distance(int D, int R, const double *mask, const double *com, const kel_particle_state *p,
							   const double *x) {
	double u[3] = {0, 0, 0};
	global_to_local(D, p, com, x, u);
	return ko_mask_sample_local(D, R, mask, u) * p->radius;
}

/* particle_porosity<T,D,PC,ParticleVoxel>::calculate (porosity.hpp:30-54) */
double ko_voxel_porosity(int D, int R, const double *mask, const double *com, const kel_particle_state *p,
						 const double *x, double eps) {
	return 1 - ko_solid_fraction(ko_mask_signed_distance(D, R, mask, com, p, x), eps);
}

/* impl::sdf_gradient (voxel_narrow.hpp:45-68) */
static void sdf_gradient(int D, int R, const double *mask, const double *com, const kel_particle_state *p,
						 const double *x, double h, double *g) {
	for (int i = 0; i < D; ++i) {
		double lo[3] = {x[0], x[1], x[2]}, hi[3] = {x[0], x[1], x[2]};
		lo[i] = x[i] - h;
		hi[i] = x[i] + h;
		double d_lo = ko_mask_signed_distance(D, R, mask, com, p, lo);
		double d_hi = ko_mask_signed_distance(D, R, mask, com, p, hi);
		g[i] = (d_hi - d_lo) / (2 * h);
	}
}

static int safe_normalize(int D, const double *in, double *out) {
	double l2 = 0;
	for (int i = 0; i < D; ++i) l2 = l2 + in[i] * in[i];
	if (!(l2 > 0)) return 0;
	double inv = 1.0 / sqrt(l2);
	for (int i = 0; i < D; ++i) out[i] = in[i] * inv;
	return 1;
}

/* voxel_contact (voxel_narrow.hpp:78-259): lattice cells of the clamped
 * intersection of the two bounding boxes, axis 0 outermost.  Returns hit. */
int ko_voxel_contact(int D, int R, const double *mask, const double *com, const kel_particle_state *lo,
					 const kel_particle_state *hi, const int64_t *extent, double eps, kel_contact_manifold *out) {
	int64_t start[3] = {0, 0, 0}, stop[3] = {1, 1, 1};
	memset(out, 0, sizeof(*out));
	for (int i = 0; i < D; ++i) {
		double a_lo = lo->position[i] - lo->radius, a_hi = hi->position[i] - hi->radius;
		double a = a_lo > a_hi ? a_lo : a_hi;
		double b_lo = lo->position[i] + lo->radius, b_hi = hi->position[i] + hi->radius;
		double b = b_lo < b_hi ? b_lo : b_hi;
		if (a < 0) a = 0;
		int64_t ai = (int64_t)floor(a);
		int64_t bi = (int64_t)ceil(b) + 1;
		if (ai < 0) ai = 0;
		if (bi > extent[i]) bi = extent[i];
		if (bi <= ai) return 0;
		start[i] = ai;
		stop[i] = bi;
	}
	double volume = 0, centroid[3] = {0, 0, 0}, grad[3] = {0, 0, 0};
	const double h = 0.5;
	for (int64_t c0 = start[0]; c0 < stop[0]; ++c0)
		for (int64_t c1 = start[1]; c1 < stop[1]; ++c1)
			for (int64_t c2 = start[2]; c2 < stop[2]; ++c2) {
				double x[3] = {(double)c0, (double)c1, D == 3 ? (double)c2 : 0.0};
				double s_lo = ko_solid_fraction(ko_mask_signed_distance(D, R, mask, com, lo, x), eps);
				if (!(s_lo > 0)) continue;
				double s_hi = ko_solid_fraction(ko_mask_signed_distance(D, R, mask, com, hi, x), eps);
				if (!(s_hi > 0)) continue;
				double w = s_lo * s_hi;
				volume += w;
				for (int i = 0; i < D; ++i) centroid[i] = centroid[i] + w * x[i];
				double g_lo[3], g_hi[3];
				sdf_gradient(D, R, mask, com, lo, x, h, g_lo);
				sdf_gradient(D, R, mask, com, hi, x, h, g_hi);
				for (int i = 0; i < D; ++i) grad[i] = grad[i] + w * (g_hi[i] - g_lo[i]);
			}
	if (!(volume > 0)) return 0;
	for (int i = 0; i < D; ++i) centroid[i] = centroid[i] / volume;
	double n[3] = {0, 0, 0};
	if (!safe_normalize(D, grad, n)) {
		double fb[3] = {0, 0, 0};
		for (int i = 0; i < D; ++i) fb[i] = lo->position[i] - hi->position[i];
		if (!safe_normalize(D, fb, n)) {
			for (int i = 0; i < D; ++i) n[i] = 0;
			n[0] = 1;
		}
	}
	double s_min = 0, s_max = 0;
	int first = 1;
	for (int64_t c0 = start[0]; c0 < stop[0]; ++c0)
		for (int64_t c1 = start[1]; c1 < stop[1]; ++c1)
			for (int64_t c2 = start[2]; c2 < stop[2]; ++c2) {
				double x[3] = {(double)c0, (double)c1, D == 3 ? (double)c2 : 0.0};
				if (!(ko_solid_fraction(ko_mask_signed_distance(D, R, mask, com, lo, x), eps) > 0.5)) continue;
				if (!(ko_solid_fraction(ko_mask_signed_distance(D, R, mask, com, hi, x), eps) > 0.5)) continue;
				double s = 0;
				for (int i = 0; i < D; ++i) s = s + x[i] * n[i];
				if (first) {
					s_min = s;
					s_max = s;
					first = 0;
				} else {
					if (s < s_min) s_min = s;
					if (s > s_max) s_max = s;
				}
			}
	double depth = first ? 1.0 : (s_max - s_min + 1.0);
	double cap = lo->radius < hi->radius ? lo->radius : hi->radius;
	if (depth > cap) depth = cap;
	out->hit = 1;
	out->depth = depth;
	for (int i = 0; i < D; ++i) {
		out->normal[i] = n[i];
		out->point[i] = centroid[i];
	}
	return 1;
}

/* ---- FP32: the voxel couple ------------------------------------------------ */

/* The body's prepared inverse transform: M = Rot(-theta) as a 3x3 matrix
 * (2D: [[c, -s], [s, c]] with c = cos(-theta), s = sin(-theta); 3D: the
 * Rodrigues matrix of the rotation vector with the negated angle), computed
 * in double and rounded to float. */
void ko_voxel_prepare(int D, const double *rot, float *M) {
	double m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
	if (D == 2) {
		double a = -rot[0];
		double c = cos(a), s = sin(a);
		m[0] = c;
		m[1] = -s;
		m[3] = s;
		m[4] = c;
	} else {
		double th2 = 0;
		for (int i = 0; i < 3; ++i) th2 = th2 + rot[i] * rot[i];
		if (th2 > 0) {
			double th = -sqrt(th2);
			double n[3];
			for (int i = 0; i < 3; ++i) n[i] = rot[i] / sqrt(th2);
			double c = cos(th), s = sin(th);
			/* out = v c + (n x v) s + n (n . v)(1 - c) */
			double K[9] = {0, -n[2], n[1], n[2], 0, -n[0], -n[1], n[0], 0};
			for (int i = 0; i < 3; ++i)
				for (int j = 0; j < 3; ++j) m[i * 3 + j] = (i == j ? c : 0.0) + K[i * 3 + j] * s + n[i] * n[j] * (1 - c);
		}
	}
	for (int i = 0; i < 9; ++i) M[i] = (float)m[i];
}

/* Float sample of the mask (float copy), mask_sample_local's operations. */
float ko_mask_sample_local_f32(int D, int R, const float *mask, const float *u) {
	const float step = 2.0f / (float)R;
	float frac[3];
	int base[3];
	float outside = 0.0f;
	for (int i = 0; i < D; ++i) {
		float g = (u[i] + 1.0f) / step - 0.5f;
		if (g < 0.0f) {
			outside += g * g * step * step;
			g = 0.0f;
		} else if (g > (float)(R - 1)) {
			float over = g - (float)(R - 1);
			outside += over * over * step * step;
			g = (float)(R - 1);
		}
		base[i] = (int)floorf(g);
		if (base[i] > R - 2) {
			base[i] = R - 2;
			if (base[i] < 0) base[i] = 0;
		}
		frac[i] = g - (float)base[i];
	}
	float acc = 0.0f;
	for (int c = 0; c < (1 << D); ++c) {
		float w = 1.0f;
		int flat = 0;
		for (int i = 0; i < D; ++i) {
			int hi = (c >> i) & 1;
			int idx = base[i] + hi;
			if (idx < 0) idx = 0;
			if (idx > R - 1) idx = R - 1;
			flat = flat * R + idx;
			w *= hi ? frac[i] : (1.0f - frac[i]);
		}
		acc += w * mask[flat];
	}
	if (outside > 0.0f) acc += sqrtf(outside);
	return acc;
}

/* The couple's factor 1 - solid of one body at a cell whose offset from the
 * body centre is r (float, exact integer part plus the body's fraction). */
float ko_voxel_factor_f32(int D, int R, const float *mask, const float *com, const float *M, float scale,
						  const float *r, float eps) {
	float q[3] = {0.f, 0.f, 0.f}, u[3] = {0.f, 0.f, 0.f};
	for (int i = 0; i < D; ++i) q[i] = r[i] / scale;
	for (int i = 0; i < D; ++i) {
		float a = M[i * 3 + 0] * q[0] + M[i * 3 + 1] * q[1];
		if (D == 3) a = a + M[i * 3 + 2] * q[2];
		u[i] = a + com[i];
	}
	float sdf = ko_mask_sample_local_f32(D, R, mask, u) * scale;
	float half = eps / 2.0f;
	float solid;
	if (sdf <= -half) solid = 1.0f;
	else if (sdf >= half) solid = 0.0f;
	else {
		float t = (sdf + half) / eps;
		float c = cosf(3.14159265358979323846f * t / 2.0f);
		solid = c * c;
	}
	return 1.0f - solid;
}

/* The voxel couple over a lattice of ext[0] x ext[1] x ext[2] cells (x
 * fastest in por): every cell starts at 1 and takes, body by body in index
 * order, the factor of each body whose box (sub-cell style, radius
 * R * reach + eps / 2) holds the image of the cell nearest the body. */
void ko_voxel_couple(int D, int R, const double *mask, const double *com, double reach, const kel_particle_state *P,
					 int np, const int64_t *ext, int periodic, double eps, double *por) {
	int64_t nx = ext[0], ny = ext[1], nz = D == 3 ? ext[2] : 1;
	int64_t n = nx * ny * nz, nm = ipow(R, D);
	float *mf = (float *)malloc(sizeof(float) * (size_t)nm);
	for (int64_t k = 0; k < nm; ++k) mf[k] = (float)mask[k];
	float comf[3] = {(float)com[0], (float)com[1], (float)com[2]};
	for (int64_t c = 0; c < n; ++c) por[c] = 1.0;
	for (int p = 0; p < np; ++p) {
		const kel_particle_state *b = &P[p];
		double rr = b->radius * reach + eps / 2;
		int64_t a[3] = {0, 0, 0}, e[3] = {1, 1, 1};
		for (int k = 0; k < D; ++k) {
			a[k] = (int64_t)floor(b->position[k] - rr - 0.5);
			e[k] = (int64_t)ceil(b->position[k] + rr + 0.5) + 1;
			if (!(periodic && k == 0)) {
				if (a[k] < 0) a[k] = 0;
				if (e[k] > ext[k]) e[k] = ext[k];
			}
		}
		float M[9];
		ko_voxel_prepare(D, b->rotation, M);
		int ic[3] = {0, 0, 0};
		float fr[3] = {0.f, 0.f, 0.f};
		for (int k = 0; k < D; ++k) {
			ic[k] = (int)llround(b->position[k]);
			fr[k] = (float)((double)ic[k] - b->position[k]);
		}
		for (int64_t iz = a[2]; iz < e[2]; ++iz)
			for (int64_t iy = a[1]; iy < e[1]; ++iy)
				for (int64_t ix = a[0]; ix < e[0]; ++ix) {
					int64_t x = periodic ? ((ix % nx) + nx) % nx : ix;
					/* the image of x nearest the body must be this one */
					double rel0 = (double)x - b->position[0];
					if (periodic) {
						if (rel0 > 0.5 * (double)nx) rel0 -= (double)nx;
						else if (rel0 < -0.5 * (double)nx) rel0 += (double)nx;
					}
					if (periodic && (int64_t)llround(b->position[0] + rel0) != ix) continue;
					int64_t cc[3] = {x, iy, iz};
					float r[3] = {0.f, 0.f, 0.f};
					for (int k = 0; k < D; ++k) {
						int d = (int)(cc[k] - ic[k]);
						if (k == 0 && periodic) {
							if (d > (int)nx / 2) d -= (int)nx;
							else if (d < -((int)nx / 2)) d += (int)nx;
						}
						r[k] = (float)d + fr[k];
					}
					float f = ko_voxel_factor_f32(D, R, mf, comf, M, (float)b->radius, r, (float)eps);
					int64_t c = x + nx * (iy + ny * (D == 3 ? iz : 0));
					por[c] = por[c] * (double)f;
				}
	}
	free(mf);
}
