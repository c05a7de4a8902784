// Particle coupling and rigid-body kernels (C ABI kel_particles_*).
//
// Reference path (keldu/lbm_mirror), per time step of
// examples/moving_poiseulle_particles_2d_psm_gpu/sim.cpp:176-224:
//   PsmReset + porosity stamp   psm.hpp:20-32, particle/porosity.hpp:56-89
//   PsmOneParticleGather        psm.hpp:95-446 (one work-item per particle,
//                               a serial loop over its AABB)
//   ParticleContact             particle/contact.hpp:466-567 (brute-force pairs)
//   ParticleIntegrate           particle/integrate.hpp:45-83,263-296
// GB300 shape:
//   couple     one thread per cell; each 32x8 tile first culls the bodies
//              whose AABB touches it (in index order), then every cell takes
//              the product of their solid-fraction complements (race free,
//              order fixed);
//   gather     one block per body, cells of its AABB spread over the block,
//              FP64 force/torque per thread, then a fixed-order warp-shuffle +
//              shared-memory reduction (deterministic);
//   contact    one thread per body over all other bodies, FP64;
//   integrate  one thread per body, FP64 position Verlet.
// This file is compiled with -fmad=false: the FP64 contact/integrate
// arithmetic and the float momentum-exchange arithmetic round exactly like
// the reference's (unfused) C++.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "lattice_internal.cuh"

using namespace kel::gb;

// A voxel shape (particle/mask.hpp): the mask on the host (double) and on
// the device (float for the couple, double for the distance and contact
// queries), its centre of mass and normalised reach.
struct kel_shape {
	int dim = 0, res = 0;
	std::vector<double> mask;
	double com[3] = {0, 0, 0};
	double reach = 0.0;
	float *d_mask_f = nullptr;
	double *d_mask_d = nullptr;
};

// Key of the captured coupled step: everything its launches bake in.
struct ParticleGraphKey {
	kel_particle_params prm;
	kel_step_program prog;
	kel::gb::SweepParams sweep;
	void *f, *por, *force, *bodies, *boxes, *partial, *rec;
	const void *shape;
	int n, gather_g, couple_g, cpt, block, direct;
};

struct kel_particles {
	kel_lattice *lat = nullptr;
	int n = 0;
	kel_particle_state *d = nullptr; // device copy of the bodies
	kel_particle_state *d_alt = nullptr; // the coupled step's second body buffer (swapped with d every step)
	float *cell_force = nullptr;     // D planes, allocated on first request
	void *boxes = nullptr;           // per-body integer boxes: current [0, n), previous couple [n, 2n)
	double *partial = nullptr;       // gather partial sums, n x gather_g x 6
	int partial_cap = 0;             // blocks per body the partial buffer holds
	int gather_g = 1;                // blocks per body of the last gather (the partials' layout)
	double max_radius = 0.0;         // largest radius of the uploaded bodies (sizes the launches)
	// value of lat->por_epoch after this set's last PSM couple (0: none); the
	// incremental couple needs the field to be untouched since then
	uint64_t epoch = 0;
	// box bookkeeping between couples: prev_is_last -- prev[] holds the boxes of
	// the last couple (the fused contact + integrate moved them there);
	// cur_fresh -- cur[] holds the boxes of the current positions, for
	// porosity mode cur_mode and ramp width cur_eps
	bool prev_is_last = false, cur_fresh = false;
	int cur_mode = 0;
	double cur_eps = 0.0;
	// the bodies' records for the fused couple + gather (CoupleRec), written by
	// the fused contact + integrate with these parameters
	void *rec = nullptr;
	int rec_mode = -1, rec_steps = 0;
	double rec_eps = 0.0;
	const kel_shape *shape = nullptr; // voxel bodies' shape (KEL_POROSITY_VOXEL)
	cudaGraphExec_t graph = nullptr; // two coupled steps from an even time step
	// fork / join of the captured steps: contact + integrate beside the sweep
	cudaStream_t side = nullptr;
	cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
	ParticleGraphKey key;
};

namespace {

constexpr double PI_D = 3.14159265358979323846;

struct PView {
	const void *f;
	int storage;
	int64_t plane;
	int nx, nxp, ny, nz, D, Q;
	int odd, periodic;
	float *por;
	float *cell_force;
	float *hN, *hD; // HLBM particle_N (D planes) and particle_D
	float *rho, *mom; // macros "density" and "velocity" (FPLBM: momentum), D planes
	float wshift[27];
	// body boxes: radius R * box_mul + box_add (1, 0 but for voxel bodies)
	double box_mul, box_add;
	// sub-cell and voxel factors may skip the FP64 nearest-image test (every
	// box narrower than half the periodic length)
	int direct;
	// voxel shape (KEL_POROSITY_VOXEL): R^D mask as float and double, centre
	// of mass, resolution
	const float *vmask_f;
	const double *vmask_d;
	float vcom_f[3];
	double vcom[3];
	int vres;
};

// ---- geometry shared by couple and gather -----------------------------------

// aabb.hpp:41-84: [a, b) per axis.  Sub-cell mode widens to every cell the
// body can touch; periodic x leaves the x range unclamped (cells wrap).
// Voxel bodies take the sub-cell rule with the radius R * rmul + radd (the
// shape's reach and half the ramp width).
__host__ __device__ inline void body_aabb(int D, const kel_particle_state &p, int nx, int ny, int nz, int periodic,
										  int subcell, int64_t *a, int64_t *b, double rmul = 1.0, double radd = 0.0) {
	const int64_t ext[3] = {nx, ny, nz};
	for (int k = 0; k < 3; ++k) {
		a[k] = 0;
		b[k] = 1;
	}
	for (int k = 0; k < D; ++k) {
		const double X = p.position[k], r = p.radius * rmul + radd;
		if (subcell) {
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

__device__ inline double rel_coord(double cell, double X, int periodic, int n) {
	double r = cell - X;
	if (periodic) {
		const double L = (double)n;
		if (r > 0.5 * L) r -= L;
		else if (r < -0.5 * L) r += L;
	}
	return r;
}

// particle_porosity<T,D,1,ParticleSpheroid>::calculate (porosity.hpp:56-89)
__device__ inline double ramp(double s, double rad, double eps) {
	const double eps_h = eps / 2;
	const double lo = rad - eps_h, hi = rad + eps_h;
	if (s <= lo) return 0.0;
	if (s >= hi) return 1.0;
	const double inner = (PI_D / (2 * eps)) * (s - lo);
	const double c = sin(inner);
	return c * c;
}

// Solid fraction by 4^D point sampling of the cell [x-1/2, x+1/2]^D, in
// FP32: r is the cell centre's offset from the body centre formed as an
// exact integer part plus the body's fraction (see Cand), the sample points
// lie at r + (2 a - 3) / 8 per axis, and a sample is inside when its squared
// distance (summed in axis order) is at most R^2, all rounded to nearest.
__device__ inline double subcell_porosity(int D, const float *r, float rad) {
	const float r2 = __fmul_rn(rad, rad);
	int inside = 0;
	for (int a = 0; a < 4; ++a)
		for (int b = 0; b < 4; ++b)
			for (int g = 0; g < (D == 3 ? 4 : 1); ++g) {
				const float px = __fadd_rn(r[0], (float)(2 * a - 3) * 0.125f);
				const float py = __fadd_rn(r[1], (float)(2 * b - 3) * 0.125f);
				float d2 = __fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py));
				if (D == 3) {
					const float pz = __fadd_rn(r[2], (float)(2 * g - 3) * 0.125f);
					d2 = __fadd_rn(d2, __fmul_rn(pz, pz));
				}
				if (d2 <= r2) ++inside;
			}
	// 1 - inside / 4^D, exact in FP32 (and so equal to the FP64 quotient)
	return (double)(1.0f - (float)inside * (D == 3 ? 0.015625f : 0.0625f));
}

// ---- couple -------------------------------------------------------------------

constexpr int TX = 32, TY = 8, TT = TX * TY;

// Every body's box (body_aabb) once per couple, as integers: the tile cull
// and the per-cell box test then need no FP64 arithmetic (FP64 issues at a
// small fraction of the FP32 rate on this GPU, and the per-tile FP64 cull
// of every body bounded the couple pass).
struct BodyBox {
	int a[3], b[3];
};

// Per body: its box for the current position into cur[i].  With shift, the
// box the previous couple used moves to prev[i] first (the incremental
// couple restores the cells it no longer covers).  With reset, the body's
// force and torque accumulators are zeroed as well (ParticleForceReset,
// integrate.hpp:195-261), which saves a launch per coupled step.
__global__ void k_pre(PView v, kel_particle_state *P, int np, int sub, BodyBox *cur, BodyBox *prev, int boxes,
					  int shift, int reset) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= np) return;
	if (reset)
		for (int k = 0; k < 3; ++k) {
			P[i].force[k] = 0.0;
			P[i].torque[k] = 0.0;
		}
	if (!boxes) return;
	if (shift) prev[i] = cur[i];
	int64_t a[3], b[3];
	body_aabb(v.D, P[i], v.nx, v.ny, v.nz, v.periodic, sub, a, b, v.box_mul, v.box_add);
	BodyBox r;
	for (int k = 0; k < 3; ++k) {
		r.a[k] = (int)a[k];
		r.b[k] = (int)b[k];
	}
	cur[i] = r;
}

// Candidate body of a couple pass, staged in shared memory.
struct Cand {
	BodyBox box;
	double X[3];
	double R;
	// squared-distance limits of the exact shortcuts (see body_factor),
	// formed once per body with the same operations
	double lim_in2, lim_out2;
	// FP32 screen: the centre's nearest lattice point, the offset of that
	// point from the centre, and the limits widened by SCREEN_MARGIN
	int ic[3];
	float fr[3];
	float s_in, s_out;
	float Rf; // the radius rounded to FP32 (the sub-cell and voxel sampling's)
	float M[9]; // voxel bodies: the inverse rotation Rot(-theta), row-major, rounded to FP32
};

// Squared-distance margin of the FP32 screen: far above its own error (the
// offset of a cell from a body is formed from an exact integer part and a
// fraction of at most 1/2, so |s2 - s2_float| stays below ~1e-4 for offsets
// up to ~100 cells) and far below the band the shortcuts leave to FP64.
constexpr float SCREEN_MARGIN = 1e-2f;

// The shortcut limits of body_factor for a body of radius R.
__device__ inline void cand_limits(Cand &c, int sub, double reach, double eps) {
	const double R = c.R;
	if (sub) {
		// margin 1e-3: far above the FP32 rounding of the sampled distances
		const double out_r = R + reach + 1e-3, in_r = R - reach - 1e-3;
		c.lim_out2 = out_r * out_r;
		c.lim_in2 = in_r > 0.0 ? in_r * in_r : -1.0;
	} else {
		const double lo = R - eps / 2, hi = R + eps / 2;
		c.lim_in2 = lo > 0.0 ? lo * lo - 1e-6 : -1.0;
		c.lim_out2 = hi * hi + 1e-6;
	}
	for (int d = 0; d < 3; ++d) {
		c.ic[d] = (int)llround(c.X[d]);
		c.fr[d] = (float)((double)c.ic[d] - c.X[d]);
	}
	c.s_out = (float)c.lim_out2 + SCREEN_MARGIN;
	c.s_in = c.lim_in2 > 0.0 ? (float)c.lim_in2 - SCREEN_MARGIN : -1.0f;
	c.Rf = (float)R;
}

// The voxel candidate's inverse rotation (mask.hpp:52-105 with the negated
// angle) as a matrix: 2D [[c, -s], [s, c]], c = cos(-theta), s = sin(-theta);
// 3D the Rodrigues matrix c I + s [n]x + (1 - c) n n^T of the rotation vector
// with the angle negated.  Formed in FP64, rounded to FP32.
__device__ inline void voxel_matrix(int D, const double *rot, float *M) {
	double m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
	if (D == 2) {
		const double a = -rot[0];
		const double c = cos(a), s = sin(a);
		m[0] = c;
		m[1] = -s;
		m[3] = s;
		m[4] = c;
	} else {
		double th2 = 0.0;
		for (int i = 0; i < 3; ++i) th2 = th2 + rot[i] * rot[i];
		if (th2 > 0.0) {
			const double th = -sqrt(th2);
			double n[3];
			for (int i = 0; i < 3; ++i) n[i] = rot[i] / sqrt(th2);
			const double c = cos(th), s = sin(th);
			const double K[9] = {0, -n[2], n[1], n[2], 0, -n[0], -n[1], n[0], 0};
			for (int i = 0; i < 3; ++i)
				for (int j = 0; j < 3; ++j) m[i * 3 + j] = (i == j ? c : 0.0) + K[i * 3 + j] * s + n[i] * n[j] * (1 - c);
		}
	}
	for (int i = 0; i < 9; ++i) M[i] = (float)m[i];
}

// Couple mode of a pass: 0 ramp, 1 sub-cell with the FP64 shortcut test,
// 2 sub-cell without it (direct), 3 voxel.
__host__ __device__ inline int couple_mode(int porosity_mode, int direct) {
	if (porosity_mode == KEL_POROSITY_SUBCELL) return direct ? 2 : 1;
	return porosity_mode == KEL_POROSITY_VOXEL ? 3 : 0;
}

// A candidate's limits and (voxel mode) its transform.  Voxel bodies have no
// distance shortcut: every cell of the box is sampled.
__device__ inline void cand_prepare(Cand &c, int cm, double reach, double eps, const double *rot, int D) {
	cand_limits(c, cm, reach, eps);
	if (cm == 3) {
		c.lim_in2 = -1.0;
		c.lim_out2 = INFINITY;
		c.s_in = -1.0f;
		c.s_out = INFINITY;
		voxel_matrix(D, rot, c.M);
	}
}

// The voxel mask sampled at body-local u in FP32: mask_sample_local
// (mask.hpp:194-264) with its order of operations, rounded to nearest.
__device__ inline float mask_sample_f32(const float *__restrict__ mask, int D, int R, const float *u) {
	const float step = __fdiv_rn(2.0f, (float)R);
	float frac[3] = {0.f, 0.f, 0.f};
	int base[3] = {0, 0, 0};
	float outside = 0.0f;
	for (int i = 0; i < D; ++i) {
		float g = __fsub_rn(__fdiv_rn(__fadd_rn(u[i], 1.0f), step), 0.5f);
		if (g < 0.0f) {
			outside = __fadd_rn(outside, __fmul_rn(__fmul_rn(__fmul_rn(g, g), step), step));
			g = 0.0f;
		} else if (g > (float)(R - 1)) {
			const float over = __fsub_rn(g, (float)(R - 1));
			outside = __fadd_rn(outside, __fmul_rn(__fmul_rn(__fmul_rn(over, over), step), step));
			g = (float)(R - 1);
		}
		base[i] = (int)floorf(g);
		if (base[i] > R - 2) {
			base[i] = R - 2;
			if (base[i] < 0) base[i] = 0;
		}
		frac[i] = __fsub_rn(g, (float)base[i]);
	}
	float acc = 0.0f;
	for (int c = 0; c < (1 << D); ++c) {
		float w = 1.0f;
		int flat = 0;
		for (int i = 0; i < D; ++i) {
			const int hi = (c >> i) & 1;
			int idx = base[i] + hi;
			if (idx < 0) idx = 0;
			if (idx > R - 1) idx = R - 1;
			flat = flat * R + idx;
			w = __fmul_rn(w, hi ? frac[i] : __fsub_rn(1.0f, frac[i]));
		}
		acc = __fadd_rn(acc, __fmul_rn(w, __ldg(mask + flat)));
	}
	if (outside > 0.0f) acc = __fadd_rn(acc, __fsqrt_rn(outside));
	return acc;
}

// Voxel body factor 1 - solid at a cell whose offset from the body centre is
// r (FP32: exact integer part plus the body's fraction): u = M r / R + com,
// the mask's signed distance times R, then solid_fraction_from_sdf
// (mask.hpp:291-311) with cos^2 in FP32.
__device__ inline float voxel_factor(const PView &v, const Cand &c, const float *r, float eps) {
	const int D = v.D;
	float q[3] = {0.f, 0.f, 0.f}, u[3] = {0.f, 0.f, 0.f};
	for (int i = 0; i < D; ++i) q[i] = __fdiv_rn(r[i], c.Rf);
	for (int i = 0; i < D; ++i) {
		float a = __fadd_rn(__fmul_rn(c.M[i * 3 + 0], q[0]), __fmul_rn(c.M[i * 3 + 1], q[1]));
		if (D == 3) a = __fadd_rn(a, __fmul_rn(c.M[i * 3 + 2], q[2]));
		u[i] = __fadd_rn(a, v.vcom_f[i]);
	}
	const float sdf = __fmul_rn(mask_sample_f32(v.vmask_f, D, v.vres, u), c.Rf);
	const float half = __fmul_rn(eps, 0.5f);
	float solid;
	if (sdf <= -half) {
		solid = 1.0f;
	} else if (sdf >= half) {
		solid = 0.0f;
	} else {
		const float t = __fdiv_rn(__fadd_rn(sdf, half), eps);
		const float cc = cosf(__fmul_rn(__fmul_rn(3.14159265358979323846f, t), 0.5f));
		solid = __fmul_rn(cc, cc);
	}
	return __fsub_rn(1.0f, solid);
}

// Per-body record of the fused couple + gather, written by the pass that
// moved the body (k_contact_integrate), so that the blocks of the next couple
// + gather read what each of them would otherwise form in FP64: the body's
// couple candidate and c_i . u_p per direction rounded to float.
struct CoupleRec {
	Cand cand;
	float upe[27];
};

// psm.hpp:178-184: u_p = (X - X_old) / (1 / sub_steps) with the raw
// sub_steps.  For a power-of-two sub_steps (and 0) the quotient is exactly
// the product (X - X_old) * sub_steps, which needs no FP64 division.
__host__ __device__ inline double wall_velocity(double dx, int steps) {
	if ((steps & (steps - 1)) == 0) return dx * (double)steps;
	return dx / (1.0 / (double)steps);
}

// Body q's factor on the porosity of cell (x, y, z), multiplied into por
// (product of complements, bodies in index order, as couple.hpp:26-58 takes
// it).  A cell none of whose images lies in the body's box is left alone.
// Two exact shortcuts skip the FP64 sampling:
//   sub-cell mode: the 16 (64) samples lie within 3 sqrt(D) / 8 of the cell
//     centre, so a centre farther than R + that radius (+ 1e-3) from the body
//     centre has no sample inside (factor 1) and one nearer than R - radius
//     (- 1e-3) has all inside (factor 0);
//   ramp mode: |r|^2 below (R - eps/2)^2 - 1e-6 gives 0, above
//     (R + eps/2)^2 + 1e-6 gives 1.
// The margins are far above the FP64 rounding of the coordinates, so the
// factors equal those of the full computation bit for bit.  With sub == 2
// (sub-cell mode where every box is narrower than half the periodic length,
// so that the image of the cell in the box is the nearest one) the cells the
// screen leaves go straight to the FP32 sampling: past either shortcut limit
// it gives the shortcut's factor itself.  An FP32 screen
// decides first the cells whose squared distance lies SCREEN_MARGIN beyond
// either limit (the same decision the FP64 test takes there; a cell that
// deep inside has its nearest image in the body's box), so that only cells
// near the limits pay for FP64, which issues at a small fraction of the FP32
// rate on this GPU.
__device__ inline void body_factor(const PView &v, int x, int y, int z, const Cand &c, int sub, double reach,
								   double eps, double &por, bool &touched) {
	const BodyBox &q = c.box;
	// integer pre-filter: no image of the cell (x, x -/+ nx when periodic) in
	// the box means the nearest image is not either
	if (y < q.a[1] || y >= q.b[1] || (v.D == 3 && (z < q.a[2] || z >= q.b[2]))) return;
	const bool in0 = x >= q.a[0] && x < q.b[0];
	const bool inm = v.periodic && x - v.nx >= q.a[0] && x - v.nx < q.b[0];
	const bool inp = v.periodic && x + v.nx >= q.a[0] && x + v.nx < q.b[0];
	if (!(in0 || inm || inp)) return;
	touched = true;
	// the cell's offset from the body in FP32: integer part (nearest image
	// when periodic) plus the body's fraction
	float rf[3];
	{
		int dx = x - c.ic[0];
		if (v.periodic) {
			if (dx > v.nx / 2) dx -= v.nx;
			else if (dx < -(v.nx / 2)) dx += v.nx;
		}
		rf[0] = __fadd_rn((float)dx, c.fr[0]);
		rf[1] = __fadd_rn((float)(y - c.ic[1]), c.fr[1]);
		rf[2] = v.D == 3 ? __fadd_rn((float)(z - c.ic[2]), c.fr[2]) : 0.f;
		if (sub == 3) {
			if (v.periodic && !v.direct) { // the image of the cell nearest the body must be the one in the box
				const int64_t xc = (int64_t)llround(c.X[0] + rel_coord((double)x, c.X[0], 1, v.nx));
				if (xc < q.a[0] || xc >= q.b[0]) return;
			}
			por = por * (double)voxel_factor(v, c, rf, (float)eps);
			return;
		}
		float s2f = __fadd_rn(__fmul_rn(rf[0], rf[0]), __fmul_rn(rf[1], rf[1]));
		if (v.D == 3) s2f = __fadd_rn(s2f, __fmul_rn(rf[2], rf[2]));
		if (s2f > c.s_out) return; // factor 1
		if (s2f < c.s_in) {        // factor 0
			por = por * 0.0;
			return;
		}
		if (sub == 2) {
			por = por * subcell_porosity(v.D, rf, c.Rf);
			return;
		}
	}
	const double X0 = c.X[0], X1 = c.X[1], X2 = c.X[2], R = c.R;
	double rel[3] = {rel_coord((double)x, X0, v.periodic, v.nx), (double)y - X1, v.D == 3 ? (double)z - X2 : 0.0};
	const double xi = X0 + rel[0];
	const int64_t xc = v.periodic ? (int64_t)llround(xi) : x;
	if (xc < q.a[0] || xc >= q.b[0]) return;
	double s2 = 0.0;
	for (int d = 0; d < v.D; ++d) s2 = s2 + rel[d] * rel[d];
	double pp;
	if (sub) {
		if (s2 > c.lim_out2) {
			return; // no sample inside: factor 1
		} else if (s2 < c.lim_in2) {
			pp = 0.0;
		} else {
			pp = subcell_porosity(v.D, rf, c.Rf);
		}
	} else {
		if (s2 < c.lim_in2) pp = 0.0;
		else if (s2 > c.lim_out2) return;
		else pp = ramp(sqrt(s2), R, eps);
	}
	por = por * pp;
	(void)reach;
}

__host__ __device__ inline double subcell_reach(int D) { return D == 3 ? 0.6495190528383290 : 0.5303300858899106; } // 3 sqrt(D) / 8

// Ordered compaction of the bodies [c0, c0 + NT) for which hit is true (one
// thread per body, NT threads) into cand[0 .. *ncand); with rec, the
// candidates are the bodies' prepared records.
template <int NT>
__device__ inline void compact_cands(bool hit, int pi, const BodyBox &bb, const kel_particle_state *P, Cand *cand,
									 int *warp_count, int *ncand, int sub, double reach, double eps, int D,
									 const CoupleRec *rec = nullptr) {
	const int tid = threadIdx.x + threadIdx.y * blockDim.x;
	const unsigned m = __ballot_sync(0xffffffffu, hit);
	if ((tid & 31) == 0) warp_count[tid >> 5] = __popc(m);
	__syncthreads();
	if (tid == 0) {
		int s = 0;
		for (int w = 0; w < NT / 32; ++w) {
			const int c = warp_count[w];
			warp_count[w] = s;
			s += c;
		}
		*ncand = s;
	}
	__syncthreads();
	if (hit && rec) {
		cand[warp_count[tid >> 5] + __popc(m & ((1u << (tid & 31)) - 1u))] = rec[pi].cand;
	} else if (hit) {
		Cand &c = cand[warp_count[tid >> 5] + __popc(m & ((1u << (tid & 31)) - 1u))];
		c.box = bb;
		for (int d = 0; d < 3; ++d) c.X[d] = P[pi].position[d];
		c.R = P[pi].radius;
		cand_prepare(c, sub, reach, eps, P[pi].rotation, D);
	}
	__syncthreads();
}

// Full couple pass.  Per tile of TX x TY cells: an ordered cull of the
// bodies whose box touches the tile, then per cell the product of the
// candidates' factors in body order (body_factor).  Every cell is written.
__global__ void __launch_bounds__(TT) k_couple(PView v, const kel_particle_state *P, const BodyBox *box, int np,
											   int mode, double eps) {
	__shared__ Cand cand[TT];
	__shared__ int warp_count[TT / 32];
	__shared__ int ncand;
	const int tid = threadIdx.y * TX + threadIdx.x;
	const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z = blockIdx.z;
	const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
	const int sub = couple_mode(mode, v.direct);
	const double reach = (sub == 1 || sub == 2) ? subcell_reach(v.D) : 0.0;
	double por = 1.0;
	bool touched = false; // some body's box holds the cell (otherwise por stays exactly 1)
	for (int c0 = 0; c0 < np; c0 += TT) {
		bool hit = false;
		const int pi = c0 + tid;
		BodyBox bb;
		if (pi < np) {
			bb = box[pi];
			const bool yz = bb.a[1] < y0 + TY && bb.b[1] > y0 && (v.D == 2 || (bb.a[2] <= z && bb.b[2] > z));
			bool xs = bb.a[0] < x0 + TX && bb.b[0] > x0;
			if (v.periodic)
				xs = xs || (bb.a[0] < x0 + TX - v.nx && bb.b[0] > x0 - v.nx) || (bb.a[0] < x0 + TX + v.nx && bb.b[0] > x0 + v.nx);
			hit = yz && xs;
		}
		compact_cands<TT>(hit, pi, bb, P, cand, warp_count, &ncand, sub, reach, eps, v.D);
		if (x < v.nx && y < v.ny)
			for (int k = 0; k < ncand; ++k) body_factor(v, x, y, z, cand[k], sub, reach, eps, por, touched);
		__syncthreads();
	}
	if (x < v.nx && y < v.ny) v.por[((int64_t)z * v.ny + y) * v.nxp + x] = touched ? (float)por : 1.0f;
}

__device__ inline int64_t box_cells(const BodyBox &q, int D) {
	const int64_t e0 = q.b[0] - q.a[0], e1 = q.b[1] - q.a[1], e2 = D == 3 ? q.b[2] - q.a[2] : 1;
	return (e0 > 0 && e1 > 0 && e2 > 0) ? e0 * e1 * e2 : 0;
}

// Do boxes p and q share a cell (some periodic image of p when periodic)?
__device__ inline bool boxes_touch(const BodyBox &p, const BodyBox &q, const PView &v) {
	if (!(p.a[1] < q.b[1] && p.b[1] > q.a[1])) return false;
	if (v.D == 3 && !(p.a[2] < q.b[2] && p.b[2] > q.a[2])) return false;
	for (int s = v.periodic ? -1 : 0; s <= (v.periodic ? 1 : 0); ++s)
		if (p.a[0] + s * v.nx < q.b[0] && p.b[0] + s * v.nx > q.a[0]) return true;
	return false;
}

constexpr int RC_CPT = 1; // cells per thread and pass of the region couple (more blocks per body instead)
constexpr int RT = 128;   // threads per block of the region couple

// Incremental couple pass.  Only cells inside some body's box can have a
// porosity other than 1, so after a couple whose boxes were prev[], the new
// field differs from the old one only inside the boxes cur[] u prev[].
// Block (b, .) recomputes the cells of body b's current box and, where it
// moved, of its previous box: each such cell gets the full product over the
// bodies (index order) whose current box holds it, or 1 when none does --
// the same value the full pass writes.  A cell in several bodies' regions is
// written by several blocks with that same value.
__global__ void __launch_bounds__(RT) k_couple_regions(PView v, const kel_particle_state *P, const BodyBox *cur,
													   const BodyBox *prev, int np, int mode, double eps) {
	__shared__ Cand cand[RT];
	__shared__ int warp_count[RT / 32];
	__shared__ int ncand;
	const int tid = threadIdx.x;
	const int b = blockIdx.x;
	const BodyBox A = cur[b], B = prev[b];
	const bool same = A.a[0] == B.a[0] && A.b[0] == B.b[0] && A.a[1] == B.a[1] && A.b[1] == B.b[1] &&
					  (v.D == 2 || (A.a[2] == B.a[2] && A.b[2] == B.b[2]));
	const int64_t n0 = box_cells(A, v.D), n1 = same ? 0 : box_cells(B, v.D);
	const int sub = couple_mode(mode, v.direct);
	const double reach = (sub == 1 || sub == 2) ? subcell_reach(v.D) : 0.0;
	for (int64_t base = (int64_t)blockIdx.y * RT * RC_CPT; base < n0 + n1; base += (int64_t)gridDim.y * RT * RC_CPT) {
		int cx[RC_CPT], cy[RC_CPT], cz[RC_CPT];
		bool ok[RC_CPT], touched[RC_CPT];
		double por[RC_CPT];
#pragma unroll
		for (int j = 0; j < RC_CPT; ++j) {
			const int64_t idx = base + (int64_t)j * RT + tid;
			ok[j] = idx < n0 + n1;
			touched[j] = false;
			por[j] = 1.0;
			cx[j] = cy[j] = cz[j] = 0;
			if (!ok[j]) continue;
			const BodyBox &q = idx < n0 ? A : B;
			const int64_t k = idx < n0 ? idx : idx - n0;
			const int64_t ex = q.b[0] - q.a[0], ey = q.b[1] - q.a[1];
			int ix = q.a[0] + (int)(k % ex);
			cy[j] = q.a[1] + (int)((k / ex) % ey);
			cz[j] = v.D == 3 ? q.a[2] + (int)(k / (ex * ey)) : 0;
			if (v.periodic) ix = ((ix % v.nx) + v.nx) % v.nx;
			cx[j] = ix;
		}
		for (int c0 = 0; c0 < np; c0 += RT) {
			bool hit = false;
			const int pi = c0 + tid;
			BodyBox bb;
			if (pi < np) {
				bb = cur[pi];
				hit = boxes_touch(bb, A, v) || (!same && boxes_touch(bb, B, v));
			}
			compact_cands<RT>(hit, pi, bb, P, cand, warp_count, &ncand, sub, reach, eps, v.D);
#pragma unroll
			for (int j = 0; j < RC_CPT; ++j)
				if (ok[j])
					for (int k = 0; k < ncand; ++k)
						body_factor(v, cx[j], cy[j], cz[j], cand[k], sub, reach, eps, por[j], touched[j]);
			__syncthreads();
		}
#pragma unroll
		for (int j = 0; j < RC_CPT; ++j)
			if (ok[j]) v.por[((int64_t)cz[j] * v.ny + cy[j]) * v.nxp + cx[j]] = touched[j] ? (float)por[j] : 1.0f;
	}
}

// ---- gather ---------------------------------------------------------------------

// Fixed-order block sum of the per-thread force/torque sums acc[0..5]
// (force[3], torque[3]) into out[0..5]: a warp-shuffle tree, then the warps in
// index order.  In 2D only force x, y and torque z can be non-zero; the other
// three are written as +0.0, the value their sums of +0.0 give.  A warp whose
// sums are all +0.0 (no contributing cell: a difference that cancels rounds to
// +0.0, so no sum is ever -0.0) writes +0.0 without the tree.  part: the
// block's NT / 32 x 6 shared scratch.
template <int D, int NT>
__device__ inline void block_sums(const double *acc, double (*part)[6], double *out) {
	constexpr int NQ = D == 2 ? 3 : 6;
	const int tid = threadIdx.x;
	bool nz = false;
#pragma unroll
	for (int j = 0; j < NQ; ++j) nz |= acc[D == 2 && j == 2 ? 3 : j] != 0.0;
	if (__any_sync(0xffffffffu, nz)) {
#pragma unroll
		for (int j = 0; j < NQ; ++j) {
			const int q = D == 2 && j == 2 ? 3 : j;
			double sum = acc[q];
			for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
			if ((tid & 31) == 0) part[tid >> 5][q] = sum;
		}
	} else if ((tid & 31) == 0) {
#pragma unroll
		for (int j = 0; j < NQ; ++j) part[tid >> 5][D == 2 && j == 2 ? 3 : j] = 0.0;
	}
	__syncthreads();
	if (tid < 6) {
		double tot = 0.0;
		if (D == 3 || tid == 0 || tid == 1 || tid == 3)
			for (int w = 0; w < NT / 32; ++w) tot += part[w][tid];
		out[tid] = tot;
	}
}

// Post-stream population f_i at a lattice cell (the buffer the next collide
// reads); outside the lattice the reference's zero ghost ring.
template <class L, int STORE>
__device__ inline float pop_post(const PView &v, int x, int y, int z, int i) {
	if (v.periodic) x = x < 0 ? x + v.nx : (x >= v.nx ? x - v.nx : x);
	if (x < 0 || x >= v.nx || y < 0 || y >= v.ny || z < 0 || z >= v.nz) return 0.f;
	int64_t idx;
	if (!v.odd) {
		idx = (int64_t)i * v.plane + ((int64_t)z * v.ny + y) * v.nxp + x;
	} else {
		int sx = x - L::cx(i);
		const int sy = y - L::cy(i), sz = z - L::cz(i);
		if (v.periodic) sx = sx < 0 ? sx + v.nxp : (sx >= v.nxp ? sx - v.nxp : sx);
		if (sx < 0 || sx >= v.nxp || sy < 0 || sy >= v.ny || sz < 0 || sz >= v.nz) return 0.f;
		idx = (int64_t)L::opp(i) * v.plane + ((int64_t)sz * v.ny + sy) * v.nxp + sx;
	}
	if (STORE == STORE_FP32) return static_cast<const float *>(v.f)[idx];
	return __half2float(static_cast<const __half *>(v.f)[idx]) + v.wshift[i];
}

constexpr int GT = 64; // threads per gather block: more blocks per body spread the FP64 sums over more SMs

// PSM (HLBM false): psm.hpp:101-446, the porosity field the couple pass
// wrote, cell force = momentum x (1 - porosity).  HLBM: hlbm.hpp:119-260,
// the body's own ramp porosity (eps) decides which cells count and the cell
// momentum enters unweighted; the cell force field is written by the HLBM
// couple pass instead (the last body wins there).
// Grid (bodies, G): block (b, g) takes the cells g, g + G, g + 2G, ... (in
// blocks of GT) of body b's box and writes its FP64 force/torque sums, after
// a fixed-order warp-shuffle and shared-memory reduction, to
// partial[(b * G + g) * 6 ..]; k_gather_finish or the contact pass adds the G
// partials of a body in order g = 0 .. G-1.  Deterministic for a given G.
template <class L, int STORE, bool HLBM>
__global__ void __launch_bounds__(GT) k_gather(PView v, const kel_particle_state *P, int steps, int mode, double eps,
											   double *partial) {
	constexpr int D = L::D;
	__shared__ double part[GT / 32][6];
	const kel_particle_state &p = P[blockIdx.x];
	int64_t a[3], b[3];
	body_aabb(D, p, v.nx, v.ny, v.nz, v.periodic, mode != KEL_POROSITY_RAMP, a, b, v.box_mul, v.box_add);
	const int64_t ex = b[0] - a[0], ey = b[1] - a[1], ez = D == 3 ? b[2] - a[2] : 1;
	const int64_t ncell = (ex > 0 && ey > 0 && ez > 0) ? ex * ey * ez : 0;
	// psm.hpp:178-184: u_p = (X - X_old) / (1 / sub_steps), raw sub_steps
	const double ts = 1.0 / (double)steps;
	double vp[3] = {0.0, 0.0, 0.0};
	for (int k = 0; k < D; ++k) vp[k] = (p.position[k] - p.position_old[k]) / ts;
	// c_i . u_p per direction, rounded to float as the reference rounds it: the
	// same for every cell of the body, so computed once (FP64 is slow here)
	float upe[L::Q];
#pragma unroll
	for (int i = 1; i < L::Q; ++i) {
		double upe_d = 0.0;
		upe_d = upe_d + (double)L::cx(i) * vp[0];
		upe_d = upe_d + (double)L::cy(i) * vp[1];
		if (D == 3) upe_d = upe_d + (double)L::cz(i) * vp[2];
		upe[i] = (float)upe_d;
	}
	double acc[6] = {0, 0, 0, 0, 0, 0}; // force[3], torque[3] (sums of minus the cell forces)
	// 32-bit index arithmetic unless the box holds 2^31 cells or more
	const bool small = ncell < ((int64_t)1 << 31);
	const int ex32 = (int)ex, ey32 = (int)ey, exy32 = small ? (int)(ex * ey) : 0;
	const int64_t stride = (int64_t)gridDim.y * GT;
	for (int64_t k = (int64_t)blockIdx.y * GT + threadIdx.x; k < ncell; k += stride) {
		int ix, iy, iz;
		if (small) {
			const int k32 = (int)k;
			ix = (int)a[0] + k32 % ex32;
			iy = (int)a[1] + (k32 / ex32) % ey32;
			iz = D == 3 ? (int)a[2] + k32 / exy32 : 0;
		} else {
			ix = (int)(a[0] + k % ex);
			iy = (int)(a[1] + (k / ex) % ey);
			iz = D == 3 ? (int)(a[2] + k / (ex * ey)) : 0;
		}
		const int x = v.periodic ? ((ix % v.nx) + v.nx) % v.nx : ix;
		const int64_t pc = ((int64_t)iz * v.ny + iy) * v.nxp + x;
		const double r[3] = {rel_coord((double)x, p.position[0], v.periodic, v.nx), (double)iy - p.position[1],
							 D == 3 ? (double)iz - p.position[2] : 0.0};
		float por;
		if (HLBM) {
			double s2 = 0.0;
			for (int d = 0; d < D; ++d) s2 = s2 + r[d] * r[d];
			por = (float)ramp(sqrt(s2), p.radius, eps);
		} else {
			por = v.por[pc];
		}
		if (por >= 1.0f) continue;
		float mom[3] = {0.f, 0.f, 0.f};
#pragma unroll
		for (int i = 1; i < L::Q; ++i) {
			const float fi = pop_post<L, STORE>(v, x, iy, iz, i);
			const float fo = pop_post<L, STORE>(v, x + L::cx(i), iy + L::cy(i), iz + L::cz(i), L::opp(i));
			const float da = __fadd_rn(__fmul_rn(fi, __fsub_rn(1.0f, upe[i])), __fmul_rn(fo, __fadd_rn(1.0f, upe[i])));
			mom[0] = __fadd_rn(mom[0], __fmul_rn((float)L::cx(i), da));
			mom[1] = __fadd_rn(mom[1], __fmul_rn((float)L::cy(i), da));
			if (D == 3) mom[2] = __fadd_rn(mom[2], __fmul_rn((float)L::cz(i), da));
		}
		const float flip = __fsub_rn(1.0f, por);
		double F[3] = {0.0, 0.0, 0.0};
		for (int d = 0; d < D; ++d) F[d] = HLBM ? (double)mom[d] : (double)__fmul_rn(mom[d], flip);
		if (!HLBM && v.cell_force)
			for (int d = 0; d < D; ++d) v.cell_force[(int64_t)d * v.plane + pc] = (float)F[d];
		for (int d = 0; d < D; ++d) acc[d] -= F[d];
		if (D == 2) {
			acc[3] -= r[0] * F[1] - r[1] * F[0];
		} else {
			acc[3] -= r[1] * F[2] - r[2] * F[1];
			acc[4] -= r[2] * F[0] - r[0] * F[2];
			acc[5] -= r[0] * F[1] - r[1] * F[0];
		}
	}
	block_sums<D, GT>(acc, part, partial + ((int64_t)blockIdx.x * gridDim.y + blockIdx.y) * 6);
}

// Incremental couple and PSM gather in one pass (the coupled step).  Block
// (b, g) takes the cells g, g + G, ... (blocks of RT) of body b's current box
// and, where it moved, its previous box, as k_couple_regions does: each cell
// gets the product of the candidates' factors, written to the porosity field.
// Cells of the current box -- body b's gather box -- then add their momentum
// exchange to the block's FP64 sums, exactly as k_gather computes it from the
// field (the porosity is the same value, computed here instead of read).
// The sums go to partial[(b * G + g) * 6 ..] in k_gather's fixed order.
// The bodies' candidates and c_i . u_p come from their records (rec).
template <class L, int STORE>
__global__ void __maxnreg__(128) k_couple_gather(PView v, const kel_particle_state *P, const BodyBox *cur,
												 const BodyBox *prev, int np, int mode, double eps,
												 const CoupleRec *rec, double *partial) {
	constexpr int D = L::D;
	__shared__ Cand cand[RT];
	__shared__ int warp_count[RT / 32];
	__shared__ int ncand;
	__shared__ double part[RT / 32][6];
	const int tid = threadIdx.x;
	const int b = blockIdx.x;
	const kel_particle_state &p = P[b];
	const BodyBox A = cur[b], B = prev[b];
	const bool same = A.a[0] == B.a[0] && A.b[0] == B.b[0] && A.a[1] == B.a[1] && A.b[1] == B.b[1] &&
					  (D == 2 || (A.a[2] == B.a[2] && A.b[2] == B.b[2]));
	const int64_t n0 = box_cells(A, D), n1 = same ? 0 : box_cells(B, D);
	const int sub = couple_mode(mode, v.direct);
	const double reach = (sub == 1 || sub == 2) ? subcell_reach(D) : 0.0;
	float upe[L::Q];
#pragma unroll
	for (int i = 1; i < L::Q; ++i) upe[i] = rec[b].upe[i];
	double acc[6] = {0, 0, 0, 0, 0, 0};
	for (int64_t base = (int64_t)blockIdx.y * RT; base < n0 + n1; base += (int64_t)gridDim.y * RT) {
		const int64_t idx = base + tid;
		const bool ok = idx < n0 + n1;
		bool touched = false;
		double por = 1.0;
		int x = 0, iy = 0, iz = 0;
		if (ok) {
			const BodyBox &q = idx < n0 ? A : B;
			const int64_t k = idx < n0 ? idx : idx - n0;
			const int64_t ex = q.b[0] - q.a[0], ey = q.b[1] - q.a[1];
			int ix = q.a[0] + (int)(k % ex);
			iy = q.a[1] + (int)((k / ex) % ey);
			iz = D == 3 ? q.a[2] + (int)(k / (ex * ey)) : 0;
			if (v.periodic) ix = ((ix % v.nx) + v.nx) % v.nx;
			x = ix;
		}
		for (int c0 = 0; c0 < np; c0 += RT) {
			bool hit = false;
			const int pi = c0 + tid;
			BodyBox bb;
			if (pi < np) {
				bb = cur[pi];
				hit = boxes_touch(bb, A, v) || (!same && boxes_touch(bb, B, v));
			}
			compact_cands<RT>(hit, pi, bb, P, cand, warp_count, &ncand, sub, reach, eps, D, rec);
			if (ok)
				for (int k = 0; k < ncand; ++k) body_factor(v, x, iy, iz, cand[k], sub, reach, eps, por, touched);
			__syncthreads();
		}
		if (!ok) continue;
		const int64_t pc = ((int64_t)iz * v.ny + iy) * v.nxp + x;
		const float porf = touched ? (float)por : 1.0f;
		v.por[pc] = porf;
		if (idx >= n0 || porf >= 1.0f) continue; // not in the gather box, or fluid
		const double r[3] = {rel_coord((double)x, p.position[0], v.periodic, v.nx), (double)iy - p.position[1],
							 D == 3 ? (double)iz - p.position[2] : 0.0};
		float mom[3] = {0.f, 0.f, 0.f};
#pragma unroll
		for (int i = 1; i < L::Q; ++i) {
			const float fi = pop_post<L, STORE>(v, x, iy, iz, i);
			const float fo = pop_post<L, STORE>(v, x + L::cx(i), iy + L::cy(i), iz + L::cz(i), L::opp(i));
			const float da = __fadd_rn(__fmul_rn(fi, __fsub_rn(1.0f, upe[i])), __fmul_rn(fo, __fadd_rn(1.0f, upe[i])));
			mom[0] = __fadd_rn(mom[0], __fmul_rn((float)L::cx(i), da));
			mom[1] = __fadd_rn(mom[1], __fmul_rn((float)L::cy(i), da));
			if (D == 3) mom[2] = __fadd_rn(mom[2], __fmul_rn((float)L::cz(i), da));
		}
		const float flip = __fsub_rn(1.0f, porf);
		double F[3] = {0.0, 0.0, 0.0};
		for (int d = 0; d < D; ++d) F[d] = (double)__fmul_rn(mom[d], flip);
		for (int d = 0; d < D; ++d) acc[d] -= F[d];
		if (D == 2) {
			acc[3] -= r[0] * F[1] - r[1] * F[0];
		} else {
			acc[3] -= r[1] * F[2] - r[2] * F[1];
			acc[4] -= r[2] * F[0] - r[0] * F[2];
			acc[5] -= r[0] * F[1] - r[1] * F[0];
		}
	}
	block_sums<D, RT>(acc, part, partial + ((int64_t)b * gridDim.y + blockIdx.y) * 6);
}

// Sum of body i's G gather partials, g = 0 .. G-1 in order.
__device__ inline void gather_total(const double *partial, int i, int G, double *tot) {
	for (int q = 0; q < 6; ++q) tot[q] = 0.0;
	for (int g = 0; g < G; ++g)
		for (int q = 0; q < 6; ++q) tot[q] += partial[((int64_t)i * G + g) * 6 + q];
}

// The gather's sums into the bodies' accumulators (force += F, torque += T).
__global__ void k_gather_finish(kel_particle_state *P, int np, int D, const double *partial, int G) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= np) return;
	double tot[6];
	gather_total(partial, i, G, tot);
	for (int d = 0; d < D; ++d) P[i].force[d] = P[i].force[d] + tot[d];
	for (int d = 0; d < (D == 2 ? 1 : 3); ++d) P[i].torque[d] = P[i].torque[d] + tot[3 + d];
}

// ---- HLBM per-cell passes ----------------------------------------------------------

// Indices (ascending) of the bodies among [c0, c0 + TT) whose AABB touches
// this tile, into cand[0 .. *ncand); every thread of the block calls it.
__device__ inline void cull_tile(const PView &v, const kel_particle_state *P, int np, int c0, int x0, int y0, int z,
								 int *cand, int *warp_count, int *ncand) {
	const int tid = threadIdx.y * TX + threadIdx.x;
	bool hit = false;
	const int pi = c0 + tid;
	if (pi < np) {
		int64_t a[3], b[3];
		body_aabb(v.D, P[pi], v.nx, v.ny, v.nz, v.periodic, 0, a, b);
		const bool yz = a[1] < y0 + TY && b[1] > y0 && (v.D == 2 || (a[2] <= z && b[2] > z));
		bool xs = a[0] < x0 + TX && b[0] > x0;
		if (v.periodic)
			xs = xs || (a[0] < x0 + TX - v.nx && b[0] > x0 - v.nx) || (a[0] < x0 + TX + v.nx && b[0] > x0 + v.nx);
		hit = yz && xs;
	}
	const unsigned m = __ballot_sync(0xffffffffu, hit);
	if ((tid & 31) == 0) warp_count[tid >> 5] = __popc(m);
	__syncthreads();
	if (tid == 0) {
		int s = 0;
		for (int w = 0; w < TT / 32; ++w) {
			const int c = warp_count[w];
			warp_count[w] = s;
			s += c;
		}
		*ncand = s;
	}
	__syncthreads();
	if (hit) cand[warp_count[tid >> 5] + __popc(m & ((1u << (tid & 31)) - 1u))] = pi;
	__syncthreads();
}

// Does body p's AABB hold cell (x, y, z)?  Returns its offset r from the body.
__device__ inline bool in_aabb(const PView &v, const kel_particle_state &p, int x, int y, int z, double *r) {
	int64_t a[3], b[3];
	body_aabb(v.D, p, v.nx, v.ny, v.nz, v.periodic, 0, a, b);
	r[0] = rel_coord((double)x, p.position[0], v.periodic, v.nx);
	r[1] = (double)y - p.position[1];
	r[2] = v.D == 3 ? (double)z - p.position[2] : 0.0;
	const int64_t xc = v.periodic ? (int64_t)llround(p.position[0] + r[0]) : x;
	return !(xc < a[0] || xc >= b[0] || y < a[1] || y >= b[1] || (v.D == 3 && (z < a[2] || z >= b[2])));
}

// HlbmReset (hlbm.hpp:27-47) and the porosity of the HLBM gathers
// (hlbm.hpp:178-186): per cell the ramp of the last body (index order) whose
// AABB holds it; with a cell-force buffer, that body's momentum exchange
// (pre-move velocity) where its porosity is below 1, as the last gather
// writing the cell leaves it.
template <int STORE>
__global__ void __launch_bounds__(TT) k_hlbm_couple(PView v, const kel_particle_state *P, int np, double eps,
													int steps) {
	__shared__ int cand[TT];
	__shared__ int warp_count[TT / 32];
	__shared__ int ncand;
	const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z = blockIdx.z;
	const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
	double por = 1.0;
	int owner = -1; // last body whose gather counts this cell (its porosity below 1)
	for (int c0 = 0; c0 < np; c0 += TT) {
		cull_tile(v, P, np, c0, x0, y0, z, cand, warp_count, &ncand);
		if (x < v.nx && y < v.ny)
			for (int k = 0; k < ncand; ++k) {
				double r[3];
				if (!in_aabb(v, P[cand[k]], x, y, z, r)) continue;
				double s2 = 0.0;
				for (int d = 0; d < v.D; ++d) s2 = s2 + r[d] * r[d];
				por = ramp(sqrt(s2), P[cand[k]].radius, eps);
				if ((float)por < 1.0f) owner = cand[k];
			}
		__syncthreads();
	}
	if (x >= v.nx || y >= v.ny) return;
	const int64_t pc = ((int64_t)z * v.ny + y) * v.nxp + x;
	v.por[pc] = (float)por;
	v.hD[pc] = 0.f;
	for (int d = 0; d < v.D; ++d) v.hN[(int64_t)d * v.plane + pc] = 0.f;
	if (!v.cell_force) return;
	float mom[2] = {0.f, 0.f};
	if (owner >= 0) {
		const kel_particle_state &p = P[owner];
		const double ts = 1.0 / (double)steps;
		double vp[2];
		for (int k = 0; k < 2; ++k) vp[k] = (p.position[k] - p.position_old[k]) / ts;
#pragma unroll
		for (int i = 1; i < 9; ++i) {
			double upe_d = 0.0;
			upe_d = upe_d + (double)D2Q9::cx(i) * vp[0];
			upe_d = upe_d + (double)D2Q9::cy(i) * vp[1];
			const float upe = (float)upe_d;
			const float fi = pop_post<D2Q9, STORE>(v, x, y, z, i);
			const float fo = pop_post<D2Q9, STORE>(v, x + D2Q9::cx(i), y + D2Q9::cy(i), z, D2Q9::opp(i));
			const float da = __fadd_rn(__fmul_rn(fi, __fsub_rn(1.0f, upe)), __fmul_rn(fo, __fadd_rn(1.0f, upe)));
			mom[0] = __fadd_rn(mom[0], __fmul_rn((float)D2Q9::cx(i), da));
			mom[1] = __fadd_rn(mom[1], __fmul_rn((float)D2Q9::cy(i), da));
		}
	}
	for (int d = 0; d < 2; ++d) v.cell_force[(int64_t)d * v.plane + pc] = mom[d];
}

// HlbmOneParticleStamp (hlbm.hpp:269-311) of every body, after the
// integrate: per cell, over the bodies (index order) whose post-move AABB
// holds it, D += 1 - por and N += u_p (1 - por), u_p = (X - X_old) sub_steps.
__global__ void __launch_bounds__(TT) k_hlbm_stamp(PView v, const kel_particle_state *P, int np, int steps) {
	__shared__ int cand[TT];
	__shared__ int warp_count[TT / 32];
	__shared__ int ncand;
	const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z = blockIdx.z;
	const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
	const bool inside = x < v.nx && y < v.ny;
	const int64_t pc = ((int64_t)z * v.ny + y) * v.nxp + x;
	const float flip = inside ? __fsub_rn(1.0f, v.por[pc]) : 0.f;
	float Dv = inside ? v.hD[pc] : 0.f;
	float N[3] = {0.f, 0.f, 0.f};
	if (inside)
		for (int d = 0; d < v.D; ++d) N[d] = v.hN[(int64_t)d * v.plane + pc];
	const double ts = 1.0 / (double)steps;
	for (int c0 = 0; c0 < np; c0 += TT) {
		cull_tile(v, P, np, c0, x0, y0, z, cand, warp_count, &ncand);
		if (inside)
			for (int k = 0; k < ncand; ++k) {
				const kel_particle_state &p = P[cand[k]];
				double r[3];
				if (!in_aabb(v, p, x, y, z, r)) continue;
				Dv = __fadd_rn(Dv, flip);
				for (int d = 0; d < v.D; ++d) {
					const float up = (float)((p.position[d] - p.position_old[d]) / ts);
					N[d] = __fadd_rn(N[d], __fmul_rn(up, flip));
				}
			}
		__syncthreads();
	}
	if (!inside) return;
	v.hD[pc] = Dv;
	for (int d = 0; d < v.D; ++d) v.hN[(int64_t)d * v.plane + pc] = N[d];
}

// ---- FPLBM (fplbm.hpp) ----------------------------------------------------------------

// FpLbmReset (fplbm.hpp:26-54), one thread per cell: porosity 1, force 0; a
// cell whose flag is in `plain` (the drivers' info 2) gets the density and
// momentum (compute_rho_momentum, macroscopic.hpp:41-60) of its current
// (post-stream) populations in the density / velocity macros.
template <int STORE>
__global__ void k_fplbm_reset(PView v, const uint8_t *flags, uint32_t plain) {
	const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
	if (x >= v.nx) return;
	const int64_t pc = (int64_t)y * v.nxp + x;
	v.por[pc] = 1.0f;
	v.cell_force[pc] = 0.0f;
	v.cell_force[v.plane + pc] = 0.0f;
	const uint8_t fl = flags[pc];
	if (fl >= 32 || !((plain >> fl) & 1u)) return;
	float r = 0.f, m0 = 0.f, m1 = 0.f;
#pragma unroll
	for (int j = 0; j < 9; ++j) {
		const float f = pop_post<D2Q9, STORE>(v, x, y, 0, j);
		r = __fadd_rn(r, f);
		if (D2Q9::cx(j) > 0) m0 = __fadd_rn(m0, f);
		if (D2Q9::cx(j) < 0) m0 = __fsub_rn(m0, f);
		if (D2Q9::cy(j) > 0) m1 = __fadd_rn(m1, f);
		if (D2Q9::cy(j) < 0) m1 = __fsub_rn(m1, f);
	}
	v.rho[pc] = r;
	v.mom[pc] = m0;
	v.mom[v.plane + pc] = m1;
}

// The AABB of body p's coupling (aabb.hpp:41-84, from the per-body boxes of
// k_pre): its own, or body 0's for every body as the reference's
// FpLbmOneParticle takes it (fplbm.hpp:186).
__device__ inline void fplbm_box(const BodyBox *box, int p, int own, int64_t *a, int64_t *b) {
	const BodyBox &q = box[own ? p : 0];
	for (int k = 0; k < 3; ++k) {
		a[k] = q.a[k];
		b[k] = q.b[k];
	}
}

// particle_porosity<float,2,1,ParticleSpheroid>::calculate (porosity.hpp:56-89):
// the angle formed in double and narrowed, its sine in float.
__device__ inline float fplbm_ramp(float s, float rad, float eps) {
	const float eps_h = __fdiv_rn(eps, 2.0f);
	const float lo = __fsub_rn(rad, eps_h), hi = __fadd_rn(rad, eps_h);
	if (s <= lo) return 0.f;
	if (s >= hi) return 1.f;
	const float inner = (float)((PI_D / (double)__fmul_rn(2.0f, eps)) * (double)__fsub_rn(s, lo));
	const float c = sinf(inner);
	return __fmul_rn(c, c);
}

// Body p's porosity and coupling force at cell (x, y): the body velocity
// (X - X_old) sub_steps and the cell's offset formed in FP64 and narrowed,
// the rest in float as the reference's T (fplbm.hpp:211-228).
__device__ inline void fplbm_cell(const PView &v, const kel_particle_state &q, float rad, double sss, int x, int y,
								  float &por, float &f0, float &f1) {
	const float vs0 = (float)((q.position[0] - q.position_old[0]) * sss);
	const float vs1 = (float)((q.position[1] - q.position_old[1]) * sss);
	const float r0 = (float)((double)x - q.position[0]), r1 = (float)((double)y - q.position[1]);
	float s2 = 0.f;
	s2 = __fadd_rn(s2, __fmul_rn(r0, r0));
	s2 = __fadd_rn(s2, __fmul_rn(r1, r1));
	por = fplbm_ramp(__fsqrt_rn(s2), rad, 1.5f);
	const float flip = __fsub_rn(1.0f, por);
	const int64_t pc = (int64_t)y * v.nxp + x;
	f0 = __fmul_rn(__fmul_rn(__fsub_rn(vs0, v.mom[pc]), 1.0f), flip);
	f1 = __fmul_rn(__fmul_rn(__fsub_rn(vs1, v.mom[v.plane + pc]), 1.0f), flip);
}

// The porosity and force fields of FpLbmOneParticle (fplbm.hpp:207-228), one
// thread per cell: of the bodies (index order) whose coupling AABB holds the
// cell, the last one's values (the reference's later writes win).
__global__ void __launch_bounds__(TT) k_fplbm_field(PView v, const kel_particle_state *P, const BodyBox *box, int np,
													int own, double sss) {
	const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
	if (x >= v.nx || y >= v.ny) return;
	int last = -1;
	for (int p = 0; p < np; ++p) {
		int64_t a[3], b[3];
		fplbm_box(box, p, own, a, b);
		if (x >= a[0] && x < b[0] && y >= a[1] && y < b[1]) last = p;
	}
	if (last < 0) return;
	const float rad = (float)(own ? P[last].radius : P[0].radius);
	float por, f0, f1;
	fplbm_cell(v, P[last], rad, sss, x, y, por, f0, f1);
	const int64_t pc = (int64_t)y * v.nxp + x;
	v.por[pc] = por;
	v.cell_force[pc] = f0;
	v.cell_force[v.plane + pc] = f1;
}

// Minus the sum of body p's coupling forces over its AABB, FP64, G blocks per
// body with fixed-order reductions into partial[(p * G + g) * 6 ..] (force
// x, y; the other four entries zero), as k_gather lays them out.
__global__ void __launch_bounds__(GT) k_fplbm_sums(PView v, const kel_particle_state *P, const BodyBox *box, int own,
												   double sss, double *partial) {
	__shared__ double part[GT / 32][2];
	const int p = blockIdx.x;
	const kel_particle_state &q = P[p];
	int64_t a[3], b[3];
	fplbm_box(box, p, own, a, b);
	const int64_t ex = b[0] - a[0], ey = b[1] - a[1];
	const int64_t ncell = (ex > 0 && ey > 0) ? ex * ey : 0;
	const float rad = (float)(own ? q.radius : P[0].radius);
	double acc0 = 0.0, acc1 = 0.0;
	for (int64_t k = (int64_t)blockIdx.y * GT + threadIdx.x; k < ncell; k += (int64_t)gridDim.y * GT) {
		const int x = (int)(a[0] + k % ex), y = (int)(a[1] + k / ex);
		float por, f0, f1;
		fplbm_cell(v, q, rad, sss, x, y, por, f0, f1);
		acc0 -= (double)f0;
		acc1 -= (double)f1;
	}
	for (int o = 16; o > 0; o >>= 1) {
		acc0 += __shfl_down_sync(0xffffffffu, acc0, o);
		acc1 += __shfl_down_sync(0xffffffffu, acc1, o);
	}
	if ((threadIdx.x & 31) == 0) {
		part[threadIdx.x >> 5][0] = acc0;
		part[threadIdx.x >> 5][1] = acc1;
	}
	__syncthreads();
	if (threadIdx.x < 6) {
		double tot = 0.0;
		if (threadIdx.x < 2)
			for (int w = 0; w < GT / 32; ++w) tot += part[w][threadIdx.x];
		partial[((int64_t)p * gridDim.y + blockIdx.y) * 6 + threadIdx.x] = tot;
	}
}

// FpLbmOneParticle's tail (fplbm.hpp:230-246), one thread per body:
// acceleration = the summed coupling force / mass + the body acceleration
// (with set_accel); then (with verlet and sub_steps > 0) the position Verlet
// sub-steps of verlet_step_lambda (particle.hpp:171-211).
__global__ void k_fplbm_integrate(kel_particle_state *P, int np, kel_particle_params prm, const double *partial, int G,
								  int set_accel, int verlet) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= np) return;
	kel_particle_state q = P[i];
	if (set_accel) {
		double tot[6];
		gather_total(partial, i, G, tot);
		for (int k = 0; k < 2; ++k) q.acceleration[k] = tot[k] / q.mass + prm.body_acceleration[k];
	}
	if (verlet && prm.sub_steps > 0) {
		const double sss = (double)prm.sub_steps, ts = 1.0 / sss, t2 = ts * ts;
		for (int s = 0; s < prm.sub_steps; ++s) {
			for (int k = 0; k < 2; ++k) {
				const double nw = q.position[k] * 2.0 - q.position_old[k] + q.acceleration[k] * t2;
				q.position_old[k] = q.position[k];
				q.position[k] = nw;
			}
			const double nw = q.rotation[0] * 2.0 - q.rotation_old[0] + q.angular_acceleration[0] * t2;
			q.rotation_old[0] = q.rotation[0];
			q.rotation[0] = nw;
		}
	}
	P[i] = q;
}

// ---- DEM contact (contact.hpp) ----------------------------------------------------

__device__ inline bool safe_normalize(int D, const double *in, double *out) {
	double l2 = 0.0;
	for (int k = 0; k < D; ++k) l2 = l2 + in[k] * in[k];
	if (!(l2 > 0)) return false;
	const double inv = 1.0 / sqrt(l2);
	for (int k = 0; k < D; ++k) out[k] = in[k] * inv;
	return true;
}

__device__ inline void surface_velocity(int D, const kel_particle_state &p, const double *r, double steps, double *v) {
	for (int k = 0; k < D; ++k) v[k] = (p.position[k] - p.position_old[k]) * steps;
	if (D == 2) {
		const double om = (p.rotation[0] - p.rotation_old[0]) * steps;
		const double t0 = -(om * r[1]), t1 = om * r[0];
		v[0] = v[0] + t0;
		v[1] = v[1] + t1;
	} else {
		double om[3];
		for (int k = 0; k < 3; ++k) om[k] = (p.rotation[k] - p.rotation_old[k]) * steps;
		const double t[3] = {om[1] * r[2] - om[2] * r[1], om[2] * r[0] - om[0] * r[2], om[0] * r[1] - om[1] * r[0]};
		for (int k = 0; k < 3; ++k) v[k] = v[k] + t[k];
	}
}

// soft_shell_response, contact.hpp:204-264
__device__ inline void soft_shell(int D, const double *n, double depth, const double *r_self, const double *v_rel,
								  double m_eff, const kel_particle_params &dem, double *F, double *T) {
	const double k_n = dem.k_n, zeta = dem.zeta_n;
	const double g_n = 2.0 * zeta * sqrt(m_eff * k_n);
	double v_n = 0.0;
	for (int k = 0; k < D; ++k) v_n = v_n + v_rel[k] * n[k];
	double f_n = k_n * depth - g_n * v_n;
	if (f_n < 0) f_n = 0;
	double v_t[3] = {0, 0, 0}, t_hat[3] = {0, 0, 0};
	for (int k = 0; k < D; ++k) v_t[k] = v_rel[k] - v_n * n[k];
	const bool have_t = safe_normalize(D, v_t, t_hat);
	double vtt = 0.0;
	for (int k = 0; k < D; ++k) vtt = vtt + v_t[k] * v_t[k];
	const double v_t_len = sqrt(vtt);
	double f_t = dem.gamma_t * v_t_len;
	const double f_t_cap = dem.mu * f_n;
	if (f_t > f_t_cap) f_t = f_t_cap;
	for (int k = 0; k < D; ++k) {
		double val = f_n * n[k];
		if (have_t) val -= f_t * t_hat[k];
		F[k] = val;
	}
	if (D == 2) {
		T[0] = r_self[0] * F[1] - r_self[1] * F[0];
	} else {
		T[0] = r_self[1] * F[2] - r_self[2] * F[1];
		T[1] = r_self[2] * F[0] - r_self[0] * F[2];
		T[2] = r_self[0] * F[1] - r_self[1] * F[0];
	}
}

__device__ inline void pdiff(int D, const double *a, const double *b, int per, double Lx, double *d) {
	for (int k = 0; k < D; ++k) d[k] = a[k] - b[k];
	if (per) {
		if (d[0] > 0.5 * Lx) d[0] -= Lx;
		else if (d[0] < -0.5 * Lx) d[0] += Lx;
	}
}

// Force and torque of the pair (self s, other j) on s, or false when they do
// not touch (particle/contact.hpp:466-512 inner body).
__device__ inline bool pair_response(const kel_particle_state &self, const kel_particle_state &other, int s, int j, int D,
									 const kel_particle_params &prm, double steps, double Lx, int periodic, double *f,
									 double *torque0) {
	double dd[3] = {0, 0, 0};
	pdiff(D, self.position, other.position, periodic, Lx, dd);
	double n2 = 0.0;
	for (int k = 0; k < D; ++k) n2 = n2 + dd[k] * dd[k];
	const double rl = self.radius, rr = other.radius;
	if (!(n2 < rl * rl + rr * rr + rr * rl * 2.0)) return false;
	const bool self_is_lo = s < j;
	const kel_particle_state &lo = self_is_lo ? self : other;
	const kel_particle_state &hi = self_is_lo ? other : self;
	double d[3] = {0, 0, 0};
	pdiff(D, lo.position, hi.position, periodic, Lx, d);
	double len2 = 0.0;
	for (int k = 0; k < D; ++k) len2 = len2 + d[k] * d[k];
	const double sum_r = lo.radius + hi.radius;
	if (!(len2 < sum_r * sum_r)) return false;
	const double len = sqrt(len2);
	double depth = sum_r - len;
	const double cap = (lo.radius < hi.radius) ? lo.radius : hi.radius;
	if (depth > cap) depth = cap;
	double n[3] = {0, 0, 0};
	if (!safe_normalize(D, d, n)) {
		for (int k = 0; k < D; ++k) n[k] = 0;
		n[0] = 1;
	}
	double off[3] = {0, 0, 0};
	for (int k = 0; k < D; ++k) off[k] = n[k] * (hi.radius - depth * 0.5);
	if (!self_is_lo)
		for (int k = 0; k < D; ++k) n[k] = -n[k];
	double r_s[3] = {0, 0, 0}, r_o[3] = {0, 0, 0};
	for (int k = 0; k < D; ++k) {
		const double pt = hi.position[k] + off[k];
		r_s[k] = pt - self.position[k];
		r_o[k] = pt - other.position[k];
	}
	if (periodic) {
		if (r_s[0] > 0.5 * Lx) r_s[0] -= Lx; else if (r_s[0] < -0.5 * Lx) r_s[0] += Lx;
		if (r_o[0] > 0.5 * Lx) r_o[0] -= Lx; else if (r_o[0] < -0.5 * Lx) r_o[0] += Lx;
	}
	double v_s[3] = {0, 0, 0}, v_o[3] = {0, 0, 0}, v_rel[3] = {0, 0, 0};
	surface_velocity(D, self, r_s, steps, v_s);
	surface_velocity(D, other, r_o, steps, v_o);
	for (int k = 0; k < D; ++k) v_rel[k] = v_s[k] - v_o[k];
	const double m_eff = (self.mass * other.mass) / (self.mass + other.mass);
	double t[3] = {0, 0, 0};
	soft_shell(D, n, depth, r_s, v_rel, m_eff, prm, f, t);
	*torque0 = t[0];
	return true;
}

// Contact of body s, by one warp (every lane calls it): the lanes evaluate
// its pairs 32 at a time, then lane 0 adds the contacts in index order (the
// reference's accumulation order, so the FP64 result is bit-identical) and
// finally the box walls, and writes the body's force (and 2D torque).  The
// sums start from the body's accumulators, or from zero with zero_start;
// with a gather partial buffer the body's gather sums are added first,
// exactly as k_gather_finish would add them.  fs / hs: this warp's scratch.
__device__ inline void contact_one(kel_particle_state *P, int s, int np, int D, const kel_particle_params &prm, int nx,
								   int ny, int nz, int periodic, const double *partial, int G, bool zero_start,
								   double (*fs)[4], int *hs, kel_particle_state *out = nullptr) {
	const int lane = threadIdx.x & 31;
	const double steps = (double)(prm.sub_steps == 0 ? 1 : prm.sub_steps);
	const double Lx = (double)nx;
	const double ext[3] = {(double)nx, (double)ny, (double)nz};
	const kel_particle_state &self = P[s];
	double force[3] = {self.force[0], self.force[1], self.force[2]};
	double torque0 = self.torque[0];
	double torque12[2] = {self.torque[1], self.torque[2]};
	if (zero_start) {
		force[0] = force[1] = force[2] = 0.0;
		torque0 = torque12[0] = torque12[1] = 0.0;
	}
	if (partial) {
		double tot[6];
		gather_total(partial, s, G, tot);
		for (int d = 0; d < D; ++d) force[d] = force[d] + tot[d];
		torque0 = torque0 + tot[3];
		if (D == 3) {
			torque12[0] = torque12[0] + tot[4];
			torque12[1] = torque12[1] + tot[5];
		}
	}
	for (int j0 = 0; j0 < np; j0 += 32) {
		const int j = j0 + lane;
		double f[3] = {0, 0, 0}, t0 = 0.0;
		const bool hit = j < np && j != s && pair_response(self, P[j], s, j, D, prm, steps, Lx, periodic, f, &t0);
		fs[lane][0] = f[0];
		fs[lane][1] = f[1];
		fs[lane][2] = f[2];
		fs[lane][3] = t0;
		hs[lane] = hit ? 1 : 0;
		__syncwarp();
		if (lane == 0) {
			for (int q = 0; q < 32; ++q) {
				if (!hs[q]) continue;
				for (int k = 0; k < D; ++k) force[k] = force[k] + fs[q][k];
				if (D == 2) torque0 = torque0 + fs[q][3];
			}
		}
		__syncwarp();
	}
	if (lane != 0) return;
	for (int ax = 0; ax < D; ++ax) {
		if (!(prm.wall_axes & (1u << ax))) continue;
		const double x = self.position[ax], r = self.radius, hb = ext[ax];
		for (int side = 0; side < 2; ++side) {
			double depth = side == 0 ? (r - x) : (x - (hb - r));
			if (!(depth > 0)) continue;
			if (depth > r) depth = r;
			double n[3] = {0, 0, 0}, pt[3] = {0, 0, 0};
			for (int k = 0; k < D; ++k) pt[k] = self.position[k];
			n[ax] = side == 0 ? 1.0 : -1.0;
			pt[ax] = side == 0 ? 0.0 : hb;
			double r_s[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
			for (int k = 0; k < D; ++k) r_s[k] = pt[k] - self.position[k];
			surface_velocity(D, self, r_s, steps, vv);
			double f[3] = {0, 0, 0}, t[3] = {0, 0, 0};
			soft_shell(D, n, depth, r_s, vv, self.mass, prm, f, t);
			for (int k = 0; k < D; ++k) force[k] = force[k] + f[k];
			if (D == 2) torque0 = torque0 + t[0];
		}
	}
	// only lane 0 of this warp writes body s (to P, or with out to *out, a
	// copy of the body); the other warps read its position fields only
	kel_particle_state &w = out ? *out : P[s];
	w.force[0] = force[0];
	w.force[1] = force[1];
	w.force[2] = force[2];
	if (D == 2 || partial || zero_start) w.torque[0] = torque0;
	if (D == 3 && (partial || zero_start)) {
		w.torque[1] = torque12[0];
		w.torque[2] = torque12[1];
	}
}

// One warp per body (four per block).
__global__ void k_contact(kel_particle_state *P, int np, int D, kel_particle_params prm, int nx, int ny, int nz,
						  int periodic, const double *partial, int G) {
	__shared__ double fs[4][32][4];
	__shared__ int hs[4][32];
	const int w = threadIdx.x >> 5;
	const int s = blockIdx.x * 4 + w;
	if (s >= np) return; // warp-uniform
	contact_one(P, s, np, D, prm, nx, ny, nz, periodic, partial, G, false, fs[w], hs[w]);
}

// integrate_particle + verlet_step_lambda (integrate.hpp:45-83, particle.hpp:171-211)
__device__ inline void integrate_state(kel_particle_state &q, int D, const kel_particle_params &prm, int nx,
									   int periodic);

__device__ inline void integrate_one(kel_particle_state *P, int pi, int D, const kel_particle_params &prm, int nx,
									 int periodic) {
	kel_particle_state q = P[pi];
	integrate_state(q, D, prm, nx, periodic);
	P[pi] = q;
}

// integrate_particle + verlet_step_lambda on a body held by the caller
__device__ inline void integrate_state(kel_particle_state &q, int D, const kel_particle_params &prm, int nx,
									   int periodic) {
	const int steps = prm.sub_steps == 0 ? 1 : prm.sub_steps;
	const double ts = 1.0 / (double)steps;
	for (int k = 0; k < D; ++k) q.acceleration[k] = q.force[k] / q.mass + prm.body_acceleration[k];
	if (D == 2) q.angular_acceleration[0] = q.torque[0] / q.inertia;
	for (int s = 0; s < steps; ++s) {
		const double t2 = ts * ts;
		for (int k = 0; k < D; ++k) {
			const double nw = q.position[k] * 2.0 - q.position_old[k] + q.acceleration[k] * t2;
			q.position_old[k] = q.position[k];
			q.position[k] = nw;
		}
		const int nr = D == 2 ? 1 : 3;
		for (int k = 0; k < nr; ++k) {
			const double nw = q.rotation[k] * 2.0 - q.rotation_old[k] + q.angular_acceleration[k] * t2;
			q.rotation_old[k] = q.rotation[k];
			q.rotation[k] = nw;
		}
	}
	if (periodic) {
		const double L = (double)nx;
		if (q.position[0] >= L) {
			q.position[0] -= L;
			q.position_old[0] -= L;
		} else if (q.position[0] < 0.0) {
			q.position[0] += L;
			q.position_old[0] += L;
		}
	}
}

__global__ void k_integrate(kel_particle_state *P, int np, int D, kel_particle_params prm, int nx, int periodic) {
	const int pi = blockIdx.x * blockDim.x + threadIdx.x;
	if (pi >= np) return;
	integrate_one(P, pi, D, prm, nx, periodic);
}

// Contact and integrate of the coupled step in one launch, one warp (block)
// per body: the contact of body s reads every body's state in P_in; lane 0
// then integrates a copy of body s with that force and writes it to P_out
// (the next step's state, so that no block reads a body another has already
// moved), and prepares the next couple's boxes and the body's record for
// the next couple + gather (its candidate for couple mode cm; lanes
// 1 .. Q-1 form c_i . u_p).
template <class L>
__global__ void __launch_bounds__(32) k_contact_integrate(const kel_particle_state *P_in, kel_particle_state *P_out,
														  PView v, kel_particle_params prm, const double *partial,
														  int G, BodyBox *cur, BodyBox *prev, int cm, double reach,
														  CoupleRec *rec) {
	__shared__ double fs[32][4];
	__shared__ int hs[32];
	const int s = blockIdx.x, np = (int)gridDim.x;
	const int lane = threadIdx.x & 31;
	kel_particle_state q;
	contact_one(const_cast<kel_particle_state *>(P_in), s, np, v.D, prm, v.nx, v.ny, v.nz, v.periodic, partial, G, true,
				fs, hs, &q);
	if (lane == 0) {
		// contact_one set q's force and torque; the rest of the body from P_in
		const kel_particle_state &o = P_in[s];
		const double f0 = q.force[0], f1 = q.force[1], f2 = q.force[2];
		const double t0 = q.torque[0], t1 = q.torque[1], t2 = q.torque[2];
		q = o;
		q.force[0] = f0;
		q.force[1] = f1;
		q.force[2] = f2;
		q.torque[0] = t0;
		if (v.D == 3) {
			q.torque[1] = t1;
			q.torque[2] = t2;
		}
		integrate_state(q, v.D, prm, v.nx, v.periodic);
		P_out[s] = q;
		int64_t a[3], b[3];
		body_aabb(v.D, q, v.nx, v.ny, v.nz, v.periodic, cm != 0, a, b, v.box_mul, v.box_add);
		BodyBox r;
		for (int k = 0; k < 3; ++k) {
			r.a[k] = (int)a[k];
			r.b[k] = (int)b[k];
		}
		prev[s] = cur[s];
		cur[s] = r;
		Cand c;
		c.box = r;
		for (int d = 0; d < 3; ++d) c.X[d] = q.position[d];
		c.R = q.radius;
		cand_prepare(c, cm, reach, prm.eps, q.rotation, v.D);
		rec[s].cand = c;
	}
	__syncwarp();
	if (lane >= 1 && lane < L::Q) {
		// the gather's c_i . u_p, rounded to float as the reference rounds it
		const kel_particle_state &n = P_out[s];
		double vp[3] = {0.0, 0.0, 0.0};
		for (int k = 0; k < L::D; ++k) vp[k] = wall_velocity(n.position[k] - n.position_old[k], prm.sub_steps);
		double upe_d = 0.0;
		upe_d = upe_d + (double)L::cx(lane) * vp[0];
		upe_d = upe_d + (double)L::cy(lane) * vp[1];
		if (L::D == 3) upe_d = upe_d + (double)L::cz(lane) * vp[2];
		rec[s].upe[lane] = (float)upe_d;
	}
}

// ---- voxel queries (FP64): mask.hpp, voxel_narrow.hpp ------------------------

// mask_sample_local (mask.hpp:194-264)
__device__ inline double mask_sample_f64(const double *__restrict__ mask, int D, int R, const double *u) {
	const double step = 2.0 / (double)R;
	double frac[3] = {0, 0, 0};
	int64_t base[3] = {0, 0, 0};
	double outside = 0;
	for (int i = 0; i < D; ++i) {
		double g = (u[i] + 1) / step - 0.5;
		if (g < 0) {
			outside += g * g * step * step;
			g = 0;
		} else if (g > (double)(R - 1)) {
			const double over = g - (double)(R - 1);
			outside += over * over * step * step;
			g = (double)(R - 1);
		}
		base[i] = (int64_t)floor(g);
		if (base[i] > (int64_t)R - 2) {
			base[i] = (int64_t)R - 2;
			if (base[i] < 0) base[i] = 0;
		}
		frac[i] = g - (double)base[i];
	}
	double acc = 0;
	for (int c = 0; c < (1 << D); ++c) {
		double w = 1;
		int64_t flat = 0;
		for (int i = 0; i < D; ++i) {
			const int hi = (c >> i) & 1;
			int64_t idx = base[i] + hi;
			if (idx < 0) idx = 0;
			if (idx > (int64_t)R - 1) idx = (int64_t)R - 1;
			flat = flat * R + idx;
			w *= hi ? frac[i] : (1 - frac[i]);
		}
		acc += w * __ldg(mask + flat);
	}
	if (outside > 0) acc += sqrt(outside);
	return acc;
}

// A body's pose for the FP64 queries: position, radius and the inverse
// rotation's terms of impl::mask_rotate (mask.hpp:52-105): 2D c, s of the
// negated angle; 3D the unit axis n, c and s of the negated angle (th2 = 0:
// no rotation).
struct VoxelPose {
	double X[3], R;
	double c, s, n[3];
	bool rot3;
};

__device__ inline VoxelPose voxel_pose(int D, const kel_particle_state &p) {
	VoxelPose q;
	for (int i = 0; i < 3; ++i) q.X[i] = p.position[i];
	q.R = p.radius;
	q.rot3 = false;
	q.n[0] = q.n[1] = q.n[2] = 0.0;
	if (D == 2) {
		const double a = -p.rotation[0];
		q.c = cos(a);
		q.s = sin(a);
	} else {
		double th2 = 0;
		for (int i = 0; i < 3; ++i) th2 = th2 + p.rotation[i] * p.rotation[i];
		q.c = 1.0;
		q.s = 0.0;
		if (th2 > 0) {
			q.rot3 = true;
			const double th = -sqrt(th2);
			for (int i = 0; i < 3; ++i) q.n[i] = p.rotation[i] / sqrt(th2);
			q.c = cos(th);
			q.s = sin(th);
		}
	}
	return q;
}

// mask_signed_distance (mask.hpp:270-282): lattice point x to body-local u
// (mask_global_to_local, mask.hpp:158-180), sampled, times the radius.
__device__ inline double voxel_sdf(const PView &v, const VoxelPose &q, const double *x) {
	const int D = v.D;
	double rel[3] = {0, 0, 0}, un[3] = {0, 0, 0};
	for (int i = 0; i < D; ++i) rel[i] = (x[i] - q.X[i]) / q.R;
	if (D == 2) {
		un[0] = rel[0] * q.c - rel[1] * q.s;
		un[1] = rel[0] * q.s + rel[1] * q.c;
	} else if (!q.rot3) {
		for (int i = 0; i < 3; ++i) un[i] = rel[i];
	} else {
		double ndv = 0;
		for (int i = 0; i < 3; ++i) ndv = ndv + q.n[i] * rel[i];
		const double cr[3] = {q.n[1] * rel[2] - q.n[2] * rel[1], q.n[2] * rel[0] - q.n[0] * rel[2],
							  q.n[0] * rel[1] - q.n[1] * rel[0]};
		for (int i = 0; i < 3; ++i) un[i] = rel[i] * q.c + cr[i] * q.s + q.n[i] * ndv * (1 - q.c);
	}
	double u[3] = {0, 0, 0};
	for (int i = 0; i < D; ++i) u[i] = un[i] + v.vcom[i];
	return mask_sample_f64(v.vmask_d, D, v.vres, u) * q.R;
}

// solid_fraction_from_sdf (mask.hpp:291-311)
__device__ inline double solid_f64(double sdf, double eps) {
	const double half = eps / 2;
	if (sdf <= -half) return 1;
	if (sdf >= half) return 0;
	const double t = (sdf + half) / eps;
	const double c = cos(PI_D * t / 2);
	return c * c;
}

// One thread per point: body b's signed distance at points[k] (3 doubles).
__global__ void k_voxel_distance(PView v, const kel_particle_state *P, int b, const double *points, int n, double *out) {
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n) return;
	const VoxelPose q = voxel_pose(v.D, P[b]);
	out[k] = voxel_sdf(v, q, points + 3 * (int64_t)k);
}

constexpr int VT = 128; // threads per pair of the voxel contact

// Fixed-order block sum of NQ doubles per thread (warp tree, then warps in
// order) into out (every thread receives it).  red: VT / 32 x NQ scratch.
template <int NQ>
__device__ inline void voxel_block_sum(double *vals, double (*red)[NQ], double *out) {
	const int tid = threadIdx.x;
#pragma unroll
	for (int j = 0; j < NQ; ++j) {
		double s = vals[j];
		for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
		if ((tid & 31) == 0) red[tid >> 5][j] = s;
	}
	__syncthreads();
#pragma unroll
	for (int j = 0; j < NQ; ++j) {
		double t = 0.0;
		for (int w = 0; w < VT / 32; ++w) t += red[w][j];
		out[j] = t;
	}
	__syncthreads();
}

// voxel_contact (voxel_narrow.hpp:78-259) of pair blockIdx.x, one block per
// pair.  The cells of the clamped intersection of the two bounding boxes are
// spread over the block (axis 0 outermost in the flat index); the overlap
// volume, centroid and weighted gradient difference are summed per thread
// and then in a fixed order that does not depend on which body is lo (the
// terms for (hi, lo) are the exact negations), so swapping a pair negates the
// normal exactly.  The depth's extent is a min / max (exact).
__global__ void __launch_bounds__(VT) k_voxel_contact(PView v, const kel_particle_state *P, const int *pairs,
													  double eps, kel_contact_manifold *out) {
	__shared__ double red[VT / 32][7];
	__shared__ double nrm[3];
	__shared__ int any_s;
	const int D = v.D, tid = threadIdx.x;
	const kel_particle_state &lo = P[pairs[2 * blockIdx.x]], &hi = P[pairs[2 * blockIdx.x + 1]];
	kel_contact_manifold res;
	memset(&res, 0, sizeof(res));
	int64_t start[3] = {0, 0, 0}, stop[3] = {1, 1, 1};
	const int64_t ext[3] = {v.nx, v.ny, v.nz};
	for (int i = 0; i < D; ++i) {
		const double a_lo = lo.position[i] - lo.radius, a_hi = hi.position[i] - hi.radius;
		double a = a_lo > a_hi ? a_lo : a_hi;
		const double b_lo = lo.position[i] + lo.radius, b_hi = hi.position[i] + hi.radius;
		const double b = b_lo < b_hi ? b_lo : b_hi;
		if (a < 0) a = 0;
		int64_t ai = (int64_t)floor(a);
		int64_t bi = (int64_t)ceil(b) + 1;
		if (ai < 0) ai = 0;
		if (bi > ext[i]) bi = ext[i];
		if (bi <= ai) { // uniform over the block
			if (tid == 0) out[blockIdx.x] = res;
			return;
		}
		start[i] = ai;
		stop[i] = bi;
	}
	const int64_t e1 = stop[1] - start[1], e2 = stop[2] - start[2];
	const int64_t ncell = (stop[0] - start[0]) * e1 * e2;
	const VoxelPose ql = voxel_pose(D, lo), qh = voxel_pose(D, hi);
	const double h = 0.5;
	double acc[7] = {0, 0, 0, 0, 0, 0, 0}; // volume, centroid[3], grad[3]
	for (int64_t k = tid; k < ncell; k += VT) {
		const double x[3] = {(double)(start[0] + k / (e1 * e2)), (double)(start[1] + (k / e2) % e1),
							 D == 3 ? (double)(start[2] + k % e2) : 0.0};
		const double s_lo = solid_f64(voxel_sdf(v, ql, x), eps);
		if (!(s_lo > 0)) continue;
		const double s_hi = solid_f64(voxel_sdf(v, qh, x), eps);
		if (!(s_hi > 0)) continue;
		const double w = s_lo * s_hi;
		acc[0] += w;
		for (int i = 0; i < D; ++i) acc[1 + i] = acc[1 + i] + w * x[i];
		for (int i = 0; i < D; ++i) { // impl::sdf_gradient by central differences, both bodies
			double xl[3] = {x[0], x[1], x[2]}, xh[3] = {x[0], x[1], x[2]};
			xl[i] = x[i] - h;
			xh[i] = x[i] + h;
			const double g_lo = (voxel_sdf(v, ql, xh) - voxel_sdf(v, ql, xl)) / (2 * h);
			const double g_hi = (voxel_sdf(v, qh, xh) - voxel_sdf(v, qh, xl)) / (2 * h);
			acc[4 + i] = acc[4 + i] + w * (g_hi - g_lo);
		}
	}
	double tot[7];
	voxel_block_sum<7>(acc, red, tot);
	if (!(tot[0] > 0)) {
		if (tid == 0) out[blockIdx.x] = res;
		return;
	}
	if (tid == 0) {
		double n[3] = {0, 0, 0}, g[3] = {tot[4], tot[5], tot[6]};
		if (!safe_normalize(D, g, n)) {
			double fb[3] = {0, 0, 0};
			for (int i = 0; i < D; ++i) fb[i] = lo.position[i] - hi.position[i];
			if (!safe_normalize(D, fb, n)) {
				n[0] = 1.0;
				n[1] = n[2] = 0.0;
			}
		}
		for (int i = 0; i < 3; ++i) nrm[i] = n[i];
		any_s = 0;
	}
	__syncthreads();
	double s_min = INFINITY, s_max = -INFINITY;
	int any = 0;
	for (int64_t k = tid; k < ncell; k += VT) {
		const double x[3] = {(double)(start[0] + k / (e1 * e2)), (double)(start[1] + (k / e2) % e1),
							 D == 3 ? (double)(start[2] + k % e2) : 0.0};
		if (!(solid_f64(voxel_sdf(v, ql, x), eps) > 0.5)) continue;
		if (!(solid_f64(voxel_sdf(v, qh, x), eps) > 0.5)) continue;
		double s = 0;
		for (int i = 0; i < D; ++i) s = s + x[i] * nrm[i];
		any = 1;
		s_min = fmin(s_min, s);
		s_max = fmax(s_max, s);
	}
	for (int o = 16; o > 0; o >>= 1) {
		s_min = fmin(s_min, __shfl_down_sync(0xffffffffu, s_min, o));
		s_max = fmax(s_max, __shfl_down_sync(0xffffffffu, s_max, o));
		any |= __shfl_down_sync(0xffffffffu, any, o);
	}
	if ((tid & 31) == 0) {
		red[tid >> 5][0] = s_min;
		red[tid >> 5][1] = s_max;
		if (any) atomicOr(&any_s, 1);
	}
	__syncthreads();
	if (tid != 0) return;
	for (int w = 0; w < VT / 32; ++w) {
		s_min = fmin(s_min, red[w][0]);
		s_max = fmax(s_max, red[w][1]);
	}
	double depth = any_s ? (s_max - s_min + 1.0) : 1.0;
	const double cap = lo.radius < hi.radius ? lo.radius : hi.radius;
	if (depth > cap) depth = cap;
	res.hit = 1;
	res.depth = depth;
	for (int i = 0; i < D; ++i) {
		res.normal[i] = nrm[i];
		res.point[i] = tot[1 + i] / tot[0];
	}
	out[blockIdx.x] = res;
}

PView make_view(kel_lattice *L) {
	PView v;
	memset(&v, 0, sizeof(v));
	v.f = L->f;
	v.storage = L->desc.storage;
	v.plane = L->plane;
	v.nx = (int)L->desc.nx;
	v.nxp = L->nxp;
	v.ny = (int)L->desc.ny;
	v.nz = (int)L->desc.nz;
	v.D = L->d.D;
	v.Q = L->d.Q;
	v.odd = (int)(L->t & 1u);
	v.periodic = (L->desc.flags & KEL_LATTICE_PERIODIC_X) ? 1 : 0;
	v.por = L->por;
	v.hN = L->hN;
	v.hD = L->hD;
	v.rho = L->rho;
	v.mom = L->u;
	for (int i = 0; i < 27; ++i) v.wshift[i] = L->wshift[i];
	v.box_mul = 1.0;
	v.box_add = 0.0;
	return v;
}

// Growth of the bodies' boxes for a porosity mode: voxel bodies reach
// R * reach + eps / 2 (the shape's extent and half the ramp).
void box_growth(const kel_particles *ps, const kel_particle_params *prm, double *mul, double *add) {
	*mul = 1.0;
	*add = 0.0;
	if (prm->porosity_mode == KEL_POROSITY_VOXEL && ps->shape) {
		*mul = ps->shape->reach;
		*add = prm->eps / 2;
	}
}

// Sub-cell and voxel factors without the FP64 nearest-image / shortcut test
// (body_factor's direct mode): every body box narrower than half the
// periodic length (boxes span at most 2 ceil(radius) + 4 cells), so that the
// image of a cell in a box is its nearest.
int direct_mode(const kel_particles *ps, const kel_particle_params *prm) {
	if (prm->porosity_mode == KEL_POROSITY_RAMP) return 0;
	const kel_lattice *L = ps->lat;
	if (!(L->desc.flags & KEL_LATTICE_PERIODIC_X)) return 1;
	double mul, add;
	box_growth(ps, prm, &mul, &add);
	return 2.0 * (ceil(ps->max_radius * mul + add) + 3.0) < 0.5 * (double)L->desc.nx ? 1 : 0;
}

// The particle passes' view: the lattice's plus the box growth, the direct
// flag and (voxel mode) the shape.
PView particle_view(kel_particles *ps, const kel_particle_params *prm) {
	PView v = make_view(ps->lat);
	box_growth(ps, prm, &v.box_mul, &v.box_add);
	v.direct = direct_mode(ps, prm);
	if (prm->porosity_mode == KEL_POROSITY_VOXEL && ps->shape) {
		const kel_shape *sh = ps->shape;
		v.vmask_f = sh->d_mask_f;
		v.vmask_d = sh->d_mask_d;
		v.vres = sh->res;
		for (int i = 0; i < 3; ++i) {
			v.vcom[i] = sh->com[i];
			v.vcom_f[i] = (float)sh->com[i];
		}
	}
	return v;
}

int check_params(const kel_particles *ps, const kel_particle_params *prm, const char *who) {
	if (!ps || !prm) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: null argument", who);
	if (prm->porosity_mode < KEL_POROSITY_RAMP || prm->porosity_mode > KEL_POROSITY_VOXEL)
		return fail(KEL_ERR_INVALID_ARGUMENT, "%s: unknown porosity mode %d", who, prm->porosity_mode);
	if (prm->porosity_mode == KEL_POROSITY_VOXEL) {
		if (prm->coupling != KEL_COUPLING_PSM)
			return fail(KEL_ERR_UNSUPPORTED, "%s: voxel porosity goes with PSM coupling", who);
		if (!ps->shape) return fail(KEL_ERR_STATE, "%s: voxel porosity needs a shape (kel_particles_set_shape)", who);
		if (!(prm->eps > 0)) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: eps must be positive", who);
	}
	if (prm->sub_steps < 0) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: negative sub_steps", who);
	if ((prm->porosity_mode == KEL_POROSITY_RAMP || prm->coupling == KEL_COUPLING_HLBM) && !(prm->eps > 0))
		return fail(KEL_ERR_INVALID_ARGUMENT, "%s: eps must be positive", who);
	if (prm->coupling < KEL_COUPLING_PSM || prm->coupling > KEL_COUPLING_FPLBM_OWN)
		return fail(KEL_ERR_INVALID_ARGUMENT, "%s: unknown coupling %d", who, prm->coupling);
	if (prm->coupling == KEL_COUPLING_FPLBM || prm->coupling == KEL_COUPLING_FPLBM_OWN) {
		if (ps->lat->d.Q != 9) return fail(KEL_ERR_UNSUPPORTED, "%s: FPLBM coupling is D2Q9 only", who);
		if (ps->lat->desc.flags & KEL_LATTICE_PERIODIC_X)
			return fail(KEL_ERR_UNSUPPORTED, "%s: FPLBM coupling needs a non-periodic lattice", who);
		int rc;
		if ((rc = ensure_field(ps->lat, &ps->lat->force, ps->lat->plane * ps->lat->d.D, 0.0f))) return rc;
	}
	if (prm->coupling == KEL_COUPLING_HLBM) {
		if (ps->lat->d.Q != 9) return fail(KEL_ERR_UNSUPPORTED, "%s: HLBM coupling is D2Q9 only", who);
		int rc;
		if ((rc = ensure_field(ps->lat, &ps->lat->hN, ps->lat->plane * ps->lat->d.D, 0.0f))) return rc;
		if ((rc = ensure_field(ps->lat, &ps->lat->hD, ps->lat->plane, 0.0f))) return rc;
	}
	return KEL_OK;
}

} // namespace

// ---------------------------------------------------------------------------
// C ABI

// Cells of a body's box per axis, at most: 2 r + 2 (ramp) or 2 r + 3
// (sub-cell and voxel, r grown by box_growth)
static int64_t box_cells_max(const kel_particles *ps, const kel_particle_params *prm) {
	double mul, add;
	box_growth(ps, prm, &mul, &add);
	const int64_t e = 2 * (int64_t)ceil(ps->max_radius * mul + add) + 4;
	return ps->lat->d.D == 3 ? e * e * e : e * e;
}

// Blocks per body of the gather: about one thread per box cell, 1 .. 64.
static int gather_blocks(const kel_particles *ps, const kel_particle_params *prm) {
	const int64_t g = (box_cells_max(ps, prm) + GT - 1) / GT;
	return (int)(g < 1 ? 1 : (g > 64 ? 64 : g));
}

// Blocks per body of the region couple (two boxes, RC_CPT cells per thread).
static int couple_blocks(const kel_particles *ps, const kel_particle_params *prm) {
	const int64_t g = (2 * box_cells_max(ps, prm) + RT * RC_CPT - 1) / (RT * RC_CPT);
	return (int)(g < 1 ? 1 : (g > 64 ? 64 : g));
}

extern "C" int kel_particles_create(kel_lattice *lat, int32_t count, kel_particles **out) {
	if (!lat || !out || count < 1) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_create: bad arguments");
	*out = nullptr;
	kel_particles *ps = new kel_particles();
	ps->lat = lat;
	ps->n = count;
	cudaError_t e = cudaMalloc(&ps->d, sizeof(kel_particle_state) * count);
	if (e == cudaSuccess) e = cudaMalloc(&ps->d_alt, sizeof(kel_particle_state) * count);
	if (e == cudaSuccess) e = cudaMalloc(&ps->boxes, sizeof(BodyBox) * 2 * (size_t)count);
	if (e == cudaSuccess) e = cudaMalloc(&ps->rec, sizeof(CoupleRec) * (size_t)count);
	if (e != cudaSuccess) {
		cudaFree(ps->d);
		cudaFree(ps->d_alt);
		cudaFree(ps->boxes);
		delete ps;
		return fail(e == cudaErrorMemoryAllocation ? KEL_ERR_OUT_OF_MEMORY : KEL_ERR_CUDA, "kel_particles_create: %s",
					cudaGetErrorString(e));
	}
	cudaMemsetAsync(ps->d, 0, sizeof(kel_particle_state) * count, lat->stream);
	int rc = ensure_field(lat, &lat->por, lat->plane, 1.0f);
	if (rc) {
		cudaFree(ps->d);
		cudaFree(ps->d_alt);
		cudaFree(ps->boxes);
		cudaFree(ps->rec);
		delete ps;
		return rc;
	}
	*out = ps;
	return KEL_OK;
}

extern "C" int kel_particles_destroy(kel_particles *ps) {
	if (!ps) return KEL_OK;
	cudaStreamSynchronize(ps->lat->stream);
	if (ps->graph) cudaGraphExecDestroy(ps->graph);
	if (ps->side) cudaStreamDestroy(ps->side);
	if (ps->ev_fork) cudaEventDestroy(ps->ev_fork);
	if (ps->ev_join) cudaEventDestroy(ps->ev_join);
	cudaFree(ps->d);
	cudaFree(ps->d_alt);
	cudaFree(ps->cell_force);
	cudaFree(ps->boxes);
	cudaFree(ps->rec);
	cudaFree(ps->partial);
	delete ps;
	return KEL_OK;
}

extern "C" int kel_particles_upload(kel_particles *ps, const kel_particle_state *host) {
	if (ps) ps->cur_fresh = false;
	if (!ps || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_upload: null argument");
	double rmax = 0.0;
	for (int i = 0; i < ps->n; ++i) {
		const double r = host[i].radius;
		if (!(r >= 0.0) || !std::isfinite(r))
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_upload: body %d has radius %g", i, r);
		if (r > rmax) rmax = r;
	}
	KEL_CUDA(cudaMemcpyAsync(ps->d, host, sizeof(kel_particle_state) * ps->n, cudaMemcpyHostToDevice, ps->lat->stream));
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	ps->max_radius = rmax;
	return KEL_OK;
}

extern "C" int kel_particles_download(kel_particles *ps, kel_particle_state *host) {
	if (!ps || !host) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_download: null argument");
	KEL_CUDA(cudaMemcpyAsync(host, ps->d, sizeof(kel_particle_state) * ps->n, cudaMemcpyDeviceToHost, ps->lat->stream));
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	return KEL_OK;
}

static BodyBox *cur_boxes(kel_particles *ps) { return static_cast<BodyBox *>(ps->boxes); }
static BodyBox *prev_boxes(kel_particles *ps) { return static_cast<BodyBox *>(ps->boxes) + ps->n; }

static int particles_reset(kel_particles *ps) {
	kel_lattice *L = ps->lat;
	k_pre<<<(ps->n + 127) / 128, 128, 0, L->stream>>>(make_view(L), ps->d, ps->n, 0, cur_boxes(ps), prev_boxes(ps), 0,
													   0, 1);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

static dim3 cell_grid(const kel_lattice *L) {
	return dim3((unsigned)((L->desc.nx + TX - 1) / TX), (unsigned)((L->desc.ny + TY - 1) / TY), (unsigned)L->desc.nz);
}

static int hlbm_steps(const kel_particle_params *prm) { return prm->sub_steps == 0 ? 1 : prm->sub_steps; }

// HLBM: porosity, reset of N / D and (with a buffer) the cell force field
static int particles_hlbm_couple(kel_particles *ps, const kel_particle_params *prm, bool want_cell_force) {
	kel_lattice *L = ps->lat;
	PView v = make_view(L);
	if (want_cell_force) {
		if (!ps->cell_force) KEL_CUDA(cudaMalloc(&ps->cell_force, sizeof(float) * L->plane * L->d.D));
		v.cell_force = ps->cell_force;
	}
	if (L->desc.storage == KEL_STORAGE_FP32)
		k_hlbm_couple<STORE_FP32><<<cell_grid(L), dim3(TX, TY), 0, L->stream>>>(v, ps->d, ps->n, prm->eps,
																				 hlbm_steps(prm));
	else
		k_hlbm_couple<STORE_FP16S><<<cell_grid(L), dim3(TX, TY), 0, L->stream>>>(v, ps->d, ps->n, prm->eps,
																				  hlbm_steps(prm));
	KEL_CUDA(cudaGetLastError());
	++L->por_epoch;
	ps->epoch = 0;
	return KEL_OK;
}

// PsmReset + couple.  The first couple of a particle set, and any couple
// after someone else wrote the porosity field, recomputes every cell; later
// ones only the cells of the bodies' current and previous boxes (identical
// field).  With reset, the bodies' force and torque are zeroed in the same
// launch.
static int particles_couple(kel_particles *ps, const kel_particle_params *prm, bool reset) {
	kel_lattice *L = ps->lat;
	if (prm->coupling == KEL_COUPLING_HLBM) {
		int rc;
		if (reset && (rc = particles_reset(ps))) return rc;
		ps->prev_is_last = ps->cur_fresh = false;
		return particles_hlbm_couple(ps, prm, false);
	}
	PView v = particle_view(ps, prm);
	const int mode = prm->porosity_mode;
	const bool incremental = ps->epoch != 0 && ps->epoch == L->por_epoch;
	// after the fused contact + integrate, the boxes are ready and nothing
	// needs resetting: no launch
	const bool ready = incremental && ps->prev_is_last && ps->cur_fresh && ps->cur_mode == mode &&
					   ps->cur_eps == prm->eps && !reset;
	if (!ready)
		k_pre<<<(ps->n + 127) / 128, 128, 0, L->stream>>>(v, ps->d, ps->n, mode != KEL_POROSITY_RAMP, cur_boxes(ps),
														   prev_boxes(ps), 1, incremental && !ps->prev_is_last ? 1 : 0,
														   reset ? 1 : 0);
	ps->prev_is_last = false;
	ps->cur_fresh = true;
	ps->cur_mode = mode;
	ps->cur_eps = prm->eps;
	if (incremental)
		k_couple_regions<<<dim3((unsigned)ps->n, (unsigned)couple_blocks(ps, prm)), RT, 0, L->stream>>>(
			v, ps->d, cur_boxes(ps), prev_boxes(ps), ps->n, prm->porosity_mode, prm->eps);
	else
		k_couple<<<cell_grid(L), dim3(TX, TY), 0, L->stream>>>(v, ps->d, cur_boxes(ps), ps->n, prm->porosity_mode,
															 prm->eps);
	KEL_CUDA(cudaGetLastError());
	ps->epoch = ++L->por_epoch;
	return KEL_OK;
}

static int particles_stamp(kel_particles *ps, const kel_particle_params *prm) {
	kel_lattice *L = ps->lat;
	k_hlbm_stamp<<<cell_grid(L), dim3(TX, TY), 0, L->stream>>>(make_view(L), ps->d, ps->n, hlbm_steps(prm));
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

static int ensure_partials(kel_particles *ps, int G) {
	if (ps->partial && ps->partial_cap >= G) return KEL_OK;
	if (ps->partial) {
		KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
		cudaFree(ps->partial);
		ps->partial = nullptr;
	}
	KEL_CUDA(cudaMalloc(&ps->partial, sizeof(double) * 6 * (size_t)ps->n * G));
	ps->partial_cap = G;
	return KEL_OK;
}

template <class Lc, int STORE>
static void launch_gather(const PView &v, kel_particles *ps, int steps, int mode, int G) {
	k_gather<Lc, STORE, false><<<dim3((unsigned)ps->n, (unsigned)G), GT, 0, ps->lat->stream>>>(v, ps->d, steps, mode,
																							  1.5, ps->partial);
}

// The gather's per-block sums into ps->partial (G blocks per body); with
// finish, they are added to the bodies' accumulators here, otherwise the
// contact pass adds them.
static int particles_gather(kel_particles *ps, const kel_particle_params *prm, bool want_cell_force, bool finish) {
	kel_lattice *L = ps->lat;
	PView v = particle_view(ps, prm);
	const int G = gather_blocks(ps, prm);
	int rc;
	if ((rc = ensure_partials(ps, G))) return rc;
	ps->gather_g = G;
	if (prm->coupling == KEL_COUPLING_HLBM) { // D2Q9 (checked); the couple pass wrote the cell forces
		const dim3 grid((unsigned)ps->n, (unsigned)G);
		if (L->desc.storage == KEL_STORAGE_FP32)
			k_gather<D2Q9, STORE_FP32, true><<<grid, GT, 0, L->stream>>>(v, ps->d, hlbm_steps(prm), KEL_POROSITY_RAMP,
																		  prm->eps, ps->partial);
		else
			k_gather<D2Q9, STORE_FP16S, true><<<grid, GT, 0, L->stream>>>(v, ps->d, hlbm_steps(prm),
																		   KEL_POROSITY_RAMP, prm->eps, ps->partial);
	} else {
		if (want_cell_force) {
			if (!ps->cell_force) KEL_CUDA(cudaMalloc(&ps->cell_force, sizeof(float) * L->plane * L->d.D));
			KEL_CUDA(cudaMemsetAsync(ps->cell_force, 0, sizeof(float) * L->plane * L->d.D, L->stream));
			v.cell_force = ps->cell_force;
		}
		const bool f32 = L->desc.storage == KEL_STORAGE_FP32;
		switch (L->d.Q) {
		case 9: f32 ? launch_gather<D2Q9, STORE_FP32>(v, ps, prm->sub_steps, prm->porosity_mode, G)
					: launch_gather<D2Q9, STORE_FP16S>(v, ps, prm->sub_steps, prm->porosity_mode, G); break;
		case 19: f32 ? launch_gather<D3Q19, STORE_FP32>(v, ps, prm->sub_steps, prm->porosity_mode, G)
					 : launch_gather<D3Q19, STORE_FP16S>(v, ps, prm->sub_steps, prm->porosity_mode, G); break;
		default: f32 ? launch_gather<D3Q27, STORE_FP32>(v, ps, prm->sub_steps, prm->porosity_mode, G)
					 : launch_gather<D3Q27, STORE_FP16S>(v, ps, prm->sub_steps, prm->porosity_mode, G); break;
		}
	}
	if (finish) k_gather_finish<<<(ps->n + 127) / 128, 128, 0, L->stream>>>(ps->d, ps->n, L->d.D, ps->partial, G);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

static bool is_fplbm(const kel_particle_params *prm) {
	return prm->coupling == KEL_COUPLING_FPLBM || prm->coupling == KEL_COUPLING_FPLBM_OWN;
}

// FPLBM couple: the bodies' boxes, FpLbmReset on every cell, then the
// porosity / force fields of the particle pass.
static int particles_fplbm_couple(kel_particles *ps, const kel_particle_params *prm) {
	kel_lattice *L = ps->lat;
	PView v = make_view(L);
	v.cell_force = L->force;
	const int own = prm->coupling == KEL_COUPLING_FPLBM_OWN;
	k_pre<<<(ps->n + 127) / 128, 128, 0, L->stream>>>(v, ps->d, ps->n, 0, cur_boxes(ps), prev_boxes(ps), 1, 0, 0);
	const dim3 rg((unsigned)((L->desc.nx + 127) / 128), (unsigned)L->desc.ny);
	if (L->desc.storage == KEL_STORAGE_FP32) k_fplbm_reset<STORE_FP32><<<rg, 128, 0, L->stream>>>(v, L->flags, L->plain_flags_fplbm);
	else k_fplbm_reset<STORE_FP16S><<<rg, 128, 0, L->stream>>>(v, L->flags, L->plain_flags_fplbm);
	k_fplbm_field<<<cell_grid(L), dim3(TX, TY), 0, L->stream>>>(v, ps->d, cur_boxes(ps), ps->n, own,
																(double)prm->sub_steps);
	KEL_CUDA(cudaGetLastError());
	++L->por_epoch;
	ps->epoch = 0;
	ps->prev_is_last = ps->cur_fresh = false;
	return KEL_OK;
}

// FPLBM gather: each body's coupling-force sum (boxes of the last couple),
// then (set_accel) its acceleration and (verlet) the Verlet sub-steps.
static int particles_fplbm_gather(kel_particles *ps, const kel_particle_params *prm, bool verlet) {
	kel_lattice *L = ps->lat;
	const int G = gather_blocks(ps, prm);
	int rc;
	if ((rc = ensure_partials(ps, G))) return rc;
	ps->gather_g = G;
	const int own = prm->coupling == KEL_COUPLING_FPLBM_OWN;
	k_fplbm_sums<<<dim3((unsigned)ps->n, (unsigned)G), GT, 0, L->stream>>>(make_view(L), ps->d, cur_boxes(ps), own,
																		   (double)prm->sub_steps, ps->partial);
	k_fplbm_integrate<<<(ps->n + 127) / 128, 128, 0, L->stream>>>(ps->d, ps->n, *prm, ps->partial, G, 1,
																   verlet ? 1 : 0);
	KEL_CUDA(cudaGetLastError());
	if (verlet) ps->cur_fresh = false;
	return KEL_OK;
}

// ParticleContact; with fold, the gather partials are added first.
static int particles_contact(kel_particles *ps, const kel_particle_params *prm, bool fold) {
	kel_lattice *L = ps->lat;
	k_contact<<<(ps->n + 3) / 4, 128, 0, L->stream>>>(ps->d, ps->n, L->d.D, *prm, (int)L->desc.nx, (int)L->desc.ny,
													   (int)L->desc.nz, (L->desc.flags & KEL_LATTICE_PERIODIC_X) ? 1 : 0,
													   fold ? ps->partial : nullptr, ps->gather_g);
	KEL_CUDA(cudaGetLastError());
	return KEL_OK;
}

static int particles_integrate(kel_particles *ps, const kel_particle_params *prm) {
	kel_lattice *L = ps->lat;
	k_integrate<<<(ps->n + 127) / 128, 128, 0, L->stream>>>(ps->d, ps->n, L->d.D, *prm, (int)L->desc.nx,
															 (L->desc.flags & KEL_LATTICE_PERIODIC_X) ? 1 : 0);
	KEL_CUDA(cudaGetLastError());
	ps->cur_fresh = false; // the bodies moved
	return KEL_OK;
}

template <class Lc, int STORE>
static void launch_couple_gather(const PView &v, kel_particles *ps, const kel_particle_params *prm, int G) {
	k_couple_gather<Lc, STORE><<<dim3((unsigned)ps->n, (unsigned)G), RT, 0, ps->lat->stream>>>(
		v, ps->d, cur_boxes(ps), prev_boxes(ps), ps->n, prm->porosity_mode, prm->eps,
		static_cast<const CoupleRec *>(ps->rec), ps->partial);
}

// Couple and gather of a coupled PSM step in one launch, when the couple is
// incremental and the boxes are prepared (*done); otherwise nothing happens.
static int particles_couple_gather(kel_particles *ps, const kel_particle_params *prm, bool *done) {
	*done = false;
	kel_lattice *L = ps->lat;
	const int mode = prm->porosity_mode;
	const bool incremental = ps->epoch != 0 && ps->epoch == L->por_epoch;
	if (!(incremental && ps->prev_is_last && ps->cur_fresh && ps->cur_mode == mode && ps->cur_eps == prm->eps))
		return KEL_OK;
	if (!(ps->rec_mode == mode && ps->rec_steps == prm->sub_steps && ps->rec_eps == prm->eps)) return KEL_OK;
	const int G = couple_blocks(ps, prm);
	int rc;
	if ((rc = ensure_partials(ps, G))) return rc;
	const PView v = particle_view(ps, prm);
	const bool f32 = L->desc.storage == KEL_STORAGE_FP32;
	switch (L->d.Q) {
	case 9: f32 ? launch_couple_gather<D2Q9, STORE_FP32>(v, ps, prm, G) : launch_couple_gather<D2Q9, STORE_FP16S>(v, ps, prm, G); break;
	case 19: f32 ? launch_couple_gather<D3Q19, STORE_FP32>(v, ps, prm, G) : launch_couple_gather<D3Q19, STORE_FP16S>(v, ps, prm, G); break;
	default: f32 ? launch_couple_gather<D3Q27, STORE_FP32>(v, ps, prm, G) : launch_couple_gather<D3Q27, STORE_FP16S>(v, ps, prm, G); break;
	}
	KEL_CUDA(cudaGetLastError());
	ps->gather_g = G;
	ps->prev_is_last = false;
	ps->cur_fresh = true;
	ps->epoch = ++L->por_epoch;
	*done = true;
	return KEL_OK;
}

// Contact (from zero, with the gather sums) and integrate of the coupled
// step in one launch, which also prepares the next couple's boxes; the
// bodies' new state lands in the second buffer, which becomes the current
// one.
static int particles_contact_integrate(kel_particles *ps, const kel_particle_params *prm, cudaStream_t st) {
	kel_lattice *L = ps->lat;
	const PView v = particle_view(ps, prm);
	const int cm = couple_mode(prm->porosity_mode, v.direct);
	const double reach = (cm == 1 || cm == 2) ? subcell_reach(L->d.D) : 0.0;
	CoupleRec *rec = static_cast<CoupleRec *>(ps->rec);
#define KEL_CI(Lc)                                                                                                     \
	k_contact_integrate<Lc><<<ps->n, 32, 0, st>>>(ps->d, ps->d_alt, v, *prm, ps->partial, ps->gather_g, cur_boxes(ps),  \
												  prev_boxes(ps), cm, reach, rec)
	switch (L->d.Q) {
	case 9: KEL_CI(D2Q9); break;
	case 19: KEL_CI(D3Q19); break;
	default: KEL_CI(D3Q27); break;
	}
#undef KEL_CI
	KEL_CUDA(cudaGetLastError());
	ps->rec_mode = prm->porosity_mode;
	ps->rec_steps = prm->sub_steps;
	ps->rec_eps = prm->eps;
	kel_particle_state *t = ps->d; // the bodies' new state is in the other buffer
	ps->d = ps->d_alt;
	ps->d_alt = t;
	ps->prev_is_last = true;
	ps->cur_fresh = true;
	ps->cur_mode = prm->porosity_mode;
	ps->cur_eps = prm->eps;
	return KEL_OK;
}

extern "C" int kel_particles_reset(kel_particles *ps) {
	if (!ps) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_reset: null argument");
	int rc = particles_reset(ps);
	if (rc) return rc;
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	return KEL_OK;
}

extern "C" int kel_particles_couple(kel_particles *ps, const kel_particle_params *prm) {
	int rc = check_params(ps, prm, "kel_particles_couple");
	if (rc) return rc;
	if (is_fplbm(prm)) rc = particles_fplbm_couple(ps, prm);
	else rc = particles_couple(ps, prm, false);
	if (rc) return rc;
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	return KEL_OK;
}

extern "C" int kel_particles_gather(kel_particles *ps, const kel_particle_params *prm, float *host_cell_force) {
	int rc = check_params(ps, prm, "kel_particles_gather");
	if (rc) return rc;
	if (is_fplbm(prm)) { // the coupling forces are the "force" field the couple wrote
		if ((rc = particles_fplbm_gather(ps, prm, false))) return rc;
		if (host_cell_force && (rc = field_to_host(ps->lat, ps->lat->force, host_cell_force, 2))) return rc;
		KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
		return KEL_OK;
	}
	// HLBM: the cell force is the momentum of the last gather writing each
	// cell, computed on the populations before the bodies move
	if (prm->coupling == KEL_COUPLING_HLBM && host_cell_force && (rc = particles_hlbm_couple(ps, prm, true)))
		return rc;
	if ((rc = particles_gather(ps, prm, host_cell_force != nullptr, true))) return rc;
	if (host_cell_force) {
		kel_lattice *L = ps->lat;
		if ((rc = field_to_host(L, ps->cell_force, host_cell_force, L->d.D))) return rc;
	}
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	return KEL_OK;
}

extern "C" int kel_particles_contact(kel_particles *ps, const kel_particle_params *prm) {
	int rc = check_params(ps, prm, "kel_particles_contact");
	if (rc || (rc = particles_contact(ps, prm, false))) return rc;
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	return KEL_OK;
}

extern "C" int kel_particles_integrate(kel_particles *ps, const kel_particle_params *prm) {
	int rc = check_params(ps, prm, "kel_particles_integrate");
	if (rc) return rc;
	if (is_fplbm(prm)) { // Verlet with the acceleration the gather set
		k_fplbm_integrate<<<(ps->n + 127) / 128, 128, 0, ps->lat->stream>>>(ps->d, ps->n, *prm, ps->partial, 1, 0, 1);
		KEL_CUDA(cudaGetLastError());
		ps->cur_fresh = false;
	} else if ((rc = particles_integrate(ps, prm))) {
		return rc;
	}
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	return KEL_OK;
}

extern "C" int kel_particles_stamp(kel_particles *ps, const kel_particle_params *prm) {
	int rc = check_params(ps, prm, "kel_particles_stamp");
	if (rc) return rc;
	if (prm->coupling != KEL_COUPLING_HLBM)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_stamp: HLBM coupling only");
	if ((rc = particles_stamp(ps, prm))) return rc;
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	return KEL_OK;
}

// One coupled step: reset + couple (one launch), gather, contact (adding the
// gather sums), integrate, (HLBM: stamp,) sweep.  With PSM coupling the
// contact starts from zero and the integrate prepares the next couple's
// boxes, so from the second step on a step is couple, gather, contact,
// integrate and the sweep.
// With a side stream (graph capture only), contact and integrate run on it
// while the sweep runs on the lattice's stream: the PSM sweep reads the
// porosity the couple wrote and the populations the gather has read, the
// bodies' pass reads and writes only the bodies and their boxes; the next
// couple waits for both.
static int coupled_step(kel_particles *ps, const kel_particle_params *prm, const kel_step_program *prog,
						uint32_t flags, cudaStream_t side = nullptr) {
	int rc;
	if (is_fplbm(prm)) {
		// examples/moving_poiseulle_particles_2d_fplbm_gpu/sim.cpp:186-258: reset
		// + particle pass (with the integration), then the sweep; its BGK
		// boundary cases store their macros every step
		if ((rc = particles_fplbm_couple(ps, prm)) || (rc = particles_fplbm_gather(ps, prm, true))) return rc;
		return kel_step(ps->lat, prog, 1, flags | KEL_STEP_ALL_MACROS);
	}
	const bool fused = prm->coupling == KEL_COUPLING_PSM;
	bool cg = false;
	if (fused && (rc = particles_couple_gather(ps, prm, &cg))) return rc;
	if (!cg && ((rc = particles_couple(ps, prm, !fused)) || (rc = particles_gather(ps, prm, false, false)))) return rc;
	if (fused && side) {
		kel_lattice *L = ps->lat;
		KEL_CUDA(cudaEventRecord(ps->ev_fork, L->stream));
		KEL_CUDA(cudaStreamWaitEvent(side, ps->ev_fork, 0));
		if ((rc = particles_contact_integrate(ps, prm, side))) return rc;
		KEL_CUDA(cudaEventRecord(ps->ev_join, side));
		if ((rc = kel_step(L, prog, 1, flags))) return rc;
		KEL_CUDA(cudaStreamWaitEvent(L->stream, ps->ev_join, 0));
		return KEL_OK;
	}
	if (fused) {
		if ((rc = particles_contact_integrate(ps, prm, ps->lat->stream))) return rc;
	} else if ((rc = particles_contact(ps, prm, true)) || (rc = particles_integrate(ps, prm))) {
		return rc;
	}
	if (prm->coupling == KEL_COUPLING_HLBM && (rc = particles_stamp(ps, prm))) return rc;
	return kel_step(ps->lat, prog, 1, flags);
}

static ParticleGraphKey graph_key(kel_particles *ps, const kel_particle_params *prm, const kel_step_program *prog) {
	ParticleGraphKey k;
	memset(&k, 0, sizeof(k));
	kel_lattice *L = ps->lat;
	k.prm = *prm;
	k.prog = *prog;
	k.sweep = sweep_params(L, prog);
	k.f = L->f;
	k.por = L->por;
	k.force = L->force;
	k.bodies = ps->d;
	k.boxes = ps->boxes;
	k.partial = ps->partial;
	k.rec = ps->rec;
	k.direct = direct_mode(ps, prm);
	k.shape = ps->shape;
	k.n = ps->n;
	k.gather_g = gather_blocks(ps, prm);
	k.couple_g = couple_blocks(ps, prm);
	k.cpt = L->cpt;
	k.block = L->block;
	return k;
}

// The captured graph of two coupled PSM steps starting at an even time step
// (incremental couples), re-captured when anything it bakes in changed.  The
// host bookkeeping the captured calls do (time step, porosity epoch) is put
// back, since nothing ran.
static int ensure_particle_graph(kel_particles *ps, const kel_particle_params *prm, const kel_step_program *prog) {
	kel_lattice *L = ps->lat;
	int rc;
	const int gmax = gather_blocks(ps, prm) > couple_blocks(ps, prm) ? gather_blocks(ps, prm) : couple_blocks(ps, prm);
	if ((rc = ensure_partials(ps, gmax))) return rc; // no allocation inside the capture
	if (!ps->side) {
		KEL_CUDA(cudaStreamCreateWithFlags(&ps->side, cudaStreamNonBlocking));
		KEL_CUDA(cudaEventCreateWithFlags(&ps->ev_fork, cudaEventDisableTiming));
		KEL_CUDA(cudaEventCreateWithFlags(&ps->ev_join, cudaEventDisableTiming));
	}
	const ParticleGraphKey k = graph_key(ps, prm, prog);
	if (ps->graph && memcmp(&k, &ps->key, sizeof(k)) == 0) return KEL_OK;
	if (ps->graph) cudaGraphExecDestroy(ps->graph);
	ps->graph = nullptr;
	const uint64_t t0 = L->t, e0 = L->por_epoch, pe0 = ps->epoch;
	const bool pl0 = ps->prev_is_last, cf0 = ps->cur_fresh;
	const int cm0 = ps->cur_mode;
	const double ce0 = ps->cur_eps;
	if (cudaStreamBeginCapture(L->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
		cudaGetLastError();
		return KEL_ERR_CUDA;
	}
	rc = coupled_step(ps, prm, prog, 0, ps->side);
	if (rc == KEL_OK) rc = coupled_step(ps, prm, prog, 0, ps->side);
	cudaGraph_t g = nullptr;
	cudaError_t e = cudaStreamEndCapture(L->stream, &g);
	L->t = t0;
	L->por_epoch = e0;
	ps->epoch = pe0;
	ps->prev_is_last = pl0;
	ps->cur_fresh = cf0;
	ps->cur_mode = cm0;
	ps->cur_eps = ce0;
	if (rc == KEL_OK && e == cudaSuccess && g) e = cudaGraphInstantiate(&ps->graph, g, 0);
	if (g) cudaGraphDestroy(g);
	if (rc != KEL_OK || e != cudaSuccess || !ps->graph) {
		cudaGetLastError();
		ps->graph = nullptr;
		return KEL_ERR_CUDA;
	}
	ps->key = k;
	return KEL_OK;
}

extern "C" int kel_particles_step(kel_particles *ps, const kel_particle_params *prm, const kel_step_program *prog,
								  uint64_t n_steps, uint32_t step_flags) {
	int rc = check_params(ps, prm, "kel_particles_step");
	if (rc) return rc;
	if (!prog) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_step: null program");
	const bool hlbm = prm->coupling == KEL_COUPLING_HLBM;
	if (hlbm != (prog->collision == KEL_COLL_HLBM))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_step: HLBM coupling goes with the KEL_COLL_HLBM collision");
	if (is_fplbm(prm) != (prog->collision == KEL_COLL_FPLBM))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_step: FPLBM coupling goes with the KEL_COLL_FPLBM collision");
	kel_lattice *L = ps->lat;
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	if (L->stream != nullptr) KEL_CUDA(cudaStreamIsCapturing(L->stream, &cap));
	// Steps without macro output replay a captured graph of two coupled steps
	// (PSM coupling, non-default stream, one-cell-per-thread style sweeps) once
	// the set is on incremental couples at an even time step.
	const uint64_t plain = (step_flags & KEL_STEP_ALL_MACROS)
							   ? 0
							   : ((step_flags & KEL_STEP_WRITE_MACROS) && n_steps > 0 ? n_steps - 1 : n_steps);
	const bool graphable = prm->coupling == KEL_COUPLING_PSM && L->stream != nullptr &&
						   cap == cudaStreamCaptureStatusNone && L->cpt != CPT_ROWS;
	uint64_t s = 0;
	for (; s < n_steps; ++s) {
		// the captured steps must find what the replayed ones leave: an
		// incremental couple and (fused path) boxes prepared by the previous step
		const bool steady = ps->prev_is_last && ps->cur_fresh;
		if (graphable && s < plain && plain - s >= 4 && (L->t & 1u) == 0 && ps->epoch != 0 &&
			ps->epoch == L->por_epoch && steady && L->have_ops && memcmp(&L->last_prog, prog, sizeof(*prog)) == 0)
			break;
		const uint32_t fl = (s + 1 == n_steps) ? step_flags : (step_flags & KEL_STEP_ALL_MACROS);
		if ((rc = coupled_step(ps, prm, prog, fl))) return rc;
	}
	if (s < n_steps) {
		const uint64_t reps = (plain - s) / 2;
		if (ensure_particle_graph(ps, prm, prog) == KEL_OK) {
			for (uint64_t r = 0; r < reps; ++r) {
				cudaError_t e = cudaGraphLaunch(ps->graph, L->stream);
				if (e != cudaSuccess)
					return fail(KEL_ERR_CUDA, "kel_particles_step: graph launch failed: %s", cudaGetErrorString(e));
			}
			s += 2 * reps;
			L->t += 2 * reps;
			ps->epoch = ++L->por_epoch; // the replays left the field of their last couple
		}
		for (; s < n_steps; ++s) {
			const uint32_t fl = (s + 1 == n_steps) ? step_flags : (step_flags & KEL_STEP_ALL_MACROS);
			if ((rc = coupled_step(ps, prm, prog, fl))) return rc;
		}
	}
	return KEL_OK;
}

// ---- voxel shapes ------------------------------------------------------------

namespace {

// solid_fraction_from_sdf (mask.hpp:291-311) on the host
double solid_host(double sdf, double eps) {
	const double half = eps / 2;
	if (sdf <= -half) return 1;
	if (sdf >= half) return 0;
	const double t = (sdf + half) / eps;
	const double c = std::cos(PI_D * t / 2);
	return c * c;
}

// Voxel k (flat, last axis fastest) -> normalised local position
// (mask_voxel_to_local, mask.hpp:111-125).
void voxel_local(int D, int R, int64_t k, double *u) {
	const double step = 2.0 / (double)R;
	int64_t idx[3] = {0, 0, 0};
	for (int i = D - 1; i >= 0; --i) {
		idx[i] = k % R;
		k /= R;
	}
	for (int i = 0; i < D; ++i) u[i] = -1 + ((double)idx[i] + 0.5) * step;
}

int64_t voxel_count(int D, int R) { return D == 3 ? (int64_t)R * R * R : (int64_t)R * R; }

// The largest |u| over the voxels at distance <= 0, plus one voxel diagonal.
double mask_reach(const kel_shape *sh) {
	double best = -1.0;
	const int64_t n = voxel_count(sh->dim, sh->res);
	for (int64_t k = 0; k < n; ++k) {
		if (!(sh->mask[k] <= 0.0)) continue;
		double u[3] = {0, 0, 0};
		voxel_local(sh->dim, sh->res, k, u);
		double s = 0;
		for (int i = 0; i < sh->dim; ++i) s = s + u[i] * u[i];
		s = std::sqrt(s);
		if (s > best) best = s;
	}
	return best < 0 ? 0.0 : best + (2.0 / (double)sh->res) * std::sqrt((double)sh->dim);
}

int shape_upload(kel_shape *sh) {
	const int64_t n = voxel_count(sh->dim, sh->res);
	std::vector<float> mf((size_t)n);
	for (int64_t k = 0; k < n; ++k) mf[k] = (float)sh->mask[k];
	cudaError_t e = cudaMalloc(&sh->d_mask_f, sizeof(float) * n);
	if (e == cudaSuccess) e = cudaMalloc(&sh->d_mask_d, sizeof(double) * n);
	if (e == cudaSuccess) e = cudaMemcpy(sh->d_mask_f, mf.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(sh->d_mask_d, sh->mask.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
	if (e != cudaSuccess)
		return fail(e == cudaErrorMemoryAllocation ? KEL_ERR_OUT_OF_MEMORY : KEL_ERR_CUDA, "kel_shape: %s",
					cudaGetErrorString(e));
	sh->reach = mask_reach(sh);
	return KEL_OK;
}

int shape_args(int32_t dim, int32_t resolution, kel_shape **out, const char *who) {
	if (!out) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: null argument", who);
	*out = nullptr;
	if (dim != 2 && dim != 3) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: dimension %d", who, dim);
	if (resolution < 2 || resolution > (dim == 2 ? 4096 : 512))
		return fail(KEL_ERR_INVALID_ARGUMENT, "%s: resolution %d", who, resolution);
	return KEL_OK;
}

} // namespace

extern "C" int kel_shape_create(int32_t dim, int32_t resolution, int32_t kind, kel_shape **out) {
	int rc = shape_args(dim, resolution, out, "kel_shape_create");
	if (rc) return rc;
	if (kind != KEL_SHAPE_SPHERE && kind != KEL_SHAPE_CUBE)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_shape_create: unknown shape %d", kind);
	kel_shape *sh = new kel_shape();
	sh->dim = dim;
	sh->res = resolution;
	const int64_t n = voxel_count(dim, resolution);
	sh->mask.resize((size_t)n);
	// fill_mask_from_sdf (mask.hpp:351-394): voxels in iteration order, the
	// centroid weighted by a one-voxel ramp
	const double step = 2.0 / (double)resolution;
	double wsum = 0, c[3] = {0, 0, 0};
	for (int64_t k = 0; k < n; ++k) {
		double u[3] = {0, 0, 0};
		voxel_local(dim, resolution, k, u);
		double d;
		if (kind == KEL_SHAPE_CUBE) { // sdf::cube (mask.hpp:328-340)
			double m = 0;
			for (int i = 0; i < dim; ++i) {
				const double a = std::fabs(u[i]);
				if (a > m) m = a;
			}
			d = m - 1;
		} else { // sdf::sphere (mask.hpp:317-322)
			double q = 0;
			for (int i = 0; i < dim; ++i) q = q + u[i] * u[i];
			d = std::sqrt(q) - 1;
		}
		sh->mask[k] = d;
		const double w = solid_host(d, step);
		wsum += w;
		for (int i = 0; i < dim; ++i) c[i] = c[i] + w * u[i];
	}
	if (wsum > 0)
		for (int i = 0; i < dim; ++i) c[i] = c[i] / wsum;
	for (int i = 0; i < 3; ++i) sh->com[i] = i < dim ? c[i] : 0.0;
	if ((rc = shape_upload(sh))) {
		kel_shape_destroy(sh);
		return rc;
	}
	*out = sh;
	return KEL_OK;
}

extern "C" int kel_shape_create_from_mask(int32_t dim, int32_t resolution, const double *mask,
										  const double *center_of_mass, kel_shape **out) {
	int rc = shape_args(dim, resolution, out, "kel_shape_create_from_mask");
	if (rc) return rc;
	if (!mask || !center_of_mass) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_shape_create_from_mask: null argument");
	const int64_t n = voxel_count(dim, resolution);
	for (int64_t k = 0; k < n; ++k)
		if (!std::isfinite(mask[k]))
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_shape_create_from_mask: voxel %lld is not finite", (long long)k);
	kel_shape *sh = new kel_shape();
	sh->dim = dim;
	sh->res = resolution;
	sh->mask.assign(mask, mask + n);
	for (int i = 0; i < 3; ++i) sh->com[i] = i < dim ? center_of_mass[i] : 0.0;
	if ((rc = shape_upload(sh))) {
		kel_shape_destroy(sh);
		return rc;
	}
	*out = sh;
	return KEL_OK;
}

extern "C" int kel_shape_info(const kel_shape *shape, double *mask, double *center_of_mass, double *reach) {
	if (!shape) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_shape_info: null shape");
	if (mask) std::memcpy(mask, shape->mask.data(), sizeof(double) * shape->mask.size());
	if (center_of_mass)
		for (int i = 0; i < 3; ++i) center_of_mass[i] = shape->com[i];
	if (reach) *reach = shape->reach;
	return KEL_OK;
}

extern "C" int kel_shape_destroy(kel_shape *shape) {
	if (!shape) return KEL_OK;
	cudaFree(shape->d_mask_f);
	cudaFree(shape->d_mask_d);
	delete shape;
	return KEL_OK;
}

extern "C" int kel_particles_set_shape(kel_particles *ps, const kel_shape *shape) {
	if (!ps) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_set_shape: null particles");
	if (shape && shape->dim != ps->lat->d.D)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_set_shape: %dD shape on a %dD lattice", shape->dim,
					ps->lat->d.D);
	KEL_CUDA(cudaStreamSynchronize(ps->lat->stream));
	ps->shape = shape;
	ps->cur_fresh = false; // voxel boxes depend on the shape's reach
	ps->rec_mode = -1;
	return KEL_OK;
}

static PView voxel_view(kel_particles *ps) {
	kel_particle_params prm;
	std::memset(&prm, 0, sizeof(prm));
	prm.porosity_mode = KEL_POROSITY_VOXEL;
	prm.eps = 1.0;
	return particle_view(ps, &prm);
}

extern "C" int kel_particles_voxel_distance(kel_particles *ps, int32_t body, const double *points, int32_t n,
											double *out) {
	if (!ps || (!points && n > 0) || (!out && n > 0) || n < 0)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_voxel_distance: bad arguments");
	if (body < 0 || body >= ps->n) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_voxel_distance: body %d", body);
	if (!ps->shape) return fail(KEL_ERR_STATE, "kel_particles_voxel_distance: no shape set");
	if (n == 0) return KEL_OK;
	kel_lattice *L = ps->lat;
	const int D = L->d.D;
	std::vector<double> p3((size_t)n * 3, 0.0);
	for (int32_t k = 0; k < n; ++k)
		for (int i = 0; i < D; ++i) p3[(size_t)k * 3 + i] = points[(size_t)k * D + i];
	double *d_buf = nullptr;
	KEL_CUDA(cudaMalloc(&d_buf, sizeof(double) * 4 * (size_t)n));
	cudaError_t e = cudaMemcpyAsync(d_buf, p3.data(), sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, L->stream);
	if (e == cudaSuccess) {
		k_voxel_distance<<<(n + 127) / 128, 128, 0, L->stream>>>(voxel_view(ps), ps->d, body, d_buf, n, d_buf + 3 * (size_t)n);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(out, d_buf + 3 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost, L->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
	cudaFree(d_buf);
	if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_particles_voxel_distance: %s", cudaGetErrorString(e));
	return KEL_OK;
}

extern "C" int kel_particles_voxel_contact(kel_particles *ps, const int32_t *pairs, int32_t npairs, double eps,
										   kel_contact_manifold *out) {
	if (!ps || npairs < 0 || (npairs > 0 && (!pairs || !out)))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_voxel_contact: bad arguments");
	if (!(eps > 0)) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_voxel_contact: eps must be positive");
	if (!ps->shape) return fail(KEL_ERR_STATE, "kel_particles_voxel_contact: no shape set");
	for (int32_t k = 0; k < 2 * npairs; ++k)
		if (pairs[k] < 0 || pairs[k] >= ps->n)
			return fail(KEL_ERR_INVALID_ARGUMENT, "kel_particles_voxel_contact: body index %d", pairs[k]);
	if (npairs == 0) return KEL_OK;
	kel_lattice *L = ps->lat;
	int *d_pairs = nullptr;
	kel_contact_manifold *d_out = nullptr;
	cudaError_t e = cudaMalloc(&d_pairs, sizeof(int) * 2 * (size_t)npairs);
	if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(kel_contact_manifold) * (size_t)npairs);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(d_pairs, pairs, sizeof(int) * 2 * (size_t)npairs, cudaMemcpyHostToDevice, L->stream);
	if (e == cudaSuccess) {
		k_voxel_contact<<<npairs, VT, 0, L->stream>>>(voxel_view(ps), ps->d, d_pairs, eps, d_out);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(out, d_out, sizeof(kel_contact_manifold) * (size_t)npairs, cudaMemcpyDeviceToHost,
							L->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
	cudaFree(d_pairs);
	cudaFree(d_out);
	if (e != cudaSuccess) return fail(KEL_ERR_CUDA, "kel_particles_voxel_contact: %s", cudaGetErrorString(e));
	return KEL_OK;
}
