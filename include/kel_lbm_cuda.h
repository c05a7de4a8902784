/*
 * kel_lbm_cuda.h -- C ABI of the GB300 lattice-Boltzmann hot path.
 *
 * Drop-in boundary for the per-cell collide + boundary + stream sweep of
 * keldu/lbm_mirror (kel::lbm).  The reference exposes that path only as
 * header-only C++ templates executed inside SYCL parallel_for lambdas; a
 * foreign caller would bind exactly these entry points.  Every function is
 * extern "C", takes plain pointers/sizes and returns an int status
 * (KEL_OK = 0, negative KEL_ERR_* on failure; kel_last_error_string() gives
 * the message of the last failure on the calling thread).
 *
 * Layout conventions (same as the reference's host data):
 *   - cell index c = x + nx*(y + ny*z)  (x fastest, flatten.hpp:11-39)
 *   - AoS populations: f[c*Q + i], direction order of df_info<T,Desc>
 *     (descriptor/d2q9.hpp:17-27, d3q19.hpp:15-37, d3q27.hpp:9-103)
 *   - flags: one uint8 per cell, meaning given by kel_step_program.ops[flag]
 *
 * Inside, the populations live in HBM as structure-of-arrays in a single
 * in-place (AA-pattern) lattice; uploads/downloads convert.
 */
#ifndef KEL_LBM_CUDA_H
#define KEL_LBM_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define KEL_OK 0
#define KEL_ERR_INVALID_ARGUMENT (-1)
#define KEL_ERR_OUT_OF_MEMORY (-2)
#define KEL_ERR_CUDA (-3)
#define KEL_ERR_DEVICE_CHECK (-4)
#define KEL_ERR_TIMEOUT (-5)
#define KEL_ERR_UNSUPPORTED (-6)
#define KEL_ERR_STATE (-7)

/* ---- lattice descriptors (df_info<T,Desc>) ------------------------------ */
#define KEL_D2Q9 9   /* descriptor/d2q9.hpp:11-57 */
#define KEL_D3Q19 19 /* descriptor/d3q19.hpp:9-70 */
#define KEL_D3Q27 27 /* descriptor/d3q27.hpp:9-103 */

/* ---- population storage in HBM ----------------------------------------- */
#define KEL_STORAGE_FP32 0  /* f_i as float */
#define KEL_STORAGE_FP16S 1 /* f_i - w_i as half, arithmetic in float */

/* ---- lattice creation flags -------------------------------------------- */
#define KEL_LATTICE_PERIODIC_X 1u /* x wraps (ghost columns copied from the opposite side) */

/* ---- per-flag boundary operation (the reference drivers' switch(info)) - *
 * Flag value 0 is the drivers' `case 0u: break;`: the cell is neither
 * collided nor streamed, and its neighbours read zero from it, as from the
 * ghost ring.  Flag values >= KEL_MAX_FLAGS take the `default: break;` path
 * (no boundary step, no collision, streamed). */
#define KEL_BC_NONE 0              /* no boundary step (collide if .collide) */
#define KEL_BC_BOUNCE_BACK 1       /* cmpt::BounceBack, full-way (boundary.hpp:32-76) */
#define KEL_BC_FLUID 2             /* no boundary step; collide if .collide */
#define KEL_BC_ZOUHE_VELOCITY_X 3  /* cmpt::ZouHeVelocityX<east> D2Q9 (boundary.hpp:759-805) */
#define KEL_BC_ZOUHE_PRESSURE_X 4  /* cmpt::ZouHePressureX<east> D2Q9/D3Q27 (boundary.hpp:175-756) */
#define KEL_BC_MOVING_WALL 5       /* lid: f_i = f_opp + 2 w_i (c_i.u_w)/cs^2 (cavity_2d_gpu.cpp:204-235) */
#define KEL_BC_ANTI_BOUNCE_BACK 6  /* cmpt::AntiBounceBack, D2Q9 y-mirror (boundary.hpp:81-133) */
#define KEL_BC_EQUILIBRIUM 7       /* cmpt::Equilibrium(rho,u) (boundary.hpp:135-161) */
/* Half-way bounce-back wall (no counterpart in the reference, whose walls
 * are full-way): a cell with this op is solid and computes nothing; a
 * population a computed cell sends towards it returns to that cell in the
 * opposite direction in the same step (the wall sits half way between the
 * two cell centres).  Populations stored at such cells are undefined.
 * Sweeps with one cell per thread; batches reject it. */
#define KEL_BC_HALFWAY_WALL 8

/* ---- collision operator applied to cells whose op has .collide = 1 ------ */
#define KEL_COLL_BGK 0     /* cmpt::BGK (collision.hpp:19-97) */
#define KEL_COLL_BGK_GUO 1 /* cmpt::BGKGuo (collision.hpp:99-205) */
#define KEL_COLL_PSM 2     /* cmpt::Psm (psm.hpp:37-90) */
#define KEL_COLL_PSM_GUO 3 /* cmpt::Psm followed by the BGKGuo forcing term */
#define KEL_COLL_HLBM 4    /* cmpt::Hlbm (hlbm.hpp:53-101), D2Q9: u <- u por + (D > 0 ? N (1 - por) / D : N) */
/* cmpt::FpLbm (fplbm.hpp:57-128) on cells whose op has no boundary step: BGK
 * plus the Guo forcing term of the cell's "force" field (the coupling force
 * the FPLBM particle pass wrote), velocity = momentum / density of the
 * populations, no global force; the density / velocity macros are left as
 * FpLbmReset wrote them (density and momentum).  Cells with a boundary step
 * collide with plain BGK (the drivers' ZouHe + BGK cases). */
#define KEL_COLL_FPLBM 5

/* ---- arithmetic mode of the sweep -------------------------------------- */
#define KEL_ARITH_FAST 0      /* float-float equilibrium bracket, fused BGK relaxation */
#define KEL_ARITH_REFERENCE 1 /* the reference's rounding sequence (double equilibrium bracket): bit-exact */
#define KEL_ARITH_SHIFTED 2   /* batches only: FP32 populations stored and relaxed as g = f - w_i (lower rounding noise) */

#define KEL_MAX_FLAGS 8

typedef struct kel_flag_op {
	int32_t bc;          /* KEL_BC_* */
	int32_t collide;     /* 1: run the program's collision after the boundary step */
	int32_t east;        /* template argument of ZouHe*X<East> */
	int32_t use_profile; /* ZouHeVelocityX: u_x taken from the inlet profile at this y */
	double rho;          /* ZouHePressureX rho setting / Equilibrium density */
	double u[3];         /* ZouHeVelocityX / MovingWall / Equilibrium velocity */
} kel_flag_op;

typedef struct kel_step_program {
	int32_t collision;  /* KEL_COLL_* */
	int32_t arithmetic; /* KEL_ARITH_* */
	double tau;         /* relaxation time */
	double global_force[3];
	kel_flag_op ops[KEL_MAX_FLAGS]; /* indexed by the cell's flag value */
} kel_step_program;

typedef struct kel_lattice_desc {
	int32_t descriptor; /* KEL_D2Q9 / KEL_D3Q19 / KEL_D3Q27 */
	int32_t storage;    /* KEL_STORAGE_* */
	int64_t nx, ny, nz; /* nz = 1 for D2Q9 */
	uint32_t flags;     /* KEL_LATTICE_* */
	uint32_t reserved;
} kel_lattice_desc;

typedef struct kel_lattice kel_lattice;

/* Dtype / layout selectors for uploads and downloads. */
#define KEL_DTYPE_F32 0
#define KEL_DTYPE_F64 1
#define KEL_LAYOUT_AOS 0 /* f[c*Q + i] (reference FixedArray order) */
#define KEL_LAYOUT_SOA 1 /* f[i*N + c] */

/* Field selectors. */
#define KEL_FIELD_POROSITY 1 /* macros "porosity" (psm.hpp:20-32), 1 fluid .. 0 solid */
#define KEL_FIELD_FORCE 2    /* macros "force" per cell, D values (collision.hpp:148-151) */
#define KEL_FIELD_HLBM_N 3   /* HLBM "particle_N" per cell, D values (hlbm.hpp:37-46) */
#define KEL_FIELD_HLBM_D 4   /* HLBM "particle_D" per cell */

/* Replaces data<ChunkStruct, encode::Sycl<>> construction + malloc_device
 * (modules/sycl/c++/data.hpp:23-61).  Initial state: every cell flag 0,
 * populations rest equilibrium f = w_i, macros rho = 1, u = 0, porosity 1,
 * force 0, time step 0. */
int kel_lattice_create(const kel_lattice_desc *desc, kel_lattice **out);
int kel_lattice_destroy(kel_lattice *lat);
/* Launches of this lattice go to `stream` (a cudaStream_t; NULL = legacy default). */
int kel_lattice_set_stream(kel_lattice *lat, void *stream);
int kel_lattice_time_step(const kel_lattice *lat, uint64_t *t);

/* Replaces device::copy_to_device of the "info" chunk (sycl/data.hpp:932-965). */
int kel_upload_flags(kel_lattice *lat, const uint8_t *host_flags);
/* Populations at the current time step (post-stream, pre-collision), as the
 * reference's buffer selected by time-step parity holds them. */
int kel_upload_populations(kel_lattice *lat, const void *host, int32_t dtype, int32_t layout);
int kel_download_populations(kel_lattice *lat, void *host, int32_t dtype, int32_t layout);
/* macros "density" / "velocity" as written by the most recent collide that
 * had KEL_STEP_WRITE_MACROS set (collision.hpp:83-89).  rho: N values, u: N*D (AoS). */
int kel_download_macros(kel_lattice *lat, float *host_rho, float *host_u);
int kel_upload_field(kel_lattice *lat, int32_t field, const float *host);
int kel_download_field(kel_lattice *lat, int32_t field, float *host);
/* Inlet velocity profile u_x(y) for ops with use_profile = 1 (ny doubles). */
int kel_upload_inlet_profile(kel_lattice *lat, const double *host_ux, int64_t n);

/* Step flags. */
#define KEL_STEP_WRITE_MACROS 1u /* store rho, u of the last of the n steps */
#define KEL_STEP_ALL_MACROS 2u   /* store rho, u on every step */

/* Replaces one iteration of the drivers' loop: the collide+BC
 * parallel_for (e.g. examples/poiseulle_2d_gpu/poiseulle_2d_gpu.cpp:169-224)
 * followed by the Stream parallel_for (:384-399), n_steps times.
 * Asynchronous on the lattice's stream.  The stream may be under a caller's
 * CUDA graph capture: the sweeps then go into that capture one launch per
 * step, and the program must have been passed to kel_step once before the
 * capture (a new program during capture is rejected).  The lattice's time
 * step advances when kel_step is called, not when a graph is replayed, so a
 * captured sequence should hold an even number of steps (the AA layout
 * depends on the parity of the time step). */
int kel_step(kel_lattice *lat, const kel_step_program *prog, uint64_t n_steps, uint32_t step_flags);

/* ---- particles: spheres (3D) / discs (2D) coupled by PSM -------------- */

/* Solid fraction used by the couple pass. */
#define KEL_POROSITY_RAMP 0    /* sin^2 ramp of width eps around R (particle/porosity.hpp:56-89) */
#define KEL_POROSITY_SUBCELL 1 /* 4^D sub-cell point sampling over the cell [x-1/2, x+1/2]^D */
/* 1 - the cos^2 solid fraction (width eps) of the signed distance read off
 * the set's voxel shape (kel_particles_set_shape), in FP32, at each cell of
 * the body's box: the sub-cell style box of radius R * reach + eps / 2
 * (reach: kel_shape_info) (particle/porosity.hpp:24-54, mask.hpp:270-311).
 * PSM coupling only. */
#define KEL_POROSITY_VOXEL 2

/* One rigid body, the fields of sch::ParticleRigidBody + collision radius
 * (particle/schema.hpp:51-115).  2D: rotation, torque and their derivatives
 * use component [0]. */
typedef struct kel_particle_state {
	double position[3];
	double position_old[3];
	double rotation[3];
	double rotation_old[3];
	double acceleration[3];
	double angular_acceleration[3];
	double force[3];  /* accumulator, zeroed by kel_particles_reset */
	double torque[3]; /* accumulator */
	double mass;
	double inertia;
	double radius;
	double density;
} kel_particle_state;

typedef struct kel_particle_params {
	int32_t porosity_mode; /* KEL_POROSITY_* */
	int32_t sub_steps;     /* Verlet sub-steps (0 acts as 1; the gather divides by the raw value) */
	double eps;            /* ramp width (the reference's gathers use 1.5) */
	double k_n, zeta_n, gamma_t, mu; /* dem_params (particle/contact.hpp:36-61) */
	double body_acceleration[3];     /* ParticleIntegrate(g) (particle/integrate.hpp:263-296) */
	uint32_t wall_axes;    /* DEM box walls at 0 and the extent on these axes (bit a = axis a) */
	int32_t coupling;      /* KEL_COUPLING_PSM (0), KEL_COUPLING_HLBM, KEL_COUPLING_FPLBM(_OWN) (D2Q9) */
} kel_particle_params;
#define KEL_COUPLING_PSM 0
/* HLBM (hlbm.hpp): couple = HlbmReset + the gathers' porosity (last body
 * wins), gather = momentum exchange without solid weight, stamp = the
 * particle_N / particle_D accumulators after the integrate, and the lattice
 * steps with KEL_COLL_HLBM. */
#define KEL_COUPLING_HLBM 1
/* FPLBM (fplbm.hpp), D2Q9, non-periodic lattices: couple = FpLbmReset
 * (porosity 1 and force 0 everywhere; density and momentum of the cells
 * whose op has no boundary step) + the particle pass of FpLbmOneParticle:
 * every body writes, over the cells of an AABB, the sin^2 ramp porosity
 * (eps 1.5) of its distance and the force (v_body - momentum) (1 - porosity)
 * (bodies in index order, the last one wins a cell); gather = each body's
 * FP64 sum of minus those forces, acceleration = sum / mass + the body
 * acceleration (force and torque are not written); integrate = the Verlet
 * sub-steps with that acceleration; no contact.  The lattice steps with
 * KEL_COLL_FPLBM.  KEL_COUPLING_FPLBM keeps the reference's choice of body
 * 0's AABB and body 0's radius (the group radius) for every body
 * (fplbm.hpp:186,194), which couples only body 0's neighbourhood;
 * KEL_COUPLING_FPLBM_OWN uses each body's own AABB and radius. */
#define KEL_COUPLING_FPLBM 2
#define KEL_COUPLING_FPLBM_OWN 3

typedef struct kel_particles kel_particles;

/* A set of `count` bodies living on `lat` (the lattice must outlive it). */
int kel_particles_create(kel_lattice *lat, int32_t count, kel_particles **out);
int kel_particles_destroy(kel_particles *ps);
int kel_particles_upload(kel_particles *ps, const kel_particle_state *host);
int kel_particles_download(kel_particles *ps, kel_particle_state *host);
/* ParticleForceReset (particle/integrate.hpp:195-261): force = torque = 0. */
int kel_particles_reset(kel_particles *ps);
/* PsmReset + ParticleFluidCouple (psm.hpp:20-32, particle/couple.hpp:26-105):
 * porosity of every cell = product over bodies of their solid-fraction
 * complement. */
int kel_particles_couple(kel_particles *ps, const kel_particle_params *prm);
/* PsmOneParticleGather (psm.hpp:95-446) for every body at once: momentum
 * exchange over the body's AABB, force -= sum of cell forces and
 * torque -= sum (x - X) x cell force, both accumulated in FP64.  When
 * `host_cell_force` is not NULL it receives the per-cell force field
 * (N*D floats, zero outside the bodies). */
int kel_particles_gather(kel_particles *ps, const kel_particle_params *prm, float *host_cell_force);
/* ParticleContact (particle/contact.hpp:466-567): pair + box-wall DEM. */
int kel_particles_contact(kel_particles *ps, const kel_particle_params *prm);
/* ParticleIntegrate (particle/integrate.hpp:45-83,263-296): position Verlet. */
int kel_particles_integrate(kel_particles *ps, const kel_particle_params *prm);
/* HLBM only: HlbmOneParticleStamp of every body (after the integrate). */
int kel_particles_stamp(kel_particles *ps, const kel_particle_params *prm);
/* One coupled time step, n times: reset, couple, gather, contact, integrate,
 * (HLBM: stamp,) then the sweep
 * (examples/moving_poiseulle_particles_2d_psm_gpu/sim.cpp:176-260,
 * examples/moving_poiseulle_particles_2d_hlbm_gpu/sim.cpp:195-262).  With
 * HLBM coupling the program's collision must be KEL_COLL_HLBM. */
int kel_particles_step(kel_particles *ps, const kel_particle_params *prm, const kel_step_program *prog,
					   uint64_t n_steps, uint32_t step_flags);

/* ---- voxel shapes: signed distance masks (particle/mask.hpp) ----------- */

/* A body shape as a signed distance on R^D voxels in normalised body-local
 * units (bounding radius 1: local [-1, 1]^D, voxel k at -1 + (k + 1/2) 2/R,
 * negative inside), scaled per body by its radius and placed by its position
 * and rotation (2D: angle rotation[0]; 3D: rotation vector, Rodrigues):
 * x = position + radius Rot(rotation) (u - center_of_mass)
 * (particle/mask.hpp:11-180).  Masks are R^D doubles, the last axis fastest. */
#define KEL_SHAPE_SPHERE 0 /* sdf::sphere (mask.hpp:317-322) */
#define KEL_SHAPE_CUBE 1   /* sdf::cube, Chebyshev distance (mask.hpp:328-340) */
typedef struct kel_shape kel_shape;

/* fill_mask_from_sdf (mask.hpp:351-394) of a built-in shape, on the host:
 * the mask and its centroid weighted by a one-voxel cos^2 solid fraction. */
int kel_shape_create(int32_t dim, int32_t resolution, int32_t kind, kel_shape **out);
/* A shape from a caller's mask (R^D doubles) and centre of mass (dim doubles). */
int kel_shape_create_from_mask(int32_t dim, int32_t resolution, const double *mask, const double *center_of_mass,
							   kel_shape **out);
/* The shape's mask (R^D doubles, may be NULL), centre of mass (3 doubles, may
 * be NULL) and normalised reach (may be NULL): the largest |u| over the
 * voxels at distance <= 0 plus one voxel diagonal 2 sqrt(dim) / R. */
int kel_shape_info(const kel_shape *shape, double *mask, double *center_of_mass, double *reach);
int kel_shape_destroy(kel_shape *shape);
/* The shape every body of the set takes (the reference's group mask,
 * sch::ParticleGroup "mask" / "center_of_mass"); NULL detaches.  The shape
 * must outlive its use and have the lattice's dimension. */
int kel_particles_set_shape(kel_particles *ps, const kel_shape *shape);

/* mask_signed_distance (mask.hpp:270-282) of body `body` of the set at
 * `n` lattice points (host, dim doubles each), FP64 on the device, into
 * out (host, n doubles). */
int kel_particles_voxel_distance(kel_particles *ps, int32_t body, const double *points, int32_t n, double *out);

/* voxel_contact (particle/voxel_narrow.hpp:78-259) of body pairs of the set,
 * FP64 on the device, one block per pair: the overlap of the two bodies'
 * solid fractions (width eps) over the lattice cells of their clamped
 * bounding-box intersection gives the contact point (overlap centroid), the
 * normal (overlap-weighted grad phi_hi - grad phi_lo, from hi toward lo) and
 * the depth (extent of the cells both hold above 1/2 along the normal, + 1,
 * capped at the smaller radius).  Sums are in a fixed order that does not
 * depend on which body is lo: swapping a pair negates the normal exactly. */
typedef struct kel_contact_manifold {
	int32_t hit;
	int32_t pad;
	double normal[3];
	double point[3];
	double depth;
} kel_contact_manifold;
/* pairs: host, 2 body indices (lo, hi) per pair; out: host, npairs entries. */
int kel_particles_voxel_contact(kel_particles *ps, const int32_t *pairs, int32_t npairs, double eps,
								kel_contact_manifold *out);

/* ---- batches: many independent D2Q9 channels in one launch ------------ */

typedef struct kel_channel_desc {
	int64_t nx, ny; /* extents of this channel */
	double tau;     /* relaxation time of this channel (BGK) */
	double u_max;   /* amplitude of its parabolic inlet: u_x(y) = 4 u_max eta (1 - eta),
					   eta = (y - 1/2) / (ny - 2), zero on the rim rows */
} kel_channel_desc;

typedef struct kel_batch kel_batch;

/* All channels packed into one allocation, laid out in tiles of `tile` cells
 * (128, 256 or 512; 0 = 256), one thread block per tile.  No counterpart in
 * the reference, which runs one compile-time-sized chunk per process
 * (modules/core/c++/chunk.hpp:25-39). */
int kel_batch_create(int32_t n_channels, const kel_channel_desc *channels, int32_t tile, kel_batch **out);
int kel_batch_destroy(kel_batch *b);
/* Flags of every channel, concatenated (nx*ny bytes each, x fastest). */
int kel_batch_upload_flags(kel_batch *b, const uint8_t *packed_flags);
/* Shared flag -> operation table; BGK only (tau comes from each channel);
 * ZouHeVelocityX ops with use_profile take the channel's parabolic inlet. */
int kel_batch_set_program(kel_batch *b, const kel_step_program *prog);
/* Time `steps` sweeps per candidate tile and keep the fastest (before the first step). */
int kel_batch_autotune(kel_batch *b, int32_t steps, int32_t *chosen_tile, float *ms_per_step);
int kel_batch_step(kel_batch *b, uint64_t n_steps);
/* Run every active channel until its relative L2 velocity change over
 * `check_every` steps, sqrt(sum |u_t - u_{t-k}|^2 / sum |u_t|^2) in FP64, is
 * below `tol`, or until `max_steps`.  With use_graph the `check_every` sweeps
 * and the residual are one captured CUDA graph, replayed.  steps_out and
 * residual_out (n values each, may be NULL) receive each channel's final time
 * step and last residual.  A channel whose residual is not finite (diverged)
 * stops too; its residual_out is NaN or inf.  Once the tiles of the active
 * channels are at most half of those launched, later sweeps launch only them. */
int kel_batch_run_until(kel_batch *b, double tol, uint64_t check_every, uint64_t max_steps, int32_t use_graph,
						uint64_t *steps_out, double *residual_out);
int kel_batch_active_count(kel_batch *b, int32_t *count);
int kel_batch_channel_time_step(const kel_batch *b, int32_t channel, uint64_t *t);
int kel_batch_info(const kel_batch *b, int64_t *cells, int64_t *padded_cells, int32_t *tile);
/* Warm start of channels [first, first + count), all at an even time step,
 * from a predicted field (no counterpart in the reference).  Channel
 * first + j reads d_pred + j * pred_stride (device): 3 floats per cell, x
 * fastest, physical (u_x, u_y, rho) = value * scale + offset with
 * d_scale / d_offset (device, 3 floats per channel).  Fluid cells get
 * f_eq(rho, u) plus, with with_neq, the non-equilibrium part
 * -(tau w_i rho / cs^2) Q_i : grad u (central differences, u = 0 in walls);
 * wall cells get the rest state at the mean density of their fluid
 * neighbours.  The residual's previous velocity becomes the predicted u. */
int kel_batch_warm_start(kel_batch *b, int32_t first, int32_t count, const float *d_pred, int64_t pred_stride,
						 const float *d_scale, const float *d_offset, int32_t with_neq);
/* Refinement of a warm start (no counterpart in the reference), same
 * prediction arguments: `iterations` times, two sweeps of every active
 * channel of the batch, then every fluid cell of channels [first, first +
 * count) keeps the non-equilibrium part of its populations and gets the
 * predicted field back: f_i <- f_i - f_eq(moments of f) + f_eq(rho_p, u_p)
 * (rho_p = the cell's own density with keep_rho).  The non-equilibrium part
 * is then the one the lattice and its boundary rules produce for the
 * predicted field.  The sweeps count as steps of the channels. */
int kel_batch_warm_refine(kel_batch *b, int32_t first, int32_t count, const float *d_pred, int64_t pred_stride,
						  const float *d_scale, const float *d_offset, int32_t iterations, int32_t keep_rho);
int kel_batch_synchronize(kel_batch *b);
/* One channel's populations (AoS, nx*ny*9) or macros (rho, u_x, u_y per cell). */
int kel_batch_download_populations(kel_batch *b, int32_t channel, float *host_aos);
int kel_batch_download_macros(kel_batch *b, int32_t channel, float *host_rho_u);

/* Relative L2 change sqrt(sum |u - u_prev|^2 / sum |u|^2) of a velocity
 * field, FP64 sums, written to *d_result (a device double) on `stream`.
 * d_u and d_u_prev hold `comps` planes of n floats each (device pointers).
 * No counterpart in the reference.  Allocates nothing: for callers that may
 * not allocate device memory while they run (cudaMalloc/cudaFree synchronise
 * the device and fail once a pooling allocator owns the memory).  Its scratch
 * is a fixed device array of 65,536 tiles, so n is limited to 16,777,216
 * cells; larger n is rejected with KEL_ERR_INVALID_ARGUMENT.  The first call
 * on a device looks up the scratch address (make it before any stream
 * capture).  Calls share the scratch: calls that overlap on the GPU race. */
int kel_velocity_residual_noalloc(const float *d_u, const float *d_u_prev, int64_t n, int32_t comps,
								  double *d_result, void *stream);

/* ---- learned warm start: conv U-Net (no counterpart in the reference) -- */

typedef struct kel_unet_desc {
	int32_t height, width;  /* grid (multiples of 8) */
	int32_t in_channels;    /* 16: mask, u_max, tau planes, zero padding */
	int32_t out_channels;   /* 3: u_x, u_y, rho (scaled) */
	int32_t widths[4];      /* channels per level, multiples of 16 (32, 64, 128, 128) */
	int32_t max_batch;
	int32_t reserved;
} kel_unet_desc;

typedef struct kel_unet kel_unet;

/* He-uniform initialisation from `seed`; FP32 master weights, bf16 copies. */
int kel_unet_create(const kel_unet_desc *desc, uint64_t seed, kel_unet **out);
int kel_unet_destroy(kel_unet *net);
int kel_unet_param_count(const kel_unet *net, int64_t *n);
int kel_unet_get_params(kel_unet *net, float *host);
int kel_unet_set_params(kel_unet *net, const float *host);
int kel_unet_get_grads(kel_unet *net, float *host);
int kel_unet_set_stream(kel_unet *net, void *stream);
int kel_unet_synchronize(kel_unet *net);
/* Input planes from device data: mask (n*H*W bytes, 1 = solid), u_max and tau
 * (n floats each).  Channels: mask, u_max / 0.08, (tau - 0.55) / 0.45, y and x
 * coordinates, the column's open fraction, the downstream resistance
 * sum 1/open^3 / W, the vertical gap height, 4 s (1 - s) across the gap,
 * the lubrication estimate of u_x / u_max (halved) and the lubrication
 * pressure S(x) / S(0), S(x) the suffix sum of 1 / sum h^3 over the columns
 * from x to the outlet; the rest zero. */
int kel_unet_make_input(kel_unet *net, const uint8_t *d_mask, const float *d_umax, const float *d_tau, int32_t n);
/* The current input (bf16 NHWC, 16 channels) copied to a device buffer. */
int kel_unet_get_input(kel_unet *net, uint16_t *d_out_bf16, int32_t n);
/* Input directly: bf16 NHWC, 16 channels (device pointer). */
int kel_unet_set_input(kel_unet *net, const uint16_t *d_input_bf16, int32_t n);
/* Forward pass; d_out (device, may be NULL) receives n*H*W*out_channels floats (NHWC). */
int kel_unet_forward(kel_unet *net, int32_t n, float *d_out);
/* After a forward with the same n: loss = mean (y - target)^2 and every
 * parameter gradient (FP32, overwritten).  *loss is written on the host. */
int kel_unet_backward(kel_unet *net, const float *d_target, int32_t n, double *loss);
int kel_unet_adam_step(kel_unet *net, float lr, float beta1, float beta2, float eps, int32_t step);
/* One training step on the input set by kel_unet_make_input / set_input:
 * forward, backward against d_target (device, copied into the net), Adam
 * (step counts from 1, as in kel_unet_adam_step) and the bf16 weight copies,
 * on the net's stream without a host synchronisation.  From the second call
 * on, the step is a captured CUDA graph, replayed while n and the Adam
 * constants beta1, beta2, eps stay the same (lr may change every step).  The
 * mean loss goes to *d_loss (device, may be NULL) and is kept for
 * kel_unet_last_loss.  The same arithmetic as forward + backward + adam_step. */
int kel_unet_train_step(kel_unet *net, const float *d_target, int32_t n, float lr, float beta1, float beta2, float eps,
						int32_t step, double *d_loss);
/* The loss of the last kel_unet_train_step (synchronises the net's stream). */
int kel_unet_last_loss(kel_unet *net, double *loss);
/* Convolution kernels: KEL_UNET_CONV_TCGEN05 (default; tcgen05.mma with the
 * accumulator in tensor memory) or KEL_UNET_CONV_MMA_SYNC (warp-level
 * mma.sync).  Both compute bf16 x bf16 -> FP32; results agree to FP32
 * summation order.  kel_unet_synchronize / kel_unet_backward return
 * KEL_ERR_TIMEOUT if a tensor-core kernel gave up on a bounded wait. */
#define KEL_UNET_CONV_TCGEN05 0
#define KEL_UNET_CONV_MMA_SYNC 1
int kel_unet_set_conv_kernel(kel_unet *net, int32_t kind);
/* Residual head (no counterpart in the reference): output channel
 * `out_channel` becomes the head's value plus `scale` times input plane
 * `in_channel`, so the network learns the correction to that plane (the
 * warm start adds the local Poiseuille estimate of u_x / u_max and the
 * lubrication pressure this way).  Each call sets one output channel (up to
 * 8); out_channel < 0 turns all of them off (the default).  Training and
 * inference use the same setting. */
int kel_unet_set_residual(kel_unet *net, int32_t out_channel, int32_t in_channel, float scale);

/* Launch shape of the sweep: cells per thread (1: one cell, 32-bit FP32 /
 * 16-bit FP16S accesses; 2: two consecutive cells, 64-bit / 32-bit accesses;
 * 4: four consecutive cells, 128-bit / 64-bit accesses) and threads per block
 * (64, 128 or 256); or KEL_LAUNCH_ROWS with block_threads = row stages (2-6): the row
 * pipeline, one thread per cell of a row, whole rows moved between HBM and
 * shared memory by bulk asynchronous copies, for rows of at most 256 cells
 * whose padded length is a multiple of 16 bytes (KEL_ERR_INVALID_ARGUMENT
 * otherwise).  Results do not depend on the shape.  If a row-pipeline sweep
 * gives up on its bounded wait for a row copy, the next
 * kel_lattice_synchronize / kel_download_populations / kel_download_macros
 * returns KEL_ERR_TIMEOUT. */
#define KEL_LAUNCH_ROWS (-1)
int kel_lattice_set_launch(kel_lattice *lat, int32_t cells_per_thread, int32_t block_threads);
int kel_lattice_get_launch(const kel_lattice *lat, int32_t *cells_per_thread, int32_t *block_threads);
/* Time `steps` sweeps of `prog` with every launch shape on the lattice's
 * current state and keep the fastest.  The populations are restored after
 * each trial and the time step does not advance. */
int kel_lattice_autotune(kel_lattice *lat, const kel_step_program *prog, int32_t steps, int32_t *cells_per_thread,
						 int32_t *block_threads, float *ms_per_step);

/* ---- geometry and initial state on the device --------------------------
 * The drivers' setup_initial_conditions (e.g. examples/poiseulle_2d_gpu/
 * poiseulle_2d_gpu.cpp:55-156) paint flags cell by cell and set
 * dfs_old = equilibrium(rho, u) on the host; here both run on the device. */
#define KEL_PAINT_BOX 0
#define KEL_PAINT_SPHERE 1
typedef struct kel_paint_op {
	int32_t shape;        /* KEL_PAINT_BOX or KEL_PAINT_SPHERE */
	int32_t flag;         /* value written (0..255) */
	int64_t lo[3], hi[3]; /* cells with lo <= x < hi on every axis: the box, or the sphere's clip */
	double center[3];     /* sphere: sum over axes (x - center)^2 <= radius^2 */
	double radius;
} kel_paint_op;
/* Apply the ops in order to the flag field (later ops win). */
int kel_lattice_paint(kel_lattice *lat, const kel_paint_op *ops, int32_t n_ops);
int kel_download_flags(kel_lattice *lat, uint8_t *host);
/* f_i(x) = equilibrium(rho, u) with the reference's rounding at the current
 * time step; rho and u from device fields (n_cells floats, x fastest; u one
 * such plane per component) or, where a pointer is NULL, from rho0 / u0 (u0
 * may be NULL: zero).  At an odd time step a boundary cell's populations that
 * come from outside the lattice have no slot (they are the zero ghost ring). */
int kel_lattice_init_equilibrium(kel_lattice *lat, const float *d_rho, const float *d_u, double rho0,
								 const double *u0);

/* ---- field output and checkpoints -------------------------------------
 * Host writers in the reference's formats (write_vtk.hpp, write_csv.hpp,
 * abstract/forst.hpp + forst_chunk.hpp): cells x fastest over dims; each
 * field one member of the reference's Struct of Chunks, in order. */
#define KEL_VALUE_U8 0
#define KEL_VALUE_F32 1
#define KEL_VALUE_F64 2
typedef struct kel_field_view {
	const char *name;   /* member key, e.g. "velocity", "density", "info" */
	int32_t value_type; /* KEL_VALUE_* */
	int32_t components; /* values per cell */
	int32_t ghost;      /* Forst only: the chunk's ghost width (zeros) */
	int32_t vector;     /* VTK: VECTORS even with one component */
	const void *data;   /* host, n_cells * components values */
} kel_field_view;
/* <out_dir>/vtk/<file_name>_<t>.vtk: ASCII STRUCTURED_POINTS, all fields. */
int kel_write_vtk(const char *out_dir, const char *file_name, uint64_t t, const int64_t *dims, int32_t n_dims,
				  const kel_field_view *fields, int32_t n_fields);
/* <out_dir>/csv/<file_name>_<name>_<t>.csv per field. */
int kel_write_csv(const char *out_dir, const char *file_name, uint64_t t, const int64_t *dims, int32_t n_dims,
				  const kel_field_view *fields, int32_t n_fields);
/* Forst encoding of the Struct of the fields' chunks (packed, no framing). */
int kel_write_forst(const char *path, const int64_t *dims, int32_t n_dims, const kel_field_view *fields,
					int32_t n_fields);
/* Inverse of kel_write_forst into the views' (writable) buffers; the file
 * size must match the layout exactly. */
int kel_read_forst(const char *path, const int64_t *dims, int32_t n_dims, kel_field_view *fields, int32_t n_fields);
#define KEL_WRITE_VTK 1
#define KEL_WRITE_CSV 2
#define KEL_WRITE_FORST 4
/* The drivers' macro output (MacroStruct {velocity, density}) of the last
 * step that wrote macros, as VTK / CSV / <out_dir>/forst/<name>_<t>.forst. */
int kel_lattice_write_fields(kel_lattice *lat, int32_t formats, const char *out_dir, const char *file_name, uint64_t t);
/* Checkpoint: Forst of {time_step UInt64, info Chunk<UInt8,0>, dfs
 * Chunk<FixedArray<Float32,Q>,1>} at the current time step; load restores
 * flags, populations and time step into a lattice of the same shape. */
int kel_lattice_save(kel_lattice *lat, const char *path);
int kel_lattice_load(kel_lattice *lat, const char *path);

/* Synchronise the lattice's stream. */
int kel_lattice_synchronize(kel_lattice *lat);

/* Thread-local message of the last failure. */
const char *kel_last_error_string(void);
/* Library version string. */
const char *kel_version(void);

#ifdef __cplusplus
}
#endif

#endif
