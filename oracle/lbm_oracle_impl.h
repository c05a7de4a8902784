/*
 * Body of the CPU restatement, instantiated twice by lbm_oracle.c with
 * REAL = float (suffix _f32) and REAL = double (suffix _f64).  TEST
 * INFRASTRUCTURE ONLY -- the oracle the CUDA path is checked against.
 *
 * It follows the reference's two-lattice scheme literally: AoS populations
 * with a one-cell zero ghost ring, dfs_old/dfs selected by time-step parity,
 * a collide+boundary pass over every cell followed by a pull stream for every
 * flag > 0 cell, and the reference's exact operation order (including the
 * double-precision bracket of the equilibrium) so that, compiled without
 * floating-point contraction, it reproduces the reference bit for bit.
 */

#define KO_CAT2(a, b) a##b
#define KO_CAT(a, b) KO_CAT2(a, b)
#define KO(name) KO_CAT(name, KO_SUFFIX)

typedef struct KO(ko_lat) {
	ko_desc d;
	int64_t nx, ny, nz, n;
	int64_t gx, gy, gz; /* ghost-padded extents */
	int periodic_x;
	uint8_t *info;
	REAL *dfs[2]; /* [0] = "dfs_old", [1] = "dfs" (ghost-padded AoS) */
	REAL *rho, *vel, *por, *force;
	REAL *hN, *hD; /* HLBM "particle_N" (D per cell) and "particle_D" */
	const double *profile;
	uint64_t t;
} KO(ko_lat);

static inline int64_t KO(gidx)(const KO(ko_lat) * L, int64_t x, int64_t y, int64_t z) {
	/* ghost-padded flat index of interior coordinate (x,y,z) */
	return (x + 1) + L->gx * ((y + 1) + L->gy * (z + (L->d.D == 3 ? 1 : 0)));
}

/* compute_rho_u, macroscopic.hpp:10-35 */
static void KO(rho_u)(const ko_desc *d, const REAL *f, REAL *rho, REAL *u) {
	REAL r = 0;
	REAL v[3] = {0, 0, 0};
	for (int j = 0; j < d->Q; ++j) {
		r = r + f[j];
		for (int k = 0; k < d->D; ++k) v[k] = v[k] + (REAL)d->c[j][k] * f[j];
	}
	for (int k = 0; k < d->D; ++k) v[k] = v[k] / r;
	*rho = r;
	for (int k = 0; k < d->D; ++k) u[k] = v[k];
}

/* equilibrium, equilibrium.hpp:7-48: the bracket is evaluated in double
 * because of the 1.0 / 0.5 literals, then narrowed on store. */
static void KO(equilibrium)(const ko_desc *d, REAL rho, const REAL *u, REAL *eq) {
	REAL vv = 0;
	for (int k = 0; k < d->D; ++k) vv = vv + u[k] * u[k];
	for (int i = 0; i < d->Q; ++i) {
		REAL vc = 0;
		for (int k = 0; k < d->D; ++k) vc = vc + u[k] * (REAL)d->c[i][k];
		REAL vcc = vc * (REAL)3.0;
		REAL wr = KO(weight)(d, i) * rho;
		double br = 1.0 + (double)vcc - (double)(REAL)3.0 * 0.5 * (double)vv + (double)(REAL)(vcc * vcc) * 0.5;
		eq[i] = (REAL)((double)wr * br);
	}
}

/* Guo forcing term F_i, collision.hpp:170-196 */
static REAL KO(guo_term)(const ko_desc *d, int i, const REAL *u, const REAL *F) {
	REAL ci[3], t1[3], t2[3];
	for (int k = 0; k < d->D; ++k) ci[k] = (REAL)d->c[i][k];
	REAL cdu = 0;
	for (int k = 0; k < d->D; ++k) cdu = cdu + ci[k] * u[k];
	REAL s = cdu * (REAL)3.0 * (REAL)3.0;
	for (int k = 0; k < d->D; ++k) {
		t1[k] = (ci[k] - u[k]) * (REAL)3.0;
		t2[k] = ci[k] * s;
	}
	REAL proj = 0;
	for (int k = 0; k < d->D; ++k) proj = proj + (t1[k] + t2[k]) * F[k];
	return KO(weight)(d, i) * proj;
}

static void KO(collide)(KO(ko_lat) * L, const kel_step_program *P, REAL *f, int64_t c) {
	const ko_desc *d = &L->d;
	REAL freq = (REAL)1 / (REAL)P->tau;
	REAL rho, u[3] = {0, 0, 0}, eq[27];
	REAL pre[27];
	for (int i = 0; i < d->Q; ++i) pre[i] = f[i];
	KO(rho_u)(d, f, &rho, u);
	if (P->collision != KEL_COLL_FPLBM) { /* FpLbm leaves FpLbmReset's density and momentum */
		L->rho[c] = rho;
		for (int k = 0; k < d->D; ++k) L->vel[c * d->D + k] = u[k];
	}
	KO(equilibrium)(d, rho, u, eq);
	REAL F[3] = {0, 0, 0};
	if (P->collision == KEL_COLL_BGK_GUO || P->collision == KEL_COLL_PSM_GUO) {
		for (int k = 0; k < d->D; ++k) F[k] = L->force[c * d->D + k] + (REAL)P->global_force[k];
	}
	if (P->collision == KEL_COLL_FPLBM) {
		for (int k = 0; k < d->D; ++k) F[k] = L->force[c * d->D + k];
	}
	switch (P->collision) {
	case KEL_COLL_BGK: /* collision.hpp:93-95 */
		for (int i = 0; i < d->Q; ++i) f[i] = f[i] + freq * (eq[i] - f[i]);
		break;
	case KEL_COLL_BGK_GUO: /* collision.hpp:170-203 */
		for (int i = 0; i < d->Q; ++i) {
			REAL Fi = KO(guo_term)(d, i, u, F);
			f[i] = f[i] + freq * (eq[i] - f[i]) + Fi * ((REAL)1 - (REAL)0.5f * freq);
		}
		break;
	case KEL_COLL_HLBM: { /* hlbm.hpp:66-101: convex combination of velocities, then BGK */
		REAL por = L->por[c];
		REAL flip = (REAL)1.0 - por;
		REAL Dv = L->hD[c];
		for (int k = 0; k < d->D; ++k) {
			REAL Nk = L->hN[c * d->D + k];
			REAL add = (Dv > 0.0) ? Nk * flip / Dv : Nk;
			u[k] = u[k] * por + add;
			L->vel[c * d->D + k] = u[k];
		}
		KO(equilibrium)(d, rho, u, eq);
		for (int i = 0; i < d->Q; ++i) f[i] = f[i] + freq * (eq[i] - f[i]);
	} break;
	case KEL_COLL_FPLBM: /* fplbm.hpp:79-127: BGK + Guo term of the cell force, macros left alone */
		for (int i = 0; i < d->Q; ++i) {
			REAL Fi = KO(guo_term)(d, i, u, F);
			f[i] = f[i] + freq * (eq[i] - f[i]) + Fi * ((REAL)1 - (REAL)0.5f * freq);
		}
		break;
	case KEL_COLL_PSM:
	case KEL_COLL_PSM_GUO: { /* psm.hpp:79-88 */
		REAL por = L->por[c];
		REAL flip = (REAL)1.0 - por;
		for (int i = 0; i < d->Q; ++i)
			f[i] = pre[i] + freq * (eq[i] - pre[i]) * por + (pre[d->opp[i]] - pre[i]) * flip;
		if (P->collision == KEL_COLL_PSM_GUO) {
			for (int i = 0; i < d->Q; ++i) {
				REAL Fi = KO(guo_term)(d, i, u, F);
				f[i] = f[i] + Fi * ((REAL)1 - (REAL)0.5f * freq);
			}
		}
	} break;
	}
}

/* D2Q9 ZouHePressureX<Dir>, boundary.hpp:186-226 */
static void KO(zouhe_pressure_d2q9)(REAL *f, int east, REAL rs) {
	if (east) {
		REAL S = f[0] + f[3] + f[4] + (f[1] + f[5] + f[7]) * (REAL)2;
		REAL rvx = rs - S;
		f[2] = f[1] + (REAL)(2.0 / 3.0) * rvx;
		f[6] = f[5] + (REAL)(1.0 / 6.0) * rvx + (REAL)0.5 * (f[3] - f[4]);
		f[8] = f[7] + (REAL)(1.0 / 6.0) * rvx + (REAL)0.5 * (f[4] - f[3]);
	} else {
		REAL S = f[0] + f[3] + f[4] + (f[2] + f[6] + f[8]) * (REAL)2;
		REAL rvx = S - rs;
		f[1] = f[2] - (REAL)(2.0 / 3.0) * rvx;
		f[5] = f[6] - (REAL)(1.0 / 6.0) * rvx + (REAL)0.5 * (f[4] - f[3]);
		f[7] = f[8] - (REAL)(1.0 / 6.0) * rvx + (REAL)0.5 * (f[3] - f[4]);
	}
}

/* D3Q27 ZouHePressureX<East>, boundary.hpp:229-756 (AtXMax = !East) */
static void KO(zouhe_pressure_d3q27)(REAL *f, int east, REAL rs) {
	const REAL two = (REAL)2.0, a = (REAL)(4.0 / 9.0), b = (REAL)(1.0 / 9.0), e = (REAL)(1.0 / 36.0);
	REAL S, rux, ruy, ruz;
	if (!east) { /* x = max: unknowns cx = -1 */
		S = f[0] + f[3] + f[6] + f[9] + f[12] + f[15] + f[18] + f[21] + f[24] +
			two * (f[2] + f[5] + f[8] + f[11] + f[14] + f[17] + f[20] + f[23] + f[26]);
		rux = S - rs;
		ruy = -f[3] + f[6] - f[12] + f[15] - f[21] + f[24] + two * (-f[5] + f[8] - f[14] + f[17] - f[23] + f[26]);
		ruz = -f[9] - f[12] - f[15] + f[18] + f[21] + f[24] + two * (-f[11] - f[14] - f[17] + f[20] + f[23] + f[26]);
		f[1] = f[2] - a * rux;
		f[4] = f[5] - b * (rux + ruy);
		f[7] = f[8] + b * (-rux + ruy);
		f[10] = f[11] - b * (rux + ruz);
		f[13] = f[14] - e * (rux + ruy + ruz);
		f[16] = f[17] + e * (-rux + ruy + ruz);
		f[19] = f[20] + b * (-rux + ruz);
		f[22] = f[23] + e * (-rux - ruy + ruz);
		f[25] = f[26] + e * (-rux + ruy + ruz);
	} else { /* x = 0: unknowns cx = +1 */
		S = f[0] + f[3] + f[6] + f[9] + f[12] + f[15] + f[18] + f[21] + f[24] +
			two * (f[1] + f[4] + f[7] + f[10] + f[13] + f[16] + f[19] + f[22] + f[25]);
		rux = rs - S;
		ruy = -f[3] + f[6] - f[12] + f[15] - f[21] + f[24] + two * (-f[4] + f[7] - f[13] + f[16] - f[22] + f[25]);
		ruz = -f[9] - f[12] - f[15] + f[18] + f[21] + f[24] + two * (-f[10] - f[13] - f[16] + f[19] + f[22] + f[25]);
		f[2] = f[1] + a * rux;
		f[5] = f[4] + b * (rux - ruy);
		f[8] = f[7] + b * (rux + ruy);
		f[11] = f[10] + b * (rux - ruz);
		f[14] = f[13] + e * (rux - ruy - ruz);
		f[17] = f[16] + e * (rux + ruy - ruz);
		f[20] = f[19] + b * (rux + ruz);
		f[23] = f[22] + e * (rux - ruy + ruz);
		f[26] = f[25] + e * (rux + ruy + ruz);
	}
}

/* D2Q9 ZouHeVelocityX<East>, boundary.hpp:775-802 */
static void KO(zouhe_velocity_d2q9)(REAL *f, int east, REAL ux, REAL uy) {
	REAL ds = east ? (f[1] + f[5] + f[7]) : (f[2] + f[6] + f[8]);
	REAL rho = (f[0] + f[4] + f[3] + ds * (REAL)2) / (ux + (REAL)1.0);
	const REAL c23 = (REAL)(2.0 / 3.0), c16 = (REAL)(1.0 / 6.0);
	if (east) {
		f[2] = f[1] + c23 * rho * ux;
		f[6] = f[5] + c16 * rho * ux + (f[3] - f[4] + rho * uy) * (REAL)0.5f;
		f[8] = f[7] + c16 * rho * ux + (f[4] - f[3] + rho * uy) * (REAL)0.5f;
	} else {
		f[1] = f[2] + c23 * rho * ux;
		f[5] = f[6] + c16 * rho * ux + (f[4] - f[3] + rho * uy) * (REAL)0.5f;
		f[7] = f[8] + c16 * rho * ux + (f[3] - f[4] + rho * uy) * (REAL)0.5f;
	}
}

static int KO(cell_step)(KO(ko_lat) * L, const kel_step_program *P, int64_t c, int64_t x, int64_t y, int64_t z, REAL *buf) {
	const ko_desc *d = &L->d;
	uint8_t info = L->info[c];
	/* `case 0u: break;` and `default: break;` of the drivers' switch(info) */
	if (info == 0u || info >= KEL_MAX_FLAGS) return 0;
	const kel_flag_op *o = &P->ops[info];
	if (o->bc == KEL_BC_HALFWAY_WALL) return 0; /* solid: computes nothing */
	REAL *f = buf + KO(gidx)(L, x, y, z) * d->Q;
	REAL cpy[27];
	switch (o->bc) {
	case KEL_BC_NONE:
	case KEL_BC_FLUID:
		break;
	case KEL_BC_BOUNCE_BACK: /* boundary.hpp:58-75 */
		for (int i = 0; i < d->Q; ++i) cpy[i] = f[i];
		for (int i = 0; i < d->Q; ++i) f[i] = cpy[d->opp[i]];
		break;
	case KEL_BC_ANTI_BOUNCE_BACK: /* boundary.hpp:119-132 */
		if (d->Q != 9) return -1;
		for (int i = 0; i < 9; ++i) cpy[i] = f[i];
		f[3] = cpy[4]; f[4] = cpy[3]; f[5] = cpy[7]; f[6] = cpy[8]; f[7] = cpy[5]; f[8] = cpy[6];
		break;
	case KEL_BC_EQUILIBRIUM: { /* boundary.hpp:147-160 */
		REAL u[3];
		for (int k = 0; k < d->D; ++k) u[k] = (REAL)o->u[k];
		KO(equilibrium)(d, (REAL)o->rho, u, f);
	} break;
	case KEL_BC_ZOUHE_PRESSURE_X:
		if (d->Q == 9) KO(zouhe_pressure_d2q9)(f, o->east, (REAL)o->rho);
		else if (d->Q == 27) KO(zouhe_pressure_d3q27)(f, o->east, (REAL)o->rho);
		else return -1;
		break;
	case KEL_BC_ZOUHE_VELOCITY_X: {
		if (d->Q != 9) return -1;
		REAL ux = (REAL)o->u[0];
		if (o->use_profile) {
			if (!L->profile) return -1;
			ux = (REAL)L->profile[y];
		}
		KO(zouhe_velocity_d2q9)(f, o->east, ux, (REAL)o->u[1]);
	} break;
	case KEL_BC_MOVING_WALL: /* cavity_2d_gpu.cpp:222-234, e.u summed over all axes */
		for (int i = 0; i < d->Q; ++i) cpy[i] = f[i];
		for (int i = 0; i < d->Q; ++i) {
			double edu = 0.0;
			for (int k = 0; k < d->D; ++k) edu = edu + (double)(REAL)d->c[i][k] * o->u[k];
			f[i] = cpy[d->opp[i]] + (REAL)(2.0 * (double)KO(weight)(d, i) * (double)(REAL)3.0 * edu);
		}
		break;
	default:
		return -1;
	}
	if (o->collide) {
		if (P->collision == KEL_COLL_FPLBM && o->bc != KEL_BC_NONE && o->bc != KEL_BC_FLUID) {
			/* the FPLBM drivers' boundary cases collide with BGK */
			kel_step_program bgk = *P;
			bgk.collision = KEL_COLL_BGK;
			KO(collide)(L, &bgk, f, c);
		} else {
			KO(collide)(L, P, f, c);
		}
	}
	return 0;
}

/* Does program P give any flag the half-way wall op?  (Only then does the
 * stream look at its neighbours' flags; P = NULL below means "none".) */
static const kel_step_program *KO(halfway_program)(const kel_step_program *P) {
	for (int k = 1; k < KEL_MAX_FLAGS; ++k)
		if (P->ops[k].bc == KEL_BC_HALFWAY_WALL) return P;
	return 0;
}

/* Is interior cell (x, y, z) a half-way wall of program P? */
static int KO(is_halfway)(const KO(ko_lat) * L, const kel_step_program *P, int64_t x, int64_t y, int64_t z) {
	if (!P || x < 0 || x >= L->nx || y < 0 || y >= L->ny || z < 0 || z >= L->nz) return 0;
	const uint8_t info = L->info[x + L->nx * (y + L->ny * z)];
	return info > 0u && info < KEL_MAX_FLAGS && P->ops[info].bc == KEL_BC_HALFWAY_WALL;
}

/* Pull stream of one cell.  Half-way bounce-back (no counterpart in the
 * reference): where the source x - c_i is a half-way wall, f_i(x) takes the
 * post-collision f_opp(i) that x itself sent towards the wall. */
static void KO(stream_cell)(KO(ko_lat) * L, const kel_step_program *P, int64_t x, int64_t y, int64_t z,
							const REAL *src, REAL *dst) {
	const ko_desc *d = &L->d;
	if (P && KO(is_halfway)(L, P, x, y, z)) return; /* solid */
	REAL *out = dst + KO(gidx)(L, x, y, z) * d->Q;
	for (int i = 0; i < d->Q; ++i) {
		int64_t sx = x - d->c[i][0], sy = y - d->c[i][1], sz = z - (d->D == 3 ? d->c[i][2] : 0);
		if (L->periodic_x) sx = (sx + L->nx) % L->nx;
		if (P && KO(is_halfway)(L, P, sx, sy, sz)) {
			out[i] = src[KO(gidx)(L, x, y, z) * d->Q + d->opp[i]];
			continue;
		}
		/* stream.hpp:256-264: ghost_at(g_index - c_i), the ghost ring holds zeros */
		out[i] = src[((sx + 1) + L->gx * ((sy + 1) + L->gy * (sz + (d->D == 3 ? 1 : 0)))) * d->Q + i];
	}
}

static int KO(run)(KO(ko_lat) * L, const kel_step_program *P, uint64_t steps) {
	const ko_desc *d = &L->d;
	const kel_step_program *hw = KO(halfway_program)(P);
	for (uint64_t s = 0; s < steps; ++s) {
		int even = (L->t % 2u) == 0u;
		REAL *old = even ? L->dfs[0] : L->dfs[1];
		REAL *nw = even ? L->dfs[1] : L->dfs[0];
		int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
		for (int64_t zy = 0; zy < L->nz * L->ny; ++zy) {
			int64_t z = zy / L->ny, y = zy % L->ny;
			for (int64_t x = 0; x < L->nx; ++x) {
				int64_t c = x + L->nx * (y + L->ny * z);
				err |= KO(cell_step)(L, P, c, x, y, z, old) != 0;
			}
		}
		if (err) return -1;
#pragma omp parallel for schedule(static)
		for (int64_t zy = 0; zy < L->nz * L->ny; ++zy) {
			int64_t z = zy / L->ny, y = zy % L->ny;
			for (int64_t x = 0; x < L->nx; ++x) {
				int64_t c = x + L->nx * (y + L->ny * z);
				if (L->info[c] > 0u) KO(stream_cell)(L, hw, x, y, z, old, nw);
			}
		}
		(void)d;
		L->t += 1;
	}
	return 0;
}

/* Throughput sample: the collide+boundary pass and the stream pass of one
 * time step restricted to rows [r0, r1) (row = z*ny + y).  The time step
 * counter does not advance; used only to time the reference algorithm on a
 * bounded part of a large lattice. */
static int KO(run_rows)(KO(ko_lat) * L, const kel_step_program *P, int64_t r0, int64_t r1) {
	const kel_step_program *hw = KO(halfway_program)(P);
	int even = (L->t % 2u) == 0u;
	REAL *old = even ? L->dfs[0] : L->dfs[1];
	REAL *nw = even ? L->dfs[1] : L->dfs[0];
	int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
	for (int64_t zy = r0; zy < r1; ++zy) {
		int64_t z = zy / L->ny, y = zy % L->ny;
		for (int64_t x = 0; x < L->nx; ++x) err |= KO(cell_step)(L, P, x + L->nx * zy, x, y, z, old) != 0;
	}
	if (err) return -1;
#pragma omp parallel for schedule(static)
	for (int64_t zy = r0; zy < r1; ++zy) {
		int64_t z = zy / L->ny, y = zy % L->ny;
		for (int64_t x = 0; x < L->nx; ++x)
			if (L->info[x + L->nx * zy] > 0u) KO(stream_cell)(L, hw, x, y, z, old, nw);
	}
	return 0;
}

/* ---- host I/O of the oracle state (AoS, no ghost) --------------------- */
static REAL *KO(current)(KO(ko_lat) * L) { return (L->t % 2u == 0u) ? L->dfs[0] : L->dfs[1]; }

static void KO(set_pops)(KO(ko_lat) * L, const double *aos) {
	REAL *cur = KO(current)(L);
	for (int64_t c = 0; c < L->n; ++c) {
		int64_t x = c % L->nx, y = (c / L->nx) % L->ny, z = c / (L->nx * L->ny);
		REAL *f = cur + KO(gidx)(L, x, y, z) * L->d.Q;
		for (int i = 0; i < L->d.Q; ++i) f[i] = (REAL)aos[c * L->d.Q + i];
	}
}

static void KO(get_pops)(KO(ko_lat) * L, double *aos) {
	REAL *cur = KO(current)(L);
	for (int64_t c = 0; c < L->n; ++c) {
		int64_t x = c % L->nx, y = (c / L->nx) % L->ny, z = c / (L->nx * L->ny);
		const REAL *f = cur + KO(gidx)(L, x, y, z) * L->d.Q;
		for (int i = 0; i < L->d.Q; ++i) aos[c * L->d.Q + i] = (double)f[i];
	}
}

/* FpLbmReset (fplbm.hpp:26-54) on every cell: porosity 1, force 0; cells
 * whose flag is in plain_mask (the drivers' info 2) get the density and
 * momentum (compute_rho_momentum, macroscopic.hpp:41-60) of their current
 * populations in the density / velocity macros. */
static void KO(fplbm_reset)(KO(ko_lat) * L, uint32_t plain_mask) {
	const ko_desc *d = &L->d;
	REAL *cur = KO(current)(L);
	for (int64_t c = 0; c < L->n; ++c) {
		L->por[c] = (REAL)1.0;
		for (int k = 0; k < d->D; ++k) L->force[c * d->D + k] = (REAL)0.0;
		const uint8_t info = L->info[c];
		if (info >= 32u || !((plain_mask >> info) & 1u)) continue;
		int64_t x = c % L->nx, y = (c / L->nx) % L->ny, z = c / (L->nx * L->ny);
		const REAL *f = cur + KO(gidx)(L, x, y, z) * d->Q;
		REAL r = 0, m[3] = {0, 0, 0};
		for (int j = 0; j < d->Q; ++j) {
			r = r + f[j];
			for (int k = 0; k < d->D; ++k) m[k] = m[k] + (REAL)d->c[j][k] * f[j];
		}
		L->rho[c] = r;
		for (int k = 0; k < d->D; ++k) L->vel[c * d->D + k] = m[k];
	}
}

/* particle_porosity<T,D,1,ParticleSpheroid>::calculate (porosity.hpp:56-89)
 * in the lattice's precision: the angle is formed in double and narrowed,
 * its sine taken in REAL. */
static REAL KO(fplbm_ramp)(REAL s, REAL rad, REAL eps) {
	REAL eps_h = eps / 2;
	REAL lo = rad - eps_h, hi = rad + eps_h;
	if (s <= lo) return 0;
	if (s >= hi) return 1;
	REAL inner = (REAL)((3.14159265358979323846 / (double)(2 * eps)) * (double)(s - lo));
	REAL c = sizeof(REAL) == 4 ? (REAL)sinf((float)inner) : (REAL)sin((double)inner);
	return c * c;
}

/* FpLbmOneParticle (fplbm.hpp:150-247) for every body in index order: over
 * the cells of an AABB (axis 0 outermost), the ramp porosity (eps 1.5) of
 * the cell's offset from the body and the force (v_body - momentum) (1 -
 * porosity) go to the porosity / force fields (a later body overwrites);
 * the body's acceleration becomes minus their sum (FP64) over its mass plus
 * the body acceleration, then its Verlet sub-steps (particle.hpp:171-211).
 * The AABB and radius are body 0's (the reference's) unless `own`.  Cell
 * quantities in REAL, body state in double. */
static void KO(fplbm_particles)(KO(ko_lat) * L, kel_particle_state *P, int np, const kel_particle_params *prm, int own) {
	const ko_desc *d = &L->d;
	const int D = d->D;
	const double sss = (double)prm->sub_steps;
	const int64_t ext[3] = {L->nx, L->ny, L->nz};
	for (int p = 0; p < np; ++p) {
		kel_particle_state *q = &P[p];
		const kel_particle_state *bx = own ? q : &P[0];
		int64_t a[3] = {0, 0, 0}, b[3] = {1, 1, 1};
		for (int k = 0; k < D; ++k) { /* aabb.hpp:41-84 */
			const double X = bx->position[k], r = bx->radius;
			a[k] = (X >= r) ? (int64_t)(X - r) : 0;
			b[k] = (int64_t)(X + r + 1.0);
			if (b[k] > ext[k]) b[k] = ext[k];
		}
		REAL vs[3] = {0, 0, 0};
		for (int k = 0; k < D; ++k) vs[k] = (REAL)((q->position[k] - q->position_old[k]) * sss);
		const REAL rad = (REAL)bx->radius;
		double fs[3] = {0, 0, 0};
		for (int64_t ix = a[0]; ix < b[0]; ++ix)
			for (int64_t iy = a[1]; iy < b[1]; ++iy)
				for (int64_t iz = a[2]; iz < b[2]; ++iz) {
					const int64_t idx[3] = {ix, iy, iz};
					const int64_t c = ix + L->nx * (iy + L->ny * iz);
					REAL s2 = 0;
					for (int k = 0; k < D; ++k) {
						const REAL rel = (REAL)((double)idx[k] - q->position[k]);
						s2 = s2 + rel * rel;
					}
					const REAL sd = sizeof(REAL) == 4 ? (REAL)sqrtf((float)s2) : (REAL)sqrt((double)s2);
					const REAL por = KO(fplbm_ramp)(sd, rad, (REAL)1.5);
					const REAL flip = (REAL)1.0 - por;
					L->por[c] = por;
					for (int k = 0; k < D; ++k) {
						const REAL fk = (vs[k] - L->vel[c * D + k]) * (REAL)1.0 * flip;
						L->force[c * D + k] = fk;
						fs[k] = fs[k] - (double)fk;
					}
				}
		for (int k = 0; k < D; ++k) q->acceleration[k] = fs[k] / q->mass + prm->body_acceleration[k];
		if (prm->sub_steps > 0) {
			const double ts = 1.0 / sss, t2 = ts * ts;
			for (int s = 0; s < prm->sub_steps; ++s) {
				for (int k = 0; k < D; ++k) {
					const double nw = q->position[k] * 2.0 - q->position_old[k] + q->acceleration[k] * t2;
					q->position_old[k] = q->position[k];
					q->position[k] = nw;
				}
				const int nr = D == 2 ? 1 : 3;
				for (int k = 0; k < nr; ++k) {
					const double nw = q->rotation[k] * 2.0 - q->rotation_old[k] + q->angular_acceleration[k] * t2;
					q->rotation_old[k] = q->rotation[k];
					q->rotation[k] = nw;
				}
			}
		}
	}
}

static void KO(set_vec)(REAL *dst, const double *src, int64_t n) {
	for (int64_t k = 0; k < n; ++k) dst[k] = (REAL)src[k];
}

static void KO(get_vec)(const REAL *src, double *dst, int64_t n) {
	for (int64_t k = 0; k < n; ++k) dst[k] = (double)src[k];
}
