/*
 * Reference harness: drives keldu/lbm_mirror's OWN hot-path components,
 * compiled unchanged from the reference tree (include path only), to produce
 * golden vectors for the CPU restatement (oracle/lbm_oracle.c) and for the
 * CUDA kernels.  Test infrastructure only: nothing in the product links it.
 *
 * What it reproduces from the reference drivers:
 *   - fields struct {info, dfs, dfs_old} with Chunk<FixedArray<T,Q>,1,dims...>
 *     (ghost ring = 1, zero-initialised, never written)
 *       examples/poiseulle_2d_gpu/poiseulle_2d_gpu.cpp:17-47
 *   - per-cell switch(info) -> component::apply, then a pull Stream for every
 *     info > 0 cell; even t collides dfs_old and streams into dfs
 *       examples/poiseulle_2d_gpu/poiseulle_2d_gpu.cpp:169-224, 384-399
 *       modules/core/c++/stream.hpp:19-58
 *   - the moving-wall lid of examples/cavity_2d_gpu/cavity_2d_gpu.cpp:204-235,
 *     generalised to D dimensions (e.u summed over all axes, in double)
 *   - PSM + Guo: cmpt::Psm followed by the BGKGuo forcing term with the same
 *     unshifted velocity (restatement; the reference has no such component)
 *
 * The one addition the reference needs for host use is a borrowed host view
 * data<sch::Ptr<sch::Chunk<...>>, enc::Native>, mirroring the device view of
 * modules/sycl/c++/data.hpp:323-396.
 *
 * Usage: ref_harness <case> <in_dir> <out_dir>
 *   in_dir/params.txt   key value lines (see read_params)
 *   in_dir/flags.u8     nx*ny*nz uint8, x fastest
 *   in_dir/init.f64     optional AoS populations (cell-major, Q per cell)
 *   in_dir/profile.f64  optional inlet u_x per y (ny values)
 *   in_dir/porosity.f64 optional per-cell porosity
 *   in_dir/force.f64    optional per-cell force (D per cell)
 *   out_dir/dfs.f64     post-stream populations at t = steps (AoS, no ghost)
 *   out_dir/rho.f64, out_dir/vel.f64   macros of the last collide
 */
#include "lbm.hpp" /* modules/core/c++/lbm.hpp, via -I */
#include "particle/voxel_narrow.hpp"
#include "forst_chunk.hpp"
#include "write_csv.hpp"
#include "write_vtk.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <filesystem>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace kel {
namespace lbm {

/* Host borrowed view over a Chunk (ghost-aware), same surface as the SYCL one. */
template <typename Sch, uint64_t Ghost, uint64_t... Sides>
class data<sch::Ptr<sch::Chunk<Sch, Ghost, Sides...>>, enc::Native> final {
public:
	using Schema = sch::Ptr<sch::Chunk<Sch, Ghost, Sides...>>;

private:
	using InnerSchema = typename sch::Chunk<Sch, Ghost, Sides...>::InnerSchema;
	using ValueSchema = typename InnerSchema::ValueType;
	data<sch::Ptr<InnerSchema>, enc::Native> values_;

public:
	data() = default;
	data(const data &) = default;
	data &operator=(const data &) = default;

	data(data<sch::Chunk<Sch, Ghost, Sides...>, enc::Native> &backing)
		: values_{backing.flat_data()} {}

	data<ValueSchema, enc::Native> &ghost_at(const data<sch::FixedArray<sch::UInt64, sizeof...(Sides)>> &index) const {
		return values_.at(index);
	}

	data<ValueSchema, enc::Native> &at(const data<sch::FixedArray<sch::UInt64, sizeof...(Sides)>> &index) const {
		data<sch::FixedArray<sch::UInt64, sizeof...(Sides)>> ind;
		for (uint64_t i = 0u; i < sizeof...(Sides); ++i) {
			ind.at({i}) = index.at({i}) + Ghost;
		}
		return values_.at(ind);
	}

	static constexpr auto get_dims() {
		return data<sch::FixedArray<sch::UInt64, sizeof...(Sides)>, enc::Native>{{Sides...}};
	}
	static constexpr auto meta() { return get_dims(); }
};

} // namespace lbm
} // namespace kel

using namespace kel::lbm;

/* Boundary / op codes; identical numbering to include/kel_lbm_cuda.h. */
enum {
	OP_NONE = 0,
	OP_BOUNCE_BACK = 1,
	OP_FLUID = 2,
	OP_ZOUHE_VELOCITY_X = 3,
	OP_ZOUHE_PRESSURE_X = 4,
	OP_MOVING_WALL = 5,
	OP_ANTI_BOUNCE_BACK = 6,
	OP_EQUILIBRIUM = 7,
};
enum { COLL_BGK = 0, COLL_BGK_GUO = 1, COLL_PSM = 2, COLL_PSM_GUO = 3 };

struct FlagOp {
	int bc = OP_NONE;
	int collide = 0;
	int east = 1; /* template flag of the Zou-He components */
	double rho = 1.0;
	double u[3] = {0, 0, 0};
	int use_profile = 0;
};

struct Params {
	uint64_t steps = 0;
	double tau = 1.0;
	int collision = COLL_BGK;
	double gforce[3] = {0, 0, 0};
	FlagOp ops[8];
};

static std::vector<char> read_file(const std::string &p, bool required) {
	std::ifstream f(p, std::ios::binary);
	if (!f) {
		if (required) {
			std::fprintf(stderr, "missing %s\n", p.c_str());
			std::exit(2);
		}
		return {};
	}
	return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

static Params read_params(const std::string &dir) {
	Params P;
	std::ifstream f(dir + "/params.txt");
	if (!f) {
		std::fprintf(stderr, "missing params.txt\n");
		std::exit(2);
	}
	std::string key;
	while (f >> key) {
		if (key == "steps") f >> P.steps;
		else if (key == "tau") f >> P.tau;
		else if (key == "collision") f >> P.collision;
		else if (key == "gforce") f >> P.gforce[0] >> P.gforce[1] >> P.gforce[2];
		else if (key == "op") {
			int flag;
			f >> flag;
			FlagOp &o = P.ops[flag & 7];
			f >> o.bc >> o.collide >> o.east >> o.rho >> o.u[0] >> o.u[1] >> o.u[2] >> o.use_profile;
		} else {
			std::fprintf(stderr, "bad key %s\n", key.c_str());
			std::exit(2);
		}
	}
	return P;
}

static void write_f64(const std::string &p, const std::vector<double> &v) {
	std::ofstream f(p, std::ios::binary);
	f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(double));
}

template <typename T, typename Desc, uint64_t... Dims>
struct Case {
	static constexpr uint64_t D = Desc::D;
	static constexpr uint64_t Q = Desc::Q;
	using dfi = df_info<T, Desc>;
	using NT = typename native_data_type<T>::type;

	using InfoChunk = sch::Chunk<sch::UInt8, 0u, Dims...>;
	using DfChunk = sch::Chunk<sch::FixedArray<T, Q>, 1u, Dims...>;
	using ChunkStruct = sch::Struct<sch::Member<InfoChunk, "info">, sch::Member<DfChunk, "dfs">, sch::Member<DfChunk, "dfs_old">>;
	using MacroStruct = sch::Struct<
		sch::Member<sch::Chunk<sch::Vector<T, D>, 0u, Dims...>, "velocity">,
		sch::Member<sch::Chunk<sch::Scalar<T>, 0u, Dims...>, "density">,
		sch::Member<sch::Chunk<sch::Scalar<T>, 0u, Dims...>, "porosity">,
		sch::Member<sch::Chunk<sch::Vector<T, D>, 0u, Dims...>, "force">>;

	static constexpr std::array<uint64_t, D> dims{Dims...};
	static constexpr uint64_t N = (Dims * ...);

	static data<sch::FixedArray<sch::UInt64, D>> unflat(uint64_t c) {
		data<sch::FixedArray<sch::UInt64, D>> idx;
		for (uint64_t d = 0; d < D; ++d) {
			idx.at({d}).set(c % dims[d]);
			c /= dims[d];
		}
		return idx;
	}

	static int run(const std::string &in, const std::string &out) {
		Params P = read_params(in);
		auto flags = read_file(in + "/flags.u8", true);
		auto init = read_file(in + "/init.f64", false);
		auto prof = read_file(in + "/profile.f64", false);
		auto por = read_file(in + "/porosity.f64", false);
		auto frc = read_file(in + "/force.f64", false);
		if (flags.size() != N) {
			std::fprintf(stderr, "flags size %zu != %llu\n", flags.size(), (unsigned long long)N);
			return 2;
		}
		if (!init.empty() && init.size() != N * Q * 8) return 3;
		if (!prof.empty() && prof.size() != dims[1] * 8) return 4;

		auto fields_own = heap<data<ChunkStruct>>();
		auto macros_own = heap<data<MacroStruct>>();
		data<sch::Ptr<ChunkStruct>> fields{*fields_own};
		data<sch::Ptr<MacroStruct>> macros{*macros_own};

		auto &info_f = fields.template get<"info">();
		auto &dfs_old_f = fields.template get<"dfs_old">();
		auto &rho_f = macros.template get<"density">();
		auto &vel_f = macros.template get<"velocity">();
		auto &por_f = macros.template get<"porosity">();
		auto &force_f = macros.template get<"force">();

		const double *initp = reinterpret_cast<const double *>(init.data());
		const double *porp = reinterpret_cast<const double *>(por.data());
		const double *frcp = reinterpret_cast<const double *>(frc.data());
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = unflat(c);
			info_f.at(idx).set(static_cast<uint8_t>(flags[c]));
			rho_f.at(idx).at({}).set(1);
			/* rest equilibrium everywhere, as every driver's setup does */
			auto eq = equilibrium<T, Desc>(rho_f.at(idx), vel_f.at(idx));
			auto &df = dfs_old_f.at(idx);
			for (uint64_t i = 0; i < Q; ++i) {
				if (initp) df.at({i}).set(static_cast<NT>(initp[c * Q + i]));
				else df.at({i}) = eq.at(i);
			}
			por_f.at(idx).at({}).set(porp ? static_cast<NT>(porp[c]) : NT(1));
			for (uint64_t d = 0; d < D; ++d) {
				force_f.at(idx).at({{d}}).set(frcp ? static_cast<NT>(frcp[c * D + d]) : NT(0));
			}
		}

		data<sch::Vector<T, D>> gforce;
		for (uint64_t d = 0; d < D; ++d) gforce.at({{d}}).set(static_cast<NT>(P.gforce[d]));

		component<T, Desc, cmpt::BGK> bgk{static_cast<NT>(P.tau)};
		component<T, Desc, cmpt::BGKGuo> guo{static_cast<NT>(P.tau), gforce};
		component<T, Desc, cmpt::Psm> psm{static_cast<NT>(P.tau)};
		component<T, Desc, cmpt::BounceBack> bb;
		component<T, Desc, cmpt::Stream> stream;

		const double *profp = reinterpret_cast<const double *>(prof.data());

		for (uint64_t t = 0; t < P.steps; ++t) {
			data<sch::UInt64> ts{t};
			for (uint64_t c = 0; c < N; ++c) {
				auto idx = unflat(c);
				uint8_t info = info_f.at(idx).get();
				const FlagOp &o = P.ops[info & 7];
				if (info > 7) continue;
				switch (o.bc) {
				case OP_NONE:
					break;
				case OP_BOUNCE_BACK:
					bb.apply(fields, idx, ts);
					break;
				case OP_FLUID:
					break;
				case OP_ZOUHE_VELOCITY_X:
					if constexpr (D == 2 && Q == 9) {
						data<sch::Vector<T, D>> u;
						for (uint64_t d = 0; d < D; ++d) u.at({{d}}).set(static_cast<NT>(o.u[d]));
						if (o.use_profile && profp) u.at({{0u}}).set(static_cast<NT>(profp[idx.at({1u}).get()]));
						if (o.east) {
							component<T, Desc, cmpt::ZouHeVelocityX<true>> zh{u};
							zh.apply(fields, idx, ts);
						} else {
							component<T, Desc, cmpt::ZouHeVelocityX<false>> zh{u};
							zh.apply(fields, idx, ts);
						}
					}
					break;
				case OP_ZOUHE_PRESSURE_X:
					if constexpr ((D == 2 && Q == 9) || (D == 3 && Q == 27)) {
						data<T> r{static_cast<NT>(o.rho)};
						if (o.east) {
							component<T, Desc, cmpt::ZouHePressureX<true>> zh{r};
							zh.apply(fields, idx, ts);
						} else {
							component<T, Desc, cmpt::ZouHePressureX<false>> zh{r};
							zh.apply(fields, idx, ts);
						}
					}
					break;
				case OP_MOVING_WALL: {
					/* examples/cavity_2d_gpu/cavity_2d_gpu.cpp:216-235, e.u over all axes */
					const bool is_even = (t % 2u) == 0u;
					auto &dfs_f = is_even ? fields.template get<"dfs_old">() : fields.template get<"dfs">();
					auto &dfs = dfs_f.at(idx);
					auto df_cpy = dfs;
					for (uint64_t i = 0u; i < Q; ++i) {
						double e_dot_u = 0.0;
						for (uint64_t d = 0; d < D; ++d)
							e_dot_u = e_dot_u + static_cast<NT>(dfi::directions[i][d]) * o.u[d];
						dfs.at({i}) = df_cpy.at({dfi::opposite_index.at(i)}) +
									  data<T>{static_cast<NT>(2.0 * dfi::weights[i] * dfi::inv_cs2 * e_dot_u)};
					}
				} break;
				case OP_ANTI_BOUNCE_BACK:
					if constexpr (D == 2 && Q == 9) {
						component<T, Desc, cmpt::AntiBounceBack<0u>> abb;
						abb.apply(fields, idx, ts);
					}
					break;
				case OP_EQUILIBRIUM: {
					data<sch::Scalar<T>> r;
					r.at({}).set(static_cast<NT>(o.rho));
					data<sch::Vector<T, D>> u;
					for (uint64_t d = 0; d < D; ++d) u.at({{d}}).set(static_cast<NT>(o.u[d]));
					component<T, Desc, cmpt::Equilibrium> eqc{r, u};
					eqc.apply(fields, idx, ts);
				} break;
				}
				if (o.collide) {
					switch (P.collision) {
					case COLL_BGK:
						bgk.apply(fields, macros, idx, ts);
						break;
					case COLL_BGK_GUO:
						guo.apply(fields, macros, idx, ts);
						break;
					case COLL_PSM:
						psm.apply(fields, macros, idx, ts);
						break;
					case COLL_PSM_GUO: {
						/* restatement: Psm, then the BGKGuo forcing term
						 * (collision.hpp:170-203) with u = sum(f c)/rho of the
						 * pre-collision populations and frequency 1/tau */
						const bool is_even = (t % 2u) == 0u;
						auto &dfs_f = is_even ? fields.template get<"dfs_old">() : fields.template get<"dfs">();
						auto &dfs = dfs_f.at(idx);
						auto pre = dfs;
						psm.apply(fields, macros, idx, ts);
						data<sch::Scalar<T>> rho;
						data<sch::Vector<T, D>> vel;
						compute_rho_u<T, Desc>(pre, rho, vel);
						auto total_force = force_f.at(idx) + gforce;
						data<sch::Scalar<T>> ics2;
						ics2.at({}).set(dfi::inv_cs2);
						data<T> freq{NT(1) / static_cast<NT>(P.tau)};
						for (uint64_t i = 0u; i < Q; ++i) {
							data<sch::Vector<T, D>> ci;
							for (uint64_t d = 0u; d < D; ++d)
								ci.at({{d}}).set(static_cast<NT>(dfi::directions[i][d]));
							auto ci_dot_u = math::dot(ci, vel);
							data<sch::Scalar<T>> w;
							w.at({}).set(dfi::weights[i]);
							auto term1 = (ci - vel) * ics2;
							auto term2 = ci * (ci_dot_u * ics2 * ics2);
							auto fp = math::dot(term1 + term2, total_force);
							auto F_i = w * fp;
							dfs.at({i}) = dfs.at({i}) + F_i.at({}) * (data<T>{1} - data<T>{0.5f} * freq);
						}
					} break;
					}
				}
			}
			for (uint64_t c = 0; c < N; ++c) {
				auto idx = unflat(c);
				if (info_f.at(idx).get() > 0u) stream.apply(fields, idx, ts);
			}
		}

		auto &final_f = (P.steps % 2u == 0u) ? fields.template get<"dfs_old">() : fields.template get<"dfs">();
		std::vector<double> dfs(N * Q), rho(N), vel(N * D);
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = unflat(c);
			for (uint64_t i = 0; i < Q; ++i) dfs[c * Q + i] = static_cast<double>(final_f.at(idx).at({i}).get());
			rho[c] = static_cast<double>(rho_f.at(idx).at({}).get());
			for (uint64_t d = 0; d < D; ++d) vel[c * D + d] = static_cast<double>(vel_f.at(idx).at({{d}}).get());
		}
		write_f64(out + "/dfs.f64", dfs);
		write_f64(out + "/rho.f64", rho);
		write_f64(out + "/vel.f64", vel);
		return 0;
	}
};


/*
 * Particle path of one coupled step, phase by phase (reset, gather, contact,
 * integrate), driving the reference's own components:
 *   ParticleForceReset, PsmOneParticleGather (psm.hpp:95-446),
 *   ParticleContact (particle/contact.hpp:522-567), ParticleIntegrate
 *   (particle/integrate.hpp:263-296),
 * on a group built by create_spheroid_particle_group (particle/particle.hpp:19-116).
 * The reference driver runs the four per particle in one work-item
 * (examples/moving_poiseulle_particles_2d_psm_gpu/sim.cpp:198-224), so later
 * particles' contacts can read positions already integrated; here every
 * phase completes for all particles before the next starts.
 *
 * in_dir/pparams.txt: sub_steps k_n zeta_n gamma_t mu gx gy walls
 * in_dir/particles.f64: per particle x y xo yo rot roto radius density
 * in_dir/init.f64: AoS populations at t = 0
 * out_dir/porosity.f64, force_field.f64, after_gather.f64, after_contact.f64,
 *   after_integrate.f64 (28 doubles per particle, kel_particle_state order)
 */
template <typename T, typename Desc, uint64_t NX, uint64_t NY, uint64_t NP>
struct ParticleCase {
	using Base = Case<T, Desc, NX, NY>;
	using NT = typename native_data_type<T>::type;
	static constexpr uint64_t D = 2, Q = Desc::Q, N = NX * NY;
	using GroupSch = sch::ParticleGroup<T, D, NP, coll::Spheroid<T>>;

	template <typename G>
	static void dump(const std::string &path, G &g) {
		std::vector<double> out;
		auto &parts = g.template get<"particles">();
		for (uint64_t p = 0; p < NP; ++p) {
			auto &rb = parts.at({p}).template get<"rigid_body">();
			double st[28] = {0};
			for (uint64_t k = 0; k < D; ++k) {
				st[0 + k] = rb.template get<"position">().at({{k}}).get();
				st[3 + k] = rb.template get<"position_old">().at({{k}}).get();
				st[12 + k] = rb.template get<"acceleration">().at({{k}}).get();
				st[18 + k] = rb.template get<"force">().at({{k}}).get();
			}
			st[6] = rb.template get<"rotation">().at({}).get();
			st[9] = rb.template get<"rotation_old">().at({}).get();
			st[15] = rb.template get<"angular_acceleration">().at({}).get();
			st[21] = rb.template get<"torque">().at({}).get();
			st[24] = rb.template get<"mass">().at({}).get();
			st[25] = rb.template get<"inertia">().at({}).get();
			st[26] = parts.at({p}).template get<"collision">().template get<"radius">().at({}).get();
			st[27] = rb.template get<"density">().at({}).get();
			out.insert(out.end(), st, st + 28);
		}
		write_f64(path, out);
	}

	static int run(const std::string &in, const std::string &out) {
		std::ifstream pf(in + "/pparams.txt");
		uint64_t sub_steps;
		double k_n, zeta, gamma_t, mu, gx, gy;
		int walls;
		pf >> sub_steps >> k_n >> zeta >> gamma_t >> mu >> gx >> gy >> walls;
		auto pv = read_file(in + "/particles.f64", true);
		auto init = read_file(in + "/init.f64", true);
		if (pv.size() != NP * 8 * 8 || init.size() != N * Q * 8) return 5;
		const double *P = reinterpret_cast<const double *>(pv.data());
		const double *I = reinterpret_cast<const double *>(init.data());

		auto fields_own = heap<data<typename Base::ChunkStruct>>();
		auto macros_own = heap<data<typename Base::MacroStruct>>();
		data<sch::Ptr<typename Base::ChunkStruct>> fields{*fields_own};
		data<sch::Ptr<typename Base::MacroStruct>> macros{*macros_own};
		auto &dfs_old_f = fields.template get<"dfs_old">();
		auto &por_f = macros.template get<"porosity">();
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			for (uint64_t i = 0; i < Q; ++i) dfs_old_f.at(idx).at({i}).set(static_cast<NT>(I[c * Q + i]));
			por_f.at(idx).at({}).set(NT(1));
			macros.template get<"density">().at(idx).at({}).set(NT(1));
		}

		data<sch::LbmMeter<sch::Scalar<T>>> r0;
		r0.at({}).set(static_cast<NT>(P[6]));
		data<sch::Scalar<T>> d0;
		d0.at({}).set(static_cast<NT>(P[7]));
		auto g = create_spheroid_particle_group<T, D, NP>(r0, d0, {4u});
		auto &parts = g.template get<"particles">();
		for (uint64_t p = 0; p < NP; ++p) {
			const double *q = P + p * 8;
			auto &pi = parts.at({p});
			auto &rb = pi.template get<"rigid_body">();
			rb.template get<"position">().at({{0u}}).set(static_cast<NT>(q[0]));
			rb.template get<"position">().at({{1u}}).set(static_cast<NT>(q[1]));
			rb.template get<"position_old">().at({{0u}}).set(static_cast<NT>(q[2]));
			rb.template get<"position_old">().at({{1u}}).set(static_cast<NT>(q[3]));
			rb.template get<"rotation">().at({}).set(static_cast<NT>(q[4]));
			rb.template get<"rotation_old">().at({}).set(static_cast<NT>(q[5]));
			/* per-particle size: mass pi r^2 rho, inertia m r^2 / 2 (particle.hpp:79-101) */
			constexpr NT pi_c = 3.14159265358979323846;
			NT r = static_cast<NT>(q[6]), rho = static_cast<NT>(q[7]);
			NT m = pi_c * r * r * rho;
			pi.template get<"collision">().template get<"radius">().at({}).set(r);
			rb.template get<"mass">().at({}).set(m);
			rb.template get<"inertia">().at({}).set(NT(0.5) * m * r * r);
			rb.template get<"density">().at({}).set(rho);
		}
		data<sch::Ptr<GroupSch>, enc::Native> view{g};

		component<T, Desc, cmpt::ParticleForceReset> reset;
		component<T, Desc, cmpt::PsmOneParticleGather> gather;
		dem_params<T> dem{static_cast<NT>(k_n), static_cast<NT>(zeta), static_cast<NT>(gamma_t), static_cast<NT>(mu)};
		data<sch::FixedArray<sch::UInt64, D>> extent{{NX, NY}};
		data<sch::LbmAcceleration<sch::Vector<T, D>>> grav;
		grav.at({{0u}}).set(static_cast<NT>(gx));
		grav.at({{1u}}).set(static_cast<NT>(gy));
		component<T, Desc, cmpt::ParticleIntegrate> integrate{grav};
		data<sch::UInt64> t0{0u}, ss{sub_steps};

		for (uint64_t p = 0; p < NP; ++p) reset.apply(view, {{p}}, t0);
		for (uint64_t p = 0; p < NP; ++p) gather.apply(fields, macros, view, {{p}}, t0, ss);
		dump(out + "/after_gather.f64", g);
		{
			std::vector<double> por(N), ff(N * D);
			for (uint64_t c = 0; c < N; ++c) {
				auto idx = Base::unflat(c);
				por[c] = por_f.at(idx).at({}).get();
				for (uint64_t k = 0; k < D; ++k) ff[c * D + k] = macros.template get<"force">().at(idx).at({{k}}).get();
			}
			write_f64(out + "/porosity.f64", por);
			write_f64(out + "/force_field.f64", ff);
		}
		if (walls) {
			component<T, Desc, cmpt::ParticleContact> contact{dem, extent};
			for (uint64_t p = 0; p < NP; ++p) contact.apply(view, {{p}}, t0, ss);
		} else {
			component<T, Desc, cmpt::ParticleContact> contact{dem};
			for (uint64_t p = 0; p < NP; ++p) contact.apply(view, {{p}}, t0, ss);
		}
		dump(out + "/after_contact.f64", g);
		for (uint64_t p = 0; p < NP; ++p) integrate.apply(view, {{p}}, t0, ss);
		dump(out + "/after_integrate.f64", g);
		return 0;
	}
};

/*
 * HLBM coupling, one time step phase by phase, driving the reference's own
 * components (hlbm.hpp): HlbmReset on every cell, ParticleForceReset,
 * HlbmOneParticleGather, ParticleIntegrate and HlbmOneParticleStamp for every
 * particle (each phase over all particles before the next), then the sweep
 * of examples/moving_poiseulle_particles_2d_hlbm_gpu/sim.cpp:237-262
 * (BounceBack on info 1, Hlbm collision on info 2) and the pull Stream.
 * in_dir: pparams.txt (sub_steps gx gy tau), particles.f64 (8 per body as
 *   ParticleCase), init.f64, flags.u8
 * out_dir: porosity.f64, force_field.f64, after_gather.f64,
 *   after_integrate.f64, hlbm_N.f64, hlbm_D.f64, dfs.f64 (t = 1), rho.f64,
 *   vel.f64
 */
template <typename T, typename Desc, uint64_t NX, uint64_t NY, uint64_t NP>
struct HlbmCase {
	using Base = Case<T, Desc, NX, NY>;
	using PC = ParticleCase<T, Desc, NX, NY, NP>;
	using NT = typename native_data_type<T>::type;
	static constexpr uint64_t D = 2, Q = Desc::Q, N = NX * NY;
	using GroupSch = sch::ParticleGroup<T, D, NP, coll::Spheroid<T>>;
	using Fields = sch::Struct<sch::Member<typename Base::InfoChunk, "info">,
							   sch::Member<typename Base::DfChunk, "dfs">,
							   sch::Member<typename Base::DfChunk, "dfs_old">,
							   sch::Member<sch::Chunk<sch::Vector<T, D>, 0u, NX, NY>, "particle_N">,
							   sch::Member<sch::Chunk<sch::Scalar<T>, 0u, NX, NY>, "particle_D">>;

	static int run(const std::string &in, const std::string &out) {
		std::ifstream pf(in + "/pparams.txt");
		uint64_t sub_steps;
		double gx, gy, tau;
		pf >> sub_steps >> gx >> gy >> tau;
		auto pv = read_file(in + "/particles.f64", true);
		auto init = read_file(in + "/init.f64", true);
		auto flags = read_file(in + "/flags.u8", true);
		if (pv.size() != NP * 8 * 8 || init.size() != N * Q * 8 || flags.size() != N) return 5;
		const double *P = reinterpret_cast<const double *>(pv.data());
		const double *I = reinterpret_cast<const double *>(init.data());

		auto fields_own = heap<data<Fields>>();
		auto macros_own = heap<data<typename Base::MacroStruct>>();
		data<sch::Ptr<Fields>> fields{*fields_own};
		data<sch::Ptr<typename Base::MacroStruct>> macros{*macros_own};
		auto &dfs_old_f = fields.template get<"dfs_old">();
		auto &info_f = fields.template get<"info">();
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			info_f.at(idx).set(static_cast<uint8_t>(flags[c]));
			for (uint64_t i = 0; i < Q; ++i) dfs_old_f.at(idx).at({i}).set(static_cast<NT>(I[c * Q + i]));
			macros.template get<"density">().at(idx).at({}).set(NT(1));
		}
		data<sch::LbmMeter<sch::Scalar<T>>> r0;
		r0.at({}).set(static_cast<NT>(P[6]));
		data<sch::Scalar<T>> d0;
		d0.at({}).set(static_cast<NT>(P[7]));
		auto g = create_spheroid_particle_group<T, D, NP>(r0, d0, {4u});
		auto &parts = g.template get<"particles">();
		for (uint64_t p = 0; p < NP; ++p) {
			const double *q = P + p * 8;
			auto &pi = parts.at({p});
			auto &rb = pi.template get<"rigid_body">();
			rb.template get<"position">().at({{0u}}).set(static_cast<NT>(q[0]));
			rb.template get<"position">().at({{1u}}).set(static_cast<NT>(q[1]));
			rb.template get<"position_old">().at({{0u}}).set(static_cast<NT>(q[2]));
			rb.template get<"position_old">().at({{1u}}).set(static_cast<NT>(q[3]));
			rb.template get<"rotation">().at({}).set(static_cast<NT>(q[4]));
			rb.template get<"rotation_old">().at({}).set(static_cast<NT>(q[5]));
			constexpr NT pi_c = 3.14159265358979323846;
			NT r = static_cast<NT>(q[6]), rho = static_cast<NT>(q[7]);
			NT m = pi_c * r * r * rho;
			pi.template get<"collision">().template get<"radius">().at({}).set(r);
			rb.template get<"mass">().at({}).set(m);
			rb.template get<"inertia">().at({}).set(NT(0.5) * m * r * r);
			rb.template get<"density">().at({}).set(rho);
		}
		data<sch::Ptr<GroupSch>, enc::Native> view{g};

		component<T, Desc, cmpt::HlbmReset> hreset;
		component<T, Desc, cmpt::ParticleForceReset> reset;
		component<T, Desc, cmpt::HlbmOneParticleGather> gather;
		component<T, Desc, cmpt::HlbmOneParticleStamp> stamp;
		data<sch::LbmAcceleration<sch::Vector<T, D>>> grav;
		grav.at({{0u}}).set(static_cast<NT>(gx));
		grav.at({{1u}}).set(static_cast<NT>(gy));
		component<T, Desc, cmpt::ParticleIntegrate> integrate{grav};
		data<sch::UInt64> t0{0u}, ss{sub_steps};

		for (uint64_t c = 0; c < N; ++c) hreset.apply(fields, macros, Base::unflat(c), t0);
		for (uint64_t p = 0; p < NP; ++p) reset.apply(view, {{p}}, t0);
		for (uint64_t p = 0; p < NP; ++p) gather.apply(fields, macros, view, {{p}}, t0, ss);
		PC::dump(out + "/after_gather.f64", g);
		{
			std::vector<double> por(N), ff(N * D);
			for (uint64_t c = 0; c < N; ++c) {
				auto idx = Base::unflat(c);
				por[c] = macros.template get<"porosity">().at(idx).at({}).get();
				for (uint64_t k = 0; k < D; ++k) ff[c * D + k] = macros.template get<"force">().at(idx).at({{k}}).get();
			}
			write_f64(out + "/porosity.f64", por);
			write_f64(out + "/force_field.f64", ff);
		}
		for (uint64_t p = 0; p < NP; ++p) integrate.apply(view, {{p}}, t0, ss);
		PC::dump(out + "/after_integrate.f64", g);
		for (uint64_t p = 0; p < NP; ++p) stamp.apply(fields, macros, view, {{p}}, t0, ss);
		{
			std::vector<double> hn(N * D), hd(N);
			for (uint64_t c = 0; c < N; ++c) {
				auto idx = Base::unflat(c);
				hd[c] = fields.template get<"particle_D">().at(idx).at({}).get();
				for (uint64_t k = 0; k < D; ++k) hn[c * D + k] = fields.template get<"particle_N">().at(idx).at({{k}}).get();
			}
			write_f64(out + "/hlbm_N.f64", hn);
			write_f64(out + "/hlbm_D.f64", hd);
		}
		component<T, Desc, cmpt::Hlbm> collision{static_cast<NT>(tau)};
		component<T, Desc, cmpt::BounceBack> bb;
		component<T, Desc, cmpt::Stream> stream;
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			switch (info_f.at(idx).get()) {
			case 1u: bb.apply(fields, idx, t0); break;
			case 2u: collision.apply(fields, macros, idx, t0); break;
			default: break;
			}
		}
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			if (info_f.at(idx).get() > 0u) stream.apply(fields, idx, t0);
		}
		auto &final_f = fields.template get<"dfs">();
		std::vector<double> dfs(N * Q), rho(N), vel(N * D);
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			for (uint64_t i = 0; i < Q; ++i) dfs[c * Q + i] = static_cast<double>(final_f.at(idx).at({i}).get());
			rho[c] = static_cast<double>(macros.template get<"density">().at(idx).at({}).get());
			for (uint64_t d = 0; d < D; ++d) vel[c * D + d] = static_cast<double>(macros.template get<"velocity">().at(idx).at({{d}}).get());
		}
		write_f64(out + "/dfs.f64", dfs);
		write_f64(out + "/rho.f64", rho);
		write_f64(out + "/vel.f64", vel);
		return 0;
	}
};

/*
 * FPLBM coupling, one time step phase by phase, driving the reference's own
 * components (fplbm.hpp): FpLbmReset on every cell (porosity 1, force 0,
 * density and momentum of the info-2 cells), FpLbmOneParticle for every
 * particle (ramp porosity and coupling force over the AABB, the body's
 * acceleration and its Verlet sub-steps), then the sweep of
 * examples/moving_poiseulle_particles_2d_fplbm_gpu/sim.cpp:229-258
 * (BounceBack on info 1, FpLbm on info 2) and the pull Stream.
 * in_dir: pparams.txt (sub_steps gx gy tau), particles.f64 (8 per body as
 *   ParticleCase), init.f64, flags.u8
 * out_dir: reset_rho.f64, reset_mom.f64 (macros after FpLbmReset),
 *   porosity.f64, force_field.f64, after_particle.f64 (bodies after
 *   FpLbmOneParticle), dfs.f64 (t = 1), rho.f64, vel.f64
 */
template <typename T, typename Desc, uint64_t NX, uint64_t NY, uint64_t NP>
struct FplbmCase {
	using Base = Case<T, Desc, NX, NY>;
	using PC = ParticleCase<T, Desc, NX, NY, NP>;
	using NT = typename native_data_type<T>::type;
	static constexpr uint64_t D = 2, Q = Desc::Q, N = NX * NY;
	using GroupSch = sch::ParticleGroup<T, D, NP, coll::Spheroid<T>>;

	static void dump_macros(const std::string &out, data<sch::Ptr<typename Base::MacroStruct>> &macros,
							const char *rho_name, const char *vel_name) {
		std::vector<double> rho(N), vel(N * D);
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			rho[c] = static_cast<double>(macros.template get<"density">().at(idx).at({}).get());
			for (uint64_t d = 0; d < D; ++d)
				vel[c * D + d] = static_cast<double>(macros.template get<"velocity">().at(idx).at({{d}}).get());
		}
		write_f64(out + "/" + rho_name, rho);
		write_f64(out + "/" + vel_name, vel);
	}

	static int run(const std::string &in, const std::string &out) {
		std::ifstream pf(in + "/pparams.txt");
		uint64_t sub_steps;
		double gx, gy, tau;
		pf >> sub_steps >> gx >> gy >> tau;
		auto pv = read_file(in + "/particles.f64", true);
		auto init = read_file(in + "/init.f64", true);
		auto flags = read_file(in + "/flags.u8", true);
		if (pv.size() != NP * 8 * 8 || init.size() != N * Q * 8 || flags.size() != N) return 5;
		const double *P = reinterpret_cast<const double *>(pv.data());
		const double *I = reinterpret_cast<const double *>(init.data());

		auto fields_own = heap<data<typename Base::ChunkStruct>>();
		auto macros_own = heap<data<typename Base::MacroStruct>>();
		data<sch::Ptr<typename Base::ChunkStruct>> fields{*fields_own};
		data<sch::Ptr<typename Base::MacroStruct>> macros{*macros_own};
		auto &dfs_old_f = fields.template get<"dfs_old">();
		auto &info_f = fields.template get<"info">();
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			info_f.at(idx).set(static_cast<uint8_t>(flags[c]));
			for (uint64_t i = 0; i < Q; ++i) dfs_old_f.at(idx).at({i}).set(static_cast<NT>(I[c * Q + i]));
			macros.template get<"density">().at(idx).at({}).set(NT(1));
		}
		data<sch::LbmMeter<sch::Scalar<T>>> r0;
		r0.at({}).set(static_cast<NT>(P[6]));
		data<sch::Scalar<T>> d0;
		d0.at({}).set(static_cast<NT>(P[7]));
		auto g = create_spheroid_particle_group<T, D, NP>(r0, d0, {4u});
		auto &parts = g.template get<"particles">();
		for (uint64_t p = 0; p < NP; ++p) {
			const double *q = P + p * 8;
			auto &pi = parts.at({p});
			auto &rb = pi.template get<"rigid_body">();
			rb.template get<"position">().at({{0u}}).set(static_cast<NT>(q[0]));
			rb.template get<"position">().at({{1u}}).set(static_cast<NT>(q[1]));
			rb.template get<"position_old">().at({{0u}}).set(static_cast<NT>(q[2]));
			rb.template get<"position_old">().at({{1u}}).set(static_cast<NT>(q[3]));
			rb.template get<"rotation">().at({}).set(static_cast<NT>(q[4]));
			rb.template get<"rotation_old">().at({}).set(static_cast<NT>(q[5]));
			constexpr NT pi_c = 3.14159265358979323846;
			NT r = static_cast<NT>(q[6]), rho = static_cast<NT>(q[7]);
			NT m = pi_c * r * r * rho;
			pi.template get<"collision">().template get<"radius">().at({}).set(r);
			rb.template get<"mass">().at({}).set(m);
			rb.template get<"inertia">().at({}).set(NT(0.5) * m * r * r);
			rb.template get<"density">().at({}).set(rho);
		}
		data<sch::Ptr<GroupSch>, enc::Native> view{g};

		component<T, Desc, cmpt::FpLbmReset> freset;
		data<sch::LbmAcceleration<sch::Vector<T, D>>> grav;
		grav.at({{0u}}).set(static_cast<NT>(gx));
		grav.at({{1u}}).set(static_cast<NT>(gy));
		component<T, Desc, cmpt::FpLbmOneParticle> one{grav};
		data<sch::UInt64> t0{0u}, ss{sub_steps};

		for (uint64_t c = 0; c < N; ++c) freset.apply(fields, macros, Base::unflat(c), t0);
		dump_macros(out, macros, "reset_rho.f64", "reset_mom.f64");
		for (uint64_t p = 0; p < NP; ++p) one.apply(fields, macros, view, {{p}}, t0, ss);
		PC::dump(out + "/after_particle.f64", g);
		{
			std::vector<double> por(N), ff(N * D);
			for (uint64_t c = 0; c < N; ++c) {
				auto idx = Base::unflat(c);
				por[c] = macros.template get<"porosity">().at(idx).at({}).get();
				for (uint64_t k = 0; k < D; ++k) ff[c * D + k] = macros.template get<"force">().at(idx).at({{k}}).get();
			}
			write_f64(out + "/porosity.f64", por);
			write_f64(out + "/force_field.f64", ff);
		}
		component<T, Desc, cmpt::FpLbm> collision{static_cast<NT>(tau)};
		component<T, Desc, cmpt::BounceBack> bb;
		component<T, Desc, cmpt::Stream> stream;
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			switch (info_f.at(idx).get()) {
			case 1u: bb.apply(fields, idx, t0); break;
			case 2u: collision.apply(fields, macros, idx, t0); break;
			default: break;
			}
		}
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			if (info_f.at(idx).get() > 0u) stream.apply(fields, idx, t0);
		}
		auto &final_f = fields.template get<"dfs">();
		std::vector<double> dfs(N * Q);
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = Base::unflat(c);
			for (uint64_t i = 0; i < Q; ++i) dfs[c * Q + i] = static_cast<double>(final_f.at(idx).at({i}).get());
		}
		write_f64(out + "/dfs.f64", dfs);
		dump_macros(out, macros, "rho.f64", "vel.f64");
		return 0;
	}
};

/*
 * Field writers of the reference on given values: write_vtk_file /
 * write_csv_file (modules/core/c++/write_vtk.hpp, write_csv.hpp) of the
 * drivers' MacroStruct {velocity, density} and of the lattice struct {info,
 * dfs, dfs_old}, and the Forst encoding (abstract/forst.hpp, forst_chunk.hpp)
 * of both, for byte comparison with the library's writers.
 *   in_dir/flags.u8, dfs.f64 (AoS, Q per cell), rho.f64, vel.f64 (D per cell)
 *   out_dir/vtk/m_37.vtk, out_dir/vtk/initial_state_0.vtk,
 *   out_dir/csv/m_velocity_37.csv, out_dir/csv/m_density_37.csv,
 *   out_dir/m.forst, out_dir/lattice.forst
 */
template <typename T, typename Desc, uint64_t... Dims>
struct WriterCase {
	using B = Case<T, Desc, Dims...>;
	static constexpr uint64_t D = Desc::D, Q = Desc::Q, N = B::N;
	using NT = typename native_data_type<T>::type;
	using Macro = sch::Struct<sch::Member<sch::Chunk<sch::Vector<T, D>, 0u, Dims...>, "velocity">,
							  sch::Member<sch::Chunk<sch::Scalar<T>, 0u, Dims...>, "density">>;

	template <typename Sch>
	static int encode(const data<Sch> &from, const std::string &path) {
		codec<Sch, enc::Forst> c;
		data<Sch, enc::Forst> bytes;
		auto eov = c.encode(from, bytes);
		if (eov.is_error()) return 3;
		std::ofstream f(path, std::ios::binary);
		f.write(reinterpret_cast<const char *>(bytes.raw()), (std::streamsize)bytes.size().get());
		return 0;
	}

	static int run(const std::string &in, const std::string &out) {
		auto flags = read_file(in + "/flags.u8", true);
		auto dfs = read_file(in + "/dfs.f64", true);
		auto rho = read_file(in + "/rho.f64", true);
		auto vel = read_file(in + "/vel.f64", true);
		const double *pd = reinterpret_cast<const double *>(dfs.data());
		const double *pr = reinterpret_cast<const double *>(rho.data());
		const double *pv = reinterpret_cast<const double *>(vel.data());
		auto macros = std::make_unique<data<Macro>>();
		auto fields = std::make_unique<data<typename B::ChunkStruct>>();
		for (uint64_t c = 0; c < N; ++c) {
			auto idx = B::unflat(c);
			for (uint64_t d = 0; d < D; ++d)
				macros->template get<"velocity">().at(idx).at({{d}}).set(static_cast<NT>(pv[c * D + d]));
			macros->template get<"density">().at(idx).at({}).set(static_cast<NT>(pr[c]));
			fields->template get<"info">().at(idx).set(static_cast<uint8_t>(flags[c]));
			for (uint64_t i = 0; i < Q; ++i) {
				fields->template get<"dfs">().at(idx).at({i}).set(static_cast<NT>(pd[c * Q + i]));
				fields->template get<"dfs_old">().at(idx).at({i}).set(static_cast<NT>(-pd[c * Q + i]));
			}
		}
		std::filesystem::path od(out);
		if (write_vtk_file(od, "m", 37u, *macros).is_error()) return 4;
		if (write_csv_file(od, "m", 37u, *macros).is_error()) return 4;
		if (write_vtk_file(od, "initial_state", 0u, *fields).is_error()) return 4;
		if (encode(*macros, out + "/m.forst")) return 3;
		if (encode(*fields, out + "/lattice.forst")) return 3;
		return 0;
	}
};

/*
 * Voxel signed-distance bodies (particle/mask.hpp, particle/porosity.hpp:24-54,
 * particle/voxel_narrow.hpp), T = Float64, a group of NB bodies made by
 * create_spheroid_particle_group (sphere mask) or refilled with sdf::cube.
 *   in_dir/vparams.txt  resolution kind(0 sphere, 1 cube) eps nx ny nz
 *   in_dir/bodies.f64   NB x (position[3], rotation[3], radius)
 *   in_dir/locals.f64   local points (3 doubles each) for mask_sample_local
 *   in_dir/points.f64   lattice points (3 doubles each)
 *   in_dir/pairs.f64    body pairs (lo, hi)
 *   in_dir/sdfs.f64     signed distances for solid_fraction_from_sdf
 * out: mask.f64 (iteration order), com.f64 (3), sample.f64, sdf.f64 and
 * porosity.f64 (body-major, per point), global.f64 (mask_local_to_global of
 * each local point per body, 3 each), solid.f64, contacts.f64 (per pair: hit,
 * depth, normal[3], point[3]).
 */
template <uint64_t D, uint64_t NB>
struct VoxelCase {
	using T = sch::Float64;
	using NT = double;

	static std::vector<double> read_f64(const std::string &p) {
		auto v = read_file(p, true);
		std::vector<double> o(v.size() / 8);
		std::memcpy(o.data(), v.data(), o.size() * 8);
		return o;
	}
	template <typename V>
	static data<sch::Vector<T, D>> vec(const V *x) {
		data<sch::Vector<T, D>> u;
		for (uint64_t i = 0; i < D; ++i) u.at({{i}}).set(static_cast<NT>(x[i]));
		return u;
	}

	static int run(const std::string &in, const std::string &out) {
		std::ifstream pf(in + "/vparams.txt");
		uint64_t R, kind, ext[3];
		double eps;
		pf >> R >> kind >> eps >> ext[0] >> ext[1] >> ext[2];
		auto B = read_f64(in + "/bodies.f64");
		auto L = read_f64(in + "/locals.f64");
		auto X = read_f64(in + "/points.f64");
		auto PR = read_f64(in + "/pairs.f64");
		auto S = read_f64(in + "/sdfs.f64");
		if (B.size() != NB * 7) return 5;
		data<sch::LbmMeter<sch::Scalar<T>>> r0;
		r0.at({}).set(B[6]);
		data<sch::Scalar<T>> d0;
		d0.at({}).set(1.0);
		auto g = create_spheroid_particle_group<T, D, NB>(r0, d0, {R});
		auto &mask = g.template get<"mask">();
		if (kind == 1)
			g.template get<"center_of_mass">().at({0u}) = fill_mask_from_sdf<T, D>(
				mask, R, [](const data<sch::Vector<T, D>> &u) { return sdf::cube<T, D>(u); });
		auto &parts = g.template get<"particles">();
		for (uint64_t p = 0; p < NB; ++p) {
			const double *q = B.data() + p * 7;
			auto &pi = parts.at({p});
			auto &rb = pi.template get<"rigid_body">();
			for (uint64_t i = 0; i < D; ++i) rb.template get<"position">().at({{i}}).set(q[i]);
			if constexpr (D == 2) rb.template get<"rotation">().at({}).set(q[3]);
			else
				for (uint64_t i = 0; i < 3; ++i) rb.template get<"rotation">().at({{i}}).set(q[3 + i]);
			pi.template get<"collision">().template get<"radius">().at({}).set(q[6]);
		}
		std::vector<double> m;
		iterator<D>::apply([&](const auto &k) { m.push_back(static_cast<double>(mask.at(k).get())); }, {},
						   mask.get_dims());
		write_f64(out + "/mask.f64", m);
		auto &com = g.template get<"center_of_mass">().at({0u});
		std::vector<double> c(3, 0.0);
		for (uint64_t i = 0; i < D; ++i) c[i] = com.at({{i}}).get();
		write_f64(out + "/com.f64", c);
		std::vector<double> samp, glob, sdf, por, sol, con;
		for (size_t k = 0; k + 3 <= L.size(); k += 3) samp.push_back(mask_sample_local<T, D>(mask, vec(&L[k]), R));
		for (uint64_t p = 0; p < NB; ++p) {
			auto &pi = parts.at({p});
			for (size_t k = 0; k + 3 <= L.size(); k += 3) {
				auto x = mask_local_to_global<T, D>(vec(&L[k]), pi, com);
				for (uint64_t i = 0; i < 3; ++i) glob.push_back(i < D ? x.at({{i}}).get() : 0.0);
			}
			for (size_t k = 0; k + 3 <= X.size(); k += 3) {
				sdf.push_back(mask_signed_distance<T, D>(g, pi, vec(&X[k]), R));
				data<sch::Scalar<T>> e;
				e.at({}).set(eps);
				por.push_back(particle_porosity<T, D, 1u, por::ParticleVoxel<T>>::calculate(g, p, vec(&X[k]), e)
								  .at({})
								  .get());
			}
		}
		for (double v : S) sol.push_back(solid_fraction_from_sdf<T>(v, eps));
		data<sch::FixedArray<sch::UInt64, D>> extent;
		for (uint64_t i = 0; i < D; ++i) extent.at({i}).set(ext[i]);
		data<sch::Scalar<T>> e;
		e.at({}).set(eps);
		for (size_t k = 0; k + 2 <= PR.size(); k += 2) {
			data<sch::ContactManifold<T, D>> mf;
			bool hit = voxel_contact<T, D>(g, parts.at({(uint64_t)PR[k]}), parts.at({(uint64_t)PR[k + 1]}), extent, e,
										  mf);
			con.push_back(hit ? 1.0 : 0.0);
			con.push_back(hit ? mf.template get<"depth">().at({}).get() : 0.0);
			for (uint64_t i = 0; i < 3; ++i) con.push_back(hit && i < D ? mf.template get<"normal">().at({{i}}).get() : 0.0);
			for (uint64_t i = 0; i < 3; ++i) con.push_back(hit && i < D ? mf.template get<"point">().at({{i}}).get() : 0.0);
		}
		write_f64(out + "/sample.f64", samp);
		write_f64(out + "/global.f64", glob);
		write_f64(out + "/sdf.f64", sdf);
		write_f64(out + "/porosity.f64", por);
		write_f64(out + "/solid.f64", sol);
		write_f64(out + "/contacts.f64", con);
		return 0;
	}
};

int main(int argc, char **argv) {
	if (argc != 4) {
		std::fprintf(stderr, "usage: %s <case> <in_dir> <out_dir>\n", argv[0]);
		return 1;
	}
	std::string c = argv[1];
	using F32 = sch::Float32;
	using F64 = sch::Float64;
	if (c == "d2q9_f32_48x20") return Case<F32, sch::D2Q9, 48, 20>::run(argv[2], argv[3]);
	if (c == "d2q9_f64_48x20") return Case<F64, sch::D2Q9, 48, 20>::run(argv[2], argv[3]);
	if (c == "d2q9_f32_256x64") return Case<F32, sch::D2Q9, 256, 64>::run(argv[2], argv[3]);
	if (c == "d3q19_f32_16x12x10") return Case<F32, sch::D3Q19, 16, 12, 10>::run(argv[2], argv[3]);
	if (c == "d3q19_f64_16x12x10") return Case<F64, sch::D3Q19, 16, 12, 10>::run(argv[2], argv[3]);
	if (c == "d3q27_f32_16x12x10") return Case<F32, sch::D3Q27, 16, 12, 10>::run(argv[2], argv[3]);
	if (c == "particles_d2q9_f64_64x48x5") return ParticleCase<F64, sch::D2Q9, 64, 48, 5>::run(argv[2], argv[3]);
	if (c == "particles_d2q9_f32_64x48x5") return ParticleCase<F32, sch::D2Q9, 64, 48, 5>::run(argv[2], argv[3]);
	if (c == "d3q27_f64_16x12x10") return Case<F64, sch::D3Q27, 16, 12, 10>::run(argv[2], argv[3]);
	if (c == "hlbm_d2q9_f64_48x40x3") return HlbmCase<F64, sch::D2Q9, 48, 40, 3>::run(argv[2], argv[3]);
	if (c == "hlbm_d2q9_f32_48x40x3") return HlbmCase<F32, sch::D2Q9, 48, 40, 3>::run(argv[2], argv[3]);
	if (c == "fplbm_d2q9_f64_48x40x1") return FplbmCase<F64, sch::D2Q9, 48, 40, 1>::run(argv[2], argv[3]);
	if (c == "fplbm_d2q9_f32_48x40x1") return FplbmCase<F32, sch::D2Q9, 48, 40, 1>::run(argv[2], argv[3]);
	if (c == "fplbm_d2q9_f32_48x40x3") return FplbmCase<F32, sch::D2Q9, 48, 40, 3>::run(argv[2], argv[3]);
	if (c == "voxel_2d_f64_4") return VoxelCase<2, 4>::run(argv[2], argv[3]);
	if (c == "voxel_3d_f64_4") return VoxelCase<3, 4>::run(argv[2], argv[3]);
	if (c == "writers_d2q9_f32_12x7") return WriterCase<F32, sch::D2Q9, 12, 7>::run(argv[2], argv[3]);
	if (c == "writers_d3q19_f64_5x4x3") return WriterCase<F64, sch::D3Q19, 5, 4, 3>::run(argv[2], argv[3]);
	std::fprintf(stderr, "unknown case %s\n", c.c_str());
	return 1;
}
