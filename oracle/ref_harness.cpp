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

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
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
	if (c == "d3q27_f64_16x12x10") return Case<F64, sch::D3Q27, 16, 12, 10>::run(argv[2], argv[3]);
	std::fprintf(stderr, "unknown case %s\n", c.c_str());
	return 1;
}
