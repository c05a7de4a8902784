// kel/lbm/cuda/lbm_cuda.hpp -- C++ face of the GB300 hot path.
//
// Keeps the spellings a keldu/lbm_mirror driver already uses for this path --
// df_info<T, Desc> (modules/core/c++/descriptor/*.hpp), sch::D2Q9 / D3Q19 /
// D3Q27, component<T, Desc, cmpt::X> with the reference's constructor
// arguments (collision.hpp, boundary.hpp, psm.hpp), error_or<T> results
// (abstract/error.hpp) -- and lowers them onto the C ABI of kel_lbm_cuda.h.
// A driver's per-cell `switch(info)` inside q.submit(parallel_for ...)
// (e.g. examples/stdkr_2d_bgk/step.hpp:22-69) becomes a step_program that maps
// each flag value to its boundary component and collision, and one call to
// lattice::step.  Header only; link libkel_lbm_cuda.so.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../../../kel_lbm_cuda.h"

namespace kel {
namespace lbm {
namespace cuda {

// ---- errors ------------------------------------------------------------------

struct error {
	int code = KEL_OK;
	std::string message;
};

template <typename T>
class error_or {
	bool ok_;
	T value_{};
	error err_;

public:
	error_or(T v) : ok_{true}, value_{std::move(v)} {}
	error_or(error e) : ok_{false}, err_{std::move(e)} {}
	bool is_error() const { return !ok_; }
	bool is_value() const { return ok_; }
	T &get_value() { return value_; }
	const error &get_error() const { return err_; }
};

template <>
class error_or<void> {
	bool ok_;
	error err_;

public:
	error_or() : ok_{true} {}
	error_or(error e) : ok_{false}, err_{std::move(e)} {}
	bool is_error() const { return !ok_; }
	bool is_value() const { return ok_; }
	const error &get_error() const { return err_; }
};

inline error_or<void> make_void() { return {}; }

inline error_or<void> status(int rc) {
	if (rc == KEL_OK) return {};
	return error{rc, kel_last_error_string()};
}

// ---- descriptors (same tables as df_info<T, Desc>) --------------------------------

namespace sch {
template <uint64_t DV, uint64_t QV>
struct Descriptor {
	static constexpr uint64_t D = DV;
	static constexpr uint64_t Q = QV;
};
using D2Q9 = Descriptor<2u, 9u>;
using D3Q19 = Descriptor<3u, 19u>;
using D3Q27 = Descriptor<3u, 27u>;
struct Float32 {};
struct Float64 {};
} // namespace sch

template <typename T, typename Desc>
struct df_info;

template <typename T>
struct df_info<T, sch::D2Q9> {
	static constexpr uint64_t D = 2u, Q = 9u;
	static constexpr std::array<std::array<int32_t, 2>, 9> directions = {
		{{0, 0}, {-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, 1}, {-1, 1}, {1, -1}}};
	static constexpr std::array<double, 9> weights = {4. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 9.,
													  1. / 36., 1. / 36., 1. / 36., 1. / 36.};
	static constexpr std::array<uint64_t, 9> opposite_index = {0, 2, 1, 4, 3, 6, 5, 8, 7};
	static constexpr double inv_cs2 = 3.0, cs2 = 1. / 3.;
	static constexpr int32_t id = KEL_D2Q9;
};

template <typename T>
struct df_info<T, sch::D3Q19> {
	static constexpr uint64_t D = 3u, Q = 19u;
	static constexpr std::array<std::array<int32_t, 3>, 19> directions = {
		{{0, 0, 0},  {-1, 0, 0}, {1, 0, 0},  {0, -1, 0}, {0, 1, 0},   {0, 0, -1}, {0, 0, 1},
		 {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 1, 0},  {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
		 {1, 0, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}, {0, 1, 1}}};
	static constexpr std::array<double, 19> weights = {1. / 3.,  1. / 18., 1. / 18., 1. / 18., 1. / 18.,
													   1. / 18., 1. / 18., 1. / 36., 1. / 36., 1. / 36.,
													   1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36.,
													   1. / 36., 1. / 36., 1. / 36., 1. / 36.};
	static constexpr std::array<uint64_t, 19> opposite_index = {0,  2,  1,  4,  3,  6,  5,  10, 9, 8,
																7,  14, 13, 12, 11, 18, 17, 16, 15};
	static constexpr double inv_cs2 = 3.0, cs2 = 1. / 3.;
	static constexpr int32_t id = KEL_D3Q19;
};

template <typename T>
struct df_info<T, sch::D3Q27> {
	static constexpr uint64_t D = 3u, Q = 27u;
	static constexpr int32_t id = KEL_D3Q27;
	static constexpr double inv_cs2 = 3.0, cs2 = 1. / 3.;
	// i = a + 3 b + 9 g with axis offsets ordered (0, -1, +1) (descriptor/d3q27.hpp:16-47)
	static constexpr int32_t axis(uint64_t a) { return a == 0 ? 0 : (a == 1 ? -1 : 1); }
	static constexpr int32_t dir(uint64_t i, uint64_t k) {
		return k == 0 ? axis(i % 3) : (k == 1 ? axis((i / 3) % 3) : axis(i / 9));
	}
};

// ---- components (parameter carriers, reference constructor arguments) -------------

namespace cmpt {
struct BGK {};
struct BGKGuo {};
struct Psm {};
struct PsmGuo {};
struct Hlbm {};
struct FpLbm {};
struct BounceBack {};
template <uint64_t I>
struct AntiBounceBack {};
struct Equilibrium {};
template <bool East>
struct ZouHePressureX {};
template <bool East>
using ZouHeHorizontal = ZouHePressureX<East>;
template <bool East>
struct ZouHeVelocityX {};
struct MovingWall {};
} // namespace cmpt

template <typename T, typename Desc, typename Cmpt>
class component;

template <typename T, typename Desc>
class component<T, Desc, cmpt::BGK> {
public:
	double relaxation;
	explicit component(double relaxation__) : relaxation{relaxation__} {}
	void lower(kel_step_program &p) const {
		p.collision = KEL_COLL_BGK;
		p.tau = relaxation;
	}
};

template <typename T, typename Desc>
class component<T, Desc, cmpt::BGKGuo> {
public:
	double relaxation;
	std::array<double, 3> global_force{};
	explicit component(double relaxation__) : relaxation{relaxation__} {}
	component(double relaxation__, const std::array<double, Desc::D> &force) : relaxation{relaxation__} {
		for (uint64_t k = 0; k < Desc::D; ++k) global_force[k] = force[k];
	}
	void lower(kel_step_program &p) const {
		p.collision = KEL_COLL_BGK_GUO;
		p.tau = relaxation;
		for (int k = 0; k < 3; ++k) p.global_force[k] = global_force[k];
	}
};

template <typename T, typename Desc>
class component<T, Desc, cmpt::Psm> {
public:
	double relaxation;
	explicit component(double relaxation__) : relaxation{relaxation__} {}
	void lower(kel_step_program &p) const {
		p.collision = KEL_COLL_PSM;
		p.tau = relaxation;
	}
};

// cmpt::Hlbm (hlbm.hpp:53-101), D2Q9: the collision of the HLBM coupling;
// the per-cell porosity / particle_N / particle_D it reads come from
// kel_particles_* with KEL_COUPLING_HLBM.
template <typename T, typename Desc>
class component<T, Desc, cmpt::Hlbm> {
public:
	double relaxation;
	explicit component(double relaxation__) : relaxation{relaxation__} {}
	void lower(kel_step_program &p) const {
		p.collision = KEL_COLL_HLBM;
		p.tau = relaxation;
	}
};

// cmpt::FpLbm (fplbm.hpp:57-128), D2Q9: the collision of the FPLBM coupling;
// the coupling force it applies comes from kel_particles_* with
// KEL_COUPLING_FPLBM (FpLbmReset + FpLbmOneParticle).
template <typename T, typename Desc>
class component<T, Desc, cmpt::FpLbm> {
public:
	double relaxation;
	explicit component(double relaxation__) : relaxation{relaxation__} {}
	void lower(kel_step_program &p) const {
		p.collision = KEL_COLL_FPLBM;
		p.tau = relaxation;
	}
};

template <typename T, typename Desc>
class component<T, Desc, cmpt::PsmGuo> {
public:
	double relaxation;
	std::array<double, 3> global_force{};
	component(double relaxation__, const std::array<double, Desc::D> &force) : relaxation{relaxation__} {
		for (uint64_t k = 0; k < Desc::D; ++k) global_force[k] = force[k];
	}
	void lower(kel_step_program &p) const {
		p.collision = KEL_COLL_PSM_GUO;
		p.tau = relaxation;
		for (int k = 0; k < 3; ++k) p.global_force[k] = global_force[k];
	}
};

template <typename T, typename Desc>
class component<T, Desc, cmpt::BounceBack> {
public:
	void lower(kel_flag_op &o) const { o.bc = KEL_BC_BOUNCE_BACK; }
};

template <typename T, typename Desc, uint64_t I>
class component<T, Desc, cmpt::AntiBounceBack<I>> {
public:
	void lower(kel_flag_op &o) const { o.bc = KEL_BC_ANTI_BOUNCE_BACK; }
};

template <typename T, typename Desc>
class component<T, Desc, cmpt::Equilibrium> {
public:
	double density;
	std::array<double, 3> velocity{};
	component(double density__, const std::array<double, Desc::D> &velocity__) : density{density__} {
		for (uint64_t k = 0; k < Desc::D; ++k) velocity[k] = velocity__[k];
	}
	void lower(kel_flag_op &o) const {
		o.bc = KEL_BC_EQUILIBRIUM;
		o.rho = density;
		for (int k = 0; k < 3; ++k) o.u[k] = velocity[k];
	}
};

template <typename T, typename Desc, bool East>
class component<T, Desc, cmpt::ZouHePressureX<East>> {
public:
	double rho_setting;
	explicit component(double rho_setting__) : rho_setting{rho_setting__} {}
	void lower(kel_flag_op &o) const {
		o.bc = KEL_BC_ZOUHE_PRESSURE_X;
		o.east = East ? 1 : 0;
		o.rho = rho_setting;
	}
};

template <typename T, typename Desc, bool East>
class component<T, Desc, cmpt::ZouHeVelocityX<East>> {
public:
	std::array<double, 3> velocity{};
	bool use_profile = false;
	explicit component(const std::array<double, Desc::D> &velocity__) {
		for (uint64_t k = 0; k < Desc::D; ++k) velocity[k] = velocity__[k];
	}
	// u_x taken per row from the lattice's inlet profile (upload_inlet_profile)
	static component from_profile() {
		component c{std::array<double, Desc::D>{}};
		c.use_profile = true;
		return c;
	}
	void lower(kel_flag_op &o) const {
		o.bc = KEL_BC_ZOUHE_VELOCITY_X;
		o.east = East ? 1 : 0;
		o.use_profile = use_profile ? 1 : 0;
		for (int k = 0; k < 3; ++k) o.u[k] = velocity[k];
	}
};

template <typename T, typename Desc>
class component<T, Desc, cmpt::MovingWall> {
public:
	std::array<double, 3> lid_velocity{};
	explicit component(const std::array<double, Desc::D> &u) {
		for (uint64_t k = 0; k < Desc::D; ++k) lid_velocity[k] = u[k];
	}
	void lower(kel_flag_op &o) const {
		o.bc = KEL_BC_MOVING_WALL;
		for (int k = 0; k < 3; ++k) o.u[k] = lid_velocity[k];
	}
};

// ---- the per-flag switch of a driver ------------------------------------------------

// Built once, then handed to lattice::step; mirrors
//   switch(info){ case 1u: bb.apply(...); break; case 2u: collision.apply(...); ... }
class step_program {
	kel_step_program p_{};

public:
	step_program() { p_.tau = 1.0; }
	explicit step_program(bool reference_arithmetic) {
		p_.tau = 1.0;
		p_.arithmetic = reference_arithmetic ? KEL_ARITH_REFERENCE : KEL_ARITH_FAST;
	}

	// flag -> boundary component only (no collision: walls, lids)
	template <typename Boundary>
	step_program &on(uint8_t flag, const Boundary &bc) {
		kel_flag_op &o = p_.ops[flag];
		o = kel_flag_op{};
		bc.lower(o);
		return *this;
	}

	// flag -> boundary component, then the collision
	template <typename Boundary, typename Collision>
	step_program &on(uint8_t flag, const Boundary &bc, const Collision &coll) {
		on(flag, bc);
		p_.ops[flag].collide = 1;
		coll.lower(p_);
		return *this;
	}

	// flag -> collision only (fluid)
	template <typename Collision>
	step_program &fluid(uint8_t flag, const Collision &coll) {
		kel_flag_op &o = p_.ops[flag];
		o = kel_flag_op{};
		o.bc = KEL_BC_FLUID;
		o.collide = 1;
		coll.lower(p_);
		return *this;
	}

	const kel_step_program &get() const { return p_; }
};

// ---- the lattice: owns device memory like data<ChunkStruct, encode::Sycl<>> ---------

enum class storage { fp32 = KEL_STORAGE_FP32, fp16_shifted = KEL_STORAGE_FP16S };

template <typename T, typename Desc>
class lattice {
	kel_lattice *h_ = nullptr;
	std::array<int64_t, 3> dims_{1, 1, 1};

public:
	lattice() = default;
	lattice(const lattice &) = delete;
	lattice &operator=(const lattice &) = delete;
	lattice(lattice &&o) noexcept : h_{o.h_}, dims_{o.dims_} { o.h_ = nullptr; }
	~lattice() { kel_lattice_destroy(h_); }

	static error_or<lattice> create(const std::array<int64_t, Desc::D> &dims, storage s = storage::fp32,
									bool periodic_x = false) {
		kel_lattice_desc d{};
		d.descriptor = df_info<T, Desc>::id;
		d.storage = static_cast<int32_t>(s);
		d.nx = dims[0];
		d.ny = dims[1];
		d.nz = Desc::D == 3 ? dims[Desc::D - 1] : 1;
		d.flags = periodic_x ? KEL_LATTICE_PERIODIC_X : 0u;
		lattice l;
		int rc = kel_lattice_create(&d, &l.h_);
		if (rc != KEL_OK) return error{rc, kel_last_error_string()};
		l.dims_ = {d.nx, d.ny, d.nz};
		return l;
	}

	int64_t cells() const { return dims_[0] * dims_[1] * dims_[2]; }
	kel_lattice *handle() const { return h_; }

	error_or<void> copy_flags_to_device(const std::vector<uint8_t> &info) {
		if ((int64_t)info.size() != cells()) return error{KEL_ERR_INVALID_ARGUMENT, "info: wrong size"};
		return status(kel_upload_flags(h_, info.data()));
	}
	error_or<void> copy_populations_to_device(const std::vector<float> &aos) {
		if ((int64_t)aos.size() != cells() * (int64_t)Desc::Q) return error{KEL_ERR_INVALID_ARGUMENT, "dfs: wrong size"};
		return status(kel_upload_populations(h_, aos.data(), KEL_DTYPE_F32, KEL_LAYOUT_AOS));
	}
	error_or<void> copy_populations_to_host(std::vector<float> &aos) {
		aos.resize(cells() * Desc::Q);
		return status(kel_download_populations(h_, aos.data(), KEL_DTYPE_F32, KEL_LAYOUT_AOS));
	}
	error_or<void> copy_macros_to_host(std::vector<float> &rho, std::vector<float> &vel) {
		rho.resize(cells());
		vel.resize(cells() * Desc::D);
		return status(kel_download_macros(h_, rho.data(), vel.data()));
	}
	error_or<void> upload_inlet_profile(const std::vector<double> &ux_per_y) {
		return status(kel_upload_inlet_profile(h_, ux_per_y.data(), (int64_t)ux_per_y.size()));
	}
	error_or<void> set_stream(void *cuda_stream) { return status(kel_lattice_set_stream(h_, cuda_stream)); }

	// n time steps of collide + boundary + stream; macros of the last one stored
	error_or<void> step(const step_program &prog, uint64_t n = 1, bool write_macros = true) {
		return status(kel_step(h_, &prog.get(), n, write_macros ? KEL_STEP_WRITE_MACROS : 0u));
	}
	error_or<void> synchronize() { return status(kel_lattice_synchronize(h_)); }
	uint64_t time_step() const {
		uint64_t t = 0;
		kel_lattice_time_step(h_, &t);
		return t;
	}
};

} // namespace cuda
} // namespace lbm
} // namespace kel
