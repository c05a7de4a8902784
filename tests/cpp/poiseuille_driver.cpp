// A keldu/lbm_mirror-style driver written against the C++ face of the GB300
// path: the geometry and the per-flag switch of examples/stdkr_2d_bgk
// (init.hpp:16-54, step.hpp:22-69) become a step_program; the time loop is
// one lattice::step call.  Writes rho and u of the last step to argv[4].
//
//   poiseuille_driver <nx> <ny> <steps> <out.bin> [reference]
#include <kel/lbm/cuda/lbm_cuda.hpp>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace kel::lbm::cuda;
using T = sch::Float32;
using Desc = sch::D2Q9;

int main(int argc, char **argv) {
	if (argc < 5) {
		std::fprintf(stderr, "usage: %s nx ny steps out.bin [reference]\n", argv[0]);
		return 2;
	}
	const int64_t nx = std::atoll(argv[1]), ny = std::atoll(argv[2]);
	const uint64_t steps = std::strtoull(argv[3], nullptr, 10);
	const bool reference = argc > 5 && std::strcmp(argv[5], "reference") == 0;

	auto eo = lattice<T, Desc>::create({nx, ny});
	if (eo.is_error()) {
		std::fprintf(stderr, "create: %s\n", eo.get_error().message.c_str());
		return 1;
	}
	auto &lat = eo.get_value();

	// info: walls 1 on the rim, fluid 2, inflow 3 at x = 0, outflow 4 at x = nx-1
	std::vector<uint8_t> info(nx * ny, 1);
	for (int64_t y = 1; y + 1 < ny; ++y)
		for (int64_t x = 0; x < nx; ++x) info[y * nx + x] = x == 0 ? 3 : (x == nx - 1 ? 4 : 2);
	// parabolic inflow, zero on the half-way wall positions
	std::vector<double> ux(ny, 0.0);
	const double u_max = 0.05;
	for (int64_t y = 1; y + 1 < ny; ++y) {
		const double eta = (y - 0.5) / (double)(ny - 2);
		ux[y] = 4.0 * u_max * eta * (1.0 - eta);
	}

	component<T, Desc, cmpt::BGK> collision{0.8};
	component<T, Desc, cmpt::BounceBack> bb;
	component<T, Desc, cmpt::ZouHeVelocityX<true>> flow_in = component<T, Desc, cmpt::ZouHeVelocityX<true>>::from_profile();
	component<T, Desc, cmpt::ZouHePressureX<false>> flow_out{1.0};

	step_program prog{reference};
	prog.on(1, bb).fluid(2, collision).on(3, flow_in, collision).on(4, flow_out, collision);

	for (auto r : {lat.copy_flags_to_device(info), lat.upload_inlet_profile(ux), lat.step(prog, steps)}) {
		if (r.is_error()) {
			std::fprintf(stderr, "error: %s\n", r.get_error().message.c_str());
			return 1;
		}
	}
	std::vector<float> rho, vel;
	auto r = lat.copy_macros_to_host(rho, vel);
	if (r.is_error()) {
		std::fprintf(stderr, "download: %s\n", r.get_error().message.c_str());
		return 1;
	}
	FILE *f = std::fopen(argv[4], "wb");
	std::fwrite(rho.data(), sizeof(float), rho.size(), f);
	std::fwrite(vel.data(), sizeof(float), vel.size(), f);
	std::fclose(f);
	std::printf("ok %lld cells %llu steps t=%llu\n", (long long)lat.cells(), (unsigned long long)steps,
				(unsigned long long)lat.time_step());
	return 0;
}
