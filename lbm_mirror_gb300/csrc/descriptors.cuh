// Lattice descriptors as compile-time tables for device code.
//
// Same direction order, weights and opposite indices as keldu/lbm_mirror's
// df_info<T, Desc> (modules/core/c++/descriptor/d2q9.hpp:17-57,
// d3q19.hpp:15-67, d3q27.hpp:16-98), so that AoS uploads/downloads compare
// index for index with the reference.
#pragma once

#include <cstdint>

namespace kel {
namespace gb {

struct D2Q9 {
	static constexpr int D = 2;
	static constexpr int Q = 9;
	static constexpr int ID = 9;
	__host__ __device__ static constexpr int cx(int i) {
		constexpr int t[9] = {0, -1, 1, 0, 0, -1, 1, -1, 1};
		return t[i];
	}
	__host__ __device__ static constexpr int cy(int i) {
		constexpr int t[9] = {0, 0, 0, -1, 1, -1, 1, 1, -1};
		return t[i];
	}
	__host__ __device__ static constexpr int cz(int) { return 0; }
	__host__ __device__ static constexpr int opp(int i) {
		constexpr int t[9] = {0, 2, 1, 4, 3, 6, 5, 8, 7};
		return t[i];
	}
	__host__ __device__ static constexpr double w(int i) {
		return i == 0 ? 4. / 9. : (i < 5 ? 1. / 9. : 1. / 36.);
	}
};

struct D3Q19 {
	static constexpr int D = 3;
	static constexpr int Q = 19;
	static constexpr int ID = 19;
	__host__ __device__ static constexpr int cx(int i) {
		constexpr int t[19] = {0, -1, 1, 0, 0, 0, 0, -1, 1, -1, 1, -1, 1, -1, 1, 0, 0, 0, 0};
		return t[i];
	}
	__host__ __device__ static constexpr int cy(int i) {
		constexpr int t[19] = {0, 0, 0, -1, 1, 0, 0, -1, -1, 1, 1, 0, 0, 0, 0, -1, 1, -1, 1};
		return t[i];
	}
	__host__ __device__ static constexpr int cz(int i) {
		constexpr int t[19] = {0, 0, 0, 0, 0, -1, 1, 0, 0, 0, 0, -1, -1, 1, 1, -1, -1, 1, 1};
		return t[i];
	}
	__host__ __device__ static constexpr int opp(int i) {
		constexpr int t[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
		return t[i];
	}
	__host__ __device__ static constexpr double w(int i) {
		return i == 0 ? 1. / 3. : (i < 7 ? 1. / 18. : 1. / 36.);
	}
};

// D3Q27: i = a + 3 b + 9 g with axis offsets ordered (0, -1, +1).
struct D3Q27 {
	static constexpr int D = 3;
	static constexpr int Q = 27;
	static constexpr int ID = 27;
	__host__ __device__ static constexpr int off(int a) { return a == 0 ? 0 : (a == 1 ? -1 : 1); }
	__host__ __device__ static constexpr int cx(int i) { return off(i % 3); }
	__host__ __device__ static constexpr int cy(int i) { return off((i / 3) % 3); }
	__host__ __device__ static constexpr int cz(int i) { return off(i / 9); }
	__host__ __device__ static constexpr int flip(int a) { return a == 0 ? 0 : 3 - a; }
	__host__ __device__ static constexpr int opp(int i) {
		return flip(i % 3) + 3 * flip((i / 3) % 3) + 9 * flip(i / 9);
	}
	__host__ __device__ static constexpr double w(int i) {
		int n = (cx(i) != 0) + (cy(i) != 0) + (cz(i) != 0);
		return n == 0 ? 8. / 27. : (n == 1 ? 2. / 27. : (n == 2 ? 1. / 54. : 1. / 216.));
	}
};

template <class L>
__host__ __device__ constexpr int cdir(int i, int k) {
	return k == 0 ? L::cx(i) : (k == 1 ? L::cy(i) : L::cz(i));
}

} // namespace gb
} // namespace kel
