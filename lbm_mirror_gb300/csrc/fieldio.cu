// Field output and checkpoints (C ABI kel_write_vtk / kel_write_csv /
// kel_write_forst / kel_read_forst and the lattice conveniences
// kel_lattice_write_fields / kel_lattice_save / kel_lattice_load).
//
// Host code only: the writers take host arrays (cells x fastest), so they run
// without a GPU; the lattice conveniences download through the lattice's own
// C ABI first.  Formats follow the reference byte for byte:
//   - ASCII VTK STRUCTURED_POINTS as modules/core/c++/write_vtk.hpp:150-255
//     writes a Struct of Chunks: fixed header, DIMENSIONS padded to 3 with 1,
//     POINT_DATA, then per member "SCALARS <key> float 1" + "LOOKUP_TABLE
//     default" or "VECTORS <key> float", one cell per line (vector components
//     space separated, padded to 3 with " 0"), a blank line after each member;
//   - CSV as modules/core/c++/write_csv.hpp:117-184: one file per member,
//     <out_dir>/csv/<name>_<key>_<t>.csv, one cell per line, components comma
//     separated;
//   - numbers as the reference's std::ostream prints them (6 significant
//     digits, %g), uint8 as an integer;
//   - Forst (modules/core/c++/abstract/forst.hpp:17-50, forst_chunk.hpp): a
//     Struct of fixed-size members is the members' packed little-endian bytes
//     in order, no framing; a Chunk covers its ghost-widened extents
//     (Sides + 2 Ghost), x fastest, the ghost ring holding zeros.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <filesystem>
#include <string>
#include <thread>
#include <vector>

#include "lattice_internal.cuh"

using namespace kel::gb;

namespace {

size_t elem_size(int32_t type) {
	switch (type) {
	case KEL_VALUE_U8: return 1;
	case KEL_VALUE_F32: return 4;
	case KEL_VALUE_F64: return 8;
	default: return 0;
	}
}

int check_fields(const int64_t *dims, int32_t n_dims, const kel_field_view *fields, int32_t n_fields,
				 const char *who) {
	if (!dims || n_dims < 1 || n_dims > 3 || !fields || n_fields < 1)
		return fail(KEL_ERR_INVALID_ARGUMENT, "%s: bad dimensions or field list", who);
	for (int d = 0; d < n_dims; ++d)
		if (dims[d] < 1) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: dimension %d is %lld", who, d, (long long)dims[d]);
	for (int k = 0; k < n_fields; ++k) {
		const kel_field_view &f = fields[k];
		if (!f.name || !f.data || elem_size(f.value_type) == 0 || f.components < 1 || f.ghost < 0)
			return fail(KEL_ERR_INVALID_ARGUMENT, "%s: field %d is malformed", who, k);
	}
	return KEL_OK;
}

int64_t cell_count(const int64_t *dims, int32_t n_dims) {
	int64_t n = 1;
	for (int d = 0; d < n_dims; ++d) n *= dims[d];
	return n;
}

// one value as the reference's ostream prints it
void put_value(std::string &s, int32_t type, const void *base, int64_t idx) {
	char buf[40];
	int len = 0;
	switch (type) {
	case KEL_VALUE_U8: len = std::snprintf(buf, sizeof(buf), "%u", (unsigned)static_cast<const uint8_t *>(base)[idx]); break;
	case KEL_VALUE_F32: len = std::snprintf(buf, sizeof(buf), "%g", (double)static_cast<const float *>(base)[idx]); break;
	default: len = std::snprintf(buf, sizeof(buf), "%g", static_cast<const double *>(base)[idx]); break;
	}
	s.append(buf, (size_t)len);
}

// Lines for cells [c0, c1) of one field: components separated by `sep`,
// padded with " 0" up to `pad_to` components (VTK vectors), '\n' per cell.
void format_cells(std::string &out, const kel_field_view &f, int64_t c0, int64_t c1, char sep, int pad_to) {
	out.reserve((size_t)(c1 - c0) * (size_t)f.components * 12);
	for (int64_t c = c0; c < c1; ++c) {
		for (int k = 0; k < f.components; ++k) {
			if (k) out.push_back(sep);
			put_value(out, f.value_type, f.data, c * f.components + k);
		}
		for (int k = f.components; k < pad_to; ++k) out.append(" 0");
		out.push_back('\n');
	}
}

// Format all cells of a field on the host threads, write in order.
bool write_cells(std::FILE *fp, const kel_field_view &f, int64_t n, char sep, int pad_to) {
	const int64_t per = 1 << 18;
	const int64_t parts = (n + per - 1) / per;
	unsigned hw = std::thread::hardware_concurrency();
	const int64_t workers = parts < (int64_t)(hw ? hw : 1) ? parts : (int64_t)(hw ? hw : 1);
	std::vector<std::string> text((size_t)parts);
	auto job = [&](int64_t w) {
		for (int64_t p = w; p < parts; p += workers) {
			const int64_t c0 = p * per, c1 = c0 + per < n ? c0 + per : n;
			format_cells(text[(size_t)p], f, c0, c1, sep, pad_to);
		}
	};
	if (workers <= 1) {
		job(0);
	} else {
		std::vector<std::thread> th;
		for (int64_t w = 0; w < workers; ++w) th.emplace_back(job, w);
		for (auto &t : th) t.join();
	}
	for (auto &s : text)
		if (std::fwrite(s.data(), 1, s.size(), fp) != s.size()) return false;
	return true;
}

int make_dir(const std::string &dir, const char *who) {
	std::error_code ec;
	std::filesystem::create_directories(dir, ec);
	if (ec) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: could not create %s: %s", who, dir.c_str(), ec.message().c_str());
	return KEL_OK;
}

} // namespace

extern "C" int kel_write_vtk(const char *out_dir, const char *file_name, uint64_t t, const int64_t *dims,
							 int32_t n_dims, const kel_field_view *fields, int32_t n_fields) {
	int rc = check_fields(dims, n_dims, fields, n_fields, "kel_write_vtk");
	if (rc) return rc;
	if (!out_dir || !file_name) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_write_vtk: null path");
	const std::string dir = std::string(out_dir) + "/vtk";
	if ((rc = make_dir(dir, "kel_write_vtk"))) return rc;
	const std::string path = dir + "/" + file_name + "_" + std::to_string(t) + ".vtk";
	std::FILE *fp = std::fopen(path.c_str(), "wb");
	if (!fp) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_write_vtk: could not open %s", path.c_str());
	const int64_t n = cell_count(dims, n_dims);
	std::string head = "# vtk DataFile Version 3.0\nLBM File\nASCII\nDATASET STRUCTURED_POINTS\n"
					   "SPACING 1.0 1.0 1.0\nORIGIN 0.0 0.0 0.0\nDIMENSIONS";
	for (int d = 0; d < 3; ++d) head += " " + std::to_string(d < n_dims ? dims[d] : 1);
	head += "\n\nPOINT_DATA " + std::to_string(n) + "\n\n";
	bool ok = std::fwrite(head.data(), 1, head.size(), fp) == head.size();
	for (int k = 0; k < n_fields && ok; ++k) {
		const kel_field_view &f = fields[k];
		const bool vec = f.components > 1 || f.vector;
		std::string h = vec ? std::string("VECTORS ") + f.name + " float\n"
							: std::string("SCALARS ") + f.name + " float 1\nLOOKUP_TABLE default\n";
		ok = std::fwrite(h.data(), 1, h.size(), fp) == h.size();
		ok = ok && write_cells(fp, f, n, ' ', vec ? 3 : 1);
		ok = ok && std::fputc('\n', fp) != EOF;
	}
	ok = (std::fclose(fp) == 0) && ok;
	if (!ok) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_write_vtk: write to %s failed", path.c_str());
	return KEL_OK;
}

extern "C" int kel_write_csv(const char *out_dir, const char *file_name, uint64_t t, const int64_t *dims,
							 int32_t n_dims, const kel_field_view *fields, int32_t n_fields) {
	int rc = check_fields(dims, n_dims, fields, n_fields, "kel_write_csv");
	if (rc) return rc;
	if (!out_dir || !file_name) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_write_csv: null path");
	const std::string dir = std::string(out_dir) + "/csv";
	if ((rc = make_dir(dir, "kel_write_csv"))) return rc;
	const int64_t n = cell_count(dims, n_dims);
	for (int k = 0; k < n_fields; ++k) {
		const kel_field_view &f = fields[k];
		const std::string path = dir + "/" + file_name + "_" + f.name + "_" + std::to_string(t) + ".csv";
		std::FILE *fp = std::fopen(path.c_str(), "wb");
		if (!fp) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_write_csv: could not open %s", path.c_str());
		bool ok = write_cells(fp, f, n, ',', 0);
		ok = (std::fclose(fp) == 0) && ok;
		if (!ok) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_write_csv: write to %s failed", path.c_str());
	}
	return KEL_OK;
}

namespace {

// bytes of one member in the Forst encoding: ghost-widened extents x components
int64_t forst_member_bytes(const int64_t *dims, int32_t n_dims, const kel_field_view &f) {
	int64_t cells = 1;
	for (int d = 0; d < n_dims; ++d) cells *= dims[d] + 2 * f.ghost;
	return cells * f.components * (int64_t)elem_size(f.value_type);
}

// interior cell c (x fastest over dims) -> its index in the ghost-widened extents
int64_t widened_index(int64_t c, const int64_t *dims, int32_t n_dims, int g) {
	int64_t idx = 0, stride = 1;
	for (int d = 0; d < n_dims; ++d) {
		const int64_t x = c % dims[d];
		c /= dims[d];
		idx += (x + g) * stride;
		stride *= dims[d] + 2 * g;
	}
	return idx;
}

bool forst_put(std::FILE *fp, const int64_t *dims, int32_t n_dims, const kel_field_view *fields, int32_t n_fields) {
	const int64_t n = cell_count(dims, n_dims);
	for (int k = 0; k < n_fields; ++k) {
		const kel_field_view &f = fields[k];
		const size_t es = elem_size(f.value_type) * (size_t)f.components;
		if (f.ghost == 0) {
			if (std::fwrite(f.data, es, (size_t)n, fp) != (size_t)n) return false;
			continue;
		}
		std::vector<uint8_t> buf((size_t)forst_member_bytes(dims, n_dims, f), 0);
		for (int64_t c = 0; c < n; ++c)
			std::memcpy(buf.data() + (size_t)widened_index(c, dims, n_dims, f.ghost) * es,
						static_cast<const uint8_t *>(f.data) + (size_t)c * es, es);
		if (std::fwrite(buf.data(), 1, buf.size(), fp) != buf.size()) return false;
	}
	return true;
}

bool forst_get(std::FILE *fp, const int64_t *dims, int32_t n_dims, const kel_field_view *fields, int32_t n_fields) {
	const int64_t n = cell_count(dims, n_dims);
	for (int k = 0; k < n_fields; ++k) {
		const kel_field_view &f = fields[k];
		const size_t es = elem_size(f.value_type) * (size_t)f.components;
		std::vector<uint8_t> buf((size_t)forst_member_bytes(dims, n_dims, f));
		if (std::fread(buf.data(), 1, buf.size(), fp) != buf.size()) return false;
		uint8_t *dst = static_cast<uint8_t *>(const_cast<void *>(f.data));
		for (int64_t c = 0; c < n; ++c)
			std::memcpy(dst + (size_t)c * es, buf.data() + (size_t)widened_index(c, dims, n_dims, f.ghost) * es, es);
	}
	return true;
}

int open_for_write(const char *path, const char *who, std::FILE **fp) {
	const std::filesystem::path p(path);
	int rc;
	if (p.has_parent_path() && (rc = make_dir(p.parent_path().string(), who))) return rc;
	*fp = std::fopen(path, "wb");
	if (!*fp) return fail(KEL_ERR_INVALID_ARGUMENT, "%s: could not open %s", who, path);
	return KEL_OK;
}

} // namespace

extern "C" int kel_write_forst(const char *path, const int64_t *dims, int32_t n_dims, const kel_field_view *fields,
							   int32_t n_fields) {
	int rc = check_fields(dims, n_dims, fields, n_fields, "kel_write_forst");
	if (rc) return rc;
	if (!path) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_write_forst: null path");
	std::FILE *fp = nullptr;
	if ((rc = open_for_write(path, "kel_write_forst", &fp))) return rc;
	bool ok = forst_put(fp, dims, n_dims, fields, n_fields);
	ok = (std::fclose(fp) == 0) && ok;
	if (!ok) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_write_forst: write to %s failed", path);
	return KEL_OK;
}

extern "C" int kel_read_forst(const char *path, const int64_t *dims, int32_t n_dims, kel_field_view *fields,
							  int32_t n_fields) {
	int rc = check_fields(dims, n_dims, fields, n_fields, "kel_read_forst");
	if (rc) return rc;
	if (!path) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_read_forst: null path");
	std::error_code ec;
	const auto size = std::filesystem::file_size(path, ec);
	if (ec) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_read_forst: %s: %s", path, ec.message().c_str());
	int64_t want = 0;
	for (int k = 0; k < n_fields; ++k) want += forst_member_bytes(dims, n_dims, fields[k]);
	if ((int64_t)size != want)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_read_forst: %s holds %llu bytes, the layout needs %lld", path,
					(unsigned long long)size, (long long)want);
	std::FILE *fp = std::fopen(path, "rb");
	if (!fp) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_read_forst: could not open %s", path);
	const bool ok = forst_get(fp, dims, n_dims, fields, n_fields);
	std::fclose(fp);
	if (!ok) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_read_forst: short read from %s", path);
	return KEL_OK;
}

// ---------------------------------------------------------------------------
// lattice conveniences

namespace {

int32_t lattice_dims(const kel_lattice *L, int64_t *dims) {
	const auto &d = L->desc;
	dims[0] = d.nx;
	dims[1] = d.ny;
	dims[2] = d.nz;
	return d.descriptor == KEL_D2Q9 ? 2 : 3;
}

kel_field_view view(const char *name, int32_t type, int32_t comps, int32_t ghost, int32_t vector, const void *data) {
	kel_field_view f;
	memset(&f, 0, sizeof(f));
	f.name = name;
	f.value_type = type;
	f.components = comps;
	f.ghost = ghost;
	f.vector = vector;
	f.data = data;
	return f;
}

} // namespace

extern "C" int kel_lattice_write_fields(kel_lattice *L, int32_t formats, const char *out_dir, const char *file_name,
										uint64_t t) {
	if (!L || !out_dir || !file_name || !(formats & (KEL_WRITE_VTK | KEL_WRITE_CSV | KEL_WRITE_FORST)))
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_write_fields: bad arguments");
	int64_t dims[3];
	const int32_t nd = lattice_dims(L, dims);
	const int64_t n = L->ncell;
	std::vector<float> rho((size_t)n), u((size_t)n * L->d.D);
	int rc = kel_download_macros(L, rho.data(), u.data());
	if (rc) return rc;
	// the drivers' MacroStruct member order: velocity, then density
	const kel_field_view f[2] = {view("velocity", KEL_VALUE_F32, L->d.D, 0, 1, u.data()),
								 view("density", KEL_VALUE_F32, 1, 0, 0, rho.data())};
	if ((formats & KEL_WRITE_VTK) && (rc = kel_write_vtk(out_dir, file_name, t, dims, nd, f, 2))) return rc;
	if ((formats & KEL_WRITE_CSV) && (rc = kel_write_csv(out_dir, file_name, t, dims, nd, f, 2))) return rc;
	if (formats & KEL_WRITE_FORST) {
		const std::string p = std::string(out_dir) + "/forst/" + file_name + "_" + std::to_string(t) + ".forst";
		if ((rc = kel_write_forst(p.c_str(), dims, nd, f, 2))) return rc;
	}
	return KEL_OK;
}

// Checkpoint: the Forst encoding of {time_step: UInt64, info: Chunk<UInt8, 0>,
// dfs: Chunk<FixedArray<Float32, Q>, 1>}, dfs holding the populations f_i(x)
// of the lattice's current time step (what the reference keeps in dfs_old at
// even and in dfs at odd time steps).
extern "C" int kel_lattice_save(kel_lattice *L, const char *path) {
	if (!L || !path) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_save: null argument");
	int64_t dims[3];
	const int32_t nd = lattice_dims(L, dims);
	const int64_t n = L->ncell;
	std::vector<float> pops((size_t)n * L->d.Q);
	int rc = kel_download_populations(L, pops.data(), KEL_DTYPE_F32, KEL_LAYOUT_AOS);
	if (rc) return rc;
	std::vector<uint8_t> flags((size_t)n);
	KEL_CUDA(cudaMemcpy2DAsync(flags.data(), (size_t)dims[0], L->flags, (size_t)L->nxp, (size_t)dims[0],
							   (size_t)(n / dims[0]), cudaMemcpyDeviceToHost, L->stream));
	KEL_CUDA(cudaStreamSynchronize(L->stream));
	const uint64_t t = L->t;
	const kel_field_view f[2] = {view("info", KEL_VALUE_U8, 1, 0, 0, flags.data()),
								 view("dfs", KEL_VALUE_F32, L->d.Q, 1, 0, pops.data())};
	std::FILE *fp = nullptr;
	if ((rc = open_for_write(path, "kel_lattice_save", &fp))) return rc;
	bool ok = std::fwrite(&t, sizeof(t), 1, fp) == 1 && forst_put(fp, dims, nd, f, 2);
	ok = (std::fclose(fp) == 0) && ok;
	if (!ok) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_save: write to %s failed", path);
	return KEL_OK;
}

// Restores flags, populations and the time step written by kel_lattice_save
// into a lattice of the same descriptor and extents; the run continues with
// the same bits as if it had not stopped.
extern "C" int kel_lattice_load(kel_lattice *L, const char *path) {
	if (!L || !path) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_load: null argument");
	int64_t dims[3];
	const int32_t nd = lattice_dims(L, dims);
	const int64_t n = L->ncell;
	std::vector<float> pops((size_t)n * L->d.Q);
	std::vector<uint8_t> flags((size_t)n);
	const kel_field_view f[2] = {view("info", KEL_VALUE_U8, 1, 0, 0, flags.data()),
								 view("dfs", KEL_VALUE_F32, L->d.Q, 1, 0, pops.data())};
	std::error_code ec;
	const auto size = std::filesystem::file_size(path, ec);
	if (ec) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_load: %s: %s", path, ec.message().c_str());
	const int64_t want = 8 + forst_member_bytes(dims, nd, f[0]) + forst_member_bytes(dims, nd, f[1]);
	if ((int64_t)size != want)
		return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_load: %s holds %llu bytes, this lattice needs %lld", path,
					(unsigned long long)size, (long long)want);
	std::FILE *fp = std::fopen(path, "rb");
	if (!fp) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_load: could not open %s", path);
	uint64_t t = 0;
	const bool ok = std::fread(&t, sizeof(t), 1, fp) == 1 && forst_get(fp, dims, nd, f, 2);
	std::fclose(fp);
	if (!ok) return fail(KEL_ERR_INVALID_ARGUMENT, "kel_lattice_load: short read from %s", path);
	int rc = kel_upload_flags(L, flags.data());
	if (rc) return rc;
	L->t = t; // uploads place f_i(x) according to the time step's parity
	return kel_upload_populations(L, pops.data(), KEL_DTYPE_F32, KEL_LAYOUT_AOS);
}
