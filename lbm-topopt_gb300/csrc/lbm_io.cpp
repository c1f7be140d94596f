// lbm_io.cpp -- the file formats the reference's applications read and write
// around the solver, on the host:
//
//   PETSc binary vectors  core/binaryIO.cc:3-33 (writeVectorToBinary /
//                         loadVectorFromBinary through PetscViewerBinary): a
//                         big-endian int32 class id 1211214, a big-endian int32
//                         length, then big-endian IEEE doubles (PETSc's published
//                         Vec file layout with 32-bit indices and real scalars).
//   VTK structured grids  latticeBoltzmann/LBSolver.cc:251-286 (outputMacros /
//                         outputFields through PetscViewerVTK): an XML
//                         StructuredGrid (.vts) with one point per lattice cell and
//                         the fields as Float64 point data, inline base64
//                         binary, UInt64 headers, little-endian.
//
// Byte order is written explicitly, so files are the same on any host.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbmgpu.h"
#include "lbm_ops.h"

namespace {

constexpr int32_t kVecClassId = 1211214;

int io_fail(int code, const std::string& msg) {
  lbm::set_global_error(msg.c_str());
  return code;
}

void put_be32(std::vector<unsigned char>& b, uint32_t v) {
  for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
}
void put_be64(std::vector<unsigned char>& b, uint64_t v) {
  for (int s = 56; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
}
void put_le64(std::vector<unsigned char>& b, uint64_t v) {
  for (int s = 0; s < 64; s += 8) b.push_back((unsigned char)(v >> s));
}
uint64_t bits_of(double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
}

std::string base64(const std::vector<unsigned char>& in) {
  static const char* tab = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
  std::string out;
  out.reserve((in.size() + 2) / 3 * 4);
  size_t i = 0;
  for (; i + 2 < in.size(); i += 3) {
    const uint32_t v = (uint32_t)in[i] << 16 | (uint32_t)in[i + 1] << 8 | in[i + 2];
    out += tab[v >> 18 & 63];
    out += tab[v >> 12 & 63];
    out += tab[v >> 6 & 63];
    out += tab[v & 63];
  }
  if (i + 1 == in.size()) {
    const uint32_t v = (uint32_t)in[i] << 16;
    out += tab[v >> 18 & 63];
    out += tab[v >> 12 & 63];
    out += "==";
  } else if (i + 2 == in.size()) {
    const uint32_t v = (uint32_t)in[i] << 16 | (uint32_t)in[i + 1] << 8;
    out += tab[v >> 18 & 63];
    out += tab[v >> 12 & 63];
    out += tab[v >> 6 & 63];
    out += '=';
  }
  return out;
}

// one DataArray: base64 of (UInt64 byte count, little-endian doubles)
void data_array(FILE* f, const char* name, int ncomp, const std::vector<double>& v) {
  std::vector<unsigned char> raw;
  raw.reserve(8 + v.size() * 8);
  put_le64(raw, (uint64_t)v.size() * 8);
  for (double d : v) put_le64(raw, bits_of(d));
  fprintf(f, "        <DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"%d\" format=\"binary\">\n",
          name, ncomp);
  std::string s = base64(raw);
  fwrite(s.data(), 1, s.size(), f);
  fprintf(f, "\n        </DataArray>\n");
}

}  // namespace

extern "C" {

int lbm_write_petsc_vec(const char* path, const double* v, int64_t n) {
  if (!path || (!v && n > 0) || n < 0) return io_fail(LBM_ERR_ARG, "null argument or negative length");
  if (n > INT32_MAX) return io_fail(LBM_ERR_ARG, "vector longer than a 32-bit PETSc index");
  std::vector<unsigned char> b;
  b.reserve(8 + (size_t)n * 8);
  put_be32(b, (uint32_t)kVecClassId);
  put_be32(b, (uint32_t)n);
  for (int64_t i = 0; i < n; ++i) put_be64(b, bits_of(v[i]));
  FILE* f = fopen(path, "wb");
  if (!f) return io_fail(LBM_ERR_ARG, std::string("cannot open ") + path);
  const size_t w = fwrite(b.data(), 1, b.size(), f);
  const int c = fclose(f);
  if (w != b.size() || c != 0) return io_fail(LBM_ERR_ARG, std::string("write failed: ") + path);
  return LBM_OK;
}

int lbm_read_petsc_vec(const char* path, double* v, int64_t n_max, int64_t* n) {
  if (!path || !n) return io_fail(LBM_ERR_ARG, "null argument");
  FILE* f = fopen(path, "rb");
  if (!f) return io_fail(LBM_ERR_ARG, std::string("cannot open ") + path);
  unsigned char h[8];
  if (fread(h, 1, 8, f) != 8) {
    fclose(f);
    return io_fail(LBM_ERR_ARG, "file too short for a PETSc Vec header");
  }
  const uint32_t id = (uint32_t)h[0] << 24 | (uint32_t)h[1] << 16 | (uint32_t)h[2] << 8 | h[3];
  const uint32_t len = (uint32_t)h[4] << 24 | (uint32_t)h[5] << 16 | (uint32_t)h[6] << 8 | h[7];
  if (id != (uint32_t)kVecClassId) {
    fclose(f);
    return io_fail(LBM_ERR_ARG, "not a PETSc Vec file (class id)");
  }
  *n = (int64_t)(int32_t)len;
  if (*n < 0) {
    fclose(f);
    return io_fail(LBM_ERR_ARG, "negative Vec length");
  }
  if (!v) {   // length query
    fclose(f);
    return LBM_OK;
  }
  if (*n > n_max) {
    fclose(f);
    return io_fail(LBM_ERR_ARG, "Vec has " + std::to_string(*n) + " entries, room for " + std::to_string(n_max));
  }
  std::vector<unsigned char> raw((size_t)*n * 8);
  const size_t r = fread(raw.data(), 1, raw.size(), f);
  fclose(f);
  if (r != raw.size()) return io_fail(LBM_ERR_ARG, "file shorter than its Vec length");
  for (int64_t i = 0; i < *n; ++i) {
    uint64_t u = 0;
    for (int k = 0; k < 8; ++k) u = u << 8 | raw[(size_t)i * 8 + k];
    memcpy(&v[i], &u, 8);
  }
  return LBM_OK;
}

int lbm_write_vts_fields(const char* path, int nx, int ny, int nz, int nfields,
                         const char* const* names, const int* ncomp, const double* const* data) {
  if (!path || nx < 1 || ny < 1 || nz < 1 || nfields < 0 || (nfields > 0 && (!names || !ncomp || !data)))
    return io_fail(LBM_ERR_ARG, "bad arguments");
  for (int k = 0; k < nfields; ++k)
    if (!names[k] || !data[k] || ncomp[k] < 1 || ncomp[k] > 9)
      return io_fail(LBM_ERR_ARG, "bad field " + std::to_string(k));
  FILE* f = fopen(path, "wb");
  if (!f) return io_fail(LBM_ERR_ARG, std::string("cannot open ") + path);
  const long long n = (long long)nx * ny * nz;
  fprintf(f, "<?xml version=\"1.0\"?>\n");
  fprintf(f, "<VTKFile type=\"StructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n");
  fprintf(f, "  <StructuredGrid WholeExtent=\"0 %d 0 %d 0 %d\">\n", nx - 1, ny - 1, nz - 1);
  fprintf(f, "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n", nx - 1, ny - 1, nz - 1);
  fprintf(f, "      <PointData>\n");
  for (int k = 0; k < nfields; ++k) {
    std::vector<double> v(data[k], data[k] + (size_t)n * ncomp[k]);
    data_array(f, names[k], ncomp[k], v);
  }
  fprintf(f, "      </PointData>\n      <Points>\n");
  std::vector<double> pts((size_t)n * 3);
  for (long long c = 0; c < n; ++c) {
    pts[3 * c] = (double)(c % nx);
    pts[3 * c + 1] = (double)((c / nx) % ny);
    pts[3 * c + 2] = (double)(c / ((long long)nx * ny));
  }
  data_array(f, "Points", 3, pts);
  fprintf(f, "      </Points>\n    </Piece>\n  </StructuredGrid>\n</VTKFile>\n");
  if (fclose(f) != 0) return io_fail(LBM_ERR_ARG, std::string("write failed: ") + path);
  return LBM_OK;
}

int lbm_write_vts(lbm_handle* h, const char* path, const double* gamma) {
  if (!h || !path) return io_fail(LBM_ERR_ARG, "null argument");
  int64_t ncell = 0;
  int npop = 0;
  int rc = lbm_get_sizes(h, &ncell, &npop);
  if (rc) return rc;
  const bool thermal = npop == 14, d3 = npop == 19;
  const int nmac = d3 || thermal ? 4 : 3;
  std::vector<double> mac((size_t)ncell * nmac);
  if ((rc = lbm_get_macros(h, mac.data()))) return rc;
  int dims[3];
  if ((rc = lbm_get_dims(h, dims))) return rc;
  std::vector<double> rho((size_t)ncell), vel((size_t)ncell * 3, 0.), T;
  for (int64_t c = 0; c < ncell; ++c) {
    rho[c] = mac[c * nmac];
    vel[3 * c] = mac[c * nmac + 1];
    vel[3 * c + 1] = mac[c * nmac + 2];
    if (d3) vel[3 * c + 2] = mac[c * nmac + 3];
  }
  std::vector<const char*> names = {"rho", "velocity"};
  std::vector<int> comps = {1, 3};
  std::vector<const double*> ptrs = {rho.data(), vel.data()};
  if (thermal) {
    T.resize((size_t)ncell);
    for (int64_t c = 0; c < ncell; ++c) T[c] = mac[c * nmac + 3];
    names.push_back("T");
    comps.push_back(1);
    ptrs.push_back(T.data());
  }
  if (gamma) {
    names.push_back("gamma");
    comps.push_back(1);
    ptrs.push_back(gamma);
  }
  return lbm_write_vts_fields(path, dims[0], dims[1], dims[2], (int)names.size(), names.data(),
                              comps.data(), ptrs.data());
}

}  // extern "C"
