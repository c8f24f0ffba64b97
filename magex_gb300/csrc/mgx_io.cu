// Spin and table outputs at scale (host code): the text writers of magex/observables.py:122-161
// (extended XYZ, VTK legacy polydata, OVF 2.0 irregular mesh) and magex/llg.py:286-297 (run table and
// the CSV half of save_spins), byte-for-byte the same text as magex's Python / numpy.savetxt writers.
// magex formats line by line in Python (about a microsecond per value); here rows are formatted in
// parallel chunks with the C library's correctly rounded printf conversions and written in order.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx {

// printf-style append of one conversion to s (any length)
static void appendf(std::string& s, const char* fmt, ...) {
  char buf[128];
  va_list ap;
  va_start(ap, fmt);
  va_list ap2;
  va_copy(ap2, ap);
  const int len = vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (len < 0) {
    va_end(ap2);
    return;
  }
  if ((size_t)len < sizeof(buf)) {
    s.append(buf, (size_t)len);
  } else {
    std::vector<char> big((size_t)len + 1);
    vsnprintf(big.data(), big.size(), fmt, ap2);
    s.append(big.data(), (size_t)len);
  }
  va_end(ap2);
}

// Format rows [0, n) with fmt_row(i, s) appending text to s, in parallel chunks, and write to f.
template <class Row>
static bool write_rows(FILE* f, int64_t n, Row fmt_row) {
  if (n <= 0) return true;
  const int64_t chunk = 1 << 16;
  const int64_t nchunks = (n + chunk - 1) / chunk;
  unsigned hw = std::thread::hardware_concurrency();
  const int nthreads = (int)std::max<int64_t>(1, std::min<int64_t>(nchunks, hw ? hw : 4));
  for (int64_t base = 0; base < nchunks; base += nthreads) {
    const int64_t batch = std::min<int64_t>(nthreads, nchunks - base);
    std::vector<std::string> out((size_t)batch);
    std::vector<std::thread> pool;
    for (int64_t t = 0; t < batch; ++t) {
      pool.emplace_back([&, t] {
        const int64_t lo = (base + t) * chunk, hi = std::min(n, lo + chunk);
        std::string& s = out[(size_t)t];
        s.reserve((size_t)(hi - lo) * 64);
        for (int64_t i = lo; i < hi; ++i) fmt_row(i, s);
      });
    }
    for (auto& th : pool) th.join();
    for (auto& s : out)
      if (fwrite(s.data(), 1, s.size(), f) != s.size()) return false;
  }
  return true;
}

// numpy.savetxt row: values formatted with fmt joined by delim, newline
static void fmt_values(std::string& s, const char* fmt, const char* delim, const double* v, int k) {
  for (int c = 0; c < k; ++c) {
    if (c) s.append(delim);
    appendf(s, fmt, v[c]);
  }
  s.push_back('\n');
}

static mgx_status open_out(const char* path, const char* mode, FILE** f) {
  if (!path) return set_error(MGX_ERR_INVALID, "output path is NULL");
  *f = fopen(path, mode);
  if (!*f) return set_error(MGX_ERR_INVALID, "cannot open %s for writing", path);
  return MGX_OK;
}

static mgx_status close_out(FILE* f, bool ok, const char* path) {
  const bool closed = fclose(f) == 0;
  if (!ok || !closed) return set_error(MGX_ERR_INVALID, "write to %s failed", path);
  return MGX_OK;
}

}  // namespace mgx

using namespace mgx;

extern "C" mgx_status mgx_write_xyz(const char* path, int64_t n, const double* pos, const double* spins,
                                    const double* mu, const int32_t* sublattice, const char* const* names,
                                    int32_t nnames, const char* comment, int32_t append) {
  if (n < 0 || (n > 0 && (!pos || !spins || !mu || !sublattice || !names)) || nnames < 1)
    return set_error(MGX_ERR_INVALID, "mgx_write_xyz: bad argument");
  for (int64_t i = 0; i < n; ++i)
    if (sublattice[i] < 0 || sublattice[i] >= nnames)
      return set_error(MGX_ERR_INVALID, "mgx_write_xyz: sublattice of site %lld out of range", (long long)i);
  FILE* f;
  mgx_status st = open_out(path, append ? "ab" : "wb", &f);
  if (st != MGX_OK) return st;
  bool ok = fprintf(f, "%lld\nProperties=species:S:1:pos:R:3:spin:R:3:mu:R:1 %s\n", (long long)n,
                    comment ? comment : "") > 0;
  ok = ok && write_rows(f, n, [&](int64_t i, std::string& out) {
         const double* p = pos + 3 * i;
         const double* v = spins + 3 * i;
         out.append(names[sublattice[i]]);
         appendf(out, " %.5f %.5f %.5f %.6f %.6f %.6f %.4f\n", p[0], p[1], p[2], v[0], v[1], v[2], mu[i]);
       });
  return close_out(f, ok, path);
}

extern "C" mgx_status mgx_write_vtk(const char* path, int64_t n, const double* pos, const double* spins,
                                    const double* scalars, const char* const* scalar_names, int32_t nscalars) {
  if (n < 0 || (n > 0 && (!pos || !spins)) || nscalars < 0 || (nscalars > 0 && (!scalars || !scalar_names)))
    return set_error(MGX_ERR_INVALID, "mgx_write_vtk: bad argument");
  FILE* f;
  mgx_status st = open_out(path, "wb", &f);
  if (st != MGX_OK) return st;
  bool ok = fprintf(f, "# vtk DataFile Version 3.0\nmagex spins\nASCII\nDATASET POLYDATA\nPOINTS %lld double\n",
                    (long long)n) > 0;
  ok = ok && write_rows(f, n, [&](int64_t i, std::string& out) { fmt_values(out, "%.6f", " ", pos + 3 * i, 3); });
  ok = ok && fprintf(f, "VERTICES %lld %lld\n", (long long)n, 2LL * n) > 0;
  ok = ok && write_rows(f, n, [&](int64_t i, std::string& out) { appendf(out, "1 %lld\n", (long long)i); });
  ok = ok && fprintf(f, "POINT_DATA %lld\nVECTORS spin double\n", (long long)n) > 0;
  ok = ok && write_rows(f, n, [&](int64_t i, std::string& out) { fmt_values(out, "%.6f", " ", spins + 3 * i, 3); });
  for (int k = 0; k < nscalars && ok; ++k) {
    ok = fprintf(f, "SCALARS %s double 1\nLOOKUP_TABLE default\n", scalar_names[k]) > 0;
    const double* a = scalars + (int64_t)k * n;
    ok = ok && write_rows(f, n, [&](int64_t i, std::string& out) { fmt_values(out, "%.6g", " ", a + i, 1); });
  }
  return close_out(f, ok, path);
}

extern "C" mgx_status mgx_write_ovf(const char* path, int64_t n, const double* pos, const double* spins) {
  if (n < 0 || (n > 0 && (!pos || !spins))) return set_error(MGX_ERR_INVALID, "mgx_write_ovf: bad argument");
  FILE* f;
  mgx_status st = open_out(path, "wb", &f);
  if (st != MGX_OK) return st;
  bool ok = fprintf(f, "# OOMMF OVF 2.0\n# Segment count: 1\n# Begin: Segment\n# Begin: Header\n# Title: magex\n"
                       "# meshtype: irregular\n# meshunit: m\n# valuedim: 3\n# valueunits: 1 1 1\n"
                       "# pointcount: %lld\n# End: Header\n# Begin: Data Text\n", (long long)n) > 0;
  ok = ok && write_rows(f, n, [&](int64_t i, std::string& out) {
         const double v[6] = {pos[3 * i] * 1e-10, pos[3 * i + 1] * 1e-10, pos[3 * i + 2] * 1e-10,
                              spins[3 * i], spins[3 * i + 1], spins[3 * i + 2]};
         fmt_values(out, "%.8e", " ", v, 6);
       });
  ok = ok && fprintf(f, "# End: Data Text\n# End: Segment\n") > 0;
  return close_out(f, ok, path);
}

extern "C" mgx_status mgx_write_csv(const char* path, int64_t nrows, int32_t ncols, const double* values,
                                    const char* fmt, const char* header) {
  if (nrows < 0 || ncols < 1 || (nrows > 0 && !values) || !fmt)
    return set_error(MGX_ERR_INVALID, "mgx_write_csv: bad argument");
  if (strcmp(fmt, "%.6f") && strcmp(fmt, "%.8g") && strcmp(fmt, "%.6g") && strcmp(fmt, "%.8e"))
    return set_error(MGX_ERR_INVALID, "mgx_write_csv: format must be one of %%.6f %%.8g %%.6g %%.8e");
  FILE* f;
  mgx_status st = open_out(path, "wb", &f);
  if (st != MGX_OK) return st;
  bool ok = true;
  if (header) ok = fprintf(f, "%s\n", header) > 0;
  ok = ok && write_rows(f, nrows, [&](int64_t i, std::string& out) {
         fmt_values(out, fmt, ",", values + (int64_t)ncols * i, ncols);
       });
  return close_out(f, ok, path);
}
