// Host-side output of the GB300 LBM library: the legacy-VTK ASCII writer
// (replaces the per-value Python loops of pytorch-lbm io_utils/vtk_writer.py
// with the same bytes).
//
// The caller supplies the header text (its float fields are formatted by the
// caller's language, as the reference's f-strings do); this file writes the
// point data: "%.6e" per value, one scalar or one "x y z" vector per line,
// solid flags as integers.  Values are formatted in parallel chunks and
// written in order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lbm_gb300.h"

namespace {

// "%.6e" of v as Python's format(v, '.6e') prints it: a NaN of either sign is
// "nan", infinities "inf" / "-inf".
inline void put_e6(std::string& s, double v) {
  if (std::isnan(v)) {
    s += "nan";
    return;
  }
  if (std::isinf(v)) {
    s += v < 0 ? "-inf" : "inf";
    return;
  }
  char b[32];
  const int n = std::snprintf(b, sizeof(b), "%.6e", v);
  s.append(b, (size_t)n);
}

// Formats lines [0, n) with fn(i, string&) in parallel chunks and writes them in order.
template <typename Fn>
bool write_lines(FILE* fp, int64_t n, Fn fn) {
  const int64_t chunk = 1 << 18;
  const int64_t nchunks = (n + chunk - 1) / chunk;
  unsigned hw = std::thread::hardware_concurrency();
  const int64_t nthreads = std::max<int64_t>(1, std::min<int64_t>(nchunks, hw ? hw : 4));
  for (int64_t c0 = 0; c0 < nchunks; c0 += nthreads) {
    const int64_t cn = std::min<int64_t>(nthreads, nchunks - c0);
    std::vector<std::string> out((size_t)cn);
    std::vector<std::thread> th;
    for (int64_t t = 0; t < cn; ++t) {
      th.emplace_back([&, t] {
        const int64_t a = (c0 + t) * chunk, b = std::min<int64_t>(n, a + chunk);
        std::string& s = out[(size_t)t];
        s.reserve((size_t)(b - a) * 16);
        for (int64_t i = a; i < b; ++i) fn(i, s);
      });
    }
    for (auto& x : th) x.join();
    for (const std::string& s : out)
      if (std::fwrite(s.data(), 1, s.size(), fp) != s.size()) return false;
  }
  return true;
}

}  // namespace

extern "C" int lbm_write_vtk(const char* path, const char* header, int64_t npoints, const double* rho,
                             const double* ux, const double* uy, const double* uz, const int32_t* solid) {
  if (!path || !header || !rho || !ux || !uy || !uz || npoints < 0) return LBM_E_ARG;
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return LBM_E_ARG;
  bool ok = std::fputs(header, fp) >= 0;
  ok = ok && std::fputs("SCALARS density float\nLOOKUP_TABLE default\n", fp) >= 0;
  ok = ok && write_lines(fp, npoints, [&](int64_t i, std::string& s) {
         put_e6(s, rho[i]);
         s += '\n';
       });
  ok = ok && std::fputs("VECTORS velocity float\n", fp) >= 0;
  ok = ok && write_lines(fp, npoints, [&](int64_t i, std::string& s) {
         put_e6(s, ux[i]);
         s += ' ';
         put_e6(s, uy[i]);
         s += ' ';
         put_e6(s, uz[i]);
         s += '\n';
       });
  if (solid) {
    ok = ok && std::fputs("SCALARS solid int\nLOOKUP_TABLE default\n", fp) >= 0;
    ok = ok && write_lines(fp, npoints, [&](int64_t i, std::string& s) {
           s += std::to_string(solid[i]);
           s += '\n';
         });
  }
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? LBM_OK : LBM_E_ARG;
}
