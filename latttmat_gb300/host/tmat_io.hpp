// Output files of the tmat driver, in the reference's formats
// (TMat/pfunc.hpp:116-200):
//   <out>_val.dat   eigenvalues / normfactor, precision 16, one per line,
//                   right-aligned to a common width (the dense-vector stream
//                   format the reference uses); complex values as (re,im)
//   <out>_vec.dat   binary: symmetric -> nconv vectors FP64 column-major;
//                   general -> complex128, or the real part only when nconv==1
//   <out>_vecl.dat  binary FP64 real part of the left vector (general only)
//   <out>_phys.dat  4 moments (precision 10, tab-separated), then on a new line
//                   the extended observables
#pragma once
#include <complex>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

namespace latttmat {

inline std::string fmt_real(double v, int prec) {
  std::ostringstream s;
  s << std::setprecision(prec) << v;
  return s.str();
}

inline std::string fmt_complex(std::complex<double> v, int prec) {
  std::ostringstream s;
  s << std::setprecision(prec) << v;
  return s.str();
}

// column-vector stream format: each coefficient right-aligned to the widest
inline std::string format_column(const std::vector<std::string>& items) {
  size_t w = 0;
  for (auto& s : items) w = std::max(w, s.size());
  std::string out;
  for (size_t i = 0; i < items.size(); ++i) {
    if (i) out += "\n";
    out += std::string(w - items[i].size(), ' ') + items[i];
  }
  return out;
}

inline void write_val(const std::string& path, const std::vector<std::complex<double>>& vals, bool symmetric) {
  std::vector<std::string> items;
  for (auto& v : vals) items.push_back(symmetric ? fmt_real(v.real(), 16) : fmt_complex(v, 16));
  std::ofstream f(path);
  f << format_column(items);
}

inline void write_vec_sym(const std::string& path, const std::vector<double>& vecs) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(vecs.data()), vecs.size() * sizeof(double));
}

// general: vecs interleaved complex (re,im), nconv columns of n
inline void write_vec_gen(const std::string& path, const std::vector<double>& vecs, int64_t n, int nconv) {
  std::ofstream f(path, std::ios::binary);
  if (nconv == 1) {
    for (int64_t i = 0; i < n; ++i) f.write(reinterpret_cast<const char*>(&vecs[2 * i]), sizeof(double));
  } else {
    f.write(reinterpret_cast<const char*>(vecs.data()), (size_t)nconv * n * 2 * sizeof(double));
  }
}

inline void write_vecl(const std::string& path, const std::vector<double>& vecl) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(vecl.data()), vecl.size() * sizeof(double));
}

inline void write_phys(const std::string& path, const double mom[4], const std::vector<double>& ext) {
  std::ofstream f(path);
  f << std::setprecision(10);
  for (int k = 0; k < 4; ++k) {
    if (k > 0) f << '\t';
    f << mom[k];
  }
  for (size_t k = 0; k < ext.size(); ++k) {
    if (k == 0)
      f << '\n';
    else
      f << '\t';
    f << ext[k];
  }
}

}  // namespace latttmat
