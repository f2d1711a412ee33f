// latttmat.hpp -- C++ adaptor over the C ABI with the shape of the
// reference's operator classes (TMat/tmat.hpp:82-144), so code written
// against the Spectra operator concept (rows/cols/perform_op) -- the
// reference's pfunc_inner (TMat/pfunc.hpp:79-202) included -- can use the GPU
// operators unchanged.
//
//   latttmat::GpuMatVecProd op(mpara_like, 'A', 2, 5, extend_cond);
//   Spectra::SymEigsSolver<double, Spectra::LARGEST_MAGN, latttmat::GpuMatVecProd> eigs(&op, nev, ncv);
//
// or, without Spectra, op.eigs(...) runs the GPU eigensolver directly.
#ifndef LATTTMAT_GB300_HPP
#define LATTTMAT_GB300_HPP

#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "latttmat.h"

namespace latttmat {

struct Error : std::runtime_error {
  tm_status code;
  Error(tm_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(tm_status s) {
  if (s != TM_OK) throw Error(s, tm_last_error());
}

// One GPU operator; the reference MatVecProd<S> counterpart.  Non-copyable,
// movable.  get_t_instance() returns the transpose view (the parent must
// outlive it), as the reference's *_T classes hold a reference to the parent.
class GpuMatVecProd {
 public:
  using Scalar = double;  // Spectra operator concept
  GpuMatVecProd(double betaJ, double kappa, double kappa2, double h, int size, char model, int dim, int axialdir,
                int extend_cond = 0) {
    tm_params p{betaJ, kappa, kappa2, h, size};
    check(tm_create(&p, model, dim, axialdir, extend_cond, &h_));
  }
  explicit GpuMatVecProd(tm_op* handle) : h_(handle) {}
  GpuMatVecProd(const GpuMatVecProd&) = delete;
  GpuMatVecProd& operator=(const GpuMatVecProd&) = delete;
  GpuMatVecProd(GpuMatVecProd&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  ~GpuMatVecProd() {
    if (h_) tm_destroy(h_);
  }

  // Spectra operator concept
  int64_t rows() const { return tm_rows(h_); }
  int64_t cols() const { return tm_cols(h_); }
  void perform_op(const double* x_in, double* y_out) const { check(tm_perform_op(h_, x_in, y_out)); }

  // reference MatVecProd extras
  int suggested_nev(int neig) const { return tm_suggested_ncv(h_, neig); }
  double getnormfactor() const { return tm_normfactor(h_); }
  int getLayerSize() const { return tm_layer_size(h_); }
  bool symmetric() const { return tm_is_symmetric(h_) == 1; }
  int64_t matvec_count() const { return tm_matvec_count(h_); }
  GpuMatVecProd get_t_instance() const {
    tm_op* t = nullptr;
    check(tm_transpose(h_, &t));
    return GpuMatVecProd(t);
  }
  int moments(const double* ql, const double* qr, double results[4]) const {
    int st = 0;
    check(tm_moments(h_, ql, qr, results, &st));
    return st;
  }
  int phys_extend(const double* ql, const double* qr, std::vector<double>& results) const {
    double buf[16];
    int n = 0, st = 0;
    check(tm_phys_extend(h_, ql, qr, buf, 16, &n, &st));
    results.assign(buf, buf + n);
    return st;
  }
  std::vector<std::pair<uint64_t, uint16_t>> orbit_table() const {
    int64_t n = 0;
    check(tm_orbit_table(h_, nullptr, nullptr, 0, &n));
    std::vector<uint64_t> idx(n);
    std::vector<uint16_t> dup(n);
    check(tm_orbit_table(h_, idx.data(), dup.data(), n, &n));
    std::vector<std::pair<uint64_t, uint16_t>> r(n);
    for (int64_t i = 0; i < n; ++i) r[i] = {idx[i], dup[i]};
    return r;
  }
  // GPU eigensolver (tm_eigs): eigenvalues / normfactor, descending magnitude;
  // vecs (rows x nev, column-major) for symmetric operators when wanted
  std::vector<double> eigs(int nev, double tol = 1e-10, int mode = TM_EIGS_F64, std::vector<double>* vecs = nullptr,
                           tm_eigs_info* info = nullptr) const {
    std::vector<double> re(nev), im(nev);
    if (vecs) vecs->assign((size_t)rows() * nev * (symmetric() ? 1 : 2), 0.0);
    check(tm_eigs(h_, nev, 0, tol, 0, mode, re.data(), im.data(), vecs ? vecs->data() : nullptr, nullptr, info));
    return re;
  }
  // d ln(lambda)/d(betaJ, kappa, kappa2, h) of the eigenpair (lambda_internal, qr)
  std::array<double, 4> grad(const double* qr, double lambda_internal, const double* ql = nullptr) const {
    std::array<double, 4> g{};
    check(tm_grad(h_, qr, ql, lambda_internal, g.data()));
    return g;
  }
  tm_op* handle() const { return h_; }

 private:
  tm_op* h_ = nullptr;
};

// Differentiable eigensolve (no reference counterpart): forward() solves for
// the two leading eigenpairs of a symmetric operator and returns ln(lambda0)
// and the correlation length xi = 1 / ln(lambda0 / |lambda1|); backward()
// maps upstream gradients of (ln lambda0, xi) to the parameters (betaJ,
// kappa, kappa2, h) through the adjoint tm_grad:
//   d ln(lambda_i) = <q_i| dT |q_i> / lambda_i      (symmetric: left = right)
//   d xi = -xi^2 (d ln lambda0 - d ln lambda1).
// The saved eigenvectors are the forward's context for the backward pass.
struct EigenForward {
  double lambda0 = 0, lambda1 = 0;  // reported eigenvalues (lambda / normfactor)
  double log_lambda0 = 0, xi = 0;
  double normfactor = 1;
  int64_t rows = 0;
  std::vector<double> q;  // eigenvectors 0 and 1, rows x 2 column-major
};

class EigenFunction {
 public:
  static EigenForward forward(const GpuMatVecProd& op, double tol = 1e-12, int mode = TM_EIGS_F64) {
    if (!op.symmetric()) throw Error(TM_ERR_UNSUPPORTED, "EigenFunction needs a symmetric operator");
    EigenForward f;
    const std::vector<double> v = op.eigs(2, tol, mode, &f.q);
    f.rows = op.rows();
    f.normfactor = op.getnormfactor();
    f.lambda0 = v[0];
    f.lambda1 = v[1];
    f.log_lambda0 = std::log(v[0]);
    f.xi = 1.0 / std::log(v[0] / std::fabs(v[1]));
    return f;
  }
  // gradient of g_log_lambda0 * ln(lambda0) + g_xi * xi w.r.t. (betaJ, kappa, kappa2, h)
  static std::array<double, 4> backward(const GpuMatVecProd& op, const EigenForward& f, double g_log_lambda0,
                                        double g_xi) {
    const std::array<double, 4> d0 = op.grad(f.q.data(), f.lambda0 * f.normfactor);
    std::array<double, 4> out{};
    if (g_xi != 0.0) {
      const std::array<double, 4> d1 = op.grad(f.q.data() + f.rows, f.lambda1 * f.normfactor);
      for (int t = 0; t < 4; ++t) out[t] = g_log_lambda0 * d0[t] - g_xi * f.xi * f.xi * (d0[t] - d1[t]);
    } else {
      for (int t = 0; t < 4; ++t) out[t] = g_log_lambda0 * d0[t];
    }
    return out;
  }
};

}  // namespace latttmat

#endif
