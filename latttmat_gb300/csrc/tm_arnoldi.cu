// Largest-magnitude eigenpairs of a general (non-symmetric) transfer matrix.
//
// Replaces Spectra::GenEigsSolver as used by pfunc_inner and getlefteigvec
// (TMat/pfunc.hpp:47-68, 84-98).  Method: Arnoldi with CGS2 in FP64 on the
// device and thick restarts on an orthonormal basis of the kept Ritz vectors
// (a Krylov-Schur style restart: A V_k = V_k H_k + f b^T with
// span(W) H-invariant, so no implicit shifts are needed).  The small dense
// eigenproblem runs on the host, where the projected matrix comes back each
// cycle anyway: Householder reduction to Hessenberg form and Francis
// double-shift QR for the eigenvalues (Golub & Van Loan, Alg. 7.4.2,
// 7.5.1-7.5.2), complex inverse iteration for the wanted eigenvectors.
// Mixed mode: FP32 matvecs until the Ritz residuals hit the FP32 floor, then
// FP64 restart cycles from the same basis until the tolerance is met.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <memory>
#include <numeric>
#include <vector>

#include "tm_blas.cuh"
#include "tm_hqr.cuh"
#include "tm_internal.h"
#include "tm_krylov.h"

namespace ltm {

void apply_refine(const Op& op, const double* x, double* y, cudaStream_t s);
double apply_internal(const Op& op, const double* x, double* y, const float* x32, float* y32, bool f32,
                      cudaStream_t s);

// ------------------------------------------------------------------ restart algebra (host)
// The small-matrix side of the Krylov-Schur restart, shared by the single
// solver below and the batched sweep (tm_sweep.cu).

// Eigen-decompose H_m ((m+1) x (m+1) column-major, leading m x m block; host:
// the routines of tm_hqr.cuh take microseconds at these sizes): Ritz values by
// |theta| descending, eigenvectors and residual estimates for the first kvec.
Ritz krylov_project(const double* Hh, int m, int kvec) {
  Ritz R;
  std::vector<double> Hm((size_t)m * m);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) Hm[i + (size_t)j * m] = Hh[i + (size_t)j * (m + 1)];
  std::vector<double> er(m), ei(m);
  if (geneig_values(Hm.data(), m, er.data(), ei.data())) fail(TM_ERR_NOCONV, "small Hessenberg QR did not converge");
  std::vector<int> ord(m);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
    double ma = std::hypot(er[a], ei[a]), mb = std::hypot(er[b], ei[b]);
    if (ma != mb) return ma > mb;
    return ei[a] > ei[b];
  });
  R.beta = Hh[m + (size_t)(m - 1) * (m + 1)];
  kvec = std::min(kvec, m);
  std::vector<double> yr((size_t)m * kvec), yi((size_t)m * kvec), Br((size_t)m * m), Bi((size_t)m * m);
  for (int c = 0; c < kvec; ++c)
    geneig_vector(Hh, m, m + 1, er[ord[c]], ei[ord[c]], Br.data(), Bi.data(), yr.data() + (size_t)c * m,
                  yi.data() + (size_t)c * m);
  for (int i = 0; i < m; ++i) R.theta.push_back({er[ord[i]], ei[ord[i]]});
  for (int c = 0; c < kvec; ++c) {
    std::vector<std::complex<double>> y(m);
    for (int i = 0; i < m; ++i) y[i] = {yr[(size_t)c * m + i], yi[(size_t)c * m + i]};
    R.resid.push_back(std::fabs(R.beta) * std::abs(y[m - 1]));
    R.y.push_back(y);
  }
  return R;
}

// Ritz vectors computed per projection, and Ritz pairs kept at a restart
int krylov_kvec(int m, int nev) { return std::min(m - 1, std::max(nev + 2, (m + nev) / 2 + 1)); }
int krylov_keep(int m, int nev, int nconv, int kvec) {
  int kk = std::min(kvec, std::max(nev + 1, nev + std::min(nconv, (m - nev) / 2)));
  return std::max(kk, std::min(kvec, (m + nev) / 2));
}

// Real orthonormal basis Wm (m x k, column-major) of the span of the first kk
// Ritz vectors (a complex pair contributes Re and Im); returns k.
int krylov_basis(const Ritz& R, int m, int kk, std::vector<double>& Wm) {
  std::vector<std::vector<double>> cols;
  for (int c = 0; c < kk; ++c) {
    bool cplx = std::fabs(R.theta[c].imag()) > 0.0;
    std::vector<double> re(m), im(m);
    for (int i = 0; i < m; ++i) {
      re[i] = R.y[c][i].real();
      im[i] = R.y[c][i].imag();
    }
    cols.push_back(re);
    if (cplx) {
      cols.push_back(im);
      ++c;  // skip the conjugate partner
    }
  }
  // modified Gram-Schmidt twice
  std::vector<std::vector<double>> q;
  for (auto& cvec : cols) {
    std::vector<double> w = cvec;
    for (int pass = 0; pass < 2; ++pass)
      for (auto& b : q) {
        double d = 0;
        for (int i = 0; i < m; ++i) d += b[i] * w[i];
        for (int i = 0; i < m; ++i) w[i] -= d * b[i];
      }
    double nr = 0;
    for (int i = 0; i < m; ++i) nr += w[i] * w[i];
    nr = std::sqrt(nr);
    if (nr < 1e-10) continue;
    for (int i = 0; i < m; ++i) w[i] /= nr;
    q.push_back(w);
  }
  int k = (int)q.size();
  Wm.assign((size_t)m * k, 0.0);
  for (int c = 0; c < k; ++c)
    for (int i = 0; i < m; ++i) Wm[(size_t)c * m + i] = q[c][i];
  return k;
}

// Projected matrix after the restart V_k = V_m W: H_k = W^T H_m W and the
// coupling row beta * W[m-1, :] below it ((m+1) x (m+1) column-major).
void krylov_restart_h(const double* Hh, int m, const std::vector<double>& Wm, int k, double beta,
                      std::vector<double>& Hn) {
  const int ld = m + 1;
  std::vector<double> HW((size_t)m * k, 0.0);
  Hn.assign((size_t)ld * ld, 0.0);
  for (int c = 0; c < k; ++c)
    for (int i = 0; i < m; ++i) {
      double acc = 0;
      for (int j = 0; j < m; ++j) acc += Hh[i + (size_t)j * ld] * Wm[(size_t)c * m + j];
      HW[(size_t)c * m + i] = acc;
    }
  for (int c = 0; c < k; ++c)
    for (int r = 0; r < k; ++r) {
      double acc = 0;
      for (int i = 0; i < m; ++i) acc += Wm[(size_t)r * m + i] * HW[(size_t)c * m + i];
      Hn[r + (size_t)c * ld] = acc;
    }
  for (int c = 0; c < k; ++c) Hn[k + (size_t)c * ld] = beta * Wm[(size_t)c * m + (m - 1)];
}

namespace {

constexpr int MMAX = 48;

// --------------------------------------------------------------- small dense
__global__ void hcolg_kernel(double* H, int ld, int j, const double* h1, const double* h2, const double* nsq) {
  int i = threadIdx.x;
  if (i <= j) H[i + j * ld] = h1[i] + h2[i];
  if (i == 0) H[(j + 1) + j * ld] = sqrt(*nsq);
}

__global__ void copyv_kernel(const double* __restrict__ a, double* __restrict__ b, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) b[i] = a[i];
}

int nblk(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 8)); }


struct Arnoldi {
  const Op& op;
  cudaStream_t s;
  int64_t n;
  int m;
  DBuf V, W, x32, y32, h1, h2, part, nsq, Hd, Wd;
  int matvecs = 0, matvecs64 = 0, restarts = 0;
  std::vector<double> Hh;  // host copy (m+1)^2

  Arnoldi(const Op& o, int ncv, cudaStream_t st_) : op(o), s(st_), n(o.n), m(ncv) {
    V.alloc((size_t)(m + 1) * n * 8);
    W.alloc((size_t)n * 8);
    h1.alloc(64 * 8);
    h2.alloc(64 * 8);
    part.alloc(red_part_bytes(16));
    nsq.alloc(8);
    Hd.alloc((size_t)(m + 1) * (m + 1) * 8);
    Wd.alloc((size_t)64 * 64 * 8);
  }
  double* v(int j) const { return V.as<double>() + (int64_t)j * n; }

  // mixed mode: the FP64 phase uses the FP64-accurate refinement products
  // (double-float where the operator has them)
  bool refine_products = false;

  void step(int j, bool f32) {
    double* w = W.as<double>();
    if (f32) {
      if (!x32.p) {
        x32.alloc((size_t)n * 4);
        y32.alloc((size_t)n * 4);
      }
      to_f32(v(j), x32.as<float>(), n, s);
      double S = apply_internal(op, nullptr, nullptr, x32.as<float>(), y32.as<float>(), true, s);
      mdot32(v(0), n, j + 1, y32.as<float>(), S, n, h1.as<double>(), part.as<double>(), s);
      maxpy32(v(0), n, j + 1, h1.as<double>(), y32.as<float>(), S, w, n, s);
    } else {
      if (refine_products)
        apply_refine(op, v(j), w, s);
      else
        apply_internal(op, v(j), w, nullptr, nullptr, false, s);
      ++matvecs64;
      mdot(v(0), n, j + 1, w, n, h1.as<double>(), part.as<double>(), s);
      maxpy(v(0), n, j + 1, h1.as<double>(), w, n, s);
    }
    ++matvecs;
    mdot(v(0), n, j + 1, w, n, h2.as<double>(), part.as<double>(), s);
    maxpy(v(0), n, j + 1, h2.as<double>(), w, n, s);
    nrm2sq(w, n, nsq.as<double>(), part.as<double>(), s);
    hcolg_kernel<<<1, 64, 0, s>>>(Hd.as<double>(), m + 1, j, h1.as<double>(), h2.as<double>(), nsq.as<double>());
    TM_CKK("hcolg");
    normalize(w, nsq.as<double>(), v(j + 1), nullptr, n, s);
  }

  void start(const double* v0, uint64_t seed) {
    TM_CK(cudaMemsetAsync(Hd.p, 0, (size_t)(m + 1) * (m + 1) * 8, s));
    if (v0)
      copyv_kernel<<<nblk(n), 256, 0, s>>>(v0, W.as<double>(), n);
    else
      fill_uniform(W.as<double>(), n, seed, s);
    nrm2sq(W.as<double>(), n, nsq.as<double>(), part.as<double>(), s);
    normalize(W.as<double>(), nsq.as<double>(), v(0), nullptr, n, s);
  }

  Ritz project(int kvec) {
    Hh.assign((size_t)(m + 1) * (m + 1), 0.0);
    TM_CK(cudaMemcpyAsync(Hh.data(), Hd.p, Hh.size() * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    return krylov_project(Hh.data(), m, kvec);
  }

  int build_basis(const Ritz& R, int kk, std::vector<double>& Wm) { return krylov_basis(R, m, kk, Wm); }

  // restart: V_k = V_m W, H_k = W^T H_m W, coupling row b = beta * W[m-1,:], v_k = v_m
  void restart(const Ritz& R, const std::vector<double>& Wm, int k) {
    TM_CK(cudaMemcpyAsync(Wd.p, Wm.data(), Wm.size() * 8, cudaMemcpyHostToDevice, s));
    basis_rotate(V.as<double>(), n, m, Wd.as<double>(), k, n, s);
    copyv_kernel<<<nblk(n), 256, 0, s>>>(v(m), v(k), n);
    TM_CKK("copyv");
    std::vector<double> Hn;
    krylov_restart_h(Hh.data(), m, Wm, k, R.beta, Hn);
    TM_CK(cudaMemcpyAsync(Hd.p, Hn.data(), Hn.size() * 8, cudaMemcpyHostToDevice, s));
    ++restarts;
  }

  // returns converged flag; R holds the final projection
  bool run(int nev, bool f32, double tol, bool tol_rel_dominant, int max_cycles, int k0, Ritz& R) {
    int k = k0;
    double best = 1e300;
    int stall = 0;
    for (int cyc = 0; cyc < max_cycles; ++cyc) {
      for (int j = k; j < m; ++j) step(j, f32);
      const int kvec = krylov_kvec(m, nev);
      R = project(kvec);
      double ref = std::abs(R.theta[0]);
      bool ok = true;
      int nconv = 0;
      double worst = 0.0;
      for (int i = 0; i < nev; ++i) {
        double lim = tol * (tol_rel_dominant ? ref : std::max(std::abs(R.theta[i]), 1e-300));
        worst = std::max(worst, R.resid[i] / std::max(ref, 1e-300));
        if (R.resid[i] <= lim)
          ++nconv;
        else
          ok = false;
      }
      if (ok) return true;
      if (f32) {  // stop the FP32 phase once its residuals stagnate at the FP32 floor
        if (worst < 0.7 * best) {
          best = worst;
          stall = 0;
        } else if (++stall >= 3 && worst < 1e-4) {
          return false;
        }
      }
      std::vector<double> Wm;
      int knew = build_basis(R, krylov_keep(m, nev, nconv, kvec), Wm);
      if (knew >= m - 1) knew = m - 2;
      restart(R, Wm, knew);
      k = knew;
    }
    return false;
  }

  // final Ritz vectors x_c = V_m y_c for c < nev (complex): host arrays
  void ritz_vectors(const Ritz& R, int nev, std::vector<double>& xr, std::vector<double>& xi) {
    std::vector<double> Yc((size_t)m * 2 * nev);
    for (int c = 0; c < nev; ++c)
      for (int i = 0; i < m; ++i) {
        Yc[(size_t)(2 * c) * m + i] = R.y[c][i].real();
        Yc[(size_t)(2 * c + 1) * m + i] = R.y[c][i].imag();
      }
    // V has m+1 columns; rotate in place into columns 0..2nev-1 (needs 2nev <= m)
    TM_CK(cudaMemcpyAsync(Wd.p, Yc.data(), Yc.size() * 8, cudaMemcpyHostToDevice, s));
    basis_rotate(V.as<double>(), n, m, Wd.as<double>(), 2 * nev, n, s);
    xr.resize((size_t)nev * n);
    xi.resize((size_t)nev * n);
    for (int c = 0; c < nev; ++c) {
      TM_CK(cudaMemcpyAsync(xr.data() + (size_t)c * n, v(2 * c), (size_t)n * 8, cudaMemcpyDeviceToHost, s));
      TM_CK(cudaMemcpyAsync(xi.data() + (size_t)c * n, v(2 * c + 1), (size_t)n * 8, cudaMemcpyDeviceToHost, s));
    }
    TM_CK(cudaStreamSynchronize(s));
  }
};

}  // namespace

// General solve: vals (complex, internal scale); vectors (complex, internal
// order) when requested.
tm_status arnoldi_solve(const Op& op, int nev, int ncv, double tol, uint64_t seed, int mode,
                        std::vector<std::complex<double>>& vals, std::vector<double>* vr, std::vector<double>* vi,
                        tm_eigs_info* info_out) {
  auto t0 = std::chrono::steady_clock::now();
  const int64_t n = op.n;
  if (nev < 1 || nev >= n) fail(TM_ERR_ARG, "nev must satisfy 1 <= nev < rows");
  if (ncv <= 0) ncv = (nev > 4) ? 2 * nev + 1 : 2 * nev + 3;
  ncv = std::max(ncv, 2 * nev + 2);
  if (ncv >= n) ncv = (int)n - 1;
  if (ncv > MMAX - 2) ncv = MMAX - 2;
  if (tol <= 0) tol = 1e-10;
  tm_eigs_info info{};
  bool done = false;
  int attempts = 0;
  std::unique_ptr<Arnoldi> Ar;
  Ritz R;
  while (!done && attempts < 3) {
    Ar.reset(new Arnoldi(op, ncv, op.stream));
    Arnoldi& a = *Ar;
    a.start(nullptr, seed);
    if (mode == TM_EIGS_MIXED) {
      const double tol32 = std::max(tol, 3e-7);
      a.run(nev, true, tol32, true, 200, 0, R);
      // FP64 Arnoldi restarted from the sum of the wanted FP32 Ritz vectors'
      // real parts (the projected matrix of the FP32 phase is only FP32
      // accurate, so it is rebuilt with FP64 products)
      std::vector<double> Yc((size_t)ncv * nev);
      for (int c = 0; c < nev; ++c)
        for (int i = 0; i < ncv; ++i) Yc[(size_t)c * ncv + i] = R.y[c][i].real();
      std::vector<double> comb(ncv, 0.0);
      for (int c = 0; c < nev; ++c)
        for (int i = 0; i < ncv; ++i) comb[i] += Yc[(size_t)c * ncv + i];
      TM_CK(cudaMemcpyAsync(a.Wd.p, comb.data(), ncv * 8, cudaMemcpyHostToDevice, op.stream));
      basis_rotate(a.V.as<double>(), n, ncv, a.Wd.as<double>(), 1, n, op.stream);
      DBuf start;
      start.alloc((size_t)n * 8);
      TM_CK(cudaMemcpyAsync(start.p, a.v(0), (size_t)n * 8, cudaMemcpyDeviceToDevice, op.stream));
      a.start(start.as<double>(), seed);
      a.refine_products = true;
      done = a.run(nev, false, tol, false, 200, 0, R);
    } else {
      done = a.run(nev, false, tol, false, 300, 0, R);
    }
    info.matvecs += a.matvecs;
    info.matvecs_f64 += a.matvecs64;
    info.restarts += a.restarts;
    info.ncv = ncv;
    ++attempts;
    if (!done) ncv = std::min(ncv + 2, std::min((int)n - 1, MMAX - 2));
  }
  vals.assign(R.theta.begin(), R.theta.begin() + nev);
  double mr = 0;
  for (int i = 0; i < nev; ++i) mr = std::max(mr, R.resid[i] / std::max(std::abs(R.theta[i]), 1e-300));
  info.max_resid = mr;
  info.nconv = done ? nev : 0;
  if (vr && vi) Ar->ritz_vectors(R, nev, *vr, *vi);
  const_cast<Op&>(op).matvecs += info.matvecs;
  info.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (info_out) *info_out = info;
  return done ? TM_OK : TM_ERR_NOCONV;
}

}  // namespace ltm
