// Largest-magnitude eigenpairs of a symmetric transfer matrix on the GPU.
//
// Replaces Spectra::SymEigsSolver as driven by pfunc_inner
// (TMat/pfunc.hpp:79-114): nev wanted values, ncv = suggested_nev
// (TMat/tmat.hpp:88), up to 3 attempts with ncv += 2 on non-convergence.
//
// Method: thick-restart Lanczos (Wu & Simon 2000), which is mathematically
// equivalent to the implicitly restarted Lanczos with exact shifts that
// ARPACK/Spectra use.  Gram-Schmidt with one full re-orthogonalisation (CGS2)
// in FP64 on the device.  The small projected eigenproblem is solved by a
// one-warp Jacobi kernel.  The host only reads Ritz values at restarts.
//
// Mixed precision (TM_EIGS_MIXED): matvecs run in FP32 until the Ritz
// residuals reach the FP32 noise floor.  Then an FP64 Rayleigh-Ritz step on
// the nev Ritz vectors (nev FP64 matvecs) gives eigenvalues whose error is
// bounded by ||r||^2/gap (Kato-Temple).  FP64 Lanczos resumes only when that
// bound misses the tolerance.
#include <algorithm>
#include <chrono>
#include <memory>
#include <cmath>
#include <numeric>
#include <vector>

#include "tm_blas.cuh"
#include "tm_internal.h"

namespace ltm {

// matvec in the operator's internal order.  f32=true: x32 -> y32 with
// T x = S * y32 (S returned).
double apply_internal(const Op& op, const double* x, double* y, const float* x32, float* y32, bool f32,
                      cudaStream_t s);
void apply_refine(const Op& op, const double* x, double* y, cudaStream_t s);

namespace {

// growth steps of the FP64 block refinement before falling back to FP64 Lanczos
constexpr int kRefineRounds = 6;

__global__ void hcol_kernel(double* H, int ld, int j, const double* h1, const double* h2, const double* nsq,
                            int write_beta) {
  int i = threadIdx.x;
  if (i <= j) {
    double v = h1[i] + h2[i];
    H[i + j * ld] = v;
    H[j + i * ld] = v;
  }
  if (i == 0 && write_beta) {
    double b = sqrt(*nsq);
    H[(j + 1) + j * ld] = b;
    H[j + (j + 1) * ld] = b;
  }
}

__global__ void copy_kernel(const double* __restrict__ a, double* __restrict__ b, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) b[i] = a[i];
}

__global__ void resid_kernel(const double* __restrict__ W, const double* __restrict__ X, int64_t ld, int k,
                             const double* __restrict__ theta, double* __restrict__ R, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st)
    for (int c = 0; c < k; ++c) R[c * ld + i] = W[c * ld + i] - theta[c] * X[c * ld + i];
}

// y = S * y32 (an FP32 product that was computed divided by S)
__global__ void f32_scaled_kernel(const float* __restrict__ y32, double S, double* __restrict__ y, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) y[i] = S * (double)y32[i];
}

int blocks_for(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 8));
}

struct Lanczos {
  const Op& op;
  cudaStream_t s;
  int64_t n;
  int m;
  DBuf V, W, x32, y32, h1, h2, part, nsq, Hd, wd, Zd, Ysel;
  int matvecs = 0, matvecs64 = 0, restarts = 0;

  Lanczos(const Op& o, int ncv, cudaStream_t st) : op(o), s(st), n(o.n), m(ncv) {
    V.alloc((size_t)(m + 1) * n * sizeof(double));
    W.alloc((size_t)n * sizeof(double));
    h1.alloc(64 * 8);
    h2.alloc(64 * 8);
    part.alloc((size_t)num_sms() * 4 * 16 * 8 + 64);
    nsq.alloc(8);
    Hd.alloc((size_t)(m + 1) * (m + 1) * 8);
    wd.alloc(64 * 8);
    Zd.alloc(64 * 64 * 8);
    Ysel.alloc(64 * 64 * 8);
  }
  double* v(int j) const { return V.as<double>() + (int64_t)j * n; }

  void ensure32() {
    if (!x32.p) {
      x32.alloc((size_t)n * 4);
      y32.alloc((size_t)n * 4);
    }
  }

  // one Lanczos step j: v(j) -> v(j+1), H column j
  void step(int j, bool f32) {
    double* w = W.as<double>();
    if (f32) {
      ensure32();
      to_f32(v(j), x32.as<float>(), n, s);
      double S = apply_internal(op, nullptr, nullptr, x32.as<float>(), y32.as<float>(), true, s);
      mdot32(v(0), n, j + 1, y32.as<float>(), S, n, h1.as<double>(), part.as<double>(), s);
      maxpy32(v(0), n, j + 1, h1.as<double>(), y32.as<float>(), S, w, n, s);
    } else {
      apply_internal(op, v(j), w, nullptr, nullptr, false, s);
      ++matvecs64;
      mdot(v(0), n, j + 1, w, n, h1.as<double>(), part.as<double>(), s);
      maxpy(v(0), n, j + 1, h1.as<double>(), w, n, s);
    }
    ++matvecs;
    mdot(v(0), n, j + 1, w, n, h2.as<double>(), part.as<double>(), s);
    maxpy(v(0), n, j + 1, h2.as<double>(), w, n, s);
    nrm2sq(w, n, nsq.as<double>(), part.as<double>(), s);
    hcol_kernel<<<1, 64, 0, s>>>(Hd.as<double>(), m + 1, j, h1.as<double>(), h2.as<double>(), nsq.as<double>(),
                                 1);
    TM_CKK("hcol");
    normalize(w, nsq.as<double>(), v(j + 1), nullptr, n, s);
  }

  struct CycleResult {
    std::vector<double> theta;     // sorted by |theta| desc
    std::vector<double> resid;     // |beta_m * y_{m-1,i}|
    std::vector<int> order;        // column indices into Z
    std::vector<double> Z;         // m x m
    double beta;
  };

  CycleResult project() {
    small_symeig(Hd.as<double>(), m, wd.as<double>(), Zd.as<double>(), s, m + 1);
    CycleResult r;
    std::vector<double> th(m), H((size_t)(m + 1) * (m + 1));
    r.Z.resize((size_t)m * m);
    TM_CK(cudaMemcpyAsync(th.data(), wd.p, m * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaMemcpyAsync(r.Z.data(), Zd.p, (size_t)m * m * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaMemcpyAsync(H.data(), Hd.p, H.size() * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    r.beta = H[m + (size_t)(m - 1) * (m + 1)];
    r.order.resize(m);
    std::iota(r.order.begin(), r.order.end(), 0);
    std::stable_sort(r.order.begin(), r.order.end(),
                     [&](int a, int b) { return std::fabs(th[a]) > std::fabs(th[b]); });
    for (int i = 0; i < m; ++i) {
      int c = r.order[i];
      r.theta.push_back(th[c]);
      r.resid.push_back(std::fabs(r.beta * r.Z[(size_t)c * m + (m - 1)]));
    }
    return r;
  }

  // V[:, 0..k) <- V[:, 0..m) * Z[:, order[0..k)]
  void rotate(const CycleResult& r, int k) {
    std::vector<double> Y((size_t)m * k);
    for (int c = 0; c < k; ++c)
      for (int j = 0; j < m; ++j) Y[(size_t)c * m + j] = r.Z[(size_t)r.order[c] * m + j];
    TM_CK(cudaMemcpyAsync(Ysel.p, Y.data(), Y.size() * 8, cudaMemcpyHostToDevice, s));
    basis_rotate(V.as<double>(), n, m, Ysel.as<double>(), k, n, s);
  }

  // restart with k kept Ritz vectors; v(k) <- v(m)
  void restart(const CycleResult& r, int k) {
    rotate(r, k);
    copy_kernel<<<blocks_for(n), 256, 0, s>>>(v(m), v(k), n);
    TM_CKK("copy");
    std::vector<double> H((size_t)(m + 1) * (m + 1), 0.0);
    for (int i = 0; i < k; ++i) {
      H[i + (size_t)i * (m + 1)] = r.theta[i];
      double cpl = r.beta * r.Z[(size_t)r.order[i] * m + (m - 1)];
      H[k + (size_t)i * (m + 1)] = cpl;
      H[i + (size_t)k * (m + 1)] = cpl;
    }
    TM_CK(cudaMemcpyAsync(Hd.p, H.data(), H.size() * 8, cudaMemcpyHostToDevice, s));
    ++restarts;
  }

  void start(const double* v0_dev, uint64_t seed) {
    TM_CK(cudaMemsetAsync(Hd.p, 0, (size_t)(m + 1) * (m + 1) * 8, s));
    if (v0_dev)
      copy_kernel<<<blocks_for(n), 256, 0, s>>>(v0_dev, W.as<double>(), n);
    else
      fill_uniform(W.as<double>(), n, seed, s);
    nrm2sq(W.as<double>(), n, nsq.as<double>(), part.as<double>(), s);
    normalize(W.as<double>(), nsq.as<double>(), v(0), nullptr, n, s);
  }

  // run restart cycles; returns the last projection.  conv(r) decides.
  template <class Conv>
  CycleResult run(int nev, bool f32, int max_cycles, Conv conv, bool* ok) {
    int k = 0;
    CycleResult r;
    *ok = false;
    double best = 1e300;
    int stall = 0;
    for (int cyc = 0; cyc < max_cycles; ++cyc) {
      for (int j = k; j < m; ++j) step(j, f32);
      r = project();
      if (conv(r)) {
        *ok = true;
        return r;
      }
      if (stagnation_stop) {
        double worst = 0.0;
        for (int i = 0; i < nev; ++i) worst = std::max(worst, r.resid[i] / std::fabs(r.theta[0]));
        if (worst < 0.7 * best) {
          best = worst;
          stall = 0;
        } else if (++stall >= 3 && worst < 1e-4) {
          return r;  // FP32 floor reached
        }
      }
      int nconv = 0;
      for (int i = 0; i < nev; ++i)
        if (conv_one(r, i)) ++nconv;
      k = std::min(m - 2, std::max(nev + 1, nev + std::min(nconv, (m - nev) / 2)));
      k = std::max(k, std::min(m - 2, (m + nev) / 2));
      restart(r, k);
    }
    return r;
  }
  double conv_tol = 1e-10;
  bool stagnation_stop = false;
  bool conv_one(const CycleResult& r, int i) const {
    return r.resid[i] <= conv_tol * std::max(std::fabs(r.theta[i]), 1e-300);
  }
};

__global__ void hcol32_kernel(double* H, int ld, int j, const double* h1, const double* h2, const double* nsq,
                              double S) {
  int i = threadIdx.x;
  if (i <= j) {
    double v = S * (h1[i] + h2[i]);
    H[i + j * ld] = v;
    H[j + i * ld] = v;
  }
  if (i == 0) {
    double b = S * sqrt(*nsq);
    H[(j + 1) + j * ld] = b;
    H[j + (j + 1) * ld] = b;
  }
}

// FP32-basis thick-restart Lanczos for the FP32 phase of mixed precision
// (ncv <= 16).  The matvec returns y = T v / S; CGS2 runs on y with FP32
// data and FP64 reductions, and S is folded into H, so no large factor ever
// enters FP32 storage.  Sweeps over the basis per step: dots, fused
// update+dots, fused update+norm (3 instead of 4).
struct Lanczos32 {
  const Op& op;
  cudaStream_t s;
  int64_t n;
  int m;
  DBuf V, W, Y, h1, h2, part, nsq, Hd, wd, Zd, Ysel;
  int matvecs = 0, restarts = 0;
  bool stagnation_stop = true;

  Lanczos32(const Op& o, int ncv, cudaStream_t st) : op(o), s(st), n(o.n), m(ncv) {
    V.alloc((size_t)(m + 1) * n * 4);
    W.alloc((size_t)n * 4);
    Y.alloc((size_t)n * 4);
    h1.alloc(64 * 8);
    h2.alloc(64 * 8);
    part.alloc((size_t)num_sms() * 4 * 16 * 8 + 64);
    nsq.alloc(8);
    Hd.alloc((size_t)(m + 1) * (m + 1) * 8);
    wd.alloc(64 * 8);
    Zd.alloc(64 * 64 * 8);
    Ysel.alloc(64 * 64 * 8);
  }
  float* v(int j) const { return V.as<float>() + (int64_t)j * n; }

  void start(uint64_t seed) {
    TM_CK(cudaMemsetAsync(Hd.p, 0, (size_t)(m + 1) * (m + 1) * 8, s));
    fill_uniform_f32(W.as<float>(), n, seed, s);
    nrm2sq_f32(W.as<float>(), n, nsq.as<double>(), part.as<double>(), s);
    normalize_f32(W.as<float>(), nsq.as<double>(), v(0), n, s);
  }

  void step(int j) {
    double S = apply_internal(op, nullptr, nullptr, v(j), Y.as<float>(), true, s);
    ++matvecs;
    mdot_f32(v(0), n, j + 1, Y.as<float>(), n, h1.as<double>(), part.as<double>(), s);
    axpy_dot_f32(v(0), n, j + 1, h1.as<double>(), Y.as<float>(), W.as<float>(), n, h2.as<double>(),
                 part.as<double>(), s);
    axpy_nrm_f32(v(0), n, j + 1, h2.as<double>(), W.as<float>(), n, nsq.as<double>(), part.as<double>(), s);
    hcol32_kernel<<<1, 64, 0, s>>>(Hd.as<double>(), m + 1, j, h1.as<double>(), h2.as<double>(), nsq.as<double>(), S);
    TM_CKK("hcol32");
    normalize_f32(W.as<float>(), nsq.as<double>(), v(j + 1), n, s);
  }

  Lanczos::CycleResult project() {
    small_symeig(Hd.as<double>(), m, wd.as<double>(), Zd.as<double>(), s, m + 1);
    Lanczos::CycleResult r;
    std::vector<double> th(m), H((size_t)(m + 1) * (m + 1));
    r.Z.resize((size_t)m * m);
    TM_CK(cudaMemcpyAsync(th.data(), wd.p, m * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaMemcpyAsync(r.Z.data(), Zd.p, (size_t)m * m * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaMemcpyAsync(H.data(), Hd.p, H.size() * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    r.beta = H[m + (size_t)(m - 1) * (m + 1)];
    r.order.resize(m);
    std::iota(r.order.begin(), r.order.end(), 0);
    std::stable_sort(r.order.begin(), r.order.end(),
                     [&](int a, int b) { return std::fabs(th[a]) > std::fabs(th[b]); });
    for (int i = 0; i < m; ++i) {
      int c = r.order[i];
      r.theta.push_back(th[c]);
      r.resid.push_back(std::fabs(r.beta * r.Z[(size_t)c * m + (m - 1)]));
    }
    return r;
  }

  std::vector<double> ysel(const Lanczos::CycleResult& r, int k) const {
    std::vector<double> Y((size_t)m * k);
    for (int c = 0; c < k; ++c)
      for (int j = 0; j < m; ++j) Y[(size_t)c * m + j] = r.Z[(size_t)r.order[c] * m + j];
    return Y;
  }

  void restart(const Lanczos::CycleResult& r, int k) {
    std::vector<double> Yh = ysel(r, k);
    TM_CK(cudaMemcpyAsync(Ysel.p, Yh.data(), Yh.size() * 8, cudaMemcpyHostToDevice, s));
    rotate_f32(V.as<float>(), n, m, Ysel.as<double>(), k, n, s);
    TM_CK(cudaMemcpyAsync(v(k), v(m), (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    std::vector<double> H((size_t)(m + 1) * (m + 1), 0.0);
    for (int i = 0; i < k; ++i) {
      H[i + (size_t)i * (m + 1)] = r.theta[i];
      double cpl = r.beta * r.Z[(size_t)r.order[i] * m + (m - 1)];
      H[k + (size_t)i * (m + 1)] = cpl;
      H[i + (size_t)k * (m + 1)] = cpl;
    }
    TM_CK(cudaMemcpyAsync(Hd.p, H.data(), H.size() * 8, cudaMemcpyHostToDevice, s));
    ++restarts;
  }

  // FP64 Ritz vectors: out[:, c] = V32 * Z[:, order[c]], c < k
  void ritz_f64(const Lanczos::CycleResult& r, int k, double* out) {
    std::vector<double> Yh = ysel(r, k);
    TM_CK(cudaMemcpyAsync(Ysel.p, Yh.data(), Yh.size() * 8, cudaMemcpyHostToDevice, s));
    combine_f32_f64(V.as<float>(), n, m, Ysel.as<double>(), k, out, n, n, s);
  }

  template <class Conv>
  Lanczos::CycleResult run(int nev, int max_cycles, Conv conv) {
    int k = 0;
    Lanczos::CycleResult r;
    double best = 1e300;
    int stall = 0;
    for (int cyc = 0; cyc < max_cycles; ++cyc) {
      for (int j = k; j < m; ++j) step(j);
      r = project();
      if (conv(r)) return r;
      double worst = 0.0;
      for (int i = 0; i < nev; ++i) worst = std::max(worst, r.resid[i] / std::fabs(r.theta[0]));
      if (stagnation_stop) {
        if (worst < 0.7 * best) {
          best = worst;
          stall = 0;
        } else if (++stall >= 3 && worst < 1e-4) {
          return r;
        }
      }
      int nconv = 0;
      for (int i = 0; i < nev; ++i)
        if (r.resid[i] <= 2e-7 * std::fabs(r.theta[0])) ++nconv;
      k = std::min(m - 2, std::max(nev + 1, nev + std::min(nconv, (m - nev) / 2)));
      k = std::max(k, std::min(m - 2, (m + nev) / 2));
      restart(r, k);
    }
    return r;
  }
};

}  // namespace

struct EigOut {
  std::vector<double> vals;      // internal eigenvalues
  std::vector<double> vecs;      // internal order, n x nev (host)
  tm_eigs_info info;
};

// Symmetric solve.  vecs_host may be null.
tm_status lanczos_solve(const Op& op, int nev, int ncv, double tol, uint64_t seed, int mode, double* vals,
                        double* vecs_host, tm_eigs_info* info_out) {
  auto t0 = std::chrono::steady_clock::now();
  cudaStream_t s = op.stream;
  const int64_t n = op.n;
  if (nev < 1 || nev >= n) fail(TM_ERR_ARG, "nev must satisfy 1 <= nev < rows");
  if (ncv <= 0) ncv = (nev > 4) ? 2 * nev + 1 : 2 * nev + 3;
  if (ncv >= n) ncv = (int)n - 1;
  if (ncv > 46) ncv = 46;
  if (ncv <= nev) fail(TM_ERR_ARG, "ncv must exceed nev");
  if (tol <= 0) tol = 1e-10;
  tm_eigs_info info{};
  std::vector<double> theta;
  bool done = false;
  int attempts = 0;
  double max_resid = 0.0;
  std::unique_ptr<Lanczos> Lz;
  while (!done && attempts < 3) {
    Lz.reset(new Lanczos(op, ncv, s));
    Lanczos& lz = *Lz;
    const bool mixed = (mode == TM_EIGS_MIXED);
    lz.start(nullptr, seed);
    bool ok = false;
    Lanczos::CycleResult r;
    if (mixed) {
      // FP32 phase: Ritz residuals down to the FP32 floor (relative to the
      // dominant Ritz value), stopping early if they stagnate
      const double tol32 = std::max(tol, 2e-7);
      const int nb0 = std::max(nev, ncv - 1);
      auto conv32 = [&](const Lanczos::CycleResult& rr) {
        for (int i = 0; i < nev; ++i)
          if (rr.resid[i] > tol32 * std::fabs(rr.theta[0])) return false;
        return true;
      };
      if (ncv <= NV32) {
        // FP32 Krylov basis (half the bytes of the FP64 basis per sweep)
        Lanczos32 l32(op, ncv, s);
        l32.start(seed);
        r = l32.run(nev, 200, conv32);
        l32.ritz_f64(r, nb0, lz.v(0));
        // the FP32 basis is orthonormal to FP32 accuracy only: re-orthonormalise
        // the FP64 Ritz block (CGS2) so Rayleigh-Ritz is a standard eigenproblem
        for (int i = 0; i < nb0; ++i) {
          double* bi = lz.v(i);
          for (int pass = 0; pass < 2 && i > 0; ++pass) {
            mdot(lz.v(0), n, i, bi, n, lz.h1.as<double>(), lz.part.as<double>(), s);
            maxpy(lz.v(0), n, i, lz.h1.as<double>(), bi, n, s);
          }
          nrm2sq(bi, n, lz.nsq.as<double>(), lz.part.as<double>(), s);
          normalize(bi, lz.nsq.as<double>(), bi, nullptr, n, s);
        }
        lz.matvecs += l32.matvecs;
        lz.restarts += l32.restarts;
      } else {
        lz.conv_tol = tol32;
        lz.stagnation_stop = true;
        r = lz.run(nev, true, 200, conv32, &ok);
        lz.stagnation_stop = false;
        lz.rotate(r, nb0);
      }
      // FP64 refinement: block Davidson with mixed-precision products.  B
      // starts as the FP32 phase's Ritz vectors; the nev wanted ones get
      // FP64-accurate products (apply_refine), the others FP32 products, and
      // each growth step appends the wanted residual block, again with FP32
      // products.  An FP32 product error reaches a Ritz pair only through the
      // pair's weight on that column, which is at the FP32 noise level for
      // the wanted pairs, so Rayleigh-Ritz values and residual estimates stay
      // FP64-accurate.  The extra Ritz vectors carry the eigenvectors next to
      // the wanted ones, which residual blocks alone resolve slowly.  When the
      // estimates meet tol, the wanted Ritz vectors get FP64-accurate products
      // and are accepted on the test of the FP64 Lanczos path and of Spectra's
      // SymEigsSolver: ||A x - theta x|| <= tol * |theta|.
      const int nx = nb0;
      const int cap = nx + 2 * nev;
      DBuf Bb, AB, XB, AXB, G, Gw, Gz, th;
      std::vector<double> thv(nev);
      bool refined = false;
      // cluster guard: FP32 Ritz values closer than 1e-5 (relative) cannot be
      // told apart from FP32-accurate vectors; solve those (and operators too
      // small for a block of cap columns) in FP64 directly
      bool cluster = (int64_t)cap * 4 > n;
      for (int i = 0; i < nev && i + 1 < (int)r.theta.size(); ++i)
        if (std::fabs(r.theta[i] - r.theta[i + 1]) < 1e-5 * std::fabs(r.theta[i])) cluster = true;
      if (!cluster) {
        Bb.alloc((size_t)cap * n * 8);
        AB.alloc((size_t)cap * n * 8);
        XB.alloc((size_t)cap * n * 8);
        AXB.alloc((size_t)cap * n * 8);
        G.alloc((size_t)cap * cap * 8);
        Gw.alloc(64 * 8);
        Gz.alloc((size_t)64 * 64 * 8);
        th.alloc(64 * 8);
      }
      double* B = Bb.as<double>();
      auto col = [&](const DBuf& b, int j) { return b.as<double>() + (int64_t)j * n; };
      auto prod32 = [&](const double* x, double* y) {
        lz.ensure32();
        to_f32(x, lz.x32.as<float>(), n, s);
        const double S = apply_internal(op, nullptr, nullptr, lz.x32.as<float>(), lz.y32.as<float>(), true, s);
        f32_scaled_kernel<<<blocks_for(n), 256, 0, s>>>(lz.y32.as<float>(), S, y, n);
        TM_CKK("f32_scaled");
        ++lz.matvecs;
      };
      auto prod64 = [&](const double* x, double* y) {
        apply_refine(op, x, y, s);
        ++lz.matvecs;
        ++lz.matvecs64;
      };
      auto norm_host = [&](const double* v) {
        double q = 0.0;
        nrm2sq(v, n, lz.nsq.as<double>(), lz.part.as<double>(), s);
        TM_CK(cudaMemcpyAsync(&q, lz.nsq.p, 8, cudaMemcpyDeviceToHost, s));
        TM_CK(cudaStreamSynchronize(s));
        return std::sqrt(std::max(q, 0.0));
      };
      // imp[j]: weight of column j on FP32-product columns (0: FP64-accurate)
      std::vector<double> imp(cap, 1.0);
      int nb = nx, verified = 0;
      if (!cluster) {
        TM_CK(cudaMemcpyAsync(B, lz.v(0), (size_t)nx * n * 8, cudaMemcpyDeviceToDevice, s));
        for (int j = 0; j < nx; ++j) {
          if (j < nev) {
            prod64(B + (int64_t)j * n, col(AB, j));
            imp[j] = 0.0;
          } else {
            prod32(B + (int64_t)j * n, col(AB, j));
          }
        }
      }
      for (int round = 0; round < kRefineRounds && !cluster; ++round) {
        // G(i, j) = B_i . (A B_j), symmetrised from the side whose product is
        // the more accurate one
        for (int j = 0; j < nb; ++j)
          mdot(B, n, nb, col(AB, j), n, G.as<double>() + (int64_t)j * nb, lz.part.as<double>(), s);
        std::vector<double> gh((size_t)nb * nb), gs((size_t)nb * nb);
        TM_CK(cudaMemcpyAsync(gh.data(), G.p, gh.size() * 8, cudaMemcpyDeviceToHost, s));
        TM_CK(cudaStreamSynchronize(s));
        for (int j = 0; j < nb; ++j)
          for (int i = 0; i < nb; ++i) {
            const double gij = gh[(size_t)j * nb + i], gji = gh[(size_t)i * nb + j];
            gs[(size_t)j * nb + i] = imp[j] < imp[i] ? gij : imp[i] < imp[j] ? gji : 0.5 * (gij + gji);
          }
        TM_CK(cudaMemcpyAsync(G.p, gs.data(), gs.size() * 8, cudaMemcpyHostToDevice, s));
        small_symeig(G.as<double>(), nb, Gw.as<double>(), Gz.as<double>(), s, nb);
        std::vector<double> gw(nb), gz((size_t)nb * nb);
        TM_CK(cudaMemcpyAsync(gw.data(), Gw.p, nb * 8, cudaMemcpyDeviceToHost, s));
        TM_CK(cudaMemcpyAsync(gz.data(), Gz.p, (size_t)nb * nb * 8, cudaMemcpyDeviceToHost, s));
        TM_CK(cudaStreamSynchronize(s));
        std::vector<int> ord(nb);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return std::fabs(gw[a]) > std::fabs(gw[b]); });
        std::vector<double> Y((size_t)nb * nb), tha(nb), impn(nb, 0.0);
        for (int c = 0; c < nb; ++c) {
          tha[c] = gw[ord[c]];
          for (int j = 0; j < nb; ++j) {
            const double y = gz[(size_t)ord[c] * nb + j];
            Y[(size_t)c * nb + j] = y;
            impn[c] += y * y * imp[j];
          }
        }
        TM_CK(cudaMemcpyAsync(lz.Ysel.p, Y.data(), Y.size() * 8, cudaMemcpyHostToDevice, s));
        basis_combine(B, n, nb, lz.Ysel.as<double>(), nb, XB.as<double>(), n, n, s);
        basis_combine(AB.as<double>(), n, nb, lz.Ysel.as<double>(), nb, AXB.as<double>(), n, n, s);
        // thick restart on the leading Ritz pairs; the wanted residual block
        // goes to the columns after them
        const int keep = std::min(nb, cap - nev);
        TM_CK(cudaMemcpyAsync(B, XB.p, (size_t)keep * n * 8, cudaMemcpyDeviceToDevice, s));
        TM_CK(cudaMemcpyAsync(AB.p, AXB.p, (size_t)keep * n * 8, cudaMemcpyDeviceToDevice, s));
        for (int c = 0; c < keep; ++c) imp[c] = impn[c];
        TM_CK(cudaMemcpyAsync(th.p, tha.data(), nev * 8, cudaMemcpyHostToDevice, s));
        resid_kernel<<<blocks_for(n), 256, 0, s>>>(AB.as<double>(), B, n, nev, th.as<double>(),
                                                     B + (int64_t)keep * n, n);
        TM_CKK("resid");
        std::vector<double> rn(nev);
        bool est_ok = true;
        max_resid = 0.0;
        for (int i = 0; i < nev; ++i) {
          thv[i] = tha[i];
          rn[i] = norm_host(B + (int64_t)(keep + i) * n);
          max_resid = std::max(max_resid, rn[i] / std::fabs(tha[i]));
          if (!(rn[i] <= 0.5 * tol * std::fabs(tha[i]))) est_ok = false;
        }
        if (est_ok && verified < 3) {
          // verification: FP64-accurate products of the wanted Ritz vectors,
          // Rayleigh quotients and true residuals
          ++verified;
          bool ok_all = true;
          max_resid = 0.0;
          for (int i = 0; i < nev; ++i) {
            double* xi = B + (int64_t)i * n;
            double* axi = col(AB, i);
            prod64(xi, axi);
            imp[i] = 0.0;
            double q = 0.0;
            mdot(xi, n, 1, axi, n, lz.h1.as<double>(), lz.part.as<double>(), s);
            TM_CK(cudaMemcpyAsync(&q, lz.h1.p, 8, cudaMemcpyDeviceToHost, s));
            TM_CK(cudaStreamSynchronize(s));
            thv[i] = q;
            tha[i] = q;
          }
          TM_CK(cudaMemcpyAsync(th.p, tha.data(), nev * 8, cudaMemcpyHostToDevice, s));
          resid_kernel<<<blocks_for(n), 256, 0, s>>>(AB.as<double>(), B, n, nev, th.as<double>(),
                                                       B + (int64_t)keep * n, n);
          TM_CKK("resid");
          for (int i = 0; i < nev; ++i) {
            rn[i] = norm_host(B + (int64_t)(keep + i) * n);
            max_resid = std::max(max_resid, rn[i] / std::fabs(thv[i]));
            if (!(rn[i] <= tol * std::max(std::fabs(thv[i]), 1e-300))) ok_all = false;
          }
          if (ok_all) {
            refined = true;
            break;
          }
        }
        if (round + 1 == kRefineRounds) break;
        // orthonormalise the residual block against B (CGS2) and give it FP32
        // products; a column that vanishes is dropped
        nb = keep;
        for (int i = 0; i < nev; ++i) {
          double* rv = B + (int64_t)(keep + i) * n;
          double* dst = B + (int64_t)nb * n;
          if (dst != rv) TM_CK(cudaMemcpyAsync(dst, rv, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
          const double r0 = norm_host(dst);
          for (int pass = 0; pass < 2; ++pass) {
            mdot(B, n, nb, dst, n, lz.h1.as<double>(), lz.part.as<double>(), s);
            maxpy(B, n, nb, lz.h1.as<double>(), dst, n, s);
          }
          nrm2sq(dst, n, lz.nsq.as<double>(), lz.part.as<double>(), s);
          double q = 0.0;
          TM_CK(cudaMemcpyAsync(&q, lz.nsq.p, 8, cudaMemcpyDeviceToHost, s));
          TM_CK(cudaStreamSynchronize(s));
          if (!(q > 1e-24 * r0 * r0) || !(r0 > 0.0)) continue;
          normalize(dst, lz.nsq.as<double>(), dst, nullptr, n, s);
          prod32(dst, col(AB, nb));
          imp[nb] = 1.0;
          ++nb;
        }
      }
      if (refined) TM_CK(cudaMemcpyAsync(XB.p, B, (size_t)nev * n * 8, cudaMemcpyDeviceToDevice, s));
      if (cluster) {
        XB.alloc((size_t)nev * n * 8);
        TM_CK(cudaMemcpyAsync(XB.p, lz.v(0), (size_t)nev * n * 8, cudaMemcpyDeviceToDevice, s));
      }
      // final Ritz vectors into V's leading columns
      TM_CK(cudaMemcpyAsync(lz.v(0), XB.p, (size_t)nev * n * 8, cudaMemcpyDeviceToDevice, s));
      if (refined) {
        theta = thv;
        done = true;
      } else {
        // FP64 continuation from the refined vectors
        DBuf start;
        start.alloc((size_t)n * 8);
        TM_CK(cudaMemsetAsync(start.p, 0, (size_t)n * 8, s));
        for (int i = 0; i < nev; ++i)
          axpby(1.0, start.as<double>(), 1.0, lz.v(i), start.as<double>(), n, s);
        int mv = lz.matvecs, mv64 = lz.matvecs64, rs = lz.restarts;
        lz.matvecs = lz.matvecs64 = lz.restarts = 0;
        lz.start(start.as<double>(), seed);
        lz.matvecs += mv;
        lz.matvecs64 += mv64;
        lz.restarts += rs;
        lz.conv_tol = tol;
        r = lz.run(nev, false, 200, [&](const Lanczos::CycleResult& rr) {
          for (int i = 0; i < nev; ++i)
            if (!lz.conv_one(rr, i)) return false;
          return true;
        }, &ok);
        lz.rotate(r, nev);
        theta.assign(r.theta.begin(), r.theta.begin() + nev);
        max_resid = 0;
        for (int i = 0; i < nev; ++i) max_resid = std::max(max_resid, r.resid[i] / std::fabs(r.theta[i]));
        done = ok;
      }
    } else {
      lz.conv_tol = tol;
      r = lz.run(nev, false, 300, [&](const Lanczos::CycleResult& rr) {
        for (int i = 0; i < nev; ++i)
          if (!lz.conv_one(rr, i)) return false;
        return true;
      }, &ok);
      lz.rotate(r, nev);
      theta.assign(r.theta.begin(), r.theta.begin() + nev);
      max_resid = 0;
      for (int i = 0; i < nev; ++i) max_resid = std::max(max_resid, r.resid[i] / std::fabs(r.theta[i]));
      done = ok;
    }
    info.matvecs += lz.matvecs;
    info.matvecs_f64 += lz.matvecs64;
    info.restarts += lz.restarts;
    info.ncv = ncv;
    ++attempts;
    if (!done) {
      ncv += 2;
      if (ncv >= n) ncv = (int)n - 1;
    }
  }
  info.nconv = done ? nev : 0;
  info.max_resid = max_resid;
  for (int i = 0; i < nev && i < (int)theta.size(); ++i) vals[i] = theta[i];
  if (vecs_host && Lz) {
    TM_CK(cudaMemcpyAsync(vecs_host, Lz->v(0), (size_t)nev * n * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
  }
  const_cast<Op&>(op).matvecs += info.matvecs;
  info.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (info_out) *info_out = info;
  return done ? TM_OK : TM_ERR_NOCONV;
}

}  // namespace ltm
