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
// Mixed precision (TM_EIGS_MIXED): Lanczos with an FP32 basis and FP32
// matvecs until the Ritz residuals reach the FP32 noise floor, then the
// refinement of refine_mixed: FP64-accurate products only for the nev wanted
// Ritz vectors, everything else in FP32, and acceptance on true FP64
// residuals (the same test as the FP64 path).  FP64 Lanczos resumes from the
// refined vectors only when the refinement does not get there.
#include <algorithm>
#include <chrono>
#include <functional>
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
// y = A x / S in double-float storage with FP64-accurate arithmetic (S: the
// FP32 products' scale)
void apply_refine_dd(const Op& op, const dfloat* x, dfloat* y, double S, cudaStream_t s);

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

int blocks_for(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 8));
}

// Eigen-decomposition of a small symmetric matrix (m <= 64) on the host:
// cyclic Jacobi (Golub & Van Loan, Alg. 8.5.2).  A: column-major with leading
// dimension lda (symmetrised on entry); w[k] eigenvalues, Z[k*m + j] the
// components of eigenvector k.  Microseconds for the projected matrices here,
// where a one-warp device kernel costs about a millisecond per call.
void sym_eig_host(const double* Ain, int m, int lda, double* w, double* Z) {
  std::vector<double> A((size_t)m * m);
  for (int c = 0; c < m; ++c)
    for (int r = 0; r < m; ++r) A[r + (size_t)c * m] = 0.5 * (Ain[r + (size_t)c * lda] + Ain[c + (size_t)r * lda]);
  for (int c = 0; c < m; ++c)
    for (int r = 0; r < m; ++r) Z[r + (size_t)c * m] = (r == c) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int c = 0; c < m; ++c)
      for (int r = 0; r < m; ++r) {
        const double v = A[r + (size_t)c * m] * A[r + (size_t)c * m];
        tot += v;
        if (r != c) off += v;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = A[p + (size_t)q * m];
        if (apq == 0.0) continue;
        const double app = A[p + (size_t)p * m], aqq = A[q + (size_t)q * m];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int r = 0; r < m; ++r) {
          const double arp = A[r + (size_t)p * m], arq = A[r + (size_t)q * m];
          A[r + (size_t)p * m] = c * arp - sn * arq;
          A[r + (size_t)q * m] = sn * arp + c * arq;
        }
        for (int r = 0; r < m; ++r) {
          const double apr = A[p + (size_t)r * m], aqr = A[q + (size_t)r * m];
          A[p + (size_t)r * m] = c * apr - sn * aqr;
          A[q + (size_t)r * m] = sn * apr + c * aqr;
        }
        for (int r = 0; r < m; ++r) {
          const double zrp = Z[r + (size_t)p * m], zrq = Z[r + (size_t)q * m];
          Z[r + (size_t)p * m] = c * zrp - sn * zrq;
          Z[r + (size_t)q * m] = sn * zrp + c * zrq;
        }
      }
  }
  for (int k = 0; k < m; ++k) w[k] = A[k + (size_t)k * m];
}

// G y = theta M y for symmetric G and symmetric positive definite M (m <=
// 64), by Cholesky M = L L^T and the standard problem L^-1 G L^-T.  Column-
// major inputs with leading dimension m.  Z[k*m + j]: eigenvector k,
// M-orthonormal.  Returns false when M is not numerically positive definite.
bool gen_sym_eig_host(const double* G, const double* M, int m, double* w, double* Z) {
  std::vector<double> L((size_t)m * m, 0.0);
  for (int j = 0; j < m; ++j) {
    double d = M[j + (size_t)j * m];
    for (int k = 0; k < j; ++k) d -= L[j + (size_t)k * m] * L[j + (size_t)k * m];
    if (!(d > 0.0)) return false;
    const double ljj = std::sqrt(d);
    L[j + (size_t)j * m] = ljj;
    for (int i = j + 1; i < m; ++i) {
      double v = 0.5 * (M[i + (size_t)j * m] + M[j + (size_t)i * m]);
      for (int k = 0; k < j; ++k) v -= L[i + (size_t)k * m] * L[j + (size_t)k * m];
      L[i + (size_t)j * m] = v / ljj;
    }
  }
  // T = L^-1 G (column by column), then A = L^-1 T^T
  std::vector<double> T((size_t)m * m), A((size_t)m * m);
  auto fsolve = [&](const double* b, double* x) {  // L x = b
    for (int i = 0; i < m; ++i) {
      double v = b[i];
      for (int k = 0; k < i; ++k) v -= L[i + (size_t)k * m] * x[k];
      x[i] = v / L[i + (size_t)i * m];
    }
  };
  std::vector<double> col(m), tr(m);
  for (int j = 0; j < m; ++j) {
    for (int i = 0; i < m; ++i) col[i] = 0.5 * (G[i + (size_t)j * m] + G[j + (size_t)i * m]);
    fsolve(col.data(), &T[(size_t)j * m]);
  }
  for (int j = 0; j < m; ++j) {
    for (int i = 0; i < m; ++i) tr[i] = T[j + (size_t)i * m];  // row j of T
    fsolve(tr.data(), &A[(size_t)j * m]);
  }
  std::vector<double> Zs((size_t)m * m);
  sym_eig_host(A.data(), m, m, w, Zs.data());
  // y = L^-T z
  for (int k = 0; k < m; ++k) {
    const double* z = &Zs[(size_t)k * m];
    double* y = &Z[(size_t)k * m];
    for (int i = m - 1; i >= 0; --i) {
      double v = z[i];
      for (int r = i + 1; r < m; ++r) v -= L[r + (size_t)i * m] * y[r];
      y[i] = v / L[i + (size_t)i * m];
    }
  }
  return true;
}

struct Lanczos {
  const Op& op;
  cudaStream_t s;
  int64_t n, ld;  // vector length, basis leading dimension
  int m;
  DBuf V, W, x32, y32, h1, h2, part, nsq, Hd, wd, Zd, Ysel;
  int matvecs = 0, matvecs64 = 0, restarts = 0;

  int vcols = 0;  // columns of V allocated (m + 1 once full)

  // cols0 > 0: allocate only that many basis columns (the mixed path needs
  // the FP64 basis for the wanted vectors only); ensure_full() grows V.
  Lanczos(const Op& o, int ncv, cudaStream_t st, int cols0 = 0) : op(o), s(st), n(o.n), ld(col_ld(o.n)), m(ncv) {
    vcols = (cols0 > 0) ? std::min(cols0, m + 1) : m + 1;
    V.alloc((size_t)vcols * ld * sizeof(double));
    W.alloc((size_t)n * sizeof(double));
    h1.alloc(64 * 8);
    h2.alloc(64 * 8);
    part.alloc(red_part_bytes(16));
    nsq.alloc(8);
    Hd.alloc((size_t)(m + 1) * (m + 1) * 8);
    wd.alloc(64 * 8);
    Zd.alloc(64 * 64 * 8);
    Ysel.alloc(64 * 64 * 8);
  }
  double* v(int j) const { return V.as<double>() + (int64_t)j * ld; }

  void ensure_full() {
    if (vcols >= m + 1) return;
    DBuf nv;
    nv.alloc((size_t)(m + 1) * ld * sizeof(double));
    TM_CK(cudaMemcpyAsync(nv.p, V.p, (size_t)vcols * ld * sizeof(double), cudaMemcpyDeviceToDevice, s));
    std::swap(V.p, nv.p);
    std::swap(V.bytes, nv.bytes);
    std::swap(V.st, nv.st);
    vcols = m + 1;
  }

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
      mdot32(v(0), ld, j + 1, y32.as<float>(), S, n, h1.as<double>(), part.as<double>(), s);
      maxpy32(v(0), ld, j + 1, h1.as<double>(), y32.as<float>(), S, w, n, s);
    } else {
      apply_internal(op, v(j), w, nullptr, nullptr, false, s);
      ++matvecs64;
      mdot(v(0), ld, j + 1, w, n, h1.as<double>(), part.as<double>(), s);
      maxpy(v(0), ld, j + 1, h1.as<double>(), w, n, s);
    }
    ++matvecs;
    mdot(v(0), ld, j + 1, w, n, h2.as<double>(), part.as<double>(), s);
    maxpy(v(0), ld, j + 1, h2.as<double>(), w, n, s);
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
    CycleResult r;
    std::vector<double> th(m), H((size_t)(m + 1) * (m + 1));
    r.Z.resize((size_t)m * m);
    TM_CK(cudaMemcpyAsync(H.data(), Hd.p, H.size() * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    sym_eig_host(H.data(), m, m + 1, th.data(), r.Z.data());
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
    basis_rotate(V.as<double>(), ld, m, Ysel.as<double>(), k, n, s);
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

// h1[i] = H(i, j) / S for i < j: the couplings of v(j) to the earlier basis
// vectors that the recurrence already knows (beta(j-1), or after a thick
// restart the couplings to the kept Ritz vectors; zero otherwise).
__global__ void hprev32_kernel(const double* H, int ld, int j, double S, double* h1) {
  const int i = threadIdx.x;
  if (i < j) h1[i] = H[i + (int64_t)j * ld] / S;
}

// FP32-basis thick-restart Lanczos for the FP32 phase of mixed precision
// (ncv <= 16).  The matvec returns y = T v / S; the Gram-Schmidt runs on y
// with FP32 data and FP64 reductions, and S is folded into H, so no large
// factor ever enters FP32 storage.  Per step: alpha = v(j) . y (one dot over
// two vectors), then y - alpha v(j) - H(0:j, j) v(0:j) with the known
// couplings and the full re-orthogonalisation dots in one sweep over the
// basis, and the correction with the norm in a second sweep (Lanczos with
// full re-orthogonalisation; the first Gram-Schmidt pass of CGS2 is the
// three-term recurrence itself).
struct Lanczos32 {
  const Op& op;
  cudaStream_t s;
  int64_t n, ld;  // vector length, basis leading dimension
  int m;
  int mp;  // size of the current projection (m, or fewer after a mid-cycle stop)
  DBuf V, W, Y, h1, h2, part, nsq, Hd, wd, Zd, Ysel;
  int matvecs = 0, restarts = 0;
  bool stagnation_stop = true;

  Lanczos32(const Op& o, int ncv, cudaStream_t st) : op(o), s(st), n(o.n), ld(col_ld(o.n)), m(ncv), mp(ncv) {
    V.alloc((size_t)(m + 1) * ld * 4);
    W.alloc((size_t)n * 4);
    Y.alloc((size_t)n * 4);
    h1.alloc(64 * 8);
    h2.alloc(64 * 8);
    part.alloc(red_part_bytes(16));
    nsq.alloc(8);
    Hd.alloc((size_t)(m + 1) * (m + 1) * 8);
    wd.alloc(64 * 8);
    Zd.alloc(64 * 64 * 8);
    Ysel.alloc(64 * 64 * 8);
  }
  float* v(int j) const { return V.as<float>() + (int64_t)j * ld; }

  void start(uint64_t seed) {
    TM_CK(cudaMemsetAsync(Hd.p, 0, (size_t)(m + 1) * (m + 1) * 8, s));
    fill_uniform_f32(W.as<float>(), n, seed, s);
    nrm2sq_f32(W.as<float>(), n, nsq.as<double>(), part.as<double>(), s);
    normalize_f32(W.as<float>(), nsq.as<double>(), v(0), n, s);
  }

  double S = 0.0;  // scale of the FP32 products: y = T v / S

  void step(int j) {
    S = apply_internal(op, nullptr, nullptr, v(j), Y.as<float>(), true, s);
    ++matvecs;
    hprev32_kernel<<<1, 64, 0, s>>>(Hd.as<double>(), m + 1, j, S, h1.as<double>());
    TM_CKK("hprev32");
    mdot_f32(v(j), ld, 1, Y.as<float>(), n, h1.as<double>() + j, part.as<double>(), s);
    axpy_dot_f32(v(0), ld, j + 1, h1.as<double>(), Y.as<float>(), W.as<float>(), n, h2.as<double>(),
                 part.as<double>(), s);
    axpy_nrm_f32(v(0), ld, j + 1, h2.as<double>(), W.as<float>(), n, nsq.as<double>(), part.as<double>(), s);
    hcol32_kernel<<<1, 64, 0, s>>>(Hd.as<double>(), m + 1, j, h1.as<double>(), h2.as<double>(), nsq.as<double>(), S);
    TM_CKK("hcol32");
    normalize_f32(W.as<float>(), nsq.as<double>(), v(j + 1), n, s);
  }

  // Rayleigh-Ritz on the first mp basis vectors
  Lanczos::CycleResult project() {
    Lanczos::CycleResult r;
    std::vector<double> th(mp), H((size_t)(m + 1) * (m + 1));
    r.Z.resize((size_t)mp * mp);
    TM_CK(cudaMemcpyAsync(H.data(), Hd.p, H.size() * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    sym_eig_host(H.data(), mp, m + 1, th.data(), r.Z.data());
    r.beta = H[mp + (size_t)(mp - 1) * (m + 1)];
    r.order.resize(mp);
    std::iota(r.order.begin(), r.order.end(), 0);
    std::stable_sort(r.order.begin(), r.order.end(),
                     [&](int a, int b) { return std::fabs(th[a]) > std::fabs(th[b]); });
    for (int i = 0; i < mp; ++i) {
      int c = r.order[i];
      r.theta.push_back(th[c]);
      r.resid.push_back(std::fabs(r.beta * r.Z[(size_t)c * mp + (mp - 1)]));
    }
    return r;
  }

  std::vector<double> ysel(const Lanczos::CycleResult& r, int k) const {
    std::vector<double> Y((size_t)mp * k);
    for (int c = 0; c < k; ++c)
      for (int j = 0; j < mp; ++j) Y[(size_t)c * mp + j] = r.Z[(size_t)r.order[c] * mp + j];
    return Y;
  }

  void restart(const Lanczos::CycleResult& r, int k) {
    std::vector<double> Yh = ysel(r, k);
    TM_CK(cudaMemcpyAsync(Ysel.p, Yh.data(), Yh.size() * 8, cudaMemcpyHostToDevice, s));
    rotate_f32(V.as<float>(), ld, mp, Ysel.as<double>(), k, n, s);
    TM_CK(cudaMemcpyAsync(v(k), v(mp), (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    std::vector<double> H((size_t)(m + 1) * (m + 1), 0.0);
    for (int i = 0; i < k; ++i) {
      H[i + (size_t)i * (m + 1)] = r.theta[i];
      double cpl = r.beta * r.Z[(size_t)r.order[i] * mp + (mp - 1)];
      H[k + (size_t)i * (m + 1)] = cpl;
      H[i + (size_t)k * (m + 1)] = cpl;
    }
    TM_CK(cudaMemcpyAsync(Hd.p, H.data(), H.size() * 8, cudaMemcpyHostToDevice, s));
    ++restarts;
  }

  // Ritz vectors first .. first+k-1 as FP32 columns (leading dimension ld)
  void ritz_f32(const Lanczos::CycleResult& r, int first, int k, float* out) {
    std::vector<double> Yh((size_t)mp * k);
    for (int c = 0; c < k; ++c)
      for (int j = 0; j < mp; ++j) Yh[(size_t)c * mp + j] = r.Z[(size_t)r.order[first + c] * mp + j];
    TM_CK(cudaMemcpyAsync(Ysel.p, Yh.data(), Yh.size() * 8, cudaMemcpyHostToDevice, s));
    combine_f32(V.as<float>(), ld, mp, Ysel.as<double>(), k, out, ld, n, s);
  }

  // Products of Ritz vectors first .. first+k-1 from the Lanczos relation
  // A V_m = V_m H + beta v_m e_m^T: A x = theta x + beta (e_m^T y) v_m, so
  // A x / S = V_{m+1} [theta y; beta y_m] / S with no product of the
  // operator (FP32 columns, leading dimension ld).
  void ritz_f32_prod(const Lanczos::CycleResult& r, int first, int k, float* out) {
    const int m1 = mp + 1;
    std::vector<double> Yh((size_t)m1 * k);
    for (int c = 0; c < k; ++c) {
      const int col = r.order[first + c];
      const double th = r.theta[first + c];
      for (int j = 0; j < mp; ++j) Yh[(size_t)c * m1 + j] = th * r.Z[(size_t)col * mp + j] / S;
      Yh[(size_t)c * m1 + mp] = r.beta * r.Z[(size_t)col * mp + (mp - 1)] / S;
    }
    TM_CK(cudaMemcpyAsync(Ysel.p, Yh.data(), Yh.size() * 8, cudaMemcpyHostToDevice, s));
    combine_f32(V.as<float>(), ld, m1, Ysel.as<double>(), k, out, ld, n, s);
  }

  // double-float Ritz vectors: out[:, c] = V32 * Z[:, order[c]], c < k <= 8
  void ritz_dd(const Lanczos::CycleResult& r, int k, dfloat* out, int64_t ldo) {
    std::vector<double> Yh = ysel(r, k);
    TM_CK(cudaMemcpyAsync(Ysel.p, Yh.data(), Yh.size() * 8, cudaMemcpyHostToDevice, s));
    combine_f32_dd(V.as<float>(), ld, mp, Ysel.as<double>(), k, out, ldo, n, s);
  }

  // FP64 Ritz vectors: out[:, c] = V32 * Z[:, order[c]], c < k (leading dimension ldo)
  void ritz_f64(const Lanczos::CycleResult& r, int k, double* out, int64_t ldo) {
    std::vector<double> Yh = ysel(r, k);
    TM_CK(cudaMemcpyAsync(Ysel.p, Yh.data(), Yh.size() * 8, cudaMemcpyHostToDevice, s));
    combine_f32_f64(V.as<float>(), ld, mp, Ysel.as<double>(), k, out, ldo, n, s);
  }

  template <class Conv>
  Lanczos::CycleResult run(int nev, int max_cycles, Conv conv) {
    int k = 0;
    Lanczos::CycleResult r;
    double best = 1e300;
    int stall = 0;
    for (int cyc = 0; cyc < max_cycles; ++cyc) {
      // once the previous cycle came within reach of the FP32 floor, test
      // after every step (a Rayleigh-Ritz of the first j + 1 vectors), so the
      // phase stops at the first product that gets there
      const bool each = cyc > 0 && best <= 5e-5;
      for (int j = k; j < m; ++j) {
        step(j);
        if (each && j + 1 < m && j + 1 > nev + 1) {
          mp = j + 1;
          r = project();
          if (conv(r)) return r;
        }
      }
      mp = m;
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
constexpr int kMaxRefineNev = 8;

// Ritz pairs of the refinement subspace [X0 | B32] (X0: nx double-float
// columns with FP64-accurate products AX0 = A X0 / S; B32: FP32 columns
// nx..nb-1 with FP32 products AB32 = A b / S).  For each wanted pair c < nv
// with coefficients Y(:, c) and ts = theta_c / S:
//   x = X0 y_x + B32 y_b,  ax/S = AX0 y_x + AB32 y_b,  r/S = ax/S - ts x,
// the X0 part in double-float, the B32 part in FP32 (its weights are at the
// FP32 noise level).  Writes r / S as FP32 into R32 (column c), x into Xo
// (double-float), and the block partial sums of ||r/S||^2 (FP32 per thread)
// into part[block * NVW + c].  All column blocks have an even leading
// dimension ld and 16-byte aligned columns; a thread takes two elements.
template <int NVW>
__global__ void __launch_bounds__(256) ritz_resid_kernel(const dfloat* __restrict__ X0,
                                                         const dfloat* __restrict__ AX0, int nx,
                                                         const float* __restrict__ B32,
                                                         const float* __restrict__ AB32, int nb,
                                                         const double* __restrict__ Y, int nv,
                                                         const double* __restrict__ theta_s,
                                                         float* __restrict__ R32, dfloat* __restrict__ Xo,
                                                         int64_t n, int64_t ld, double* __restrict__ part) {
  __shared__ dfloat Yd[48 * NVW];
  __shared__ float Yf[48 * NVW];
  __shared__ dfloat th[NVW];
  for (int t = threadIdx.x; t < nb * nv; t += blockDim.x) {
    Yd[t] = dfloat(Y[t]);
    Yf[t] = (float)Y[t];
  }
  if (threadIdx.x < nv) th[threadIdx.x] = dfloat(-theta_s[threadIdx.x]);
  __syncthreads();
  float acc[NVW];
#pragma unroll
  for (int c = 0; c < NVW; ++c) acc[c] = 0.f;
  auto ld2 = [](const dfloat* p, int64_t i, dfloat& a, dfloat& b) {
    const float4 v = reinterpret_cast<const float4*>(p)[i];
    a = dfloat(v.x, v.y);
    b = dfloat(v.z, v.w);
  };
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += st) {
    dfloat x0[NVW], x1[NVW], a0[NVW], a1[NVW];
    float2 xs[NVW], axs[NVW];
#pragma unroll
    for (int c = 0; c < NVW; ++c) {
      x0[c] = x1[c] = a0[c] = a1[c] = dfloat(0.f, 0.f);
      xs[c] = axs[c] = make_float2(0.f, 0.f);
    }
    // unrolled so that several columns' loads are in flight per thread
#pragma unroll 4
    for (int j = 0; j < nx; ++j) {
      dfloat xa, xb, aa, ab;
      ld2(X0 + (int64_t)j * ld, i, xa, xb);
      ld2(AX0 + (int64_t)j * ld, i, aa, ab);
#pragma unroll
      for (int c = 0; c < NVW; ++c)
        if (c < nv) {
          const dfloat y = Yd[c * nb + j];
          x0[c] = df_fma(xa, y, x0[c]);
          x1[c] = df_fma(xb, y, x1[c]);
          a0[c] = df_fma(aa, y, a0[c]);
          a1[c] = df_fma(ab, y, a1[c]);
        }
    }
#pragma unroll 4
    for (int j = nx; j < nb; ++j) {
      const float2 bv = reinterpret_cast<const float2*>(B32 + (int64_t)j * ld)[i];
      const float2 abv = reinterpret_cast<const float2*>(AB32 + (int64_t)j * ld)[i];
#pragma unroll
      for (int c = 0; c < NVW; ++c)
        if (c < nv) {
          const float y = Yf[c * nb + j];
          xs[c].x = fmaf(bv.x, y, xs[c].x);
          xs[c].y = fmaf(bv.y, y, xs[c].y);
          axs[c].x = fmaf(abv.x, y, axs[c].x);
          axs[c].y = fmaf(abv.y, y, axs[c].y);
        }
    }
#pragma unroll
    for (int c = 0; c < NVW; ++c)
      if (c < nv) {
        const dfloat xx0 = x0[c] + dfloat(xs[c].x, 0.f), xx1 = x1[c] + dfloat(xs[c].y, 0.f);
        const dfloat r0 = df_fma(th[c], xx0, a0[c] + dfloat(axs[c].x, 0.f));
        const dfloat r1 = df_fma(th[c], xx1, a1[c] + dfloat(axs[c].y, 0.f));
        const float f0 = r0.hi + r0.lo, f1 = r1.hi + r1.lo;
        reinterpret_cast<float2*>(R32 + (int64_t)c * ld)[i] = make_float2(f0, f1);
        reinterpret_cast<float4*>(Xo + (int64_t)c * ld)[i] = make_float4(xx0.hi, xx0.lo, xx1.hi, xx1.lo);
        acc[c] = fmaf(f0, f0, fmaf(f1, f1, acc[c]));
      }
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t i = n - 1;
    for (int c = 0; c < nv; ++c) {
      dfloat x(0.f, 0.f), ax(0.f, 0.f);
      float xs = 0.f, axs = 0.f;
      for (int j = 0; j < nx; ++j) {
        x = df_fma(X0[(int64_t)j * ld + i], Yd[c * nb + j], x);
        ax = df_fma(AX0[(int64_t)j * ld + i], Yd[c * nb + j], ax);
      }
      for (int j = nx; j < nb; ++j) {
        xs = fmaf(B32[(int64_t)j * ld + i], Yf[c * nb + j], xs);
        axs = fmaf(AB32[(int64_t)j * ld + i], Yf[c * nb + j], axs);
      }
      const dfloat xx = x + dfloat(xs, 0.f);
      const dfloat r = df_fma(th[c], xx, ax + dfloat(axs, 0.f));
      const float f = r.hi + r.lo;
      R32[(int64_t)c * ld + i] = f;
      Xo[(int64_t)c * ld + i] = xx;
      acc[c] = fmaf(f, f, acc[c]);
    }
  }
  __shared__ double sh[8][NVW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NVW; ++c) {
    double v = (double)acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < NVW) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q][threadIdx.x];
    part[(int64_t)blockIdx.x * NVW + threadIdx.x] = t;
  }
}

// out = (float)(in * scale)
__global__ void f64_to_f32_scaled_kernel(const double* __restrict__ in, double scale, float* __restrict__ out,
                                         int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)(in[i] * scale);
}

// Y = R^-1 for the Cholesky factor G = R^T R of a k x k Gram matrix
// (column-major, symmetrised): X R^-1 has orthonormal columns when G = X^T X.
// Y column-major (Y[c*k + j] = (R^-1)(j, c)).  False when G is not
// numerically positive definite.
bool chol_qr_inverse(const std::vector<double>& Gin, int k, std::vector<double>& Y) {
  std::vector<double> R((size_t)k * k, 0.0);  // R[c*k + r], r <= c
  for (int c = 0; c < k; ++c) {
    for (int r = 0; r <= c; ++r) {
      double v = 0.5 * (Gin[(size_t)r + (size_t)c * k] + Gin[(size_t)c + (size_t)r * k]);
      for (int t = 0; t < r; ++t) v -= R[(size_t)r * k + t] * R[(size_t)c * k + t];
      if (r < c) {
        R[(size_t)c * k + r] = v / R[(size_t)r * k + r];
      } else {
        if (!(v > 1e-8)) return false;
        R[(size_t)c * k + c] = std::sqrt(v);
      }
    }
  }
  Y.assign((size_t)k * k, 0.0);
  for (int c = 0; c < k; ++c) {
    Y[(size_t)c * k + c] = 1.0 / R[(size_t)c * k + c];
    for (int r = c - 1; r >= 0; --r) {
      double v = 0.0;
      for (int t = r + 1; t <= c; ++t) v += R[(size_t)t * k + r] * Y[(size_t)c * k + t];
      Y[(size_t)c * k + r] = -v / R[(size_t)r * k + r];
    }
  }
  return true;
}

// FP64-accurate refinement of the FP32 phase's Ritz pairs.
//
// On GB300 FP64 arithmetic runs at a small fraction of the FP32 rate, so the
// refinement keeps FP64-level accuracy where the result needs it, in
// double-float storage and arithmetic (FP32 pipes), and FP32 everywhere
// else.  The subspace is [X0 | C]: X0 = the nev wanted Ritz vectors
// (double-float, with FP64-accurate products), C = the other FP32 Ritz vectors
// and, each round, the wanted residual block (FP32 storage, FP32 products,
// FP32 Gram-Schmidt).  C's weight in a wanted Ritz vector is at the FP32 noise
// level (~1e-7), so FP32 errors in C, in A C and in the C-rows of the projected
// matrix reach the wanted pairs only at ~1e-14 relative.  The projected matrix
// takes each entry from the side whose product is the more accurate one (A X0
// for the X0 rows).  The extra Ritz vectors carry the eigenvectors next to
// the wanted ones, which residual blocks alone resolve slowly.  When the
// estimated residuals meet tol, the Ritz vectors get FP64-accurate products
// and are accepted on the test of the FP64 path and of Spectra's
// SymEigsSolver, ||A x - theta x|| <= tol |theta|, with theta the Rayleigh
// quotient; else the verified vectors become the new X0 and the rounds go on.
// All products are kept divided by S, the FP32 products' scale, so they stay
// in the FP32 exponent range.
//
// In: fill_x0 writes the wanted Ritz vectors (orthonormal, double-float,
// leading dimension lz.ld) into the nev columns it is given; the other
// nx - nev Ritz vectors come from fill_extras (FP32 columns, and their FP32
// products A x / S when it returns the scale S > 0) or, without it, from
// lz.v(nev..nx-1).
// Out: lz.v(0..nev-1) the best Ritz vectors (FP64); thv, max_resid; true when
// accepted.
bool refine_mixed(const Op& op, Lanczos& lz, int nev, int nx, double tol, std::vector<double>& thv,
                  double& max_resid, const std::function<void(dfloat*)>& fill_x0,
                  const std::function<double(float*, float*)>& fill_extras, tm_eigs_info& info) {
  cudaStream_t s = lz.s;
  const int64_t n = lz.n, ld = lz.ld;  // every column block below has leading dimension ld
  const int cap = std::min(48, nx + 5 * nev);
  const int gblocks = blocks_for(n);
  DBuf XA, B32, AB32, R32, Xo, AXo, Wd, Yd, thd, part, bpart, dpart, Hd, hd;
  // XA = [X0 | A X0 / S] (double-float, contiguous so one sweep gives both
  // coupling rows)
  XA.alloc((size_t)2 * nev * ld * 8);
  bpart.alloc(mdot_block_part_bytes());
  dpart.alloc(dd_part_bytes(kMaxBlockW * 4));
  Hd.alloc((size_t)48 * 2 * kMaxBlockW * 8);
  hd.alloc(64 * 8);
  B32.alloc((size_t)cap * ld * 4);
  AB32.alloc((size_t)cap * ld * 4);
  R32.alloc((size_t)nev * ld * 4);
  Xo.alloc((size_t)nev * ld * 8);
  AXo.alloc((size_t)nev * ld * 8);
  Wd.alloc((size_t)ld * 8);
  Yd.alloc((size_t)48 * kMaxRefineNev * 8);
  thd.alloc(kMaxRefineNev * 8);
  part.alloc((size_t)gblocks * kMaxRefineNev * 8);
  auto f32col = [&](const DBuf& b, int j) { return b.as<float>() + (int64_t)j * ld; };
  auto x0 = [&](int j) { return XA.as<dfloat>() + (int64_t)j * ld; };          // X0 column j
  auto ax0 = [&](int j) { return XA.as<dfloat>() + (int64_t)(nev + j) * ld; };  // A X0 / S column j
  auto xo = [&](int c) { return Xo.as<dfloat>() + (int64_t)c * ld; };
  auto axo = [&](int c) { return AXo.as<dfloat>() + (int64_t)c * ld; };
  auto host_sync = [&]() { TM_CK(cudaStreamSynchronize(s)); };
  double S = 0.0;
  auto prod32 = [&](const float* x, float* y) {
    const double Sj = apply_internal(op, nullptr, nullptr, x, y, true, s);
    ++lz.matvecs;
    if (S == 0.0) S = Sj;
    if (Sj != S) fail(TM_ERR_CUDA, "inconsistent FP32 product scale");
  };
  auto proddd = [&](const dfloat* x, dfloat* y) {
    apply_refine_dd(op, x, y, S, s);
    ++lz.matvecs;
    ++lz.matvecs64;
  };
  // the final vectors back to the FP64 basis
  auto to_lz = [&](const dfloat* X) {
    for (int c = 0; c < nev; ++c) df_to_f64(X + (int64_t)c * ld, 1.0, lz.v(c), n, s);
  };

  // projected matrix G = B^T A B and Gram matrix M = B^T B of B = [X0 | C].
  // The X0 rows take FP64-accurate dots against the exact FP32 values of C: C
  // is orthogonal to X0 only to FP32 accuracy (~1e-7), the size of the
  // couplings that carry the correction, so those entries and the Gram block
  // must be exact.  The C-C block is FP32 (second order).
  std::vector<double> G((size_t)cap * cap, 0.0), M((size_t)cap * cap, 0.0);
  auto g = [&](int i, int j) -> double& { return G[(size_t)j * cap + i]; };
  auto mm = [&](int i, int j) -> double& { return M[(size_t)j * cap + i]; };
  // X0 rows of C columns j0 .. j0+cnt-1 (cnt <= 4): one sweep over XA gives
  // X0 . c (Gram) and (A X0 / S) . c (projected matrix) for the whole block
  auto x0_rows = [&](int j0, int cnt) {
    F32Cols w{};
    for (int c = 0; c < cnt; ++c) w.c[c] = f32col(B32, j0 + c);
    mdot_dd_block(XA.as<dfloat>(), ld, 2 * nev, w, cnt, n, Hd.as<double>(), 48, dpart.as<double>(), s);
    std::vector<double> h((size_t)48 * cnt);
    TM_CK(cudaMemcpyAsync(h.data(), Hd.p, h.size() * 8, cudaMemcpyDeviceToHost, s));
    host_sync();
    for (int c = 0; c < cnt; ++c) {
      const int j = j0 + c;
      for (int i = 0; i < nev; ++i) {
        mm(i, j) = mm(j, i) = h[(size_t)48 * c + i];
        g(i, j) = g(j, i) = S * h[(size_t)48 * c + nev + i];
      }
    }
  };
  // C columns j0 .. j0+cnt-1 (cnt <= 4) against columns 0 .. j0+cnt-1: one
  // sweep over B32 gives b . A w for the whole block.  The C-C blocks enter
  // the wanted pairs at second order: one side of the symmetric product
  // suffices, and the C-C Gram block is the identity (C is orthonormal to
  // FP32 accuracy, ~1e-6, which moves the wanted pairs by ~1e-6 of the
  // squared C weights, ~1e-14).
  auto add_gcols = [&](int j0, int cnt) {
    const int nv = j0 + cnt;
    F32Cols w1{};
    for (int c = 0; c < cnt; ++c) w1.c[c] = f32col(AB32, j0 + c);
    mdot_block_f32(B32.as<float>(), ld, nv, w1, cnt, n, Hd.as<double>(), 48, bpart.as<double>(), s);
    std::vector<double> h((size_t)48 * cnt);
    TM_CK(cudaMemcpyAsync(h.data(), Hd.p, h.size() * 8, cudaMemcpyDeviceToHost, s));
    host_sync();
    for (int c = 0; c < cnt; ++c) {
      const int j = j0 + c;
      const double* gl = &h[(size_t)48 * c];  // b_i . A b_j / S
      for (int i = nev; i <= j; ++i) {
        g(i, j) = g(j, i) = S * gl[i];
        mm(i, j) = mm(j, i) = (i == j) ? 1.0 : 0.0;
      }
    }
    x0_rows(j0, cnt);
  };
  // X0 block (FP64-accurate products and dots) and its rows against every C
  // column
  auto set_x0 = [&](int nb) {
    if (nev <= 4) {
      // X0^T [X0 | A X0 / S] in one sweep over XA
      mdot_dd_gram(x0(0), ld, nev, 2 * nev, n, hd.as<double>(), dpart.as<double>(), s);
      std::vector<double> gg((size_t)2 * nev * nev);
      TM_CK(cudaMemcpyAsync(gg.data(), hd.p, gg.size() * 8, cudaMemcpyDeviceToHost, s));
      host_sync();
      for (int j = 0; j < nev; ++j)
        for (int i = 0; i < nev; ++i) {
          mm(i, j) = gg[(size_t)i + (size_t)j * nev];
          g(i, j) = S * gg[(size_t)i + (size_t)(nev + j) * nev];
        }
    } else {
      for (int j = 0; j < nev; ++j) {
      std::vector<double> h(nev), q(nev);
      mdot_dd(x0(0), ld, nev, ax0(j), n, hd.as<double>(), dpart.as<double>(), s);
      TM_CK(cudaMemcpyAsync(h.data(), hd.p, nev * 8, cudaMemcpyDeviceToHost, s));
      host_sync();
      mdot_dd(x0(0), ld, nev, x0(j), n, hd.as<double>(), dpart.as<double>(), s);
      TM_CK(cudaMemcpyAsync(q.data(), hd.p, nev * 8, cudaMemcpyDeviceToHost, s));
      host_sync();
      for (int i = 0; i < nev; ++i) {
        g(i, j) = S * h[i];
        mm(i, j) = q[i];
      }
      }
    }
    for (int j = 0; j < nev; ++j)
      for (int i = 0; i < j; ++i) {
        g(i, j) = g(j, i) = 0.5 * (g(i, j) + g(j, i));
        mm(i, j) = mm(j, i) = 0.5 * (mm(i, j) + mm(j, i));
      }
    for (int j = 0; j < nev; ++j)  // FP32 copy of X0 for the FP32 Gram-Schmidt of C
      df_to_f32(x0(j), f32col(B32, j), n, s);
    for (int j = nev; j < nb; j += 4) x0_rows(j, std::min(4, nb - j));
  };
  // start: the extra Ritz vectors to FP32 with FP32 products, the wanted ones
  // with FP64-accurate products
  fill_x0(x0(0));
  for (int j = 0; j < nev; ++j) df_to_f32(x0(j), f32col(B32, j), n, s);
  bool extras_prod = false;
  if (fill_extras) {
    if (nx > nev) {
      const double Se = fill_extras(f32col(B32, nev), f32col(AB32, nev));
      if (Se > 0.0) {
        S = Se;
        extras_prod = true;
      }
    }
  } else {
    for (int j = nev; j < nx; ++j) {
      f64_to_f32_scaled_kernel<<<gblocks, 256, 0, s>>>(lz.v(j), 1.0, f32col(B32, j), n);
      TM_CKK("to_f32");
    }
  }
  if (!extras_prod)
    for (int j = nev; j < nx; ++j) prod32(f32col(B32, j), f32col(AB32, j));
  if (S == 0.0) prod32(f32col(B32, 0), f32col(AB32, 0));  // only its scale is used; set_x0 overwrites it
  for (int i = 0; i < nev; ++i) proddd(x0(i), ax0(i));
  int nb = nx;
  set_x0(nev);
  for (int j = nev; j < nb; j += 4) add_gcols(j, std::min(4, nb - j));
  int verified = 0;
  bool have_x = false;
  // after a failed verification: grow before verifying again, and accept
  // only verified pairs from then on
  bool force_grow = false, trust_bound = true;
  for (int round = 0; round < 3 * kRefineRounds; ++round) {
    // Rayleigh-Ritz on [X0 | C]
    std::vector<double> Gc((size_t)nb * nb), Mc((size_t)nb * nb);
    for (int j = 0; j < nb; ++j)
      for (int i = 0; i < nb; ++i) {
        Gc[(size_t)j * nb + i] = g(i, j);
        Mc[(size_t)j * nb + i] = mm(i, j);
      }
    std::vector<double> gw(nb), gz((size_t)nb * nb);
    if (!gen_sym_eig_host(Gc.data(), Mc.data(), nb, gw.data(), gz.data())) break;
    std::vector<int> ord(nb);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return std::fabs(gw[a]) > std::fabs(gw[b]); });
    std::vector<double> Y((size_t)nb * nev), tha(nev), ths(nev);
    for (int c = 0; c < nev; ++c) {
      tha[c] = gw[ord[c]];
      ths[c] = tha[c] / S;
      for (int j = 0; j < nb; ++j) Y[(size_t)c * nb + j] = gz[(size_t)ord[c] * nb + j];
    }
    TM_CK(cudaMemcpyAsync(Yd.p, Y.data(), Y.size() * 8, cudaMemcpyHostToDevice, s));
    TM_CK(cudaMemcpyAsync(thd.p, ths.data(), nev * 8, cudaMemcpyHostToDevice, s));
    // wanted Ritz vectors (double-float) and residuals (FP32 copy and norms)
    auto ritz_kernel = (nev <= 4) ? ritz_resid_kernel<4> : ritz_resid_kernel<kMaxRefineNev>;
    const int pstride = (nev <= 4) ? 4 : kMaxRefineNev;  // the kernel's per-block stride
    ritz_kernel<<<gblocks, 256, 0, s>>>(x0(0), ax0(0), nev, B32.as<float>(), AB32.as<float>(), nb, Yd.as<double>(),
                                        nev, thd.as<double>(), R32.as<float>(), Xo.as<dfloat>(), n, ld,
                                        part.as<double>());
    TM_CKK("ritz_resid");
    std::vector<double> ph((size_t)gblocks * kMaxRefineNev), rn(nev, 0.0);
    TM_CK(cudaMemcpyAsync(ph.data(), part.p, ph.size() * 8, cudaMemcpyDeviceToHost, s));
    host_sync();
    have_x = true;
    for (int b = 0; b < gblocks; ++b)
      for (int c = 0; c < nev; ++c) rn[c] += ph[(size_t)b * pstride + c];
    // The estimate differs from the true residual of x only through the
    // FP32 products in the C block: |r - r_est| <= eps32 ||A|| ||y_c||, with
    // eps32 = (2L + 8) 2^-24 per FP32 product (one rounding per butterfly
    // level and scaling step; A is entrywise non-negative, so ||A|x||| <=
    // ||A|| ||x||) taken 4x, and ||A|| <= 1.01 |theta_0|.  The FP64-accurate
    // products of X0 are the ones a verification would use too.
    const double eps32 = 4.0 * (2.0 * op.L + 8.0) * std::ldexp(1.0, -24);
    bool est_ok = true, certified = true;
    max_resid = 0.0;
    ++info.refine_rounds;
    for (int c = 0; c < nev; ++c) {
      rn[c] = S * std::sqrt(std::max(rn[c], 0.0));
      thv[c] = tha[c];
      max_resid = std::max(max_resid, rn[c] / std::fabs(tha[c]));
      double yc2 = 0.0;
      for (int j = nev; j < nb; ++j) yc2 += Y[(size_t)c * nb + j] * Y[(size_t)c * nb + j];
      const double bound = eps32 * 1.01 * std::fabs(tha[0]) * std::sqrt(yc2);
      if (!(rn[c] <= 0.5 * tol * std::fabs(tha[c]))) est_ok = false;
      if (!(rn[c] + bound <= tol * std::fabs(tha[c]))) certified = false;
    }
    info.refine_est = max_resid;
    if (est_ok && certified && trust_bound) {
      to_lz(xo(0));
      info.refine_outcome = 1;
      return true;
    }
    if (est_ok && !force_grow && verified < 3) {
      // verification with FP64-accurate products of the Ritz vectors
      ++verified;
      bool ok_all = true;
      max_resid = 0.0;
      for (int c = 0; c < nev; ++c) {
        proddd(xo(c), axo(c));
        double q[2];
        mdot_dd(xo(c), ld, 1, axo(c), n, hd.as<double>(), dpart.as<double>(), s);
        TM_CK(cudaMemcpyAsync(&q[0], hd.p, 8, cudaMemcpyDeviceToHost, s));
        nrm2sq_dd(xo(c), n, hd.as<double>() + 1, dpart.as<double>(), s);
        TM_CK(cudaMemcpyAsync(&q[1], hd.as<double>() + 1, 8, cudaMemcpyDeviceToHost, s));
        host_sync();
        const double ts = q[0] / q[1];  // theta / S
        axpby_dd(1.0, axo(c), -ts, xo(c), Wd.as<dfloat>(), n, s);
        double rr = 0.0;
        nrm2sq_dd(Wd.as<dfloat>(), n, hd.as<double>(), dpart.as<double>(), s);
        TM_CK(cudaMemcpyAsync(&rr, hd.p, 8, cudaMemcpyDeviceToHost, s));
        host_sync();
        const double th = S * ts;
        const double res = S * std::sqrt(std::max(rr, 0.0) / q[1]);
        thv[c] = th;
        max_resid = std::max(max_resid, res / std::fabs(th));
        if (!(res <= tol * std::max(std::fabs(th), 1e-300))) ok_all = false;
      }
      ++info.refine_checks;
      info.refine_true = max_resid;
      // the verified vectors become X0 either way
      TM_CK(cudaMemcpyAsync(x0(0), Xo.p, (size_t)nev * ld * 8, cudaMemcpyDeviceToDevice, s));
      TM_CK(cudaMemcpyAsync(ax0(0), AXo.p, (size_t)nev * ld * 8, cudaMemcpyDeviceToDevice, s));
      if (ok_all) {
        to_lz(x0(0));
        info.refine_outcome = 2;
        return true;
      }
      // re-orthonormalise X0 (its products follow linearly) and rebuild its rows
      for (int i = 0; i < nev; ++i) {
        for (int pass = 0; pass < 2 && i > 0; ++pass) {
          mdot_dd(x0(0), ld, i, x0(i), n, hd.as<double>(), dpart.as<double>(), s);
          maxpy_dd(x0(0), ld, i, hd.as<double>(), x0(i), n, s);
          maxpy_dd(ax0(0), ld, i, hd.as<double>(), ax0(i), n, s);
        }
        double q = 0.0;
        nrm2sq_dd(x0(i), n, hd.as<double>(), dpart.as<double>(), s);
        TM_CK(cudaMemcpyAsync(&q, hd.p, 8, cudaMemcpyDeviceToHost, s));
        host_sync();
        const double inv = 1.0 / std::sqrt(q);
        axpby_dd(inv, x0(i), 0.0, x0(i), x0(i), n, s);
        axpby_dd(inv, ax0(i), 0.0, ax0(i), ax0(i), n, s);
      }
      set_x0(nb);
      force_grow = true;
      trust_bound = false;
      continue;
    }
    force_grow = false;
    if (verified >= 3 || round + 1 >= 3 * kRefineRounds || nb + nev > cap) break;
    // grow: the residuals of the wanted pairs not yet well converged (all of
    // them if none is left), orthonormalised against the subspace and within
    // the block; FP32 products; a column that vanishes is dropped.  A residual
    // already below a quarter of the tolerance (half of it is accepted) adds
    // little, and its product costs as much as any other.
    {
      std::vector<int> keep;
      for (int c = 0; c < nev; ++c)
        if (!(rn[c] <= 0.25 * tol * std::fabs(thv[c]))) keep.push_back(c);
      if (keep.empty())
        for (int c = 0; c < nev; ++c) keep.push_back(c);
      const int nk = (int)keep.size();
      for (int k = 0; k < nk; ++k)
        TM_CK(cudaMemcpyAsync(f32col(B32, nb + k), R32.as<float>() + (size_t)keep[k] * ld, (size_t)n * 4,
                              cudaMemcpyDeviceToDevice, s));
      std::vector<double> q0(nk, 0.0);  // squared norms before the projection
      F32Cols wc{};
      F32ColsMut wm{};
      for (int k = 0; k < nk; ++k) {
        wc.c[k] = f32col(B32, nb + k);
        wm.c[k] = f32col(B32, nb + k);
      }
      // Block Gram-Schmidt against the subspace, then Cholesky QR within the
      // block.  One sweep gives [B | W]^T W: the couplings H = B^T W and the
      // block's own Gram matrix; W -= B H is the second sweep.  The Gram
      // matrix of the updated block follows as W^T W - H^T H (B orthonormal
      // to FP32 accuracy), and a third sweep maps W to W R^-1.  A column whose
      // norm the projection more than halves gets a second projection first
      // ("twice is enough"), with the Gram matrix taken afresh.
      const int nv = nb + nk;
      auto block_dots = [&](std::vector<double>& g) {
        mdot_block_f32(B32.as<float>(), ld, nv, wc, nk, n, Hd.as<double>(), 48, bpart.as<double>(), s);
        g.resize((size_t)48 * nk);
        TM_CK(cudaMemcpyAsync(g.data(), Hd.p, g.size() * 8, cudaMemcpyDeviceToHost, s));
        host_sync();
      };
      std::vector<double> gq;
      block_dots(gq);
      auto gram_after = [&](const std::vector<double>& g, std::vector<double>& gp) {
        gp.assign((size_t)nk * nk, 0.0);
        for (int a = 0; a < nk; ++a)
          for (int b = 0; b < nk; ++b) {
            double v = g[(size_t)48 * b + nb + a];
            for (int i = 0; i < nb; ++i) v -= g[(size_t)48 * a + i] * g[(size_t)48 * b + i];
            gp[(size_t)b * nk + a] = v;
          }
      };
      std::vector<double> gp;
      gram_after(gq, gp);
      for (int k = 0; k < nk; ++k) q0[k] = gq[(size_t)48 * k + nb + k];
      bool again = false;
      for (int k = 0; k < nk; ++k)
        if (!(gp[(size_t)k * nk + k] >= 0.5 * q0[k])) again = true;
      maxpy_block_f32(B32.as<float>(), ld, nb, Hd.as<double>(), 48, wm, nk, n, s);
      if (again) {
        block_dots(gq);
        gram_after(gq, gp);
        maxpy_block_f32(B32.as<float>(), ld, nb, Hd.as<double>(), 48, wm, nk, n, s);
      }
      // Cholesky of the block's Gram matrix, dropping a column whose remaining
      // norm is below 1e-10 of its norm before the projection (it adds no
      // direction); Rk: the kept columns' triangular factor
      std::vector<int> kept;
      std::vector<double> Rk((size_t)nk * nk, 0.0);  // Rk[c * nk + r], r <= c, over kept indices
      for (int k = 0; k < nk; ++k) {
        const int c = (int)kept.size();
        std::vector<double> col(c + 1, 0.0);
        for (int r = 0; r < c; ++r) {
          double v = gp[(size_t)k * nk + kept[r]];
          for (int t = 0; t < r; ++t) v -= Rk[(size_t)r * nk + t] * col[t];
          col[r] = v / Rk[(size_t)r * nk + r];
        }
        double d = gp[(size_t)k * nk + k];
        for (int t = 0; t < c; ++t) d -= col[t] * col[t];
        if (!(q0[k] > 0.0) || !(d > 1e-10 * q0[k])) continue;
        col[c] = std::sqrt(d);
        for (int r = 0; r <= c; ++r) Rk[(size_t)c * nk + r] = col[r];
        kept.push_back(k);
      }
      const int nkept = (int)kept.size();
      int pos = nb;
      if (nkept > 0) {
        // Y = R^-1 over the kept columns (back substitution), rows indexed by
        // the block's columns: new column c = sum_k W_k Y[c * nk + k]
        std::vector<double> Rinv((size_t)nkept * nkept, 0.0), Y((size_t)nk * nkept, 0.0);
        for (int c = 0; c < nkept; ++c) {
          Rinv[(size_t)c * nkept + c] = 1.0 / Rk[(size_t)c * nk + c];
          for (int r = c - 1; r >= 0; --r) {
            double v = 0.0;
            for (int t = r + 1; t <= c; ++t) v += Rk[(size_t)t * nk + r] * Rinv[(size_t)c * nkept + t];
            Rinv[(size_t)c * nkept + r] = -v / Rk[(size_t)r * nk + r];
          }
        }
        for (int c = 0; c < nkept; ++c)
          for (int r = 0; r <= c; ++r) Y[(size_t)c * nk + kept[r]] = Rinv[(size_t)c * nkept + r];
        TM_CK(cudaMemcpyAsync(hd.p, Y.data(), Y.size() * 8, cudaMemcpyHostToDevice, s));
        rotate_f32(f32col(B32, nb), ld, nk, hd.as<double>(), nkept, n, s);
        pos = nb + nkept;
      }
      for (int j = nb; j < pos; ++j) prod32(f32col(B32, j), f32col(AB32, j));
      if (pos > nb) add_gcols(nb, pos - nb);
      nb = pos;
    }
  }
  to_lz(have_x ? xo(0) : x0(0));
  info.refine_outcome = 3;
  return false;
}

tm_status lanczos_solve(const Op& op, int nev, int ncv, double tol, uint64_t seed, int mode, double* vals,
                        double* vecs_host, tm_eigs_info* info_out) {
  auto t0 = std::chrono::steady_clock::now();
  cudaStream_t s = op.stream;
  const int64_t n = op.n;
  if (nev < 1 || nev >= n) fail(TM_ERR_ARG, "nev must satisfy 1 <= nev < rows");
  // The reference's rule (suggested_nev); the mixed mode takes at least 16
  // columns: its FP32 phase keeps more Ritz vectors next to the wanted ones,
  // and the refinement resolves the wanted ones against them in fewer rounds
  // (L = 32 headline: 41 products against 45 with 11 columns).
  if (ncv <= 0) {
    ncv = (nev > 4) ? 2 * nev + 1 : 2 * nev + 3;
    if (mode == TM_EIGS_MIXED) ncv = std::max(ncv, std::min(NV32, 2 * nev + 8));
  }
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
    const bool mixed_nv32 = (mode == TM_EIGS_MIXED) && ncv <= NV32;
    Lz.reset(new Lanczos(op, ncv, s, mixed_nv32 ? nev + 1 : 0));
    Lanczos& lz = *Lz;
    const bool mixed = (mode == TM_EIGS_MIXED);
    // the FP64 basis starts here unless the FP32 basis runs the first phase
    // (it then holds the refined vectors, and restarts from them if needed)
    if (!mixed_nv32) lz.start(nullptr, seed);
    bool ok = false;
    Lanczos::CycleResult r;
    if (mixed) {
      // FP32 phase: Ritz residuals down to the FP32 floor, relative to each
      // wanted Ritz value (but no further than 1e-8 of the dominant one),
      // stopping early if they stagnate.  A wanted pair that stops short of
      // the floor costs the refinement more than the Lanczos steps that
      // would have taken it there.
      const double tol32 = std::max(tol, 2e-7);
      int nb0 = std::max(nev, ncv - 1);
      auto conv32 = [&](const Lanczos::CycleResult& rr) {
        for (int i = 0; i < nev; ++i)
          if (rr.resid[i] > tol32 * std::max(std::fabs(rr.theta[i]), 0.05 * std::fabs(rr.theta[0]))) return false;
        return true;
      };
      std::unique_ptr<Lanczos32> l32;
      std::function<double(float*, float*)> extras;
      std::function<void(dfloat*)> fill_x0;
      std::function<void()> x0_f64;
      if (ncv <= NV32) {
        // FP32 Krylov basis (half the bytes of the FP64 basis per sweep)
        l32.reset(new Lanczos32(op, ncv, s));
        l32->start(seed);
        r = l32->run(nev, 200, conv32);
        nb0 = std::min(nb0, l32->mp);  // a mid-cycle stop leaves fewer Ritz vectors
        // the wanted Ritz vectors in double-float for the refinement,
        // re-orthonormalised (CGS2): the FP32 basis is orthonormal to FP32
        // accuracy only
        Lanczos32* lp = l32.get();
        Lanczos* lzp = &lz;
        fill_x0 = [lp, lzp, &r, nev](dfloat* X) {
          const int64_t ld = lzp->ld, nn = lzp->n;
          lp->ritz_dd(r, nev, X, ld);
          if (nev <= 4) {
            // Cholesky QR: one sweep for the Gram matrix G = X^T X (close to
            // the identity), X <- X R^-1 in a second
            DBuf gpart;
            gpart.alloc(dd_part_bytes(32));
            mdot_dd_gram(X, ld, nev, nev, nn, lzp->h1.as<double>(), gpart.as<double>(), lzp->s);
            std::vector<double> G((size_t)nev * nev);
            TM_CK(cudaMemcpyAsync(G.data(), lzp->h1.p, G.size() * 8, cudaMemcpyDeviceToHost, lzp->s));
            TM_CK(cudaStreamSynchronize(lzp->s));
            std::vector<double> Y;
            if (chol_qr_inverse(G, nev, Y)) {
              TM_CK(cudaMemcpyAsync(lzp->h2.p, Y.data(), Y.size() * 8, cudaMemcpyHostToDevice, lzp->s));
              combine_dd_inplace(X, ld, nev, lzp->h2.as<double>(), nn, lzp->s);
              TM_CK(cudaStreamSynchronize(lzp->s));
              return;
            }
          }
          for (int i = 0; i < nev; ++i) {
            dfloat* xi = X + (int64_t)i * ld;
            for (int pass = 0; pass < 2 && i > 0; ++pass) {
              mdot_dd(X, ld, i, xi, nn, lzp->h1.as<double>(), lzp->part.as<double>(), lzp->s);
              maxpy_dd(X, ld, i, lzp->h1.as<double>(), xi, nn, lzp->s);
            }
            nrm2sq_dd(xi, nn, lzp->nsq.as<double>(), lzp->part.as<double>(), lzp->s);
            normalize_dd(xi, lzp->nsq.as<double>(), nn, lzp->s);
          }
        };
        // the same in FP64 in V, for the FP64 continuation when the
        // refinement does not run
        x0_f64 = [lp, lzp, &r, nev]() {
          const int64_t nn = lzp->n;
          lp->ritz_f64(r, nev, lzp->v(0), lzp->ld);
          for (int i = 0; i < nev; ++i) {
            double* bi = lzp->v(i);
            for (int pass = 0; pass < 2 && i > 0; ++pass) {
              mdot(lzp->v(0), lzp->ld, i, bi, nn, lzp->h1.as<double>(), lzp->part.as<double>(), lzp->s);
              maxpy(lzp->v(0), lzp->ld, i, lzp->h1.as<double>(), bi, nn, lzp->s);
            }
            nrm2sq(bi, nn, lzp->nsq.as<double>(), lzp->part.as<double>(), lzp->s);
            normalize(bi, lzp->nsq.as<double>(), bi, nullptr, nn, lzp->s);
          }
        };
        // the other Ritz vectors stay FP32
        extras = [lp, &r, nev, nb0](float* out, float* aout) {
          lp->ritz_f32(r, nev, nb0 - nev, out);
          lp->ritz_f32_prod(r, nev, nb0 - nev, aout);
          return lp->S;
        };
        lz.matvecs += l32->matvecs;
        lz.restarts += l32->restarts;
        info.matvecs_phase1 = l32->matvecs;
      } else {
        lz.conv_tol = tol32;
        lz.stagnation_stop = true;
        r = lz.run(nev, true, 200, conv32, &ok);
        lz.stagnation_stop = false;
        info.matvecs_phase1 = lz.matvecs;
        lz.rotate(r, nb0);
        Lanczos* lzp = &lz;
        fill_x0 = [lzp, nev](dfloat* X) {
          for (int i = 0; i < nev; ++i) f64_to_df(lzp->v(i), 1.0, X + (int64_t)i * lzp->ld, lzp->n, lzp->s);
        };
      }
      TM_CK(cudaStreamSynchronize(s));
      const auto t1 = std::chrono::steady_clock::now();
      info.seconds_phase1 = std::chrono::duration<double>(t1 - t0).count();
      // FP64-accurate refinement (refine_mixed); leaves the best Ritz
      // vectors in V's leading columns either way
      std::vector<double> thv(nev);
      bool cluster = false;
      for (int i = 0; i < nev && i + 1 < (int)r.theta.size(); ++i)
        if (std::fabs(r.theta[i] - r.theta[i + 1]) < 1e-5 * std::fabs(r.theta[i])) cluster = true;
      const bool run_refine = !cluster && nev <= kMaxRefineNev && (int64_t)(nb0 + 6 * nev) * 4 <= n;
      const bool refined = run_refine && refine_mixed(op, lz, nev, nb0, tol, thv, max_resid, fill_x0, extras, info);
      if (!run_refine && x0_f64) x0_f64();
      if (!refined && info.refine_outcome == 0) info.refine_outcome = 3;
      TM_CK(cudaStreamSynchronize(s));
      info.seconds_refine = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
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
        lz.ensure_full();
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
  stage_err_check(s);  // the staged Krylov sweeps' bounded waits all completed
  for (int i = 0; i < nev && i < (int)theta.size(); ++i) vals[i] = theta[i];
  if (vecs_host && Lz) {
    // eigenvectors in the reference's order.  Host memory the device can
    // address (pinned and mapped) is filled by a gather kernel that reads the
    // pi-order vectors from HBM and stores coalesced over the host link;
    // other host memory gets the pi -> reference scatter on the device, then
    // one copy.
    // Only page-locked memory (cudaHostGetFlags knows it) takes the direct
    // path: a system that lets the device reach pageable memory through the
    // host's page tables reports it as addressable too, but stores through
    // those translations are far slower than one copy.
    cudaPointerAttributes pa{};
    unsigned int hflags = 0;
    double* hdev = nullptr;
    if (cudaHostGetFlags(&hflags, vecs_host) == cudaSuccess && cudaPointerGetAttributes(&pa, vecs_host) == cudaSuccess) {
      if (pa.type == cudaMemoryTypeHost && pa.devicePointer) hdev = static_cast<double*>(pa.devicePointer);
    } else {
      (void)cudaGetLastError();
    }
    if (op.has_pi && hdev) {
      gather_cols_f64(Lz->v(0), Lz->ld, op.pinv.as<uint32_t>(), hdev, n, nev, s);
      TM_CK(cudaStreamSynchronize(s));
    } else if (op.has_pi) {
      DBuf ref;
      ref.alloc((size_t)nev * n * 8);
      for (int c = 0; c < nev; ++c)
        scatter_f64(Lz->v(c), op.pi.as<uint32_t>(), ref.as<double>() + (int64_t)c * n, n, s);
      TM_CK(cudaMemcpyAsync(vecs_host, ref.p, (size_t)nev * n * 8, cudaMemcpyDeviceToHost, s));
      TM_CK(cudaStreamSynchronize(s));
    } else {
      TM_CK(cudaMemcpy2DAsync(vecs_host, (size_t)n * 8, Lz->v(0), (size_t)Lz->ld * 8, (size_t)n * 8, nev,
                              cudaMemcpyDeviceToHost, s));
      TM_CK(cudaStreamSynchronize(s));
    }
  }
  const_cast<Op&>(op).matvecs += info.matvecs;
  info.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (info_out) *info_out = info;
  return done ? TM_OK : TM_ERR_NOCONV;
}

}  // namespace ltm
