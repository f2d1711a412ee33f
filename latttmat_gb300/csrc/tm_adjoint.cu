// Adjoint of the leading eigenvalues: d ln(lambda)/d(betaJ, kappa, kappa2, h).
//
// No reference counterpart (the reference only reports eigenvalues and the
// magnetisation / domain-wall moments of TMat/tmatphys.cpp).  For an
// eigenpair (lambda, r) with left vector l (l = r for symmetric operators):
//   d lambda = l^T (dT) r / (l^T r).
// Every operator here is T = p * Tv' * Th * Tv' (Tv' = the operator's Tvec:
// the square-root intra-layer Boltzmann weight, times nf^(1/2) / sqrt(dup) in
// the reduced forms).  Tv' is diagonal, so with g(s) = d ln Tv'(s)/d theta:
//   d ln lambda = 2 <g>_{l r} + l^T (p Tv' dTh Tv') r / (lambda l^T r),
// where <g>_{l r} = sum l_i r_i g(s_i) / sum l_i r_i.  The first term is a
// fused weighted reduction over the basis.  The second is nonzero only for
// theta = betaJ (Th depends on K = betaJ alone for the Kronecker-core
// operators).  It comes from a tangent sweep: the butterflies carry
// (value, derivative) pairs, t = [[e^K, e^-K], [e^-K, e^K]] and
// dt/dK = [[e^K, -e^-K], [-e^-K, e^K]].  The normfactor terms cancel: the
// result is the derivative of the reported eigenvalue lambda/normfactor.
#include <cmath>
#include <vector>

#include "tm_chain.h"
#include "tm_group.cuh"
#include "tm_internal.h"

namespace ltm {

namespace {

struct GradParams {
  int kind, L, s1, s2, boundary;
  double bj, k, k2, h;
};

// d(exponent of Tv')/d theta without the normfactor terms, theta = (bJ, k, k2, h)
__device__ void gvec(const GradParams& p, uint64_t s, double g[4]) {
  const int L = p.L;
  const uint64_t mask = (1ull << L) - 1;
  int n0 = popc64(s);
  g[0] = g[1] = g[2] = g[3] = 0.0;
  if (p.kind == K_XAT) {
    int n1, n2, ns1 = L, ns2 = L;
    uint64_t a, b;
    switch (p.boundary) {
      case 0:
        n1 = popc64(s ^ rotr(s, L, 1));
        n2 = popc64(s ^ rotr(s, L, 2));
        break;
      case 1:
        n1 = popc64((s & (mask >> 1)) ^ (s >> 1));
        n2 = popc64((s & (mask >> 2)) ^ (s >> 2));
        ns1 = L - 1;
        ns2 = L - 2;
        break;
      case 5:
      case 9:
        a = (s << 1) | (p.boundary == 9 ? 1ull : 0ull);
        b = s >> 1;
        n1 = popc64(s ^ a);
        n2 = popc64((a & mask) ^ b);
        ns1 = L + 1;
        break;
      default:
        a = (s << 1) | (p.boundary == 17 ? 1ull : 0ull);
        b = (s << 2) | (p.boundary == 17 ? 3ull : 0ull);
        n1 = popc64(s ^ a);
        n2 = popc64(s ^ b);
        ns1 = L + 1;
        ns2 = L + 2;
        break;
    }
    g[0] = -0.5 * (2.0 * n1 - ns1) + 0.5 * p.k * (2.0 * n2 - ns2) - 0.5 * p.h * (2.0 * n0 - L);
    g[1] = 0.5 * p.bj * (2.0 * n2 - ns2);
    g[3] = -0.5 * p.bj * (2.0 * n0 - L);
  } else if (p.kind == K_XAM) {
    int n1, n2;
    if (!p.boundary) {
      n1 = popc64(s ^ rotr(s, L, 1));
      n2 = popc64(s ^ rotr(s, L, 2));
    } else {
      n1 = popc64((s & (mask >> 1)) ^ (s >> 1));
      n2 = popc64((s & (mask >> 2)) ^ (s >> 2));
    }
    g[0] = -0.5 * (2 * n1 - L) + 0.5 * p.k * (2 * n2 - L) - 0.5 * p.h * (2 * n0 - L);
    g[1] = 0.5 * p.bj * (2 * n2 - L);
    g[3] = -0.5 * p.bj * (2 * n0 - L);
  } else if (p.kind == K_ZBT || p.kind == K_ZBM || p.kind == K_XDT || p.kind == K_XDM) {
    aux_tvec_grad(p.kind, L, p.boundary, p.bj, p.k2, p.h, s, g);
  } else if (p.kind == K_XAM3) {
    int n1a = popc64(s ^ rshift3d(s, p.s1, p.s2, 1));
    int n1b = popc64(s ^ dshift3d(s, p.s1, p.s2, 1));
    int n2 = popc64(s ^ rshift3d(s, p.s1, p.s2, 2));
    g[0] = -(n1a + n1b - L) + 0.5 * p.k * (2 * n2 - L) - 0.5 * p.h * (2 * n0 - L);
    g[1] = 0.5 * p.bj * (2 * n2 - L);
    g[3] = -0.5 * p.bj * (2 * n0 - L);
  }
}

__global__ void diag_grad_kernel(GradParams p, const double* __restrict__ qr, const double* __restrict__ ql,
                                 const uint32_t* __restrict__ idx, int64_t n, double* __restrict__ part) {
  double acc[5] = {0, 0, 0, 0, 0};
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) {
    uint64_t s = idx ? (uint64_t)idx[i] : (uint64_t)i;
    double w = qr[i] * (ql ? ql[i] : qr[i]);
    double g[4];
    gvec(p, s, g);
    for (int k = 0; k < 4; ++k) acc[k] += w * g[k];
    acc[4] += w;
  }
  __shared__ double sh[5][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < 5; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double t = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[threadIdx.x][q];
    part[(int64_t)blockIdx.x * 5 + threadIdx.x] = t;
  }
}

// v = Tvec .* qr expanded to the full space (reduced: through smap)
__global__ void tangent_expand(const double* __restrict__ qr, const double* __restrict__ tv,
                               const uint32_t* __restrict__ smap, int64_t N, double* __restrict__ v,
                               double* __restrict__ dv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < N; i += st) {
    int64_t r = smap ? (int64_t)smap[i] : i;
    v[i] = qr[r] * tv[r];
    dv[i] = 0.0;
  }
}

__device__ __forceinline__ int spad(int e) { return e + (e >> 5); }

// dual-number butterfly pass over bits [lo, lo+nb) (+ cb contiguous bits)
__global__ void dual_sweep_kernel(double* __restrict__ v, double* __restrict__ dv, int lo, int nb, int cb, double a,
                                  double b) {
  extern __shared__ double sm[];
  const int tile = 1 << (nb + cb);
  double* sv = sm;
  double* sd = sm + tile + tile / 32 + 1;
  const uint64_t outer = blockIdx.x;
  const uint64_t lob = (uint64_t)(lo - cb);
  const uint64_t base = ((outer & ((1ull << lob) - 1)) << cb) | ((outer >> lob) << (lo + nb));
  auto gidx = [&](int e) -> uint64_t {
    return base | (uint64_t)(e & ((1 << cb) - 1)) | ((uint64_t)(e >> cb) << lo);
  };
  for (int e = threadIdx.x; e < tile; e += blockDim.x) {
    uint64_t i = gidx(e);
    sv[spad(e)] = v[i];
    sd[spad(e)] = dv[i];
  }
  __syncthreads();
  for (int bb = 0; bb < nb; ++bb) {
    const int bit = cb + bb;
    for (int q = threadIdx.x; q < tile / 2; q += blockDim.x) {
      int lowm = (1 << bit) - 1;
      int e0 = ((q & ~lowm) << 1) | (q & lowm), e1 = e0 | (1 << bit);
      double x0 = sv[spad(e0)], x1 = sv[spad(e1)];
      double d0 = sd[spad(e0)], d1 = sd[spad(e1)];
      sv[spad(e0)] = a * x0 + b * x1;
      sv[spad(e1)] = b * x0 + a * x1;
      sd[spad(e0)] = a * d0 + b * d1 + (a * x0 - b * x1);
      sd[spad(e1)] = b * d0 + a * d1 + (-b * x0 + a * x1);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < tile; e += blockDim.x) {
    uint64_t i = gidx(e);
    v[i] = sv[spad(e)];
    dv[i] = sd[spad(e)];
  }
}

// quad = sum_r ql_r * post_r * dv[state(r)]
__global__ void tangent_contract(const double* __restrict__ dv, const double* __restrict__ ql,
                                 const uint32_t* __restrict__ idx, const uint16_t* __restrict__ dup,
                                 const double* __restrict__ tv, double pc, int64_t n, double* __restrict__ part) {
  double acc = 0.0;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) {
    int64_t s = idx ? (int64_t)idx[i] : i;
    double post = pc * tv[i] * (dup ? (double)dup[i] : 1.0);
    acc += ql[i] * post * dv[s];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    part[blockIdx.x] = t;
  }
}

int nblocks(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 4));
}

}  // namespace

void ensure_state_map(Op& op);

void matvec_aux_tangent(const Op& op, const double* x, double* y, const AuxCoef& db, int dir, cudaStream_t s);

// Aux-bit operators (DNNI, diagonal BNNNI): T = D_out C D_in with the
// diagonal Boltzmann weights D (Tvec, times dup in the reduced output) and
// the chain C of local step gates built from b1 = e^{+-bJ}, b2 = e^{-+bJ k},
// b3 = e^{-+bJ k2}.  d ln(lambda) = 2 <g>_{lr} + <l, D_out (dC) D_in r> /
// (lambda <l, r>); the second term is a tangent product of the chain
// (matvec_aux_tangent) per parameter the gates depend on.
static void adjoint_grad_aux(const Op& op, const double* dqr, const double* qlp, double lam, double wsum,
                             double grad[4]) {
  cudaStream_t s = op.stream;
  const int64_t n = op.n;
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  DBuf y;
  y.alloc((size_t)n * 8);
  std::vector<double> yh(n), lh(n);
  TM_CK(cudaMemcpyAsync(lh.data(), qlp ? qlp : dqr, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
  for (int t = 0; t < 3; ++t) {
    if (t == 2 && !zb) break;  // DNNI gates do not depend on kappa2
    const AuxCoef db = aux_coef_derivative(op.mp.betaJ, op.mp.kappa, op.mp.kappa2, t);
    matvec_aux_tangent(op, dqr, y.as<double>(), db, 0, s);
    TM_CK(cudaMemcpyAsync(yh.data(), y.p, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    double quad = 0.0;
    for (int64_t i = 0; i < n; ++i) quad += lh[i] * yh[i];
    grad[t] += quad / (lam * wsum);
  }
}

void adjoint_grad(const Op& op, const double* qr_h, const double* ql_h, double lam, double grad[4]) {
  const bool aux = (op.kind == K_ZBT || op.kind == K_ZBM || op.kind == K_XDT || op.kind == K_XDM);
  if (op.kind != K_XAT && op.kind != K_XAM && op.kind != K_XAM3 && !aux)
    fail(TM_ERR_UNSUPPORTED, "adjoint provided for the x-ANNNI, DNNI and diagonal BNNNI operators");
  cudaStream_t s = op.stream;
  const int64_t n = op.n;
  const bool reduced = (op.kind == K_XAM || op.kind == K_XAM3 || op.kind == K_ZBM || op.kind == K_XDM);
  DBuf dqr, dql, part;
  dqr.alloc((size_t)n * 8);
  TM_CK(cudaMemcpyAsync(dqr.p, qr_h, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  const double* qlp = nullptr;
  if (ql_h) {
    dql.alloc((size_t)n * 8);
    TM_CK(cudaMemcpyAsync(dql.p, ql_h, (size_t)n * 8, cudaMemcpyHostToDevice, s));
    qlp = dql.as<double>();
  }
  GradParams gp{op.kind, op.L, op.size1, op.size2, op.boundary, op.mp.betaJ, op.mp.kappa, op.mp.kappa2, op.mp.h};
  int nb = nblocks(n);
  part.alloc((size_t)nb * 5 * 8 + 64);
  diag_grad_kernel<<<nb, 256, 0, s>>>(gp, dqr.as<double>(), qlp, reduced ? op.idx.as<uint32_t>() : nullptr, n,
                                      part.as<double>());
  TM_CKK("diag_grad");
  std::vector<double> hp((size_t)nb * 5);
  TM_CK(cudaMemcpyAsync(hp.data(), part.p, hp.size() * 8, cudaMemcpyDeviceToHost, s));
  TM_CK(cudaStreamSynchronize(s));
  double sums[5] = {0, 0, 0, 0, 0};
  for (int b = 0; b < nb; ++b)
    for (int k = 0; k < 5; ++k) sums[k] += hp[(size_t)b * 5 + k];
  const double wsum = sums[4];
  for (int k = 0; k < 4; ++k) grad[k] = 2.0 * sums[k] / wsum;
  if (aux) {
    adjoint_grad_aux(op, dqr.as<double>(), qlp, lam, wsum, grad);
    return;
  }

  // tangent term for betaJ through the full space
  if (reduced) ensure_state_map(const_cast<Op&>(op));
  const int L = op.L;
  const int64_t N = 1ll << L;
  DBuf v, dv;
  v.alloc((size_t)N * 8);
  dv.alloc((size_t)N * 8);
  tangent_expand<<<nblocks(N) * 4, 256, 0, s>>>(dqr.as<double>(), op.tvec.as<double>(),
                                               reduced ? op.smap.as<uint32_t>() : nullptr, N, v.as<double>(),
                                               dv.as<double>());
  TM_CKK("tangent_expand");
  const double K = op.mp.betaJ, a = std::exp(K), b = std::exp(-K);
  const int NB = 11, CB = 4;
  int lo = 0;
  while (lo < L) {
    int cb = (lo == 0) ? 0 : std::min(CB, lo);
    int nbits = std::min(L - lo, NB - cb);
    int tile = 1 << (nbits + cb);
    size_t shm = (size_t)2 * (tile + tile / 32 + 1) * 8;
    int64_t nblk = (int64_t)1 << (L - nbits - cb);
    dual_sweep_kernel<<<(unsigned)nblk, std::min(256, std::max(32, tile / 2)), shm, s>>>(v.as<double>(),
                                                                                      dv.as<double>(), lo, nbits,
                                                                                      cb, a, b);
    TM_CKK("dual_sweep");
    lo += nbits;
  }
  const double pc = (op.kind == K_XAT) ? op.normfactor : 1.0;
  DBuf part2;
  int nb2 = nblocks(n);
  part2.alloc((size_t)nb2 * 8 + 64);
  tangent_contract<<<nb2, 256, 0, s>>>(dv.as<double>(), qlp ? qlp : dqr.as<double>(),
                                       reduced ? op.idx.as<uint32_t>() : nullptr,
                                       reduced ? op.dup.as<uint16_t>() : nullptr, op.tvec.as<double>(), pc, n,
                                       part2.as<double>());
  TM_CKK("tangent_contract");
  std::vector<double> h2(nb2);
  TM_CK(cudaMemcpyAsync(h2.data(), part2.p, nb2 * 8, cudaMemcpyDeviceToHost, s));
  TM_CK(cudaStreamSynchronize(s));
  double quad = 0;
  for (double x : h2) quad += x;
  grad[0] += quad / (lam * wsum);
}

}  // namespace ltm
