// Aux-bit transfer-matrix cores: DNNI (one carried bit) and diagonal
// BNNNI+3NN (two carried bits), full operators and their reduced forms.
//
// DNNI (XDTMatVecProd2D, TMat/tmat.cpp:322-476): the inter-layer factor couples
// each new spin to three old ones (same site and both diagonals), so it is
// swept site by site with the previous old spin carried in an auxiliary bit.
// The diagonal BNNNI TM (ZBTMatVecProd2D, TMat/tmat.cpp:480-662) sweeps two
// sites per step with two carried bits; its transpose swaps the roles of the
// coupling factors (optdirection = 1).
//
// GPU form: every sweep step is one output-centric kernel over all
// (lastbit pass, aux, state) elements at once.  The reference runs its
// lastbit passes (2 for DNNI, 4 for BNNNI) one after another; here they are
// independent slices of one launch.  Each output element is computed directly
// from its 2 or 4 inputs (no scatter).  Steps are scaled by the inverse of
// their largest row sum, so FP32 intermediates stay in range; the product of
// the scales is applied in FP64 at the fold.  Reduced operators (XDM, ZBM)
// expand through the state->rank map, run the same core, and contract at the
// orbit representatives.
#include <algorithm>
#include <cmath>

#include "tm_internal.h"

namespace ltm {

namespace {

struct AuxCoef {
  double b1[2], b2[2], b3[2];
};

template <class T>
struct AuxCoefT {
  T b1[2], b2[2], b3[2];
  T g;  // step normalisation (multiply)
};

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)num_sms() * 32));
}

// ------------------------------------------------------------------ DNNI
// element e of a 2*2*N buffer: e = (lb << (L+1)) | (aux << L) | r
template <class T>
__global__ void xdt_init(const T* __restrict__ x, const double* __restrict__ pre, int L, int bc,
                         AuxCoefT<T> c, int npass, T* __restrict__ P) {
  const int64_t N = 1ll << L;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < N * npass; i += st) {
    const int lb = (int)(i >> L);
    const uint64_t rp = (uint64_t)(i & (N - 1));
    T* Q = P + (int64_t)lb * 2 * N;
    T v = pre ? (T)((double)x[rp] * pre[rp]) : x[rp];
    if (bc == 0) {
      // TMat/tmat.cpp:392-405: aux bit = copy of the top bit
      const uint64_t rpb = ((rp & (uint64_t)(N >> 1)) << 1) | rp;
      Q[rpb] = ((int)(rp & 1) == lb) ? v : (T)0;
      Q[rpb ^ (uint64_t)N] = 0;
    } else if (bc == 5) {
      // TMat/tmat.cpp:440-449
      Q[rp] = v * c.b2[rp & 1] * c.b2[rp >> (L - 1)];
      Q[rp | (uint64_t)N] = 0;
    } else {
      // bc 9, TMat/tmat.cpp:452-457
      Q[rp | (uint64_t)N] = v * c.b2[(rp & 1) ^ 1] * c.b2[rp >> (L - 1)];
      Q[rp] = 0;
    }
  }
}

// one sweep step (permute_mult_T1 / _last, TMat/tmat.cpp:344-376), output-centric
template <class T>
__global__ void xdt_step(const T* __restrict__ X, T* __restrict__ Y, int L, AuxCoefT<T> c, int last,
                         int bc, int npass) {
  const int64_t N = 1ll << L;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < 2 * N * npass; i += st) {
    const int lb = (int)(i >> (L + 1));
    const uint64_t loc = (uint64_t)(i & (2 * N - 1));
    const uint64_t a = loc >> L, r = loc & (uint64_t)(N - 1);
    const uint64_t rp = rotl(r, L, 1);
    const uint64_t s = rp & 1;
    const uint64_t rq = (rp & ~1ull) | a;
    const uint64_t nb = last ? (bc == 0 ? (uint64_t)lb : 0ull) : ((rq >> 1) & 1);
    const T* Xp = X + (int64_t)lb * 2 * N;
    T v = c.b1[s ^ a] * c.b2[nb ^ s] * (c.b2[s] * Xp[rq] + c.b2[s ^ 1] * Xp[rq | (uint64_t)N]);
    Y[i] = v * c.g;
  }
}

template <class T>
__global__ void xdt_fold(const T* __restrict__ P, const double* __restrict__ post, double postc, int L, int npass,
                         T* __restrict__ y) {
  const int64_t N = 1ll << L;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < N; i += st) {
    double acc = 0.0;
    for (int lb = 0; lb < npass; ++lb) acc += (double)P[(int64_t)lb * 2 * N + i] + (double)P[(int64_t)lb * 2 * N + N + i];
    if (post) acc *= post[i];
    y[i] = (T)(acc * postc);
  }
}

// ------------------------------------------------------------------ diagonal BNNNI
// element e of a 4*4*N buffer: e = (lb << (L+2)) | (aux << L) | r
template <class T>
__global__ void zbt_init(const T* __restrict__ x, const double* __restrict__ pre, int L, T* __restrict__ P) {
  const int64_t N = 1ll << L;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < N * 4; i += st) {
    const int lb = (int)(i >> L);
    const uint64_t rp = (uint64_t)(i & (N - 1));
    T* Q = P + (int64_t)lb * 4 * N;
    // TMat/tmat.cpp:607-619: aux bits = copy of the top two bits
    const uint64_t nc = (uint64_t)((N >> 1) | (N >> 2));
    const uint64_t rpb = ((rp & nc) << 2) | rp;
    T v = pre ? (T)((double)x[rp] * pre[rp]) : x[rp];
    Q[rpb] = ((int)(rp & 3) == lb) ? v : (T)0;
    Q[rpb ^ (uint64_t)N] = 0;
    Q[rpb ^ (uint64_t)(2 * N)] = 0;
    Q[rpb ^ (nc << 2)] = 0;
  }
}

// permute_mult_T1 / _last of ZBTMatVecProd2D (TMat/tmat.cpp:521-588), output-centric
template <class T>
__global__ void zbt_step(const T* __restrict__ X, T* __restrict__ Y, int L, AuxCoefT<T> c, int last, int dir) {
  const int64_t N = 1ll << L;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < 16 * N; i += st) {
    const uint64_t lb = (uint64_t)(i >> (L + 2));
    const uint64_t loc = (uint64_t)(i & (4 * N - 1));
    const uint64_t aux = loc >> L, r = loc & (uint64_t)(N - 1);
    const uint64_t rp = rotl(r, L, 2);
    const uint64_t rq = (rp & ~3ull) | aux;
    const uint64_t sl = (rp >> 1) & 1, sr = rp & 1, pl = aux >> 1, pr = aux & 1;
    const uint64_t fl = last ? (lb >> 1) : ((rp >> 3) & 1), fr = last ? (lb & 1) : ((rp >> 2) & 1);
    T v;
    if (!dir)
      v = c.b1[sr ^ pl] * c.b2[sr ^ fr] * c.b2[sl ^ fl] * c.b3[sr ^ pr] * c.b3[sl ^ pl];
    else
      v = c.b1[sl ^ fr] * c.b1[sl ^ pr] * c.b2[sr ^ fr] * c.b2[sl ^ fl] * c.b3[sr ^ pr] * c.b3[sl ^ pl];
    const T* Xp = X + (int64_t)lb * 4 * N;
    T d = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint64_t al = (uint64_t)q >> 1, ar = (uint64_t)q & 1;
      const T xv = Xp[((uint64_t)q << L) | rq];
      if (!dir)
        d += xv * c.b1[sr ^ al] * c.b2[sr ^ ar] * c.b2[sl ^ al];
      else
        d += xv * c.b2[sr ^ ar] * c.b2[sl ^ al];
    }
    Y[i] = v * d * c.g;
  }
}

template <class T>
__global__ void zbt_fold(const T* __restrict__ P, const double* __restrict__ post, double postc, int L,
                         T* __restrict__ y) {
  const int64_t N = 1ll << L;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < N; i += st) {
    double acc = 0.0;
    for (int lb = 0; lb < 4; ++lb)
      for (int a = 0; a < 4; ++a) acc += (double)P[(int64_t)lb * 4 * N + (int64_t)a * N + i];
    if (post) acc *= post[i];
    y[i] = (T)(acc * postc);
  }
}

// ------------------------------------------------------------------ reduced expand / contract
template <class T>
__global__ void red_expand(const T* __restrict__ x, const double* __restrict__ tv, const uint32_t* __restrict__ smap,
                           int64_t N, T* __restrict__ v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < N; i += st) {
    uint32_t r = smap[i];
    v[i] = (T)((double)x[r] * tv[r]);
  }
}

template <class T>
__global__ void red_contract(const T* __restrict__ z, const uint32_t* __restrict__ idx, const uint16_t* __restrict__ dup,
                             const double* __restrict__ tv, double post, T* __restrict__ y, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) y[i] = (T)((double)z[idx[i]] * post * (double)dup[i] * tv[i]);
}

AuxCoef coef_of(const Op& op) {
  AuxCoef c;
  const double bj = op.mp.betaJ;
  c.b1[0] = std::exp(bj);
  c.b1[1] = 1.0 / c.b1[0];
  c.b2[0] = std::exp(-bj * op.mp.kappa);
  c.b2[1] = 1.0 / c.b2[0];
  c.b3[0] = std::exp(-bj * op.mp.kappa2);
  c.b3[1] = 1.0 / c.b3[0];
  return c;
}

// largest row sum of one sweep step (bound used to normalise FP32 steps)
double step_bound(const Op& op, const AuxCoef& c, int dir) {
  double best = 0.0;
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  if (!zb) {
    for (int s = 0; s < 2; ++s)
      for (int a = 0; a < 2; ++a)
        for (int nb = 0; nb < 2; ++nb)
          best = std::max(best, c.b1[s ^ a] * c.b2[nb ^ s] * (c.b2[s] + c.b2[s ^ 1]));
  } else {
    for (int sl = 0; sl < 2; ++sl)
      for (int sr = 0; sr < 2; ++sr)
        for (int pl = 0; pl < 2; ++pl)
          for (int pr = 0; pr < 2; ++pr)
            for (int fl = 0; fl < 2; ++fl)
              for (int fr = 0; fr < 2; ++fr) {
                double v = !dir ? c.b1[sr ^ pl] * c.b2[sr ^ fr] * c.b2[sl ^ fl] * c.b3[sr ^ pr] * c.b3[sl ^ pl]
                                : c.b1[sl ^ fr] * c.b1[sl ^ pr] * c.b2[sr ^ fr] * c.b2[sl ^ fl] * c.b3[sr ^ pr] *
                                      c.b3[sl ^ pl];
                double d = 0.0;
                for (int q = 0; q < 4; ++q) {
                  int al = q >> 1, ar = q & 1;
                  d += !dir ? c.b1[sr ^ al] * c.b2[sr ^ ar] * c.b2[sl ^ al] : c.b2[sr ^ ar] * c.b2[sl ^ al];
                }
                best = std::max(best, v * d);
              }
  }
  return best;
}

}  // namespace

void build_aux(Op& op) {
  const int L = op.L;
  const int64_t N = 1ll << L;
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  if (op.kind == K_ZBT || op.kind == K_ZBM) {
    if (L % 2) fail(TM_ERR_ARG, "diagonal BNNNI operators need an even width");
  }
  const int64_t per = zb ? 16 * N : 4 * N;  // elements per sweep buffer
  op.ws_a.alloc((size_t)per * 8);
  op.ws_b.alloc((size_t)per * 8);
  if (op.kind == K_XDM || op.kind == K_ZBM) op.xp.alloc((size_t)N * 8);  // expanded / contracted full vector
}

// y = T x (or T^T x for transposed views); scaled: FP32 result divided by the
// returned factor.
template <class T>
double matvec_aux_dir(const Op& op, const T* x, T* y, bool scaled, int dir, cudaStream_t s) {
  const int L = op.L;
  const int64_t N = 1ll << L;
  const bool reduced = (op.kind == K_XDM || op.kind == K_ZBM);
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  AuxCoef c64 = coef_of(op);
  const double gb = step_bound(op, c64, dir);
  const bool norm = (sizeof(T) == 4);
  AuxCoefT<T> c;
  for (int k = 0; k < 2; ++k) {
    c.b1[k] = (T)c64.b1[k];
    c.b2[k] = (T)c64.b2[k];
    c.b3[k] = (T)c64.b3[k];
  }
  c.g = norm ? (T)(1.0 / gb) : (T)1;
  const int nsteps = zb ? L / 2 : L;
  const double gscale = norm ? std::pow(gb, (double)nsteps) : 1.0;
  T* A = op.ws_a.as<T>();
  T* B = op.ws_b.as<T>();
  const T* xin = x;
  const double* pre = op.tvec.as<double>();
  if (reduced) {
    T* v = op.xp.as<T>();
    red_expand<T><<<grid_for(N), 256, 0, s>>>(x, op.tvec.as<double>(), op.smap.as<uint32_t>(), N, v);
    TM_CKK("red_expand");
    xin = v;
    pre = nullptr;
  }
  const double sf = scaled ? 1.0 : gscale;
  T* fold_out = reduced ? op.xp.as<T>() : y;
  if (!zb) {
    const int bc = op.boundary;
    const int npass = (bc == 0) ? 2 : 1;
    xdt_init<T><<<grid_for(N * npass), 256, 0, s>>>(xin, pre, L, bc, c, npass, A);
    TM_CKK("xdt_init");
    for (int st = 0; st < L; ++st) {
      xdt_step<T><<<grid_for(2 * N * npass), 256, 0, s>>>(A, B, L, c, st == L - 1, bc, npass);
      TM_CKK("xdt_step");
      std::swap(A, B);
    }
    const double postc = reduced ? sf : op.normfactor * sf;
    xdt_fold<T><<<grid_for(N), 256, 0, s>>>(A, reduced ? nullptr : op.tvec.as<double>(), postc, L, npass, fold_out);
    TM_CKK("xdt_fold");
  } else {
    zbt_init<T><<<grid_for(4 * N), 256, 0, s>>>(xin, pre, L, A);
    TM_CKK("zbt_init");
    for (int st = 0; st < L / 2; ++st) {
      zbt_step<T><<<grid_for(16 * N), 256, 0, s>>>(A, B, L, c, st == L / 2 - 1, dir);
      TM_CKK("zbt_step");
      std::swap(A, B);
    }
    zbt_fold<T><<<grid_for(N), 256, 0, s>>>(A, reduced ? nullptr : op.tvec.as<double>(), sf, L, fold_out);
    TM_CKK("zbt_fold");
  }
  if (reduced) {
    red_contract<T><<<grid_for(op.n), 256, 0, s>>>(fold_out, op.idx.as<uint32_t>(), op.dup.as<uint16_t>(),
                                                   op.tvec.as<double>(), 1.0, y, op.n);
    TM_CKK("red_contract");
  }
  return scaled ? gscale : 1.0;
}

template <class T>
double matvec_aux(const Op& op, const T* x, T* y, bool scaled, cudaStream_t s) {
  const Op& base = op.parent ? *op.parent : op;
  return matvec_aux_dir<T>(base, x, y, scaled, op.transposed ? 1 : 0, s);
}

template double matvec_aux<float>(const Op&, const float*, float*, bool, cudaStream_t);
template double matvec_aux<double>(const Op&, const double*, double*, bool, cudaStream_t);

}  // namespace ltm
