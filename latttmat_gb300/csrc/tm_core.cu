// Full-space transfer-matrix cores and the generic reduced-basis path.
//
// Kronecker sweep (x-ANNNI perpendicular TM, 3D ANNNI): the inter-layer
// factor Th = (x)_{i<L} t with t = [[e^K, e^-K], [e^-K, e^K]]
// (TMat/tmat.cpp:79-93, the L in-place butterflies of XATMatVecProd2D and of
// permute_mult_TL).  Here the butterflies run in shared-memory tiles: a pass
// takes up to NB bits at once, so L bits cost ceil(L/NB) passes over HBM
// instead of L.  The coefficients are normalised, a' = e^K/(e^K+e^-K), so
// intermediates stay bounded in FP32; (e^K+e^-K)^L is folded into the FP64
// output scale.  The Boltzmann-weight scaling (Tv^(1/2) x) is fused into the
// first pass's load and nf*Tv^(1/2) into the last pass's store.
//
// Generic reduced path (any reduced operator): expand the representative
// vector to the full space through the state->rank map, run the full core,
// then gather the representatives (TMat/tmatreduce.cpp:406-529 restated as
// y = D^(1/2) Tv^(1/2) Th Tv^(1/2) P D^(-1/2) x evaluated at representatives).
#include <cmath>

#include "tm_internal.h"

namespace ltm {

namespace {

template <class T>
struct Coef {
  T a, b;
};

// smem index with one pad word every 32 elements (bank-conflict relief for
// strided butterfly partners)
__device__ __forceinline__ int spad(int e) { return e + (e >> 5); }

// One sweep pass.  Elements handled by a CTA: 2^nb butterfly positions (bits
// [lo, lo+nb)) times 2^cb contiguous positions (bits [0, cb), only when lo>0),
// for one value of the remaining "outer" bits.
//   load_mode 0: v = x[i]; 1: v = x[i]*pre[i]; 2: v = x[map[i]]
//   store_mode 0: out[i] = v; 1: out[i] = v*post*scale[i] (FP64 product)
template <class T>
__global__ void __launch_bounds__(512) sweep_kernel(const T* __restrict__ x, T* __restrict__ out,
                                                    int L, int lo, int nb, int cb, Coef<T> c,
                                                    int load_mode, const double* __restrict__ pre,
                                                    const uint32_t* __restrict__ map,
                                                    int store_mode, const double* __restrict__ scale,
                                                    double post) {
  extern __shared__ unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int tile_bits = nb + cb;
  const int tile = 1 << tile_bits;
  // outer index -> the bits not in [0,cb) U [lo,lo+nb)
  const uint64_t outer = blockIdx.x;
  const uint64_t low_outer_bits = (uint64_t)(lo - cb);  // bits [cb, lo)
  const uint64_t o_lo = outer & ((1ull << low_outer_bits) - 1);
  const uint64_t o_hi = outer >> low_outer_bits;
  const uint64_t base = (o_lo << cb) | (o_hi << (lo + nb));
  auto gidx = [&](int e) -> uint64_t {
    uint64_t k = (uint64_t)(e & ((1 << cb) - 1));
    uint64_t j = (uint64_t)(e >> cb);
    return base | k | (j << lo);
  };
  for (int e = threadIdx.x; e < tile; e += blockDim.x) {
    uint64_t i = gidx(e);
    T v;
    if (load_mode == 0)
      v = x[i];
    else if (load_mode == 1)
      v = (T)((double)x[i] * pre[i]);
    else
      v = x[map[i]];
    sm[spad(e)] = v;
  }
  __syncthreads();
  const int npair = tile >> 1;
  for (int b = 0; b < nb; ++b) {
    const int bit = cb + b;  // position inside the tile index
    for (int p = threadIdx.x; p < npair; p += blockDim.x) {
      int lowm = (1 << bit) - 1;
      int e0 = ((p & ~lowm) << 1) | (p & lowm);
      int e1 = e0 | (1 << bit);
      T v0 = sm[spad(e0)], v1 = sm[spad(e1)];
      sm[spad(e0)] = c.a * v0 + c.b * v1;
      sm[spad(e1)] = c.b * v0 + c.a * v1;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < tile; e += blockDim.x) {
    uint64_t i = gidx(e);
    T v = sm[spad(e)];
    if (store_mode == 1) v = (T)((double)v * post * scale[i]);
    out[i] = v;
  }
}

template <class T>
void run_sweep(const Op& op, const T* x, T* out, int L, int load_mode, const double* pre,
               const uint32_t* map, int store_mode, const double* scale, double post,
               cudaStream_t s) {
  const double K = op.mp.betaJ;
  const double ea = std::exp(K), eb = std::exp(-K);
  Coef<T> c;
  c.a = (T)(ea / (ea + eb));
  c.b = (T)(eb / (ea + eb));
  const int NB = (sizeof(T) == 8) ? 12 : 13;  // tile bits (32 KB per tile either way)
  const int CB = (sizeof(T) == 8) ? 4 : 5;
  int lo = 0;
  bool first = true;
  const T* src = x;
  while (lo < L) {
    int cb = (lo == 0) ? 0 : std::min(CB, lo);
    int nb = std::min(L - lo, NB - cb);
    bool last = (lo + nb >= L);
    int tile = 1 << (nb + cb);
    int64_t nblocks = (int64_t)1 << (L - nb - cb);
    int threads = std::min(512, std::max(32, tile / 2));
    size_t shm = (size_t)(tile + tile / 32 + 1) * sizeof(T);
    sweep_kernel<T><<<(unsigned)nblocks, threads, shm, s>>>(
        src, out, L, lo, nb, cb, c, first ? load_mode : 0, pre, map, last ? store_mode : 0, scale,
        post);
    TM_CKK("sweep");
    src = out;
    first = false;
    lo += nb;
  }
}

// ---- generic reduced path kernels
template <class T>
__global__ void scale_in_kernel(const T* __restrict__ x, const double* __restrict__ tv, T* __restrict__ u,
                                int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) u[i] = (T)((double)x[i] * tv[i]);
}

// y[r] = post * dup[r] * tv[r] * z[idx[r]]
template <class T>
__global__ void contract_kernel(const T* __restrict__ z, const uint32_t* __restrict__ idx,
                                const uint16_t* __restrict__ dup, const double* __restrict__ tv,
                                double post, T* __restrict__ y, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) y[i] = (T)((double)z[idx[i]] * post * (double)dup[i] * tv[i]);
}

int grid_for(int64_t n, int threads = 256) {
  int64_t b = (n + threads - 1) / threads;
  int64_t cap = (int64_t)num_sms() * 16;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

}  // namespace

// y = T x on the full space (K_XAT) or on the reduced basis through the full
// space (reduced kinds whose core is the Kronecker sweep).  scaled=true:
// the result is divided by S = (e^K+e^-K)^L and S is returned.
template <class T>
double matvec_bfly(const Op& op, const T* x, T* y, bool scaled, cudaStream_t s) {
  const double K = op.mp.betaJ;
  const double S = std::pow(std::exp(K) + std::exp(-K), (double)op.L);
  const double sf = scaled ? 1.0 : S;
  if (op.kind == K_XAT) {
    // y = nf * Tv^(1/2) * Th * Tv^(1/2) * x   (TMat/tmat.cpp:71-102)
    run_sweep<T>(op, x, y, op.L, 1, op.tvec.as<double>(), nullptr, 1, op.tvec.as<double>(),
                 op.normfactor * sf, s);
    return scaled ? S : 1.0;
  }
  // reduced: u = Tvec .* x ; v = P u ; z = Th v ; y = dup .* Tvec .* z[idx]
  T* u = static_cast<T*>(op.ws_c.p);
  T* full = static_cast<T*>(op.ws_a.p);
  scale_in_kernel<T><<<grid_for(op.n), 256, 0, s>>>(x, op.tvec.as<double>(), u, op.n);
  TM_CKK("scale_in");
  run_sweep<T>(op, u, full, op.L, 2, nullptr, op.smap.as<uint32_t>(), 0, nullptr, 1.0, s);
  contract_kernel<T><<<grid_for(op.n), 256, 0, s>>>(full, op.idx.as<uint32_t>(), op.dup.as<uint16_t>(),
                                                    op.tvec.as<double>(), sf, y, op.n);
  TM_CKK("contract");
  return scaled ? S : 1.0;
}

template double matvec_bfly<float>(const Op&, const float*, float*, bool, cudaStream_t);
template double matvec_bfly<double>(const Op&, const double*, double*, bool, cudaStream_t);

// ---- permutation helpers
namespace {
template <class T>
__global__ void gather_kernel(const T* __restrict__ src, const uint32_t* __restrict__ idx,
                              T* __restrict__ dst, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) dst[i] = src[idx[i]];
}
// dst[c*n + i] = src[c*lds + idx[i]] for nvec columns, two consecutive
// outputs per thread in one 16-byte store where dst allows it (the stores may
// go to host memory over the host link, where wide stores count)
__global__ void gather_cols_f64_kernel(const double* __restrict__ src, int64_t lds, const uint32_t* __restrict__ idx,
                                       double* __restrict__ dst, int64_t n, int nvec) {
  const int64_t half = (n + 1) >> 1;
  const int64_t total = half * nvec;
  const bool pairs = (n % 2 == 0) && ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / half, i = (t - c * half) * 2;
    const double* sc = src + c * lds;
    double* dc = dst + c * n;
    if (pairs) {
      const double a = sc[idx[i]], b = sc[idx[i + 1]];
      *reinterpret_cast<double2*>(dc + i) = make_double2(a, b);
    } else {
      dc[i] = sc[idx[i]];
      if (i + 1 < n) dc[i + 1] = sc[idx[i + 1]];
    }
  }
}

template <class T>
__global__ void scatter_kernel(const T* __restrict__ src, const uint32_t* __restrict__ idx,
                               T* __restrict__ dst, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) dst[idx[i]] = src[i];
}
}  // namespace

void gather_f64(const double* src, const uint32_t* idx, double* dst, int64_t n, cudaStream_t s) {
  gather_kernel<double><<<grid_for(n), 256, 0, s>>>(src, idx, dst, n);
  TM_CKK("gather");
}
void gather_cols_f64(const double* src, int64_t lds, const uint32_t* idx, double* dst, int64_t n, int nvec,
                     cudaStream_t s) {
  gather_cols_f64_kernel<<<grid_for(((n + 1) / 2) * nvec), 256, 0, s>>>(src, lds, idx, dst, n, nvec);
  TM_CKK("gather_cols");
}
void scatter_f64(const double* src, const uint32_t* idx, double* dst, int64_t n, cudaStream_t s) {
  scatter_kernel<double><<<grid_for(n), 256, 0, s>>>(src, idx, dst, n);
  TM_CKK("scatter");
}
void gather_f32(const float* src, const uint32_t* idx, float* dst, int64_t n, cudaStream_t s) {
  gather_kernel<float><<<grid_for(n), 256, 0, s>>>(src, idx, dst, n);
  TM_CKK("gather");
}
void scatter_f32(const float* src, const uint32_t* idx, float* dst, int64_t n, cudaStream_t s) {
  scatter_kernel<float><<<grid_for(n), 256, 0, s>>>(src, idx, dst, n);
  TM_CKK("scatter");
}

}  // namespace ltm
