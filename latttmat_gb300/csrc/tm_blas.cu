// Krylov-solver vector kernels (FP64 Gram-Schmidt, norms, basis rotation) and
// the small dense symmetric eigensolver, all on the device.
#include <cmath>
#include <mutex>

#include "tm_blas.cuh"
#include "tm_stage.cuh"

namespace ltm {

namespace {

constexpr int BT = 256;        // threads per block
constexpr int NVMAX = 16;      // vectors per fused pass

int red_blocks(int64_t n) {
  int64_t b = (n + BT * 4 - 1) / (BT * 4);
  int64_t cap = (int64_t)num_sms() * kRedBlocksPerSM;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <int NV, bool W32>
__global__ void __launch_bounds__(BT) mdot_kernel(const double* __restrict__ V, int64_t ldv, int nv,
                                                  const double* __restrict__ w, const float* __restrict__ w32,
                                                  double scale, int64_t n, double* __restrict__ part) {
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  // two elements per iteration: twice the loads in flight per thread
  for (; i + st < n; i += 2 * st) {
    const int64_t i2 = i + st;
    const double wa = W32 ? scale * (double)w32[i] : w[i];
    const double wb = W32 ? scale * (double)w32[i2] : w[i2];
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (k < nv) {
        const double va = V[k * ldv + i], vb = V[k * ldv + i2];
        acc[k] = fma(va, wa, acc[k]);
        acc[k] = fma(vb, wb, acc[k]);
      }
  }
  if (i < n) {
    double wi = W32 ? scale * (double)w32[i] : w[i];
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (k < nv) acc[k] = fma(V[k * ldv + i], wi, acc[k]);
  }
  __shared__ double sh[BT / 32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double v = warp_sum(acc[k]);
    if (lane == 0) sh[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double t = 0.0;
    for (int q = 0; q < BT / 32; ++q) t += sh[q][threadIdx.x];
    part[(int64_t)blockIdx.x * NV + threadIdx.x] = t;
  }
}

__global__ void mdot_final(const double* __restrict__ part, int nb, int nv, int stride, double* __restrict__ h) {
  int k = blockIdx.x;
  if (k >= nv) return;
  double t = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) t += part[(int64_t)b * stride + k];
  t = warp_sum(t);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += sh[q];
    h[k] = s;
  }
}

template <int NV, bool W32>
__global__ void __launch_bounds__(BT) maxpy_kernel(const double* __restrict__ V, int64_t ldv, int nv,
                                                   const double* __restrict__ h, const float* __restrict__ w32,
                                                   double scale, double* __restrict__ w, int64_t n) {
  __shared__ double hs[NV];
  if (threadIdx.x < NV) hs[threadIdx.x] = (threadIdx.x < nv) ? h[threadIdx.x] : 0.0;
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i + st < n; i += 2 * st) {
    const int64_t i2 = i + st;
    double a = W32 ? scale * (double)w32[i] : w[i];
    double b = W32 ? scale * (double)w32[i2] : w[i2];
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (k < nv) {
        a = fma(-V[k * ldv + i], hs[k], a);
        b = fma(-V[k * ldv + i2], hs[k], b);
      }
    w[i] = a;
    w[i2] = b;
  }
  if (i < n) {
    double acc = W32 ? scale * (double)w32[i] : w[i];
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (k < nv) acc = fma(-V[k * ldv + i], hs[k], acc);
    w[i] = acc;
  }
}

__global__ void nrm_kernel(const double* __restrict__ w, int64_t n, double* __restrict__ part) {
  double acc = 0.0;
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) acc = fma(w[i], w[i], acc);
  __shared__ double sh[BT / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < BT / 32; ++q) t += sh[q];
    part[blockIdx.x] = t;
  }
}

__global__ void normalize_kernel(const double* __restrict__ w, const double* __restrict__ nsq,
                                 double* __restrict__ v, float* __restrict__ v32, int64_t n) {
  double inv = 1.0 / sqrt(*nsq);
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    double x = w[i] * inv;
    v[i] = x;
    if (v32) v32[i] = (float)x;
  }
}

// row-wise in-place V[:, :k] = V[:, :m] Y  (m <= 64)
__global__ void __launch_bounds__(BT) rotate_kernel(double* __restrict__ V, int64_t ldv, int m,
                                                    const double* __restrict__ Y, int k, int64_t n) {
  __shared__ double Ys[64 * 64];
  for (int t = threadIdx.x; t < m * k; t += BT) Ys[t] = Y[t];
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    double row[64];
    for (int j = 0; j < m; ++j) row[j] = V[j * ldv + i];
    for (int c = 0; c < k; ++c) {
      double acc = 0.0;
      for (int j = 0; j < m; ++j) acc = fma(row[j], Ys[c * m + j], acc);
      V[c * ldv + i] = acc;
    }
  }
}

__global__ void __launch_bounds__(BT) combine_kernel(const double* __restrict__ V, int64_t ldv, int m,
                                                     const double* __restrict__ Y, int k, double* __restrict__ out,
                                                     int64_t ldo, int64_t n) {
  __shared__ double Ys[64 * 64];
  for (int t = threadIdx.x; t < m * k; t += BT) Ys[t] = Y[t];
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    double row[64];
    for (int j = 0; j < m; ++j) row[j] = V[j * ldv + i];
    for (int c = 0; c < k; ++c) {
      double acc = 0.0;
      for (int j = 0; j < m; ++j) acc = fma(row[j], Ys[c * m + j], acc);
      out[c * ldo + i] = acc;
    }
  }
}

__global__ void to_f32_kernel(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) out[i] = (float)in[i];
}

__global__ void axpby_kernel(double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                             double* __restrict__ out, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) out[i] = a * x[i] + b * y[i];
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void uniform_kernel(double* __restrict__ v, int64_t n, uint64_t seed) {
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    uint64_t r = splitmix64(seed * 0x100000001b3ull + (uint64_t)i);
    v[i] = (double)(r >> 11) * (1.0 / 9007199254740992.0);
  }
}

__global__ void nonfinite_kernel(const double* __restrict__ v, int64_t n, unsigned int* cnt) {
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  unsigned int c = 0;
  for (; i < n; i += st) c += !isfinite(v[i]);
  if (c) atomicAdd(cnt, c);
}

// One-warp cyclic Jacobi for a small symmetric matrix (m <= 48).  Rotation
// parameters follow the classical formulation (Golub & Van Loan, Alg. 8.5.2).
__global__ void symeig_kernel(const double* __restrict__ Ain, int m, int lda, double* __restrict__ w,
                              double* __restrict__ Z) {
  __shared__ double A[48 * 48];
  __shared__ double Q[48 * 48];
  const int lane = threadIdx.x;
  for (int t = lane; t < m * m; t += 32) {
    int r = t % m, c = t / m;
    A[t] = 0.5 * (Ain[r + c * lda] + Ain[c + r * lda]);
    Q[t] = (r == c) ? 1.0 : 0.0;
  }
  __syncwarp();
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int t = lane; t < m * m; t += 32) {
      int r = t % m, c = t / m;
      double v = A[t] * A[t];
      tot += v;
      if (r != c) off += v;
    }
    off = warp_sum(off);
    tot = warp_sum(tot);
    off = __shfl_sync(0xffffffffu, off, 0);
    tot = __shfl_sync(0xffffffffu, tot, 0);
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < m - 1; ++p) {
      for (int q = p + 1; q < m; ++q) {
        double apq = A[p + q * m];
        if (apq == 0.0) continue;
        double app = A[p + p * m], aqq = A[q + q * m];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        __syncwarp();
        // A <- J^T A J ; columns p,q then rows p,q
        for (int r = lane; r < m; r += 32) {
          double arp = A[r + p * m], arq = A[r + q * m];
          A[r + p * m] = c * arp - s * arq;
          A[r + q * m] = s * arp + c * arq;
        }
        __syncwarp();
        for (int r = lane; r < m; r += 32) {
          double apr = A[p + r * m], aqr = A[q + r * m];
          A[p + r * m] = c * apr - s * aqr;
          A[q + r * m] = s * apr + c * aqr;
        }
        __syncwarp();
        for (int r = lane; r < m; r += 32) {
          double qrp = Q[r + p * m], qrq = Q[r + q * m];
          Q[r + p * m] = c * qrp - s * qrq;
          Q[r + q * m] = s * qrp + c * qrq;
        }
        __syncwarp();
      }
    }
  }
  for (int t = lane; t < m; t += 32) w[t] = A[t + t * m];
  for (int t = lane; t < m * m; t += 32) Z[t] = Q[t];
}

// ---------------------------------------------------------------- FP32 basis
template <int NV>
__device__ __forceinline__ void block_reduce_store(float (&acc)[NV], int nv, double* __restrict__ part) {
  __shared__ double sh[BT / 32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double v = warp_sum((double)acc[k]);
    if (lane == 0) sh[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double t = 0.0;
    for (int q = 0; q < BT / 32; ++q) t += sh[q][threadIdx.x];
    part[(int64_t)blockIdx.x * NV + threadIdx.x] = t;
  }
}

__global__ void __launch_bounds__(BT) mdot_f32_kernel(const float* __restrict__ V, int64_t ldv, int nv,
                                                      const float* __restrict__ w, int64_t n,
                                                      double* __restrict__ part) {
  float acc[NV32];
#pragma unroll
  for (int k = 0; k < NV32; ++k) acc[k] = 0.f;
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i + st < n; i += 2 * st) {
    const int64_t i2 = i + st;
    const float wa = w[i], wb = w[i2];
#pragma unroll
    for (int k = 0; k < NV32; ++k)
      if (k < nv) {
        const float va = V[k * ldv + i], vb = V[k * ldv + i2];
        acc[k] = fmaf(va, wa, acc[k]);
        acc[k] = fmaf(vb, wb, acc[k]);
      }
  }
  if (i < n) {
    const float wi = w[i];
#pragma unroll
    for (int k = 0; k < NV32; ++k)
      if (k < nv) acc[k] = fmaf(V[k * ldv + i], wi, acc[k]);
  }
  block_reduce_store<NV32>(acc, nv, part);
}

__global__ void __launch_bounds__(BT) axpy_dot_f32_kernel(const float* __restrict__ V, int64_t ldv, int nv,
                                                          const double* __restrict__ h,
                                                          const float* __restrict__ win, float* __restrict__ wout,
                                                          int64_t n, double* __restrict__ part) {
  __shared__ float hs[NV32];
  if (threadIdx.x < NV32) hs[threadIdx.x] = (threadIdx.x < nv) ? (float)h[threadIdx.x] : 0.f;
  __syncthreads();
  float acc[NV32];
#pragma unroll
  for (int k = 0; k < NV32; ++k) acc[k] = 0.f;
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    float v[NV32];
    float w = win[i];
#pragma unroll
    for (int k = 0; k < NV32; ++k)
      if (k < nv) {
        v[k] = V[k * ldv + i];
        w = fmaf(-v[k], hs[k], w);
      }
    wout[i] = w;
#pragma unroll
    for (int k = 0; k < NV32; ++k)
      if (k < nv) acc[k] = fmaf(v[k], w, acc[k]);
  }
  block_reduce_store<NV32>(acc, nv, part);
}

__global__ void __launch_bounds__(BT) axpy_nrm_f32_kernel(const float* __restrict__ V, int64_t ldv, int nv,
                                                          const double* __restrict__ h, float* __restrict__ w,
                                                          int64_t n, double* __restrict__ part) {
  __shared__ float hs[NV32];
  if (threadIdx.x < NV32) hs[threadIdx.x] = (threadIdx.x < nv) ? (float)h[threadIdx.x] : 0.f;
  __syncthreads();
  float acc[1] = {0.f};
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i + st < n; i += 2 * st) {
    const int64_t i2 = i + st;
    float x = w[i], y = w[i2];
#pragma unroll
    for (int k = 0; k < NV32; ++k)
      if (k < nv) {
        x = fmaf(-V[k * ldv + i], hs[k], x);
        y = fmaf(-V[k * ldv + i2], hs[k], y);
      }
    w[i] = x;
    w[i2] = y;
    acc[0] = fmaf(x, x, acc[0]);
    acc[0] = fmaf(y, y, acc[0]);
  }
  if (i < n) {
    float x = w[i];
#pragma unroll
    for (int k = 0; k < NV32; ++k)
      if (k < nv) x = fmaf(-V[k * ldv + i], hs[k], x);
    w[i] = x;
    acc[0] = fmaf(x, x, acc[0]);
  }
  block_reduce_store<1>(acc, 1, part);
}

// w -= V h with FP32 data and FP32 arithmetic (h rounded to FP32)
__global__ void __launch_bounds__(BT) maxpy_f32_kernel(const float* __restrict__ V, int64_t ldv, int nv,
                                                       const double* __restrict__ h, float* __restrict__ w,
                                                       int64_t n) {
  __shared__ float hs[NV32];
  if (threadIdx.x < NV32) hs[threadIdx.x] = (threadIdx.x < nv) ? (float)h[threadIdx.x] : 0.f;
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    float acc = w[i];
#pragma unroll
    for (int k = 0; k < NV32; ++k)
      if (k < nv) acc = fmaf(-V[k * ldv + i], hs[k], acc);
    w[i] = acc;
  }
}

// Block dots: part[b][k*NW + j] = partial sums of V[k] . W[j] (FP32 data,
// FP32 per-thread accumulation, FP64 block reduction).  One sweep over KV
// basis columns serves NW vectors.
template <int KV, int NW>
__global__ void __launch_bounds__(BT) mdot_block_f32_kernel(const float* __restrict__ V, int64_t ldv, int kv,
                                                            F32Cols W, int nw, int64_t n,
                                                            double* __restrict__ part) {
  float acc[KV][NW];
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) acc[k][j] = 0.f;
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i + st < n; i += 2 * st) {
    const int64_t i2 = i + st;
    float wa[NW], wb[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      wa[j] = (j < nw) ? W.c[j][i] : 0.f;
      wb[j] = (j < nw) ? W.c[j][i2] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < KV; ++k)
      if (k < kv) {
        const float va = V[k * ldv + i], vb = V[k * ldv + i2];
#pragma unroll
        for (int j = 0; j < NW; ++j) {
          acc[k][j] = fmaf(va, wa[j], acc[k][j]);
          acc[k][j] = fmaf(vb, wb[j], acc[k][j]);
        }
      }
  }
  if (i < n) {
    float wv[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) wv[j] = (j < nw) ? W.c[j][i] : 0.f;
#pragma unroll
    for (int k = 0; k < KV; ++k)
      if (k < kv) {
        const float v = V[k * ldv + i];
#pragma unroll
        for (int j = 0; j < NW; ++j) acc[k][j] = fmaf(v, wv[j], acc[k][j]);
      }
  }
  __shared__ double sh[BT / 32][KV * NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      double v = warp_sum((double)acc[k][j]);
      if (lane == 0) sh[wid][k * NW + j] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < KV * NW; t += BT) {
    double a = 0.0;
    for (int q = 0; q < BT / 32; ++q) a += sh[q][t];
    part[(int64_t)blockIdx.x * (KV * NW) + t] = a;
  }
}

// FP64 block dots of FP64 columns against FP32 vectors (exact FP32 values,
// FP64 products and sums): part[b][k*NW + j] partial sums of V[k] . W[j].
template <int KV, int NW>
__global__ void __launch_bounds__(BT) mdot64_block_kernel(const double* __restrict__ V, int64_t ldv, int kv,
                                                          F32Cols W, int nw, int64_t n, double* __restrict__ part) {
  double acc[KV][NW];
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) acc[k][j] = 0.0;
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    double wv[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) wv[j] = (j < nw) ? (double)W.c[j][i] : 0.0;
#pragma unroll
    for (int k = 0; k < KV; ++k)
      if (k < kv) {
        const double v = V[k * ldv + i];
#pragma unroll
        for (int j = 0; j < NW; ++j)
          if (j < nw) acc[k][j] = fma(v, wv[j], acc[k][j]);
      }
  }
  __shared__ double sh[BT / 32][KV * NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      double v = warp_sum(acc[k][j]);
      if (lane == 0) sh[wid][k * NW + j] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < KV * NW; t += BT) {
    double a = 0.0;
    for (int q = 0; q < BT / 32; ++q) a += sh[q][t];
    part[(int64_t)blockIdx.x * (KV * NW) + t] = a;
  }
}

// H[(k0 + k) + j * ldh] = sum over blocks of part[b][k*NW + j]
__global__ void mdot_block_final(const double* __restrict__ part, int nb, int kv, int nw, int stride, int nws,
                                 double* H, int64_t ldh, int k0) {
  const int t = blockIdx.x;
  const int k = t / nw, j = t % nw;
  if (k >= kv) return;
  double a = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) a += part[(int64_t)b * stride + k * nws + j];
  a = warp_sum(a);
  __shared__ double shr[32];
  if ((threadIdx.x & 31) == 0) shr[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r += shr[q];
    H[(k0 + k) + (int64_t)j * ldh] = r;
  }
}

// W[j] -= sum_k V[k] H[k0 + k, j]  (FP32 data and arithmetic)
template <int KV, int NW>
__global__ void __launch_bounds__(BT) maxpy_block_f32_kernel(const float* __restrict__ V, int64_t ldv, int kv,
                                                             const double* __restrict__ H, int64_t ldh, int k0,
                                                             F32ColsMut W, int nw, int64_t n) {
  __shared__ float hs[KV][NW];
  for (int t = threadIdx.x; t < KV * NW; t += BT) {
    const int k = t / NW, j = t % NW;
    hs[k][j] = (k < kv && j < nw) ? (float)H[(k0 + k) + (int64_t)j * ldh] : 0.f;
  }
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    float v[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) v[k] = (k < kv) ? V[k * ldv + i] : 0.f;
#pragma unroll
    for (int j = 0; j < NW; ++j)
      if (j < nw) {
        float w = W.c[j][i];
#pragma unroll
        for (int k = 0; k < KV; ++k) w = fmaf(-v[k], hs[k][j], w);
        W.c[j][i] = w;
      }
  }
}

__global__ void normalize_f32_kernel(const float* __restrict__ w, const double* __restrict__ nsq,
                                     float* __restrict__ v, int64_t n) {
  const float inv = (float)(1.0 / sqrt(*nsq));
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) v[i] = w[i] * inv;
}

template <int MM>
__global__ void __launch_bounds__(BT) rotate_f32_kernel(float* __restrict__ V, int64_t ldv, int m,
                                                        const double* __restrict__ Y, int k, int64_t n) {
  __shared__ float Ys[MM * MM];
  for (int t = threadIdx.x; t < m * k; t += BT) Ys[t] = (float)Y[t];
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    float row[MM];
#pragma unroll
    for (int j = 0; j < MM; ++j) row[j] = (j < m) ? V[j * ldv + i] : 0.f;
#pragma unroll
    for (int c = 0; c < MM; ++c) {
      if (c < k) {
        float acc = 0.f;
#pragma unroll
        for (int j = 0; j < MM; ++j)
          if (j < m) acc = fmaf(row[j], Ys[c * m + j], acc);
        V[c * ldv + i] = acc;
      }
    }
  }
}

template <int MM>
__global__ void __launch_bounds__(BT) combine_f32_f64_kernel(const float* __restrict__ V, int64_t ldv, int m,
                                                             const double* __restrict__ Y, int k,
                                                             double* __restrict__ out, int64_t ldo, int64_t n) {
  __shared__ double Ys[MM * MM];
  for (int t = threadIdx.x; t < m * k; t += BT) Ys[t] = Y[t];
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    float row[MM];
#pragma unroll
    for (int j = 0; j < MM; ++j) row[j] = (j < m) ? V[j * ldv + i] : 0.f;
    for (int c = 0; c < k; ++c) {
      double acc = 0.0;
#pragma unroll
      for (int j = 0; j < MM; ++j)
        if (j < m) acc = fma((double)row[j], Ys[c * m + j], acc);
      out[c * ldo + i] = acc;
    }
  }
}

template <int MM>
__global__ void __launch_bounds__(BT) combine_f32_f32_kernel(const float* __restrict__ V, int64_t ldv, int m,
                                                             const double* __restrict__ Y, int k,
                                                             float* __restrict__ out, int64_t ldo, int64_t n) {
  __shared__ float Ys[MM * MM];
  for (int t = threadIdx.x; t < m * k; t += BT) Ys[t] = (float)Y[t];
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    float row[MM];
#pragma unroll
    for (int j = 0; j < MM; ++j) row[j] = (j < m) ? V[j * ldv + i] : 0.f;
    for (int c = 0; c < k; ++c) {
      float acc = 0.f;
#pragma unroll
      for (int j = 0; j < MM; ++j)
        if (j < m) acc = fmaf(row[j], Ys[c * m + j], acc);
      out[c * ldo + i] = acc;
    }
  }
}

__global__ void uniform_f32_kernel(float* __restrict__ v, int64_t n, uint64_t seed) {
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) {
    uint64_t r = splitmix64(seed * 0x100000001b3ull + (uint64_t)i);
    v[i] = (float)((double)(r >> 11) * (1.0 / 9007199254740992.0));
  }
}

__global__ void nrm_f32_kernel(const float* __restrict__ w, int64_t n, double* __restrict__ part) {
  float acc[1] = {0.f};
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (; i < n; i += st) acc[0] = fmaf(w[i], w[i], acc[0]);
  block_reduce_store<1>(acc, 1, part);
}

// ------------------------------------------------------- 16-byte vector forms
// Used when every column starts on a 16-byte boundary (ldv a multiple of 4
// floats / 2 doubles).  Each thread moves float4 / double2 per column, with
// U of them per column in flight for narrow bases; the n % 4 (n % 2) tail
// elements go to block 0.  Widths NVT are matched to the basis so the
// accumulators and loads in flight fit the registers.
__device__ __forceinline__ float dot4(const float4& a, const float4& b, float c) {
  c = fmaf(a.x, b.x, c);
  c = fmaf(a.y, b.y, c);
  c = fmaf(a.z, b.z, c);
  return fmaf(a.w, b.w, c);
}
__device__ __forceinline__ void sub4(float4& x, const float4& v, float h) {
  x.x = fmaf(-v.x, h, x.x);
  x.y = fmaf(-v.y, h, x.y);
  x.z = fmaf(-v.z, h, x.z);
  x.w = fmaf(-v.w, h, x.w);
}
__device__ __forceinline__ const float4* col4(const float* V, int64_t ldv, int k) {
  return reinterpret_cast<const float4*>(V + (int64_t)k * ldv);
}

template <int NVT, int U>
__global__ void __launch_bounds__(BT) mdot_f32v_kernel(const float* __restrict__ V, int64_t ldv, int nv,
                                                       const float* __restrict__ w, int64_t n,
                                                       double* __restrict__ part) {
  float acc[NVT];
#pragma unroll
  for (int k = 0; k < NVT; ++k) acc[k] = 0.f;
  const int64_t n4 = n >> 2;
  const int64_t st = (int64_t)gridDim.x * BT;
  const float4* w4 = reinterpret_cast<const float4*>(w);
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  for (; i + (U - 1) * st < n4; i += U * st) {
    float4 wv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) wv[u] = w4[i + u * st];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        const float4* vk = col4(V, ldv, k);
#pragma unroll
        for (int u = 0; u < U; ++u) acc[k] = dot4(vk[i + u * st], wv[u], acc[k]);
      }
  }
  for (; i < n4; i += st) {
    const float4 wv = w4[i];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) acc[k] = dot4(col4(V, ldv, k)[i], wv, acc[k]);
  }
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = (n4 << 2) + threadIdx.x;
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) acc[k] = fmaf(V[(int64_t)k * ldv + t], w[t], acc[k]);
  }
  block_reduce_store<NVT>(acc, nv, part);
}

// wout = win - V h ; part <- V . wout  (the V values stay in registers)
template <int NVT>
__global__ void __launch_bounds__(BT) axpy_dot_f32v_kernel(const float* __restrict__ V, int64_t ldv, int nv,
                                                           const double* __restrict__ h,
                                                           const float* __restrict__ win, float* __restrict__ wout,
                                                           int64_t n, double* __restrict__ part) {
  __shared__ float hs[NVT];
  if (threadIdx.x < NVT) hs[threadIdx.x] = (threadIdx.x < nv) ? (float)h[threadIdx.x] : 0.f;
  __syncthreads();
  float acc[NVT];
#pragma unroll
  for (int k = 0; k < NVT; ++k) acc[k] = 0.f;
  const int64_t n4 = n >> 2;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n4; i += st) {
    float4 v[NVT];
    float4 x = reinterpret_cast<const float4*>(win)[i];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        v[k] = col4(V, ldv, k)[i];
        sub4(x, v[k], hs[k]);
      }
    reinterpret_cast<float4*>(wout)[i] = x;
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) acc[k] = dot4(v[k], x, acc[k]);
  }
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = (n4 << 2) + threadIdx.x;
    float x = win[t];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) x = fmaf(-V[(int64_t)k * ldv + t], hs[k], x);
    wout[t] = x;
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) acc[k] = fmaf(V[(int64_t)k * ldv + t], x, acc[k]);
  }
  block_reduce_store<NVT>(acc, nv, part);
}

// ---- staged forms (columns streamed through shared memory by bulk copies)
// A chunk is kChunk floats of every column: 256 threads x one float4.  The
// chunks cover the first 4 * (n / 4) elements; block 0 takes the n % 4 tail
// with plain loads after the sweep.
constexpr int kChunk = 4 * BT;

// wout = win - V h ; part <- V . wout, for wide bases (9..16 columns): the
// update reads V and win from the stage, the dots read V again from there
template <int NVT>
__global__ void __launch_bounds__(BT, 1) axpy_dot_f32_staged(const float* __restrict__ V, int64_t ldv, int nv,
                                                             const double* __restrict__ h,
                                                             const float* __restrict__ win,
                                                             float* __restrict__ wout, int64_t n,
                                                             double* __restrict__ part, int nstage, int* err) {
  extern __shared__ __align__(128) float stg[];
  __shared__ __align__(8) uint64_t full[kStageMax];
  __shared__ float hs[NVT];
  if (threadIdx.x < NVT) hs[threadIdx.x] = (threadIdx.x < nv) ? (float)h[threadIdx.x] : 0.f;
  float acc[NVT];
#pragma unroll
  for (int k = 0; k < NVT; ++k) acc[k] = 0.f;
  const int ncol = nv + 1;  // V columns, then win
  const int64_t nf = (n >> 2) << 2;
  const int64_t nch = (nf + kChunk - 1) / kChunk;
  staged_sweep(
      full, nstage, nch, err,
      [&](int64_t c, int st, uint64_t* bar) {
        const int64_t e0 = c * kChunk;
        const uint32_t bytes = (uint32_t)(min((int64_t)kChunk, nf - e0) * 4);
        mbar_arrive_expect_tx(bar, bytes * ncol);
        float* d = stg + (int64_t)st * ncol * kChunk;
        for (int k = 0; k < nv; ++k) bulk_g2s(d + k * kChunk, V + (int64_t)k * ldv + e0, bytes, bar);
        bulk_g2s(d + nv * kChunk, win + e0, bytes, bar);
      },
      [&](int64_t c, int st) {
        const int64_t e0 = c * kChunk;
        const int t4 = threadIdx.x * 4;
        if (e0 + t4 >= nf) return;
        const float* d = stg + (int64_t)st * ncol * kChunk + t4;
        float4 x = *reinterpret_cast<const float4*>(d + nv * kChunk);
#pragma unroll
        for (int k = 0; k < NVT; ++k)
          if (k < nv) sub4(x, *reinterpret_cast<const float4*>(d + k * kChunk), hs[k]);
        __stcs(reinterpret_cast<float4*>(wout + e0 + t4), x);
#pragma unroll
        for (int k = 0; k < NVT; ++k)
          if (k < nv) acc[k] = dot4(*reinterpret_cast<const float4*>(d + k * kChunk), x, acc[k]);
      });
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = nf + threadIdx.x;
    float x = win[t];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) x = fmaf(-V[(int64_t)k * ldv + t], hs[k], x);
    wout[t] = x;
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) acc[k] = fmaf(V[(int64_t)k * ldv + t], x, acc[k]);
  }
  block_reduce_store<NVT>(acc, nv, part);
}

// part[b][k*NW + j] = partial sums of V[k] . W[j] (kv <= KV, nw <= NW), the
// kv + nw columns staged together
template <int KV, int NW>
__global__ void __launch_bounds__(BT, 1) mdot_block_f32_staged(const float* __restrict__ V, int64_t ldv, int kv,
                                                               F32Cols W, int nw, int64_t n,
                                                               double* __restrict__ part, int nstage, int* err) {
  extern __shared__ __align__(128) float stg[];
  __shared__ __align__(8) uint64_t full[kStageMax];
  float acc[KV][NW];
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) acc[k][j] = 0.f;
  const int ncol = kv + nw;  // V columns, then W columns
  const int64_t nf = (n >> 2) << 2;
  const int64_t nch = (nf + kChunk - 1) / kChunk;
  staged_sweep(
      full, nstage, nch, err,
      [&](int64_t c, int st, uint64_t* bar) {
        const int64_t e0 = c * kChunk;
        const uint32_t bytes = (uint32_t)(min((int64_t)kChunk, nf - e0) * 4);
        mbar_arrive_expect_tx(bar, bytes * ncol);
        float* d = stg + (int64_t)st * ncol * kChunk;
        for (int k = 0; k < kv; ++k) bulk_g2s(d + k * kChunk, V + (int64_t)k * ldv + e0, bytes, bar);
        for (int j = 0; j < nw; ++j) bulk_g2s(d + (kv + j) * kChunk, W.c[j] + e0, bytes, bar);
      },
      [&](int64_t c, int st) {
        const int t4 = threadIdx.x * 4;
        if (c * kChunk + t4 >= nf) return;
        const float* d = stg + (int64_t)st * ncol * kChunk + t4;
        float4 wv[NW];
#pragma unroll
        for (int j = 0; j < NW; ++j)
          wv[j] = (j < nw) ? *reinterpret_cast<const float4*>(d + (kv + j) * kChunk) : make_float4(0, 0, 0, 0);
#pragma unroll
        for (int k = 0; k < KV; ++k)
          if (k < kv) {
            const float4 v = *reinterpret_cast<const float4*>(d + k * kChunk);
#pragma unroll
            for (int j = 0; j < NW; ++j) acc[k][j] = dot4(v, wv[j], acc[k][j]);
          }
      });
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = nf + threadIdx.x;
#pragma unroll
    for (int k = 0; k < KV; ++k)
      if (k < kv) {
        const float v = V[(int64_t)k * ldv + t];
#pragma unroll
        for (int j = 0; j < NW; ++j)
          if (j < nw) acc[k][j] = fmaf(v, W.c[j][t], acc[k][j]);
      }
  }
  __shared__ double sh[BT / 32][KV * NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      double v = warp_sum((double)acc[k][j]);
      if (lane == 0) sh[wid][k * NW + j] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < KV * NW; t += BT) {
    double a = 0.0;
    for (int q = 0; q < BT / 32; ++q) a += sh[q][t];
    part[(int64_t)blockIdx.x * (KV * NW) + t] = a;
  }
}

// w -= V h in place; with NRM, part <- ||w||^2
template <int NVT, int U, bool NRM>
__global__ void __launch_bounds__(BT) axpy_f32v_kernel(const float* __restrict__ V, int64_t ldv, int nv,
                                                       const double* __restrict__ h, float* __restrict__ w,
                                                       int64_t n, double* __restrict__ part) {
  __shared__ float hs[NVT];
  if (threadIdx.x < NVT) hs[threadIdx.x] = (threadIdx.x < nv) ? (float)h[threadIdx.x] : 0.f;
  __syncthreads();
  float acc[1] = {0.f};
  const int64_t n4 = n >> 2;
  const int64_t st = (int64_t)gridDim.x * BT;
  float4* w4 = reinterpret_cast<float4*>(w);
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  for (; i + (U - 1) * st < n4; i += U * st) {
    float4 x[U];
#pragma unroll
    for (int u = 0; u < U; ++u) x[u] = w4[i + u * st];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        const float4* vk = col4(V, ldv, k);
#pragma unroll
        for (int u = 0; u < U; ++u) sub4(x[u], vk[i + u * st], hs[k]);
      }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      w4[i + u * st] = x[u];
      if (NRM) acc[0] = dot4(x[u], x[u], acc[0]);
    }
  }
  for (; i < n4; i += st) {
    float4 x = w4[i];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) sub4(x, col4(V, ldv, k)[i], hs[k]);
    w4[i] = x;
    if (NRM) acc[0] = dot4(x, x, acc[0]);
  }
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = (n4 << 2) + threadIdx.x;
    float x = w[t];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) x = fmaf(-V[(int64_t)k * ldv + t], hs[k], x);
    w[t] = x;
    if (NRM) acc[0] = fmaf(x, x, acc[0]);
  }
  if (NRM) block_reduce_store<1>(acc, 1, part);
}

// W[j] -= sum_k V[k] H[k0 + k, j]
template <int KV, int NW>
__global__ void __launch_bounds__(BT) maxpy_block_f32v_kernel(const float* __restrict__ V, int64_t ldv, int kv,
                                                              const double* __restrict__ H, int64_t ldh, int k0,
                                                              F32ColsMut W, int nw, int64_t n) {
  __shared__ float hs[KV][NW];
  for (int t = threadIdx.x; t < KV * NW; t += BT) {
    const int k = t / NW, j = t % NW;
    hs[k][j] = (k < kv && j < nw) ? (float)H[(k0 + k) + (int64_t)j * ldh] : 0.f;
  }
  __syncthreads();
  const int64_t n4 = n >> 2;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n4; i += st) {
    float4 v[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) v[k] = (k < kv) ? col4(V, ldv, k)[i] : make_float4(0, 0, 0, 0);
#pragma unroll
    for (int j = 0; j < NW; ++j)
      if (j < nw) {
        float4* wj = reinterpret_cast<float4*>(W.c[j]);
        float4 x = wj[i];
#pragma unroll
        for (int k = 0; k < KV; ++k) sub4(x, v[k], hs[k][j]);
        wj[i] = x;
      }
  }
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = (n4 << 2) + threadIdx.x;
    for (int j = 0; j < nw; ++j) {
      float x = W.c[j][t];
      for (int k = 0; k < kv; ++k) x = fmaf(-V[(int64_t)k * ldv + t], hs[k][j], x);
      W.c[j][t] = x;
    }
  }
}

// W[j] -= sum_{k < nv} V[k] H[k, j] in one sweep (nv <= 48): each W element
// is loaded and stored once however many basis columns there are
template <int NW>
__global__ void __launch_bounds__(BT) maxpy_block_all_f32v_kernel(const float* __restrict__ V, int64_t ldv, int nv,
                                                                  const double* __restrict__ H, int64_t ldh,
                                                                  F32ColsMut W, int nw, int64_t n) {
  __shared__ float hs[48][NW];
  for (int t = threadIdx.x; t < 48 * NW; t += BT) {
    const int k = t / NW, j = t % NW;
    hs[k][j] = (k < nv && j < nw) ? (float)H[k + (int64_t)j * ldh] : 0.f;
  }
  __syncthreads();
  const int64_t n4 = n >> 2;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n4; i += st) {
    float4 x[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) x[j] = (j < nw) ? reinterpret_cast<const float4*>(W.c[j])[i] : make_float4(0, 0, 0, 0);
    int k = 0;
    for (; k + 4 <= nv; k += 4) {
      float4 v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = col4(V, ldv, k + q)[i];
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int j = 0; j < NW; ++j) sub4(x[j], v[q], hs[k + q][j]);
    }
    for (; k < nv; ++k) {
      const float4 v = col4(V, ldv, k)[i];
#pragma unroll
      for (int j = 0; j < NW; ++j) sub4(x[j], v, hs[k][j]);
    }
#pragma unroll
    for (int j = 0; j < NW; ++j)
      if (j < nw) reinterpret_cast<float4*>(W.c[j])[i] = x[j];
  }
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = (n4 << 2) + threadIdx.x;
    for (int j = 0; j < nw; ++j) {
      float x = W.c[j][t];
      for (int k = 0; k < nv; ++k) x = fmaf(-V[(int64_t)k * ldv + t], hs[k][j], x);
      W.c[j][t] = x;
    }
  }
}

__global__ void normalize_f32v_kernel(const float* __restrict__ w, const double* __restrict__ nsq,
                                      float* __restrict__ v, int64_t n) {
  const float inv = (float)(1.0 / sqrt(*nsq));
  const int64_t n4 = n >> 2;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n4; i += st) {
    float4 x = reinterpret_cast<const float4*>(w)[i];
    x.x *= inv;
    x.y *= inv;
    x.z *= inv;
    x.w *= inv;
    reinterpret_cast<float4*>(v)[i] = x;
  }
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = (n4 << 2) + threadIdx.x;
    v[t] = w[t] * inv;
  }
}

__global__ void nrm_f32v_kernel(const float* __restrict__ w, int64_t n, double* __restrict__ part) {
  float acc[1] = {0.f};
  const int64_t n4 = n >> 2;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n4; i += st) {
    const float4 x = reinterpret_cast<const float4*>(w)[i];
    acc[0] = dot4(x, x, acc[0]);
  }
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const float x = w[(n4 << 2) + threadIdx.x];
    acc[0] = fmaf(x, x, acc[0]);
  }
  block_reduce_store<1>(acc, 1, part);
}

// out[:, c] = V[:, 0..m) Y[:, c] for c < k (in place when out == V: every
// row is read before any is written), m <= MM; FP32 or FP64 output
template <int MM, class OutT>
__global__ void __launch_bounds__(BT) combine_f32v_kernel(const float* V, int64_t ldv, int m,
                                                          const double* __restrict__ Y, int k, OutT* out,
                                                          int64_t ldo, int64_t n) {
  using AccT = OutT;
  __shared__ AccT Ys[MM * MM];
  for (int t = threadIdx.x; t < m * k; t += BT) Ys[t] = (AccT)Y[t];
  __syncthreads();
  const int64_t n4 = n >> 2;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n4; i += st) {
    float4 row[MM];
#pragma unroll
    for (int j = 0; j < MM; ++j) row[j] = (j < m) ? col4(V, ldv, j)[i] : make_float4(0, 0, 0, 0);
    for (int c = 0; c < k; ++c) {
      AccT a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma unroll
      for (int j = 0; j < MM; ++j)
        if (j < m) {
          const AccT y = Ys[c * m + j];
          a0 = fma((AccT)row[j].x, y, a0);
          a1 = fma((AccT)row[j].y, y, a1);
          a2 = fma((AccT)row[j].z, y, a2);
          a3 = fma((AccT)row[j].w, y, a3);
        }
      OutT* o = out + (int64_t)c * ldo + (i << 2);
      if (sizeof(OutT) == 4) {
        *reinterpret_cast<float4*>(o) = make_float4((float)a0, (float)a1, (float)a2, (float)a3);
      } else {
        reinterpret_cast<double2*>(o)[0] = make_double2((double)a0, (double)a1);
        reinterpret_cast<double2*>(o)[1] = make_double2((double)a2, (double)a3);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < (int)(n & 3)) {
    const int64_t t = (n4 << 2) + threadIdx.x;
    AccT row[MM];
    for (int j = 0; j < m; ++j) row[j] = (AccT)V[(int64_t)j * ldv + t];
    for (int c = 0; c < k; ++c) {
      AccT a = 0;
      for (int j = 0; j < m; ++j) a = fma(row[j], Ys[c * m + j], a);
      out[(int64_t)c * ldo + t] = (OutT)a;
    }
  }
}

// ---- FP64 columns, double2 loads
__device__ __forceinline__ const double2* col2(const double* V, int64_t ldv, int k) {
  return reinterpret_cast<const double2*>(V + (int64_t)k * ldv);
}

// part <- V . w  (w FP64, or scale * w32 with W32)
template <int NVT, int U, bool W32>
__global__ void __launch_bounds__(BT) mdot_v2_kernel(const double* __restrict__ V, int64_t ldv, int nv,
                                                     const double* __restrict__ w, const float* __restrict__ w32,
                                                     double scale, int64_t n, double* __restrict__ part) {
  double acc[NVT];
#pragma unroll
  for (int k = 0; k < NVT; ++k) acc[k] = 0.0;
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  auto wload = [&](int64_t i) -> double2 {
    if (W32) {
      const float2 f = reinterpret_cast<const float2*>(w32)[i];
      return make_double2(scale * (double)f.x, scale * (double)f.y);
    }
    return reinterpret_cast<const double2*>(w)[i];
  };
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  for (; i + (U - 1) * st < n2; i += U * st) {
    double2 wv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) wv[u] = wload(i + u * st);
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        const double2* vk = col2(V, ldv, k);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const double2 v = vk[i + u * st];
          acc[k] = fma(v.x, wv[u].x, acc[k]);
          acc[k] = fma(v.y, wv[u].y, acc[k]);
        }
      }
  }
  for (; i < n2; i += st) {
    const double2 wv = wload(i);
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        const double2 v = col2(V, ldv, k)[i];
        acc[k] = fma(v.x, wv.x, acc[k]);
        acc[k] = fma(v.y, wv.y, acc[k]);
      }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) {
    const int64_t t = n - 1;
    const double wt = W32 ? scale * (double)w32[t] : w[t];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) acc[k] = fma(V[(int64_t)k * ldv + t], wt, acc[k]);
  }
  __shared__ double sh[BT / 32][NVT];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NVT; ++k) {
    const double v = warp_sum(acc[k]);
    if (lane == 0) sh[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < NVT) {
    double t = 0.0;
    for (int q = 0; q < BT / 32; ++q) t += sh[q][threadIdx.x];
    part[(int64_t)blockIdx.x * NVT + threadIdx.x] = t;
  }
}

// w = (W32 ? scale * w32 : w) - V h
template <int NVT, int U, bool W32>
__global__ void __launch_bounds__(BT) maxpy_v2_kernel(const double* __restrict__ V, int64_t ldv, int nv,
                                                      const double* __restrict__ h, const float* __restrict__ w32,
                                                      double scale, double* __restrict__ w, int64_t n) {
  __shared__ double hs[NVT];
  if (threadIdx.x < NVT) hs[threadIdx.x] = (threadIdx.x < nv) ? h[threadIdx.x] : 0.0;
  __syncthreads();
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  double2* w2 = reinterpret_cast<double2*>(w);
  int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x;
  for (; i + (U - 1) * st < n2; i += U * st) {
    double2 x[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (W32) {
        const float2 f = reinterpret_cast<const float2*>(w32)[i + u * st];
        x[u] = make_double2(scale * (double)f.x, scale * (double)f.y);
      } else {
        x[u] = w2[i + u * st];
      }
    }
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        const double2* vk = col2(V, ldv, k);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const double2 v = vk[i + u * st];
          x[u].x = fma(-v.x, hs[k], x[u].x);
          x[u].y = fma(-v.y, hs[k], x[u].y);
        }
      }
#pragma unroll
    for (int u = 0; u < U; ++u) w2[i + u * st] = x[u];
  }
  for (; i < n2; i += st) {
    double2 x;
    if (W32) {
      const float2 f = reinterpret_cast<const float2*>(w32)[i];
      x = make_double2(scale * (double)f.x, scale * (double)f.y);
    } else {
      x = w2[i];
    }
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        const double2 v = col2(V, ldv, k)[i];
        x.x = fma(-v.x, hs[k], x.x);
        x.y = fma(-v.y, hs[k], x.y);
      }
    w2[i] = x;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) {
    const int64_t t = n - 1;
    double x = W32 ? scale * (double)w32[t] : w[t];
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) x = fma(-V[(int64_t)k * ldv + t], hs[k], x);
    w[t] = x;
  }
}

// part[b][k*NW + j] = partial sums of V[k] . W[j], V FP64, W FP32 (exact in FP64)
template <int KV, int NW>
__global__ void __launch_bounds__(BT) mdot64_block_v2_kernel(const double* __restrict__ V, int64_t ldv, int kv,
                                                             F32Cols W, int nw, int64_t n,
                                                             double* __restrict__ part) {
  double acc[KV][NW];
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) acc[k][j] = 0.0;
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n2; i += st) {
    double2 wv[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      if (j < nw) {
        const float2 f = reinterpret_cast<const float2*>(W.c[j])[i];
        wv[j] = make_double2((double)f.x, (double)f.y);
      } else {
        wv[j] = make_double2(0.0, 0.0);
      }
    }
#pragma unroll
    for (int k = 0; k < KV; ++k)
      if (k < kv) {
        const double2 v = col2(V, ldv, k)[i];
#pragma unroll
        for (int j = 0; j < NW; ++j)
          if (j < nw) {
            acc[k][j] = fma(v.x, wv[j].x, acc[k][j]);
            acc[k][j] = fma(v.y, wv[j].y, acc[k][j]);
          }
      }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) {
    const int64_t t = n - 1;
#pragma unroll
    for (int k = 0; k < KV; ++k)
      if (k < kv)
#pragma unroll
        for (int j = 0; j < NW; ++j)
          if (j < nw) acc[k][j] = fma(V[(int64_t)k * ldv + t], (double)W.c[j][t], acc[k][j]);
  }
  __shared__ double sh[BT / 32][KV * NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      const double v = warp_sum(acc[k][j]);
      if (lane == 0) sh[wid][k * NW + j] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < KV * NW; t += BT) {
    double a = 0.0;
    for (int q = 0; q < BT / 32; ++q) a += sh[q][t];
    part[(int64_t)blockIdx.x * (KV * NW) + t] = a;
  }
}

__global__ void nrm_v2_kernel(const double* __restrict__ w, int64_t n, double* __restrict__ part) {
  double acc = 0.0;
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n2; i += st) {
    const double2 x = reinterpret_cast<const double2*>(w)[i];
    acc = fma(x.x, x.x, acc);
    acc = fma(x.y, x.y, acc);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) acc = fma(w[n - 1], w[n - 1], acc);
  __shared__ double sh[BT / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < BT / 32; ++q) t += sh[q];
    part[blockIdx.x] = t;
  }
}

inline bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
inline bool al8(const void* p) { return ((uintptr_t)p & 7u) == 0; }
// every column of a float basis on a 16-byte boundary
inline bool cols4(const float* V, int64_t ldv) { return al16(V) && (ldv & 3) == 0; }
inline bool cols2(const double* V, int64_t ldv) { return al16(V) && (ldv & 1) == 0; }

}  // namespace

int* stage_err_word() {
  static std::mutex mu;
  static int* words[64] = {};
  int dev = 0;
  TM_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) fail(TM_ERR_CUDA, "device index out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!words[dev]) {
    int* p = nullptr;
    TM_CK(cudaMalloc(&p, sizeof(int)));
    TM_CK(cudaMemset(p, 0, sizeof(int)));
    words[dev] = p;
  }
  return words[dev];
}

void stage_err_check(cudaStream_t s) {
  int* w = stage_err_word();
  int h = 0;
  TM_CK(cudaMemcpyAsync(&h, w, sizeof(int), cudaMemcpyDeviceToHost, s));
  TM_CK(cudaStreamSynchronize(s));
  if (h) {
    TM_CK(cudaMemsetAsync(w, 0, sizeof(int), s));
    fail(TM_ERR_CUDA, "a shared-memory stage of a Krylov sweep was not filled in time");
  }
}

int stage_count(int64_t chunk_bytes) {
  return (int)std::max<int64_t>(2, std::min<int64_t>(kStageMax, kStageBytes / chunk_bytes));
}

namespace {
// Grid of a staged launch: as many CTAs per SM as the stages' shared memory
// lets reside (at most kRedBlocksPerSM, the partial-sum buffers' bound).
template <class K>
int staged_grid(K kernel, size_t shm) {
  raise_smem_limit((const void*)kernel, shm);
  int occ = 0;
  TM_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, BT, shm));
  return num_sms() * std::max(1, std::min(occ, kRedBlocksPerSM));
}
}  // namespace

void mdot_f32(const float* V, int64_t ldv, int nv, const float* w, int64_t n, double* h, double* part,
              cudaStream_t s) {
  const bool vec = cols4(V, ldv) && al16(w);
  for (int k0 = 0; k0 < nv; k0 += NV32) {
    const int kk = std::min(NV32, nv - k0);
    const int nb = red_blocks(n);
    const float* Vk = V + (int64_t)k0 * ldv;
    int stride = NV32;
    if (!vec) {
      mdot_f32_kernel<<<nb, BT, 0, s>>>(Vk, ldv, kk, w, n, part);
    } else if (kk <= 3) {
      mdot_f32v_kernel<4, 2><<<nb, BT, 0, s>>>(Vk, ldv, kk, w, n, part);
      stride = 4;
    } else if (kk <= 8) {
      mdot_f32v_kernel<8, 2><<<nb, BT, 0, s>>>(Vk, ldv, kk, w, n, part);
      stride = 8;
    } else if (kk <= 12) {
      mdot_f32v_kernel<12, 1><<<nb, BT, 0, s>>>(Vk, ldv, kk, w, n, part);
      stride = 12;
    } else {
      mdot_f32v_kernel<16, 1><<<nb, BT, 0, s>>>(Vk, ldv, kk, w, n, part);
    }
    TM_CKK("mdot_f32");
    mdot_final<<<kk, 256, 0, s>>>(part, nb, kk, stride, h + k0);
    TM_CKK("mdot_final");
  }
}

static bool cols_al16(const float* const* c, int nw) {
  for (int j = 0; j < nw; ++j)
    if (!al16(c[j])) return false;
  return true;
}
static bool cols_al8(const float* const* c, int nw) {
  for (int j = 0; j < nw; ++j)
    if (!al8(c[j])) return false;
  return true;
}

void mdot_block_f32(const float* V, int64_t ldv, int nv, const F32Cols& W, int nw, int64_t n, double* H,
                    int64_t ldh, double* part, cudaStream_t s) {
  if (nw < 1 || nw > kMaxBlockW) fail(TM_ERR_LIMIT, "mdot_block_f32: 1..8 vectors");
  constexpr int KV = 8;
  const int nb = red_blocks(n);
  const bool vec = cols4(V, ldv) && cols_al16(W.c, nw);
  for (int k0 = 0; k0 < nv; k0 += KV) {
    const int kv = std::min(KV, nv - k0);
    const float* Vk = V + (int64_t)k0 * ldv;
    if (vec) {
      // the kv + nw columns staged together (the accumulators halve when the
      // block is narrow)
      const int nst = stage_count((int64_t)(kv + nw) * kChunk * 4);
      const size_t shm = (size_t)nst * (kv + nw) * kChunk * 4;
      const int nws = (nw <= 4) ? 4 : kMaxBlockW;
      auto kfn = (nw <= 4) ? mdot_block_f32_staged<KV, 4> : mdot_block_f32_staged<KV, kMaxBlockW>;
      const int gs = staged_grid(kfn, shm);
      kfn<<<gs, BT, shm, s>>>(Vk, ldv, kv, W, nw, n, part, nst, stage_err_word());
      TM_CKK("mdot_block_f32");
      mdot_block_final<<<kv * nw, 256, 0, s>>>(part, gs, kv, nw, KV * nws, nws, H, ldh, k0);
    } else if (nw <= 4) {  // half the accumulators when the block is narrow
      mdot_block_f32_kernel<KV, 4><<<nb, BT, 0, s>>>(Vk, ldv, kv, W, nw, n, part);
      TM_CKK("mdot_block_f32");
      mdot_block_final<<<kv * nw, 256, 0, s>>>(part, nb, kv, nw, KV * 4, 4, H, ldh, k0);
    } else {
      mdot_block_f32_kernel<KV, kMaxBlockW><<<nb, BT, 0, s>>>(Vk, ldv, kv, W, nw, n, part);
      TM_CKK("mdot_block_f32");
      mdot_block_final<<<kv * nw, 256, 0, s>>>(part, nb, kv, nw, KV * kMaxBlockW, kMaxBlockW, H, ldh, k0);
    }
    TM_CKK("mdot_block_final");
  }
}

void maxpy_block_f32(const float* V, int64_t ldv, int nv, const double* H, int64_t ldh, const F32ColsMut& W, int nw,
                     int64_t n, cudaStream_t s) {
  if (nw < 1 || nw > kMaxBlockW) fail(TM_ERR_LIMIT, "maxpy_block_f32: 1..8 vectors");
  constexpr int KV = 8;
  const bool vec = cols4(V, ldv) && cols_al16(W.c, nw);
  if (vec && nv <= 48) {
    if (nw <= 4)
      maxpy_block_all_f32v_kernel<4><<<red_blocks(n), BT, 0, s>>>(V, ldv, nv, H, ldh, W, nw, n);
    else
      maxpy_block_all_f32v_kernel<kMaxBlockW><<<red_blocks(n), BT, 0, s>>>(V, ldv, nv, H, ldh, W, nw, n);
    TM_CKK("maxpy_block_f32");
    return;
  }
  for (int k0 = 0; k0 < nv; k0 += KV) {
    const int kv = std::min(KV, nv - k0);
    const float* Vk = V + (int64_t)k0 * ldv;
    if (vec && nw <= 4)
      maxpy_block_f32v_kernel<KV, 4><<<red_blocks(n), BT, 0, s>>>(Vk, ldv, kv, H, ldh, k0, W, nw, n);
    else if (vec)
      maxpy_block_f32v_kernel<KV, kMaxBlockW><<<red_blocks(n), BT, 0, s>>>(Vk, ldv, kv, H, ldh, k0, W, nw, n);
    else
      maxpy_block_f32_kernel<KV, kMaxBlockW><<<red_blocks(n), BT, 0, s>>>(Vk, ldv, kv, H, ldh, k0, W, nw, n);
    TM_CKK("maxpy_block_f32");
  }
}

void mdot64_block(const double* V, int64_t ldv, int nv, const F32Cols& W, int nw, int64_t n, double* H,
                  int64_t ldh, double* part, cudaStream_t s) {
  if (nw < 1 || nw > 4) fail(TM_ERR_LIMIT, "mdot64_block: 1..4 vectors");
  constexpr int KV = 8, NW = 4;
  const int nb = red_blocks(n);
  const bool vec = cols2(V, ldv) && cols_al8(W.c, nw);
  for (int k0 = 0; k0 < nv; k0 += KV) {
    const int kv = std::min(KV, nv - k0);
    if (vec)
      mdot64_block_v2_kernel<KV, NW><<<nb, BT, 0, s>>>(V + (int64_t)k0 * ldv, ldv, kv, W, nw, n, part);
    else
      mdot64_block_kernel<KV, NW><<<nb, BT, 0, s>>>(V + (int64_t)k0 * ldv, ldv, kv, W, nw, n, part);
    TM_CKK("mdot64_block");
    mdot_block_final<<<kv * nw, 256, 0, s>>>(part, nb, kv, nw, KV * NW, NW, H, ldh, k0);
    TM_CKK("mdot_block_final");
  }
}

size_t mdot_block_part_bytes() { return red_part_bytes(8 * kMaxBlockW); }
size_t red_part_bytes(int width) { return (size_t)num_sms() * kRedBlocksPerSM * width * sizeof(double) + 64; }

void maxpy_f32(const float* V, int64_t ldv, int nv, const double* h, float* w, int64_t n, cudaStream_t s) {
  const bool vec = cols4(V, ldv) && al16(w);
  for (int k0 = 0; k0 < nv; k0 += NV32) {
    const int kk = std::min(NV32, nv - k0);
    const float* Vk = V + (int64_t)k0 * ldv;
    const int nb = red_blocks(n);
    if (!vec)
      maxpy_f32_kernel<<<nb, BT, 0, s>>>(Vk, ldv, kk, h + k0, w, n);
    else if (kk <= 4)
      axpy_f32v_kernel<4, 2, false><<<nb, BT, 0, s>>>(Vk, ldv, kk, h + k0, w, n, nullptr);
    else if (kk <= 8)
      axpy_f32v_kernel<8, 1, false><<<nb, BT, 0, s>>>(Vk, ldv, kk, h + k0, w, n, nullptr);
    else
      axpy_f32v_kernel<16, 1, false><<<nb, BT, 0, s>>>(Vk, ldv, kk, h + k0, w, n, nullptr);
    TM_CKK("maxpy_f32");
  }
}

void axpy_dot_f32(const float* V, int64_t ldv, int nv, const double* h, const float* win, float* wout, int64_t n,
                  double* h2, double* part, cudaStream_t s) {
  if (nv > NV32) fail(TM_ERR_LIMIT, "axpy_dot_f32: too many vectors");
  int nb = red_blocks(n);
  int stride = NV32;
  if (!(cols4(V, ldv) && al16(win) && al16(wout))) {
    axpy_dot_f32_kernel<<<nb, BT, 0, s>>>(V, ldv, nv, h, win, wout, n, part);
  } else if (nv <= 4) {
    axpy_dot_f32v_kernel<4><<<nb, BT, 0, s>>>(V, ldv, nv, h, win, wout, n, part);
    stride = 4;
  } else if (nv <= 8) {
    axpy_dot_f32v_kernel<8><<<nb, BT, 0, s>>>(V, ldv, nv, h, win, wout, n, part);
    stride = 8;
  } else {
    // wide bases: staged, so the sweep is not limited by the registers that
    // hold one vector of every column
    const int nst = stage_count((int64_t)(nv + 1) * kChunk * 4);
    const size_t shm = (size_t)nst * (nv + 1) * kChunk * 4;
    auto kfn = axpy_dot_f32_staged<NV32>;
    const int gs = staged_grid(kfn, shm);
    kfn<<<gs, BT, shm, s>>>(V, ldv, nv, h, win, wout, n, part, nst, stage_err_word());
    nb = gs;
  }
  TM_CKK("axpy_dot_f32");
  mdot_final<<<nv, 256, 0, s>>>(part, nb, nv, stride, h2);
  TM_CKK("mdot_final");
}

void axpy_nrm_f32(const float* V, int64_t ldv, int nv, const double* h, float* w, int64_t n, double* nsq,
                  double* part, cudaStream_t s) {
  if (nv > NV32) fail(TM_ERR_LIMIT, "axpy_nrm_f32: too many vectors");
  const int nb = red_blocks(n);
  if (!(cols4(V, ldv) && al16(w)))
    axpy_nrm_f32_kernel<<<nb, BT, 0, s>>>(V, ldv, nv, h, w, n, part);
  else if (nv <= 4)
    axpy_f32v_kernel<4, 2, true><<<nb, BT, 0, s>>>(V, ldv, nv, h, w, n, part);
  else if (nv <= 8)
    axpy_f32v_kernel<8, 1, true><<<nb, BT, 0, s>>>(V, ldv, nv, h, w, n, part);
  else
    axpy_f32v_kernel<16, 1, true><<<nb, BT, 0, s>>>(V, ldv, nv, h, w, n, part);
  TM_CKK("axpy_nrm_f32");
  mdot_final<<<1, 256, 0, s>>>(part, nb, 1, 1, nsq);
  TM_CKK("mdot_final");
}

void normalize_f32(const float* w, const double* nsq, float* v, int64_t n, cudaStream_t s) {
  if (al16(w) && al16(v))
    normalize_f32v_kernel<<<red_blocks(n), BT, 0, s>>>(w, nsq, v, n);
  else
    normalize_f32_kernel<<<red_blocks(n), BT, 0, s>>>(w, nsq, v, n);
  TM_CKK("normalize_f32");
}

void rotate_f32(float* V, int64_t ldv, int m, const double* Y, int k, int64_t n, cudaStream_t s) {
  if (m <= 16 && cols4(V, ldv))
    combine_f32v_kernel<16, float><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, V, ldv, n);
  else if (m <= 16)
    rotate_f32_kernel<16><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, n);
  else if (m <= 32)
    rotate_f32_kernel<32><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, n);
  else
    fail(TM_ERR_LIMIT, "rotate_f32: basis too large");
  TM_CKK("rotate_f32");
}

void combine_f32_f64(const float* V, int64_t ldv, int m, const double* Y, int k, double* out, int64_t ldo, int64_t n,
                     cudaStream_t s) {
  if (m <= 16 && cols4(V, ldv) && al16(out) && (ldo & 1) == 0)
    combine_f32v_kernel<16, double><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  else if (m <= 16)
    combine_f32_f64_kernel<16><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  else if (m <= 32)
    combine_f32_f64_kernel<32><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  else
    fail(TM_ERR_LIMIT, "combine_f32_f64: basis too large");
  TM_CKK("combine_f32_f64");
}

void combine_f32(const float* V, int64_t ldv, int m, const double* Y, int k, float* out, int64_t ldo, int64_t n,
                 cudaStream_t s) {
  if (m <= 16 && cols4(V, ldv) && cols4(out, ldo))
    combine_f32v_kernel<16, float><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  else if (m <= 16)
    combine_f32_f32_kernel<16><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  else if (m <= 32)
    combine_f32_f32_kernel<32><<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  else
    fail(TM_ERR_LIMIT, "combine_f32: basis too large");
  TM_CKK("combine_f32");
}

void fill_uniform_f32(float* v, int64_t n, uint64_t seed, cudaStream_t s) {
  uniform_f32_kernel<<<red_blocks(n), BT, 0, s>>>(v, n, seed);
  TM_CKK("uniform_f32");
}

void nrm2sq_f32(const float* w, int64_t n, double* out, double* part, cudaStream_t s) {
  int nb = red_blocks(n);
  if (al16(w))
    nrm_f32v_kernel<<<nb, BT, 0, s>>>(w, n, part);
  else
    nrm_f32_kernel<<<nb, BT, 0, s>>>(w, n, part);
  TM_CKK("nrm_f32");
  mdot_final<<<1, 256, 0, s>>>(part, nb, 1, 1, out);
  TM_CKK("mdot_final");
}

static void mdot_impl(const double* V, int64_t ldv, int nv, const double* w, const float* w32, double scale,
                      int64_t n, double* h, double* part, cudaStream_t s) {
  const bool vec = cols2(V, ldv) && (w32 ? al8(w32) : al16(w));
  for (int k0 = 0; k0 < nv; k0 += NVMAX) {
    const int kk = std::min(NVMAX, nv - k0);
    const int nb = red_blocks(n);
    const double* Vk = V + (int64_t)k0 * ldv;
    int stride = NVMAX;
    if (vec) {
#define TM_MDOT_V(NVT, U)                                                                            \
  do {                                                                                                \
    if (w32)                                                                                          \
      mdot_v2_kernel<NVT, U, true><<<nb, BT, 0, s>>>(Vk, ldv, kk, nullptr, w32, scale, n, part);      \
    else                                                                                              \
      mdot_v2_kernel<NVT, U, false><<<nb, BT, 0, s>>>(Vk, ldv, kk, w, nullptr, 1.0, n, part);         \
    stride = NVT;                                                                                     \
  } while (0)
      if (kk <= 4)
        TM_MDOT_V(4, 2);
      else if (kk <= 8)
        TM_MDOT_V(8, 1);
      else
        TM_MDOT_V(16, 1);
#undef TM_MDOT_V
    } else if (w32) {
      mdot_kernel<NVMAX, true><<<nb, BT, 0, s>>>(Vk, ldv, kk, nullptr, w32, scale, n, part);
    } else {
      mdot_kernel<NVMAX, false><<<nb, BT, 0, s>>>(Vk, ldv, kk, w, nullptr, 1.0, n, part);
    }
    TM_CKK("mdot");
    mdot_final<<<kk, 256, 0, s>>>(part, nb, kk, stride, h + k0);
    TM_CKK("mdot_final");
  }
}

void mdot(const double* V, int64_t ldv, int nv, const double* w, int64_t n, double* h, double* part,
          cudaStream_t s) {
  mdot_impl(V, ldv, nv, w, nullptr, 1.0, n, h, part, s);
}
void mdot32(const double* V, int64_t ldv, int nv, const float* w32, double scale, int64_t n, double* h,
            double* part, cudaStream_t s) {
  mdot_impl(V, ldv, nv, nullptr, w32, scale, n, h, part, s);
}

// w = (w32 ? scale * w32 : w) - V h over one chunk of <= NVMAX columns
static void maxpy_chunk(const double* V, int64_t ldv, int kk, const double* h, const float* w32, double scale,
                        double* w, int64_t n, cudaStream_t s) {
  const int nb = red_blocks(n);
  if (cols2(V, ldv) && al16(w) && (!w32 || al8(w32))) {
#define TM_MAXPY_V(NVT, U)                                                                           \
  do {                                                                                                \
    if (w32)                                                                                          \
      maxpy_v2_kernel<NVT, U, true><<<nb, BT, 0, s>>>(V, ldv, kk, h, w32, scale, w, n);               \
    else                                                                                              \
      maxpy_v2_kernel<NVT, U, false><<<nb, BT, 0, s>>>(V, ldv, kk, h, nullptr, 1.0, w, n);            \
  } while (0)
    if (kk <= 4)
      TM_MAXPY_V(4, 2);
    else if (kk <= 8)
      TM_MAXPY_V(8, 1);
    else
      TM_MAXPY_V(16, 1);
#undef TM_MAXPY_V
  } else if (w32) {
    maxpy_kernel<NVMAX, true><<<nb, BT, 0, s>>>(V, ldv, kk, h, w32, scale, w, n);
  } else {
    maxpy_kernel<NVMAX, false><<<nb, BT, 0, s>>>(V, ldv, kk, h, nullptr, 1.0, w, n);
  }
  TM_CKK("maxpy");
}

void maxpy(const double* V, int64_t ldv, int nv, const double* h, double* w, int64_t n, cudaStream_t s) {
  for (int k0 = 0; k0 < nv; k0 += NVMAX)
    maxpy_chunk(V + (int64_t)k0 * ldv, ldv, std::min(NVMAX, nv - k0), h + k0, nullptr, 1.0, w, n, s);
}

void maxpy32(const double* V, int64_t ldv, int nv, const double* h, const float* w32, double scale, double* w,
             int64_t n, cudaStream_t s) {
  maxpy_chunk(V, ldv, std::min(NVMAX, nv), h, w32, scale, w, n, s);
  if (nv > NVMAX) maxpy(V + NVMAX * ldv, ldv, nv - NVMAX, h + NVMAX, w, n, s);
}

void nrm2sq(const double* w, int64_t n, double* out, double* part, cudaStream_t s) {
  int nb = red_blocks(n);
  if (al16(w))
    nrm_v2_kernel<<<nb, BT, 0, s>>>(w, n, part);
  else
    nrm_kernel<<<nb, BT, 0, s>>>(w, n, part);
  TM_CKK("nrm");
  mdot_final<<<1, 256, 0, s>>>(part, nb, 1, 1, out);
  TM_CKK("nrm_final");
}

void normalize(const double* w, const double* nsq, double* v, float* v32, int64_t n, cudaStream_t s) {
  normalize_kernel<<<red_blocks(n), BT, 0, s>>>(w, nsq, v, v32, n);
  TM_CKK("normalize");
}

void basis_rotate(double* V, int64_t ldv, int m, const double* Y, int k, int64_t n, cudaStream_t s) {
  rotate_kernel<<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, n);
  TM_CKK("rotate");
}

void basis_combine(const double* V, int64_t ldv, int m, const double* Y, int k, double* out, int64_t ldo, int64_t n,
                   cudaStream_t s) {
  if (m > 64 || m * k > 64 * 64) fail(TM_ERR_LIMIT, "basis_combine: block too large");
  combine_kernel<<<red_blocks(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  TM_CKK("combine");
}

void to_f32(const double* in, float* out, int64_t n, cudaStream_t s) {
  to_f32_kernel<<<red_blocks(n), BT, 0, s>>>(in, out, n);
  TM_CKK("to_f32");
}

void axpby(double a, const double* x, double b, const double* y, double* out, int64_t n, cudaStream_t s) {
  axpby_kernel<<<red_blocks(n), BT, 0, s>>>(a, x, b, y, out, n);
  TM_CKK("axpby");
}

void fill_uniform(double* v, int64_t n, uint64_t seed, cudaStream_t s) {
  uniform_kernel<<<red_blocks(n), BT, 0, s>>>(v, n, seed);
  TM_CKK("uniform");
}

void count_nonfinite(const double* v, int64_t n, unsigned int* cnt, cudaStream_t s) {
  nonfinite_kernel<<<red_blocks(n), BT, 0, s>>>(v, n, cnt);
  TM_CKK("nonfinite");
}

void small_symeig(const double* A, int m, double* w, double* Z, cudaStream_t s, int lda) {
  if (m > 48) fail(TM_ERR_LIMIT, "small eigenproblem larger than 48");
  symeig_kernel<<<1, 32, 0, s>>>(A, m, lda, w, Z);
  TM_CKK("symeig");
}

}  // namespace ltm
