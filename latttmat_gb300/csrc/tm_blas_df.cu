// Krylov kernels on double-float vectors: each element is a (hi, lo) pair of
// FP32 values, hi + lo with about 48 significant bits (tm_df.cuh), 8 bytes
// like an FP64 element.  The refinement keeps its FP64-accurate vectors (the
// wanted Ritz vectors and their products) in this form, so their arithmetic
// runs on the FP32 pipes: on GB300 an FP64 FMA costs about as much issue time
// as 64 FP32 operations, while a double-float multiply-add is about 14.
//
// Columns start on 16-byte boundaries (leading dimension even): the kernels
// move two elements per 16-byte load.  Results of dot products come back in
// FP64 (per-block double-float partials, summed in FP64).
#include <cmath>

#include "tm_blas.cuh"
#include "tm_df.cuh"

namespace ltm {

namespace {

constexpr int BT = 256;

int blocks_df(int64_t n) {
  const int64_t b = (n + 2 * BT - 1) / (2 * BT);
  const int64_t cap = (int64_t)num_sms() * kRedBlocksPerSM;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// acc + a * b for an FP32 a (exact TwoProduct of a * b.hi, plus a * b.lo)
__device__ __forceinline__ dfloat df_fma_f(float a, dfloat b, dfloat acc) {
  const float p = a * b.hi;
  float e = fmaf(a, b.hi, -p);
  e = fmaf(a, b.lo, e);
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  float err = (acc.hi - (s - bb)) + (p - bb);
  err += e + acc.lo;
  return df_renorm(s, err);
}

// two consecutive elements of a double-float column
struct df2 {
  dfloat a, b;
};
__device__ __forceinline__ df2 ld2(const dfloat* p, int64_t i) {
  const float4 v = reinterpret_cast<const float4*>(p)[i];
  return df2{dfloat(v.x, v.y), dfloat(v.z, v.w)};
}
__device__ __forceinline__ void st2(dfloat* p, int64_t i, const df2& v) {
  reinterpret_cast<float4*>(p)[i] = make_float4(v.a.hi, v.a.lo, v.b.hi, v.b.lo);
}

// block reduction of NV double-float partials into part[block * NV + k]
template <int NV>
__device__ __forceinline__ void block_store_df(const dfloat (&acc)[NV], double* __restrict__ part) {
  __shared__ double sh[BT / 32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double v = warp_sum_d((double)acc[k].hi + (double)acc[k].lo);
    if (lane == 0) sh[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double t = 0.0;
    for (int q = 0; q < BT / 32; ++q) t += sh[q][threadIdx.x];
    part[(int64_t)blockIdx.x * NV + threadIdx.x] = t;
  }
}

__global__ void final_df_kernel(const double* __restrict__ part, int nb, int nv, int stride, double* __restrict__ h) {
  const int k = blockIdx.x;
  if (k >= nv) return;
  double t = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) t += part[(int64_t)b * stride + k];
  t = warp_sum_d(t);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += sh[q];
    h[k] = s;
  }
}

// part <- V[k] . w, k < nv
template <int NVT>
__global__ void __launch_bounds__(BT) mdot_dd_kernel(const dfloat* __restrict__ V, int64_t ldv, int nv,
                                                     const dfloat* __restrict__ w, int64_t n,
                                                     double* __restrict__ part) {
  dfloat acc[NVT];
#pragma unroll
  for (int k = 0; k < NVT; ++k) acc[k] = dfloat(0.f, 0.f);
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n2; i += st) {
    const df2 x = ld2(w, i);
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        const df2 v = ld2(V + (int64_t)k * ldv, i);
        acc[k] = df_fma(v.a, x.a, acc[k]);
        acc[k] = df_fma(v.b, x.b, acc[k]);
      }
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t t = n - 1;
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) acc[k] = df_fma(V[(int64_t)k * ldv + t], w[t], acc[k]);
  }
  block_store_df<NVT>(acc, part);
}

// w -= sum_k V[k] h[k]  (h FP64 on the device)
template <int NVT>
__global__ void __launch_bounds__(BT) maxpy_dd_kernel(const dfloat* __restrict__ V, int64_t ldv, int nv,
                                                      const double* __restrict__ h, dfloat* __restrict__ w,
                                                      int64_t n) {
  __shared__ dfloat hs[NVT];
  if (threadIdx.x < NVT) hs[threadIdx.x] = (threadIdx.x < nv) ? dfloat(-h[threadIdx.x]) : dfloat(0.f, 0.f);
  __syncthreads();
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n2; i += st) {
    df2 x = ld2(w, i);
#pragma unroll
    for (int k = 0; k < NVT; ++k)
      if (k < nv) {
        const df2 v = ld2(V + (int64_t)k * ldv, i);
        x.a = df_fma(v.a, hs[k], x.a);
        x.b = df_fma(v.b, hs[k], x.b);
      }
    st2(w, i, x);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t t = n - 1;
    dfloat x = w[t];
    for (int k = 0; k < nv; ++k) x = df_fma(V[(int64_t)k * ldv + t], hs[k], x);
    w[t] = x;
  }
}

__global__ void __launch_bounds__(BT) nrm_dd_kernel(const dfloat* __restrict__ w, int64_t n,
                                                    double* __restrict__ part) {
  dfloat acc[1] = {dfloat(0.f, 0.f)};
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n2; i += st) {
    const df2 x = ld2(w, i);
    acc[0] = df_fma(x.a, x.a, acc[0]);
    acc[0] = df_fma(x.b, x.b, acc[0]);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) acc[0] = df_fma(w[n - 1], w[n - 1], acc[0]);
  block_store_df<1>(acc, part);
}

// out = a x + b y; with nsq != nullptr, a is replaced by a / sqrt(*nsq).
// Element-wise, so out may be x or y (in-place updates and normalisation).
__global__ void __launch_bounds__(BT) axpby_dd_kernel(double a, const dfloat* x, double b, const dfloat* y,
                                                      dfloat* out, int64_t n, const double* __restrict__ nsq) {
  __shared__ dfloat ab[2];
  if (threadIdx.x == 0) {
    ab[0] = dfloat(nsq ? a / sqrt(*nsq) : a);
    ab[1] = dfloat(b);
  }
  __syncthreads();
  const dfloat ca = ab[0], cb = ab[1];
  const bool two = (b != 0.0);
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n2; i += st) {
    const df2 u = ld2(x, i);
    df2 r{ca * u.a, ca * u.b};
    if (two) {
      const df2 v = ld2(y, i);
      r.a = df_fma(cb, v.a, r.a);
      r.b = df_fma(cb, v.b, r.b);
    }
    st2(out, i, r);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t t = n - 1;
    dfloat r = ca * x[t];
    if (two) r = df_fma(cb, y[t], r);
    out[t] = r;
  }
}

// out[:, c] = V32[:, 0..m) Y[:, c] in double-float (Y FP64, m <= MM, k <= 8)
template <int MM>
__global__ void __launch_bounds__(BT) combine_f32_dd_kernel(const float* __restrict__ V, int64_t ldv, int m,
                                                            const double* __restrict__ Y, int k,
                                                            dfloat* __restrict__ out, int64_t ldo, int64_t n) {
  __shared__ dfloat Ys[MM * 8];
  for (int t = threadIdx.x; t < m * k; t += BT) Ys[t] = dfloat(Y[t]);
  __syncthreads();
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n2; i += st) {
    float2 row[MM];
#pragma unroll
    for (int j = 0; j < MM; ++j)
      row[j] = (j < m) ? reinterpret_cast<const float2*>(V + (int64_t)j * ldv)[i] : make_float2(0.f, 0.f);
    for (int c = 0; c < k; ++c) {
      df2 acc{dfloat(0.f, 0.f), dfloat(0.f, 0.f)};
#pragma unroll
      for (int j = 0; j < MM; ++j)
        if (j < m) {
          const dfloat y = Ys[c * m + j];
          acc.a = df_fma_f(row[j].x, y, acc.a);
          acc.b = df_fma_f(row[j].y, y, acc.b);
        }
      st2(out + (int64_t)c * ldo, i, acc);
    }
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t t = n - 1;
    for (int c = 0; c < k; ++c) {
      dfloat acc(0.f, 0.f);
      for (int j = 0; j < m; ++j) acc = df_fma_f(V[(int64_t)j * ldv + t], Ys[c * m + j], acc);
      out[(int64_t)c * ldo + t] = acc;
    }
  }
}

// part[b][k*NW + j] partial sums of V[k] . W[j]: V double-float, W FP32
template <int KV, int NW>
__global__ void __launch_bounds__(BT) mdot_dd_block_kernel(const dfloat* __restrict__ V, int64_t ldv, int kv,
                                                           F32Cols W, int nw, int64_t n,
                                                           double* __restrict__ part) {
  dfloat acc[KV][NW];
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) acc[k][j] = dfloat(0.f, 0.f);
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t i = (int64_t)blockIdx.x * BT + threadIdx.x; i < n2; i += st) {
    float2 wv[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j)
      wv[j] = (j < nw) ? reinterpret_cast<const float2*>(W.c[j])[i] : make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < KV; ++k)
      if (k < kv) {
        const df2 v = ld2(V + (int64_t)k * ldv, i);
#pragma unroll
        for (int j = 0; j < NW; ++j) {
          acc[k][j] = df_fma_f(wv[j].x, v.a, acc[k][j]);
          acc[k][j] = df_fma_f(wv[j].y, v.b, acc[k][j]);
        }
      }
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t t = n - 1;
    for (int k = 0; k < kv; ++k)
      for (int j = 0; j < nw; ++j) acc[k][j] = df_fma_f(W.c[j][t], V[(int64_t)k * ldv + t], acc[k][j]);
  }
  __shared__ double sh[BT / 32][KV * NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      const double v = warp_sum_d((double)acc[k][j].hi + (double)acc[k][j].lo);
      if (lane == 0) sh[wid][k * NW + j] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < KV * NW; t += BT) {
    double a = 0.0;
    for (int q = 0; q < BT / 32; ++q) a += sh[q][t];
    part[(int64_t)blockIdx.x * (KV * NW) + t] = a;
  }
}

// part[b][i * NY + j] partial sums of V[i] . V[j], i < nx, j < ny (all
// double-float columns of one block)
template <int NX, int NY>
__global__ void __launch_bounds__(BT) mdot_dd_gram_kernel(const dfloat* __restrict__ V, int64_t ldv, int nx,
                                                          int ny, int64_t n, double* __restrict__ part) {
  dfloat acc[NX][NY];
#pragma unroll
  for (int i = 0; i < NX; ++i)
#pragma unroll
    for (int j = 0; j < NY; ++j) acc[i][j] = dfloat(0.f, 0.f);
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t t = (int64_t)blockIdx.x * BT + threadIdx.x; t < n2; t += st) {
    df2 row[NY];
#pragma unroll
    for (int j = 0; j < NY; ++j)
      row[j] = (j < ny) ? ld2(V + (int64_t)j * ldv, t) : df2{dfloat(0.f, 0.f), dfloat(0.f, 0.f)};
#pragma unroll
    for (int i = 0; i < NX; ++i)
#pragma unroll
      for (int j = 0; j < NY; ++j)
        if (i < nx && j < ny) {
          acc[i][j] = df_fma(row[i].a, row[j].a, acc[i][j]);
          acc[i][j] = df_fma(row[i].b, row[j].b, acc[i][j]);
        }
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t t = n - 1;
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j) acc[i][j] = df_fma(V[(int64_t)i * ldv + t], V[(int64_t)j * ldv + t], acc[i][j]);
  }
  __shared__ double sh[BT / 32][NX * NY];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NX; ++i)
#pragma unroll
    for (int j = 0; j < NY; ++j) {
      const double v = warp_sum_d((double)acc[i][j].hi + (double)acc[i][j].lo);
      if (lane == 0) sh[wid][i * NY + j] = v;
    }
  __syncthreads();
  for (int q = threadIdx.x; q < NX * NY; q += BT) {
    double a = 0.0;
    for (int w = 0; w < BT / 32; ++w) a += sh[w][q];
    part[(int64_t)blockIdx.x * (NX * NY) + q] = a;
  }
}

// V[:, c] = sum_j V[:, j] Y[c * k + j], c < k <= KK, in place (each thread
// reads its rows of all k columns before writing any)
template <int KK>
__global__ void __launch_bounds__(BT) combine_dd_inplace_kernel(dfloat* __restrict__ V, int64_t ldv, int k,
                                                                const double* __restrict__ Y, int64_t n) {
  __shared__ double ys[KK * KK];
  for (int q = threadIdx.x; q < k * k; q += BT) ys[q] = Y[q];
  __syncthreads();
  dfloat yd[KK * KK];
#pragma unroll
  for (int q = 0; q < KK * KK; ++q) yd[q] = (q < k * k) ? dfloat(ys[q]) : dfloat(0.f, 0.f);
  const int64_t n2 = n >> 1;
  const int64_t st = (int64_t)gridDim.x * BT;
  for (int64_t t = (int64_t)blockIdx.x * BT + threadIdx.x; t < n2; t += st) {
    df2 row[KK];
#pragma unroll
    for (int j = 0; j < KK; ++j)
      if (j < k) row[j] = ld2(V + (int64_t)j * ldv, t);
#pragma unroll
    for (int c = 0; c < KK; ++c)
      if (c < k) {
        df2 o{dfloat(0.f, 0.f), dfloat(0.f, 0.f)};
#pragma unroll
        for (int j = 0; j < KK; ++j)
          if (j < k) {
            o.a = df_fma(yd[c * k + j], row[j].a, o.a);
            o.b = df_fma(yd[c * k + j], row[j].b, o.b);
          }
        st2(V + (int64_t)c * ldv, t, o);
      }
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int64_t t = n - 1;
    dfloat r[KK];
    for (int j = 0; j < k; ++j) r[j] = V[(int64_t)j * ldv + t];
    for (int c = 0; c < k; ++c) {
      dfloat o(0.f, 0.f);
      for (int j = 0; j < k; ++j) o = df_fma(yd[c * k + j], r[j], o);
      V[(int64_t)c * ldv + t] = o;
    }
  }
}

__global__ void block_final_df_kernel(const double* __restrict__ part, int nb, int kv, int nw, int stride, int nws,
                                      double* H, int64_t ldh, int k0) {
  const int t = blockIdx.x;
  const int k = t / nw, j = t % nw;
  if (k >= kv) return;
  double a = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) a += part[(int64_t)b * stride + k * nws + j];
  a = warp_sum_d(a);
  __shared__ double shr[32];
  if ((threadIdx.x & 31) == 0) shr[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r += shr[q];
    H[(k0 + k) + (int64_t)j * ldh] = r;
  }
}

// Conversions, two elements (16 bytes of double-float or FP64) per access and
// four accesses per thread in flight; the odd tail element goes to block 0.
// Every column starts on a 16-byte boundary.
constexpr int kConvU = 4;

__global__ void df_to_f32_kernel(const dfloat* __restrict__ x, float* __restrict__ out, int64_t n) {
  const int64_t n2 = n >> 1, st = (int64_t)gridDim.x * blockDim.x;
  const float4* x4 = reinterpret_cast<const float4*>(x);
  float2* o2 = reinterpret_cast<float2*>(out);
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + (kConvU - 1) * st < n2; i += kConvU * st) {
    float4 v[kConvU];
#pragma unroll
    for (int u = 0; u < kConvU; ++u) v[u] = __ldcs(x4 + i + u * st);
#pragma unroll
    for (int u = 0; u < kConvU; ++u) o2[i + u * st] = make_float2(v[u].x + v[u].y, v[u].z + v[u].w);
  }
  for (; i < n2; i += st) {
    const float4 v = __ldcs(x4 + i);
    o2[i] = make_float2(v.x + v.y, v.z + v.w);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) out[n - 1] = x[n - 1].hi + x[n - 1].lo;
}

__global__ void df_to_f64_kernel(const dfloat* __restrict__ x, double scale, double* __restrict__ out, int64_t n) {
  const int64_t n2 = n >> 1, st = (int64_t)gridDim.x * blockDim.x;
  const float4* x4 = reinterpret_cast<const float4*>(x);
  double2* o2 = reinterpret_cast<double2*>(out);
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  auto cv = [&](const float4& v) {
    return make_double2(((double)v.x + (double)v.y) * scale, ((double)v.z + (double)v.w) * scale);
  };
  for (; i + (kConvU - 1) * st < n2; i += kConvU * st) {
    float4 v[kConvU];
#pragma unroll
    for (int u = 0; u < kConvU; ++u) v[u] = __ldcs(x4 + i + u * st);
#pragma unroll
    for (int u = 0; u < kConvU; ++u) o2[i + u * st] = cv(v[u]);
  }
  for (; i < n2; i += st) o2[i] = cv(__ldcs(x4 + i));
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0)
    out[n - 1] = ((double)x[n - 1].hi + (double)x[n - 1].lo) * scale;
}

__global__ void f64_to_df_kernel(const double* __restrict__ x, double scale, dfloat* __restrict__ out, int64_t n) {
  const int64_t n2 = n >> 1, st = (int64_t)gridDim.x * blockDim.x;
  const double2* x2 = reinterpret_cast<const double2*>(x);
  float4* o4 = reinterpret_cast<float4*>(out);
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  auto cv = [&](const double2& v) {
    const dfloat a(v.x * scale), b(v.y * scale);
    return make_float4(a.hi, a.lo, b.hi, b.lo);
  };
  for (; i + (kConvU - 1) * st < n2; i += kConvU * st) {
    double2 v[kConvU];
#pragma unroll
    for (int u = 0; u < kConvU; ++u) v[u] = __ldcs(x2 + i + u * st);
#pragma unroll
    for (int u = 0; u < kConvU; ++u) o4[i + u * st] = cv(v[u]);
  }
  for (; i < n2; i += st) o4[i] = cv(__ldcs(x2 + i));
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) out[n - 1] = dfloat(x[n - 1] * scale);
}

}  // namespace

void mdot_dd(const dfloat* V, int64_t ldv, int nv, const dfloat* w, int64_t n, double* h, double* part,
             cudaStream_t s) {
  if (nv < 1) return;
  if (nv > 8) fail(TM_ERR_LIMIT, "mdot_dd: at most 8 columns");
  const int nb = blocks_df(n);
  int stride = 8;
  if (nv <= 4) {
    mdot_dd_kernel<4><<<nb, BT, 0, s>>>(V, ldv, nv, w, n, part);
    stride = 4;
  } else {
    mdot_dd_kernel<8><<<nb, BT, 0, s>>>(V, ldv, nv, w, n, part);
  }
  TM_CKK("mdot_dd");
  final_df_kernel<<<nv, 256, 0, s>>>(part, nb, nv, stride, h);
  TM_CKK("mdot_dd_final");
}

void maxpy_dd(const dfloat* V, int64_t ldv, int nv, const double* h, dfloat* w, int64_t n, cudaStream_t s) {
  if (nv < 1) return;
  if (nv > 8) fail(TM_ERR_LIMIT, "maxpy_dd: at most 8 columns");
  if (nv <= 4)
    maxpy_dd_kernel<4><<<blocks_df(n), BT, 0, s>>>(V, ldv, nv, h, w, n);
  else
    maxpy_dd_kernel<8><<<blocks_df(n), BT, 0, s>>>(V, ldv, nv, h, w, n);
  TM_CKK("maxpy_dd");
}

void nrm2sq_dd(const dfloat* w, int64_t n, double* out, double* part, cudaStream_t s) {
  const int nb = blocks_df(n);
  nrm_dd_kernel<<<nb, BT, 0, s>>>(w, n, part);
  TM_CKK("nrm_dd");
  final_df_kernel<<<1, 256, 0, s>>>(part, nb, 1, 1, out);
  TM_CKK("nrm_dd_final");
}

void axpby_dd(double a, const dfloat* x, double b, const dfloat* y, dfloat* out, int64_t n, cudaStream_t s) {
  axpby_dd_kernel<<<blocks_df(n), BT, 0, s>>>(a, x, b, y, out, n, nullptr);
  TM_CKK("axpby_dd");
}

void normalize_dd(dfloat* w, const double* nsq, int64_t n, cudaStream_t s) {
  axpby_dd_kernel<<<blocks_df(n), BT, 0, s>>>(1.0, w, 0.0, w, w, n, nsq);
  TM_CKK("normalize_dd");
}

void combine_f32_dd(const float* V, int64_t ldv, int m, const double* Y, int k, dfloat* out, int64_t ldo, int64_t n,
                    cudaStream_t s) {
  if (k > 8) fail(TM_ERR_LIMIT, "combine_f32_dd: at most 8 outputs");
  if (m <= 16)
    combine_f32_dd_kernel<16><<<blocks_df(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  else if (m <= 32)
    combine_f32_dd_kernel<32><<<blocks_df(n), BT, 0, s>>>(V, ldv, m, Y, k, out, ldo, n);
  else
    fail(TM_ERR_LIMIT, "combine_f32_dd: basis too large");
  TM_CKK("combine_f32_dd");
}

void mdot_dd_block(const dfloat* V, int64_t ldv, int nv, const F32Cols& W, int nw, int64_t n, double* H, int64_t ldh,
                   double* part, cudaStream_t s) {
  if (nw < 1 || nw > 4) fail(TM_ERR_LIMIT, "mdot_dd_block: 1..4 vectors");
  // four double-float columns per launch: 16 accumulators keep the kernel
  // near 64 registers, so an SM holds enough warps to cover the loads
  constexpr int KV = 4, NW = 4;
  const int nb = blocks_df(n);
  for (int k0 = 0; k0 < nv; k0 += KV) {
    const int kv = std::min(KV, nv - k0);
    mdot_dd_block_kernel<KV, NW><<<nb, BT, 0, s>>>(V + (int64_t)k0 * ldv, ldv, kv, W, nw, n, part);
    TM_CKK("mdot_dd_block");
    block_final_df_kernel<<<kv * nw, 256, 0, s>>>(part, nb, kv, nw, KV * NW, NW, H, ldh, k0);
    TM_CKK("mdot_dd_block_final");
  }
}

void mdot_dd_gram(const dfloat* V, int64_t ldv, int nx, int ny, int64_t n, double* G, double* part, cudaStream_t s) {
  if (nx < 1 || nx > 4 || ny < nx || ny > 8) fail(TM_ERR_LIMIT, "mdot_dd_gram: 1..4 of up to 8 columns");
  constexpr int NX = 4, NY = 8;
  const int nb = blocks_df(n);
  mdot_dd_gram_kernel<NX, NY><<<nb, BT, 0, s>>>(V, ldv, nx, ny, n, part);
  TM_CKK("mdot_dd_gram");
  // column-major G (ld nx): entry (i, j) from the partials' slot i * NY + j
  block_final_df_kernel<<<nx * ny, 256, 0, s>>>(part, nb, nx, ny, NX * NY, NY, G, nx, 0);
  TM_CKK("mdot_dd_gram_final");
}

void combine_dd_inplace(dfloat* V, int64_t ldv, int k, const double* Y, int64_t n, cudaStream_t s) {
  if (k < 1 || k > 4) fail(TM_ERR_LIMIT, "combine_dd_inplace: 1..4 columns");
  combine_dd_inplace_kernel<4><<<blocks_df(n), BT, 0, s>>>(V, ldv, k, Y, n);
  TM_CKK("combine_dd_inplace");
}

void df_to_f32(const dfloat* x, float* out, int64_t n, cudaStream_t s) {
  df_to_f32_kernel<<<blocks_df(2 * n), BT, 0, s>>>(x, out, n);
  TM_CKK("df_to_f32");
}

void df_to_f64(const dfloat* x, double scale, double* out, int64_t n, cudaStream_t s) {
  df_to_f64_kernel<<<blocks_df(2 * n), BT, 0, s>>>(x, scale, out, n);
  TM_CKK("df_to_f64");
}

void f64_to_df(const double* x, double scale, dfloat* out, int64_t n, cudaStream_t s) {
  f64_to_df_kernel<<<blocks_df(2 * n), BT, 0, s>>>(x, scale, out, n);
  TM_CKK("f64_to_df");
}

size_t dd_part_bytes(int width) { return (size_t)num_sms() * kRedBlocksPerSM * width * sizeof(double) + 64; }

}  // namespace ltm
