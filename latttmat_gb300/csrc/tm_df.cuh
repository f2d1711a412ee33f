// Double-float ("float-float") arithmetic for FP64-accurate products on the
// FP32 pipes.
//
// A value is hi + lo with |lo| <= ulp(hi)/2 (about 48 significant bits).
// Addition uses Knuth's TwoSum, multiplication the FMA-based TwoProduct,
// each followed by a fast renormalisation (Dekker 1971; Knuth, TAOCP vol. 2,
// sec. 4.2.2).  On GB300 the FP32 pipes are roughly 64x faster than FP64,
// so a double-float butterfly (about 20 FP32 operations per output) beats a
// native FP64 one several times over, at relative error ~1e-14 per sweep.
#pragma once
#include <cuda_runtime.h>

namespace ltm {

struct __align__(8) dfloat {
  float hi, lo;
  __host__ __device__ dfloat() {}
  __host__ __device__ dfloat(int v) : hi((float)v), lo(0.f) {}
  __host__ __device__ dfloat(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ dfloat(double v) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
  }
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dfloat df_renorm(float s, float e) {
  float h = s + e;
  return dfloat(h, e - (h - s));
}

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  return df_renorm(s, e);
}

__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_renorm(p, e);
}

// a * b + c with one renormalisation (TwoProduct by FMA, then TwoSum)
__device__ __forceinline__ dfloat df_fma(dfloat a, dfloat b, dfloat c) {
  float p = a.hi * b.hi;
  float pe = fmaf(a.hi, b.hi, -p);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  float s = p + c.hi;
  float bb = s - p;
  float se = (p - (s - bb)) + (c.hi - bb);
  se += pe + c.lo;
  return df_renorm(s, se);
}

// df_fma without the final renormalisation: hi + lo still carries the exact
// TwoSum error, but |lo| may exceed ulp(hi)/2 by a few ulps.  For chains of
// a few such steps (the butterfly levels of one round) followed by df_norm;
// the operands' lo enter only as correction terms, so accuracy is unchanged
// up to a few units of 2^-48.
__device__ __forceinline__ dfloat df_fma_unnorm(dfloat a, dfloat b, dfloat c) {
  float p = a.hi * b.hi;
  float pe = fmaf(a.hi, b.hi, -p);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  float s = p + c.hi;
  float bb = s - p;
  float se = (p - (s - bb)) + (c.hi - bb);
  se += pe + c.lo;
  return dfloat(s, se);
}

__device__ __forceinline__ dfloat df_norm(dfloat a) { return df_renorm(a.hi, a.lo); }

__device__ __forceinline__ dfloat& operator+=(dfloat& a, dfloat b) {
  a = a + b;
  return a;
}
__device__ __forceinline__ dfloat& operator*=(dfloat& a, dfloat b) {
  a = a * b;
  return a;
}

// Forward-mode tangent pair (value, derivative with respect to one
// parameter): the adjoint's tangent products of the aux-bit chains run the
// chain steps in this type, d(a b) = da b + a db, d(a + b) = da + db.  Both
// parts are double-float, so the products run on the FP32 pipes at
// FP64-level accuracy (~1e-14), in the FP32 exponent range (the chains
// normalise their steps as the other double-float products do).
struct __align__(16) tangent {
  dfloat v, d;
  __host__ __device__ tangent() {}
  __host__ __device__ tangent(double x) : v(x), d(0.0) {}
  __host__ __device__ tangent(double x, double dx) : v(x), d(dx) {}
  __host__ __device__ tangent(dfloat x, dfloat dx) : v(x), d(dx) {}
};

__device__ __forceinline__ tangent operator+(tangent a, tangent b) { return tangent(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ tangent operator*(tangent a, tangent b) {
  return tangent(a.v * b.v, df_fma(a.d, b.v, a.v * b.d));
}
__device__ __forceinline__ tangent& operator+=(tangent& a, tangent b) {
  a = a + b;
  return a;
}
__device__ __forceinline__ tangent& operator*=(tangent& a, tangent b) {
  a = a * b;
  return a;
}

}  // namespace ltm
