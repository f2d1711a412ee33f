// Spin-state bit utilities shared by host and device code.
//
// States are L-bit integers (bit i = spin at site i, 1 = down).  These helpers
// restate the reference's Spin namespace (TMat/utility.hpp:36-128,
// TMat/utility.cpp:17-120) with integer semantics that must match bit-exactly:
// popcounts, cyclic shifts, bit reversal of the low nbit bits, and the exact
// integer power used for Kronecker factors.  Device code uses the hardware
// popcount / bit-reverse / funnel-shift instructions.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define TM_HD __host__ __device__ __forceinline__
#else
#define TM_HD inline
#endif

namespace ltm {

TM_HD int popc64(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __popcll(v);
#else
  return __builtin_popcountll(v);
#endif
}

// Spin::offsetState (TMat/utility.hpp:120-123): cyclic right shift by d of an
// n-bit state (site i moves to site i-d).
TM_HD uint64_t rotr(uint64_t s, int n, int d) {
  if (d == 0) return s;
  return (s >> d) | ((s & ((1ull << d) - 1)) << (n - d));
}

// Spin::lffsetState (TMat/utility.hpp:128-131): cyclic left shift by d.
TM_HD uint64_t rotl(uint64_t s, int n, int d) {
  if (d == 0) return s;
  uint64_t m = (n >= 64) ? ~0ull : ((1ull << n) - 1);
  return ((s << d) & m) | (s >> (n - d));
}

// Spin::bitreversal (TMat/utility.cpp:17-31): reverse the low nbit bits.
TM_HD uint64_t brev(uint64_t s, int nbit) {
#if defined(__CUDA_ARCH__)
  return __brevll(s) >> (64 - nbit);
#else
  s = ((s >> 1) & 0x5555555555555555ull) | ((s & 0x5555555555555555ull) << 1);
  s = ((s >> 2) & 0x3333333333333333ull) | ((s & 0x3333333333333333ull) << 2);
  s = ((s >> 4) & 0x0f0f0f0f0f0f0f0full) | ((s & 0x0f0f0f0f0f0f0f0full) << 4);
  s = ((s >> 8) & 0x00ff00ff00ff00ffull) | ((s & 0x00ff00ff00ff00ffull) << 8);
  s = ((s >> 16) & 0x0000ffff0000ffffull) | ((s & 0x0000ffff0000ffffull) << 16);
  s = (s >> 32) | (s << 32);
  return s >> (64 - nbit);
#endif
}

// Spin::powdi (TMat/utility.hpp:65-84): a[0]^(-b) by repeated squaring, with
// a = {base, 1/base}.  Same multiplication order as the reference so the
// result is the same double.
TM_HD double powdi(const double a0, const double a1, int b) {
  double result = 1.0;
  double t;
  if (b < 0) {
    b = -b;
    t = a0;
  } else {
    t = a1;
  }
  while (b) {
    if (b & 1) result *= t;
    t *= t;
    b >>= 1;
  }
  return result;
}

// Spin::spinBzexp (TMat/utility.hpp:104-115)
TM_HD int bzexp(uint64_t s, int n) { return 2 * popc64(s) - n; }
TM_HD int bzexp2(uint64_t a, uint64_t b, int n) { return 2 * popc64(a ^ b) - n; }

// Spin::nnode (TMat/utility.cpp:35-47): number of domain walls in a layer.
TM_HD int nnode(uint64_t s, int n, int open_boundary) {
  uint64_t t = s >> 1;
  if (!open_boundary)
    t |= (s & 1) << (n - 1);
  else
    t |= (s & (uint64_t)(n - 1)) << 1;  // reference quirk kept verbatim
  return popc64(s ^ t);
}

// 3D layer helpers (TMat/utility.cpp:52-120).  A 3D layer of size1 rows by
// size2 columns is packed row-major: bit r*size2+c.
TM_HD uint64_t rshift3d(uint64_t s, int size1, int size2, int d) {
  uint64_t mask = (1ull << size2) - 1, r = 0;
  for (int row = 0; row < size1; ++row) {
    r |= rotr(s & mask, size2, d) << (row * size2);
    s >>= size2;
  }
  return r;
}
TM_HD uint64_t dshift3d(uint64_t s, int size1, int size2, int d) {
  uint64_t mask = (1ull << (size2 * d)) - 1;
  return (s >> (size2 * d)) | ((s & mask) << ((size1 - d) * size2));
}
TM_HD uint64_t rotate3d(uint64_t s, int size) {
  uint64_t r = 0;
  for (int a = 0; a < size; ++a)
    for (int b = 0; b < size; ++b)
      if (s & (1ull << (a * size + b))) r |= 1ull << ((b + 1) * size - (a + 1));
  return r;
}
TM_HD uint64_t reflect3d(uint64_t s, int size1, int size2, int axis) {
  uint64_t mask = (1ull << size2) - 1, r = 0;
  if (!axis) {
    for (int row = 0; row < size1; ++row) {
      r |= brev(s & mask, size2) << (row * size2);
      s >>= size2;
    }
  } else {
    for (int row = 0; row < size1; ++row) {
      r <<= size2;
      r |= s & mask;
      s >>= size2;
    }
  }
  return r;
}

}  // namespace ltm
