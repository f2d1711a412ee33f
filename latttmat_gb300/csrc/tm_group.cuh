// Symmetry groups of the reduced operators, as device functions.
//
// A reduced basis vector is the normalised sum over one orbit of spin states.
// The reference enumerates orbits with a serial bitset scan:
//   X-2D  genX2DDuplist  (TMat/tmatreduce.cpp:19-111): rotations x reflection (x flip)
//   Z-2D  genZ2DDuplist  (TMat/tmatreduce.cpp:242-334): shift-by-2 x
//         R(s)=bitreversal(rotate1(s)) (x flip)
//   X-3D  genX3DDuplist  (TMat/tmat3d.cpp:17-98): row shifts x column shifts x
//         two mirrors (x flip) (x 90-degree rotation)
// Those scans keep the first unvisited state (the orbit minimum), so idxlist
// is the ascending list of orbit minima and duplist the orbit sizes.  Here the
// same tables come from a per-state test: s is a representative iff no group
// image is smaller, and |orbit| = |group list| / #{list elements fixing s}.
#pragma once
#include "tm_bits.cuh"
#include "tm_internal.h"

namespace ltm {

struct GroupDev {
  int kind, L, size1, size2, periodic, flip, rotate;
  uint64_t mask;
};

inline GroupDev to_dev(const GroupDesc& g) {
  GroupDev d;
  d.kind = g.kind;
  d.L = g.L;
  d.size1 = g.size1;
  d.size2 = g.size2;
  d.periodic = g.periodic;
  d.flip = g.flip;
  d.rotate = g.rotate;
  const int nb = g.nbits ? g.nbits : g.L;
  d.mask = (nb >= 64) ? ~0ull : ((1ull << nb) - 1);
  return d;
}

// Visit every element of the enumerated group list applied to s.  The
// visitor returns false to stop early.  F: bool(uint64_t image)
template <class F>
TM_HD void for_each_image(const GroupDev& g, uint64_t s, F&& f) {
  const uint64_t mask = g.mask;
  if (g.kind == G_X2D) {
    if (g.periodic) {
      for (int k = 0; k < g.L; ++k) {
        uint64_t a = rotr(s, g.L, k);
        uint64_t b = brev(a, g.L);
        if (!f(a)) return;
        if (!f(b)) return;
        if (g.flip) {
          if (!f(~a & mask)) return;
          if (!f(~b & mask)) return;
        }
      }
    } else {
      uint64_t b = brev(s, g.L);
      if (!f(s)) return;
      if (!f(b)) return;
      if (g.flip) {
        if (!f(~s & mask)) return;
        if (!f(~b & mask)) return;
      }
    }
  } else if (g.kind == G_Z2D) {
    uint64_t r = brev(rotr(s, g.L, 1), g.L);
    if (g.periodic) {
      int ncyc = (g.L & 1) ? g.L : g.L / 2;
      int d = 0;
      for (int j = 0; j < ncyc; ++j) {
        uint64_t a = rotr(s, g.L, d);
        uint64_t b = rotr(r, g.L, d);
        if (!f(a)) return;
        if (!f(b)) return;
        if (g.flip) {
          if (!f(~a & mask)) return;
          if (!f(~b & mask)) return;
        }
        d += 2;
        if (d >= g.L) d -= g.L;
      }
    } else {
      if (!f(s)) return;
      if (!f(r)) return;
      if (g.flip) {
        if (!f(~s & mask)) return;
        if (!f(~r & mask)) return;
      }
    }
  } else if (g.kind == G_Y2D) {
    // two-layer states (left layer in the high L bits): translations and
    // reflection of both layers at once (x flip of both), the orbit walk of
    // genY2DDuplist (TMat/tmatreduce.cpp:113-240)
    const uint64_t lm = (1ull << g.L) - 1;
    const uint64_t hi = s >> g.L, lo = s & lm;
    for (int k = 0; k < g.L; ++k) {
      const uint64_t ah = rotr(hi, g.L, k), al = rotr(lo, g.L, k);
      const uint64_t a = ah << g.L | al;
      const uint64_t b = brev(ah, g.L) << g.L | brev(al, g.L);
      if (!f(a)) return;
      if (!f(b)) return;
      if (g.flip) {
        if (!f(~a & mask)) return;
        if (!f(~b & mask)) return;
      }
    }
  } else if (g.kind == G_X3D) {
    for (int rr = 0; rr <= g.rotate; ++rr) {
      uint64_t s0 = rr ? rotate3d(s, g.size1) : s;
      for (int c = 0; c <= g.flip; ++c) {
        uint64_t s1 = c ? (~s0 & mask) : s0;
        for (int a = 0; a < 2; ++a) {
          uint64_t s2 = a ? reflect3d(s1, g.size1, g.size2, 0) : s1;
          for (int b = 0; b < 2; ++b) {
            uint64_t s3 = b ? reflect3d(s2, g.size1, g.size2, 1) : s2;
            uint64_t t1 = s3;
            for (int dx = 0; dx < g.size2; ++dx) {
              uint64_t t2 = t1;
              for (int dy = 0; dy < g.size1; ++dy) {
                if (!f(t2)) return;
                t2 = dshift3d(t2, g.size1, g.size2, 1);
              }
              t1 = rshift3d(t1, g.size1, g.size2, 1);
            }
          }
        }
      }
    }
  }
}

TM_HD int group_order(const GroupDev& g) {
  switch (g.kind) {
    case G_X2D: return (g.periodic ? 2 * g.L : 2) * (g.flip ? 2 : 1);
    case G_Z2D: return (g.periodic ? 2 * ((g.L & 1) ? g.L : g.L / 2) : 2) * (g.flip ? 2 : 1);
    case G_X3D: return g.size1 * g.size2 * 4 * (g.flip ? 2 : 1) * (g.rotate ? 2 : 1);
    case G_Y2D: return 2 * g.L * (g.flip ? 2 : 1);
  }
  return 1;
}

// X-2D periodic group on L <= 32 bits in 32-bit arithmetic: the same images
// as for_each_image (rotations, their reflections, and the flips of both),
// tested in rotation order with an early exit.  The orbit-table build spends
// its time here (2^L states at L = 32).
TM_HD bool is_rep_x2d32(uint32_t s, int L, int flip) {
  const uint32_t mask = (L == 32) ? 0xffffffffu : ((1u << L) - 1u);
  uint32_t a = s;
  for (int k = 0; k < L; ++k) {
#if defined(__CUDA_ARCH__)
    const uint32_t b = __brev(a) >> (32 - L);
#else
    uint32_t b = 0;
    for (int i = 0; i < L; ++i) b |= ((a >> i) & 1u) << (L - 1 - i);
#endif
    if (a < s || b < s) return false;
    if (flip && ((~a & mask) < s || (~b & mask) < s)) return false;
    a = ((a >> 1) | (a << (L - 1))) & mask;  // rotate right by one site
  }
  return true;
}

// Orbit minimum under the X-2D periodic group, L <= 32, in 32-bit
// arithmetic.  The smallest image has the most leading zeros: a longest
// cyclic run of zeros of s (or of its mirror image, which has the same runs)
// rotated to the front, or with the spin flip a longest run of ones.  Growing
// the run-start mask one bit at a time gives the longest length and where
// those runs start, so only a few rotations need comparing.
TM_HD uint32_t rotr32_l(uint32_t x, int L, int k, uint32_t mask) {
  return k ? (((x >> k) | (x << (L - k))) & mask) : x;
}
TM_HD uint32_t brev32_l(uint32_t x, int L) {
#if defined(__CUDA_ARCH__)
  return __brev(x) >> (32 - L);
#else
  uint32_t b = 0;
  for (int i = 0; i < L; ++i) b |= ((x >> i) & 1u) << (L - 1 - i);
  return b;
#endif
}
// length of the longest cyclic run of ones in y (y != 0, y != mask) and, in
// *starts, the bits where runs of that length start
TM_HD int longest_run32(uint32_t y, int L, uint32_t mask, uint32_t* starts) {
  uint32_t t = y;
  int k = 1;
  for (;;) {  // ends with k <= L - 1: y has a zero bit
    const uint32_t nt = t & rotr32_l(y, L, k, mask);
    if (!nt) break;
    t = nt;
    ++k;
  }
  *starts = t;
  return k;
}
TM_HD uint32_t canon_x2d32(uint32_t s, int L, int flip) {
  const uint32_t mask = (L == 32) ? 0xffffffffu : ((1u << L) - 1u);
  if (s == 0 || (flip && s == mask)) return 0;
  if (s == mask) return s;  // no flip: every image is s
  const uint32_t r = brev32_l(s, L);
  uint32_t zs, zr;
  const int Z = longest_run32(~s & mask, L, mask, &zs);
  uint32_t os = 0, orr = 0;
  const int O = flip ? longest_run32(s, L, mask, &os) : -1;
  uint32_t best = mask;
  auto scan = [&](uint32_t v, uint32_t t, int k0, bool inv) {
    while (t) {
#if defined(__CUDA_ARCH__)
      const int i = __ffs(t) - 1;
#else
      const int i = __builtin_ctz(t);
#endif
      t &= t - 1;
      const int k = (i + k0 >= L) ? i + k0 - L : i + k0;
      uint32_t a = rotr32_l(v, L, k, mask);
      if (inv) a = ~a & mask;
      if (a < best) best = a;
    }
  };
  if (Z >= O) {
    longest_run32(~r & mask, L, mask, &zr);
    scan(s, zs, Z, false);
    scan(r, zr, Z, false);
  }
  if (flip && O >= Z) {
    longest_run32(r, L, mask, &orr);
    scan(s, os, O, true);
    scan(r, orr, O, true);
  }
  return best;
}

#if defined(__CUDACC__)
// ---- warp-cooperative forms for the X-2D periodic group on L <= 32 bits.
// Lane k < L takes the images of rotation k (a = rotr(s, k), b = its
// reflection, and their flips), so one warp covers the whole group list in
// one step.  All 32 lanes must call these with the same s.

// rotate right by k within L bits, 1 <= k <= L - 1
__device__ __forceinline__ uint32_t rotr_l32(uint32_t x, int L, int k, uint32_t mask) {
  return ((x >> k) | (x << (L - k))) & mask;
}

// true iff the L-bit word y has a cyclic run of ones of length >= k (1 <= k <= L)
__device__ __forceinline__ bool has_run32(uint32_t y, int L, int k, uint32_t mask) {
  uint32_t t = y;
  int len = 1;
  while (2 * len <= k && len < L) {
    t &= rotr_l32(t, L, len, mask);
    len *= 2;
  }
  if (k > len) t &= rotr_l32(t, L, k - len, mask);
  return t != 0;
}

// Necessary condition for s to be its orbit's minimum: no cyclic run of
// zeros longer than s's leading zeros (rotating it to the front gives a
// smaller image), and with the spin flip no such run of ones either.
__device__ __forceinline__ bool rep_candidate_x2d32(uint32_t s, int L, int flip) {
  if (s == 0) return true;
  const uint32_t mask = (L == 32) ? 0xffffffffu : ((1u << L) - 1u);
  const int z = __clz(s) - (32 - L);  // leading zeros within L bits
  if (z + 1 > L) return true;
  if (has_run32(~s & mask, L, z + 1, mask)) return false;
  if (flip && has_run32(s, L, z + 1, mask)) return false;
  return true;
}

// true iff y has a (non-cyclic) run of ones of length >= k (1 <= k <= 32)
__device__ __forceinline__ bool has_run_linear32(uint32_t y, int k) {
  uint32_t t = y;
  int len = 1;
  while (2 * len <= k) {
    t &= t >> len;
    len *= 2;
  }
  if (k > len) t &= t >> (k - len);
  return t != 0;
}

// The 32 states w*32 + b (b < 32) share bits [5, L), and for w > 0 their
// leading-zero count z.  A run of more than z zeros inside those bits (or,
// with the spin flip, of more than z ones) fails rep_candidate_x2d32 for every
// state of the word, so the word holds no representative.
__device__ __forceinline__ bool word_rejected_x2d32(uint64_t w, int L, int flip) {
  if (w == 0 || L <= 6) return false;
  const uint32_t up = (uint32_t)(w << 5);  // w < 2^(L-5), so this fits in L bits
  const int z = __clz(up) - (32 - L);
  if (z + 1 > L - 5) return false;
  const uint32_t umask = ((L == 32) ? 0xffffffffu : ((1u << L) - 1u)) & ~31u;
  if (has_run_linear32(~up & umask, z + 1)) return true;
  return flip && has_run_linear32(up & umask, z + 1);
}

// Bit i set iff bits i .. i+k-1 (cyclic, L-bit word) of y are all ones;
// every bit for k = 0.  (0 <= k < L)
__device__ __forceinline__ uint32_t run_starts32(uint32_t y, int L, int k, uint32_t mask) {
  if (k == 0) return mask;
  uint32_t t = y;
  int len = 1;
  while (2 * len <= k) {
    t &= rotr_l32(t, L, len, mask);
    len *= 2;
  }
  if (k > len) t &= rotr_l32(t, L, k - len, mask);
  return t;
}

// One thread's exact test of s against the periodic X-2D group (L <= 32):
// true iff no image of s is smaller, and then *fix = the number of group
// elements fixing s (orbit size = group order / *fix).  An image no larger
// than s starts with at least z zeros (z = s's leading zeros within L bits),
// so only the rotations that bring a run of z zeros of s or of its mirror
// image to the front -- or, for the flipped images, a run of z ones -- need a
// comparison: rotation by k = i + z for each run start i.  Images equal to s
// are among them too, so the same pass counts the stabiliser.
__device__ __forceinline__ bool lane_rep_x2d32(uint32_t s, int L, int flip, int* fix) {
  const uint32_t mask = (L == 32) ? 0xffffffffu : ((1u << L) - 1u);
  if (s == 0) {
    *fix = 2 * L;  // rotations and reflections; the flip moves 0 to the all-ones state
    return true;
  }
  const int z = __clz(s) - (32 - L);
  const uint32_t r = __brev(s) >> (32 - L);
  int f = 0;
  for (int v4 = 0; v4 < (flip ? 4 : 2); ++v4) {
    const uint32_t v = (v4 & 1) ? r : s;
    const bool inv = v4 >= 2;
    uint32_t t = run_starts32(inv ? v : (~v & mask), L, z, mask);
    while (t) {
      const int i = __ffs(t) - 1;
      t &= t - 1;
      const int k = (i + z >= L) ? i + z - L : i + z;
      uint32_t a = k ? rotr_l32(v, L, k, mask) : v;
      if (inv) a = ~a & mask;
      if (a < s) return false;
      f += (a == s);
    }
  }
  *fix = f;
  return true;
}

#endif

TM_HD bool is_rep(const GroupDev& g, uint64_t s) {
  if (g.kind == G_X2D && g.periodic && g.L <= 32) return is_rep_x2d32((uint32_t)s, g.L, g.flip);
  bool rep = true;
  for_each_image(g, s, [&](uint64_t im) {
    if (im < s) {
      rep = false;
      return false;
    }
    return true;
  });
  return rep;
}

TM_HD uint64_t canon(const GroupDev& g, uint64_t s) {
  if (g.kind == G_X2D && g.periodic && g.L <= 32) return canon_x2d32((uint32_t)s, g.L, g.flip);
  uint64_t m = s;
  for_each_image(g, s, [&](uint64_t im) {
    if (im < m) m = im;
    return true;
  });
  return m;
}

TM_HD int orbit_size(const GroupDev& g, uint64_t s) {
  int fix = 0;
  for_each_image(g, s, [&](uint64_t im) {
    fix += (im == s);
    return true;
  });
  return group_order(g) / fix;
}

}  // namespace ltm
