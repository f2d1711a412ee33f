// Even/odd two-pass product for the reduced x-ANNNI operator (XAMMatVecProd2D,
// TMat/tmatreduce.cpp:406-529), periodic boundary, even L.
//
// The reference expands the representative vector into 2^(L-nleadbit)-state
// slices, one slice per leading-bit pattern, and sweeps each slice.  That
// costs O(2^L * L) work per product, plus O(n_rep * L) scatter probes per slice.
//
// GB300 design.  Split the L sites into even sites (e, m = L/2 bits) and odd
// sites (o, m bits).  The inter-layer factor factorises as Th = Th_E (x) Th_O.
// The subgroup H of the layer group that maps even sites to even sites
// (rotations by 2, the reflection s -> bitreversal(rotate1(s)), spin flip)
// commutes with Th_E and Th_O separately.  So:
//   pass 1: w = Th_E v needs only the tiles {(e, o): o = o_rep} for o_rep an
//           H-representative of the odd pattern (about 2^m / (L or 2L) tiles).
//           v on such a tile is gathered from the representative vector
//           through a precomputed index (map1).
//   pass 2: z = Th_O w needs only tiles with e = e_rep, one per H-class of e.
//           Each w value is read from its H-image in a pass-1 tile.  The output
//           is the value at one designated state of every orbit.
// Work and HBM traffic are about 2^(L+1)/|H| elements instead of 2^L * L.
//
// Memory layout.  Both passes walk a tile in an "iteration order" of the
// m-bit patterns: grouped by the top ct bits (the cluster split, below), then
// by H-class.  A warp's 32 elements are then a few whole H-classes, and
//   - the reduced vector is kept in "pi order": per pass-2 tile, the
//     designated outputs in pass 2's iteration order, so pass 1's gathers of
//     one class land in a few contiguous runs of the vector, and each CTA of
//     pass 2 writes one contiguous range (pi maps back to idxlist order);
//   - w1 is class-major: the block of e-class C holds, for each pass-1 tile,
//     the |C| values of C's members, so pass 1 writes and pass 2 reads whole
//     runs, and pass 2 reads one contiguous block per tile.
// Gathers go straight to shared memory with cp.async.
//
// Arithmetic.  The butterfly [[a, b], [b, a]] is applied as x0 + r x1,
// x1 + r x0 with r = min(a, b) / max(a, b): one FMA per element and level.
// The input is scaled by (1 + r)^-L so magnitudes match the normalised
// operator, and the output factor stays (e^K + e^-K)^L.
//
// A tile of 2^m elements is split over a cluster of 2^c CTAs (FP32 m=16: two
// CTAs x 2^15 elements in 135 KB of shared memory), CTA `rank` holding the
// patterns whose top c bits are `rank`.  The butterflies on those top bits
// combine the CTAs' tiles through DSMEM once all local rounds are done.
// Inside a CTA each thread owns 2^KB elements per round: KB butterfly levels
// in registers, with a padded shared-memory transpose between rounds.
#include <atomic>
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <type_traits>
#include <vector>

#include "tm_df.cuh"
#include "tm_group.cuh"
#include "tm_internal.h"

namespace cg = cooperative_groups;

namespace ltm {

// ------------------------------------------------------------- bit helpers
TM_HD uint32_t rotr_m(uint32_t x, int m, int d) {
  d %= m;
  return d ? (((x >> d) | (x << (m - d))) & ((m == 32) ? 0xffffffffu : ((1u << m) - 1u))) : x;
}
TM_HD uint32_t rotl_m(uint32_t x, int m, int d) { return rotr_m(x, m, (m - d % m) % m); }
TM_HD uint32_t brev_m(uint32_t x, int m) {
#if defined(__CUDA_ARCH__)
  return __brev(x) >> (32 - m);
#else
  uint32_t r = 0;
  for (int i = 0; i < m; ++i) r |= ((x >> i) & 1u) << (m - 1 - i);
  return r;
#endif
}
// H element g = j + m*refl + 2m*flip acting on the odd / even halves.
TM_HD uint32_t act_o(int g, uint32_t o, int m) {
  int j = g % m, refl = (g / m) & 1, fl = g / (2 * m);
  uint32_t r = rotr_m(o, m, j);
  if (refl) r = brev_m(r, m);
  if (fl) r ^= (1u << m) - 1u;
  return r;
}
TM_HD uint32_t act_e(int g, uint32_t e, int m) {
  int j = g % m, refl = (g / m) & 1, fl = g / (2 * m);
  uint32_t r = rotr_m(e, m, j);
  if (refl) r = rotl_m(brev_m(r, m), m, 1);
  if (fl) r ^= (1u << m) - 1u;
  return r;
}
// interleave e (even sites) and o (odd sites) into an L=2m-bit state
TM_HD uint32_t spread16(uint32_t x) {
  x &= 0xffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}
TM_HD uint32_t gather16(uint32_t x) {
  x &= 0x55555555u;
  x = (x | (x >> 1)) & 0x33333333u;
  x = (x | (x >> 2)) & 0x0f0f0f0fu;
  x = (x | (x >> 4)) & 0x00ff00ffu;
  x = (x | (x >> 8)) & 0x0000ffffu;
  return x;
}
TM_HD uint32_t join_eo(uint32_t e, uint32_t o) { return spread16(e) | (spread16(o) << 1); }

namespace {

struct EOArgs {
  int m, c, n, p;       // tile bits, cluster bits, local bits, thread bits
  int ct;               // top bits grouping the iteration orders (c <= ct)
  int ng;               // H elements
  int64_t n_orep;       // pass-1 tiles
  // Butterfly [[a, b], [b, a]] / max(a, b) on every site: with r = min/max,
  // x0' = x0 + r x1, x1' = x1 + r x0 (swap = 0, a >= b) or the outputs
  // exchanged (swap = 1).  The factor max(a, b)^L is applied at the output.
  float r32;
  double r64;
  int swap;
};

__device__ __forceinline__ int spad(int e) { return e + (e >> 5); }

template <class T>
__device__ __forceinline__ T coef_r(const EOArgs& A);
template <>
__device__ __forceinline__ float coef_r<float>(const EOArgs& A) { return A.r32; }
template <>
__device__ __forceinline__ double coef_r<double>(const EOArgs& A) { return A.r64; }
template <>
__device__ __forceinline__ dfloat coef_r<dfloat>(const EOArgs& A) { return dfloat(A.r64); }

// r * x + y in the engine's arithmetic
__device__ __forceinline__ float fma_t(float r, float x, float y) { return fmaf(r, x, y); }
__device__ __forceinline__ double fma_t(double r, double x, double y) { return fma(r, x, y); }
__device__ __forceinline__ dfloat fma_t(dfloat r, dfloat x, dfloat y) { return df_fma_unnorm(r, x, y); }

// In-register butterflies on all NB levels of the 2^NB elements held by one
// thread.  Output pair of level lv: (x0 + r x1, x1 + r x0), or exchanged
// (swap).
template <class T, int NB>
__device__ __forceinline__ void reg_bfly(T (&v)[1 << NB], T r, int swap) {
  if (!swap) {
#pragma unroll
    for (int lv = 0; lv < NB; ++lv)
#pragma unroll
      for (int i = 0; i < (1 << NB); ++i)
        if (!(i & (1 << lv))) {
          const T x0 = v[i], x1 = v[i | (1 << lv)];
          v[i] = fma_t(r, x1, x0);
          v[i | (1 << lv)] = fma_t(r, x0, x1);
        }
  } else {
#pragma unroll
    for (int lv = 0; lv < NB; ++lv)
#pragma unroll
      for (int i = 0; i < (1 << NB); ++i)
        if (!(i & (1 << lv))) {
          const T x0 = v[i], x1 = v[i | (1 << lv)];
          v[i] = fma_t(r, x0, x1);
          v[i | (1 << lv)] = fma_t(r, x1, x0);
        }
  }
}

// The FP32 butterflies with the elements held in pairs (v[k] = elements 2k,
// 2k + 1): level 0 pairs the two halves of one register pair (two scalar
// FMAs per pair); every higher level pairs whole register pairs, two
// butterflies per packed FMA (sm_100+ FFMA2).
template <int NB>
__device__ __forceinline__ void reg_bfly_f2(float2 (&v)[1 << (NB - 1)], float r, int swap) {
  const float2 r2 = make_float2(r, r);
  if (!swap) {
#pragma unroll
    for (int k = 0; k < (1 << (NB - 1)); ++k) {
      const float x0 = v[k].x, x1 = v[k].y;
      v[k].x = fmaf(r, x1, x0);
      v[k].y = fmaf(r, x0, x1);
    }
#pragma unroll
    for (int lv = 1; lv < NB; ++lv)
#pragma unroll
      for (int k = 0; k < (1 << (NB - 1)); ++k)
        if (!(k & (1 << (lv - 1)))) {
          const float2 a = v[k], b = v[k | (1 << (lv - 1))];
          v[k] = __ffma2_rn(r2, b, a);
          v[k | (1 << (lv - 1))] = __ffma2_rn(r2, a, b);
        }
  } else {
#pragma unroll
    for (int k = 0; k < (1 << (NB - 1)); ++k) {
      const float x0 = v[k].x, x1 = v[k].y;
      v[k].x = fmaf(r, x0, x1);
      v[k].y = fmaf(r, x1, x0);
    }
#pragma unroll
    for (int lv = 1; lv < NB; ++lv)
#pragma unroll
      for (int k = 0; k < (1 << (NB - 1)); ++k)
        if (!(k & (1 << (lv - 1)))) {
          const float2 a = v[k], b = v[k | (1 << (lv - 1))];
          v[k] = __ffma2_rn(r2, a, b);
          v[k | (1 << (lv - 1))] = __ffma2_rn(r2, b, a);
        }
  }
}

// Double-float values two to a lane pair: hi words in one float2, lo words in
// another.  df2_fma_unnorm is df_fma_unnorm (tm_df.cuh) on both lanes with the
// same operation sequence (so the same results), on the packed FP32 pipes;
// differences are taken as fma(b, -1, a), and -p comes from -r.hi, so no
// operand needs a separate negation.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ void df2_fma_unnorm(float2 rh, float2 rl, float2 rhn, float2 xh, float2 xl, float2 yh,
                                               float2 yl, float2& oh, float2& ol) {
  const float2 np = __fmul2_rn(rhn, xh);  // -p, p = r.hi x.hi
  float2 pe = __ffma2_rn(rh, xh, np);     // r.hi x.hi - p (exact)
  pe = __ffma2_rn(rh, xl, pe);
  pe = __ffma2_rn(rl, xh, pe);
  const float2 sm = sub2(yh, np);            // p + y.hi
  const float2 bb = __fadd2_rn(sm, np);      // s - p
  const float2 t = sub2(sm, bb);             // s - bb
  const float2 e2 = sub2(yh, bb);            // y.hi - bb
  const float2 se = sub2(e2, __fadd2_rn(np, t));  // (p - (s - bb)) + (y.hi - bb)
  oh = sm;
  ol = __fadd2_rn(se, __fadd2_rn(pe, yl));
}

// reg_bfly for double-float values held as (hi pair, lo pair) per two
// elements: level 0 within a pair (scalar), every higher level on whole
// pairs, then one renormalisation per element
template <int NB>
__device__ __forceinline__ void reg_bfly_df2(float2 (&h)[1 << (NB - 1)], float2 (&l)[1 << (NB - 1)], dfloat r,
                                             int swap) {
  const float2 rh = make_float2(r.hi, r.hi), rl = make_float2(r.lo, r.lo), rhn = make_float2(-r.hi, -r.hi);
  if (!swap) {
#pragma unroll
    for (int k = 0; k < (1 << (NB - 1)); ++k) {
      const dfloat x0(h[k].x, l[k].x), x1(h[k].y, l[k].y);
      const dfloat o0 = df_fma_unnorm(r, x1, x0), o1 = df_fma_unnorm(r, x0, x1);
      h[k] = make_float2(o0.hi, o1.hi);
      l[k] = make_float2(o0.lo, o1.lo);
    }
  } else {
#pragma unroll
    for (int k = 0; k < (1 << (NB - 1)); ++k) {
      const dfloat x0(h[k].x, l[k].x), x1(h[k].y, l[k].y);
      const dfloat o0 = df_fma_unnorm(r, x0, x1), o1 = df_fma_unnorm(r, x1, x0);
      h[k] = make_float2(o0.hi, o1.hi);
      l[k] = make_float2(o0.lo, o1.lo);
    }
  }
  // no swap: (a + r b, b + r a); swap: (b + r a, a + r b)
  if (!swap) {
#pragma unroll
    for (int lv = 1; lv < NB; ++lv)
#pragma unroll
      for (int k = 0; k < (1 << (NB - 1)); ++k)
        if (!(k & (1 << (lv - 1)))) {
          const int k1 = k | (1 << (lv - 1));
          const float2 ah = h[k], al = l[k], bh = h[k1], bl = l[k1];
          df2_fma_unnorm(rh, rl, rhn, bh, bl, ah, al, h[k], l[k]);
          df2_fma_unnorm(rh, rl, rhn, ah, al, bh, bl, h[k1], l[k1]);
        }
  } else {
#pragma unroll
    for (int lv = 1; lv < NB; ++lv)
#pragma unroll
      for (int k = 0; k < (1 << (NB - 1)); ++k)
        if (!(k & (1 << (lv - 1)))) {
          const int k1 = k | (1 << (lv - 1));
          const float2 ah = h[k], al = l[k], bh = h[k1], bl = l[k1];
          df2_fma_unnorm(rh, rl, rhn, ah, al, bh, bl, h[k], l[k]);
          df2_fma_unnorm(rh, rl, rhn, bh, bl, ah, al, h[k1], l[k1]);
        }
  }
  // renormalise: hi' = hi + lo, lo' = lo - (hi' - hi)
#pragma unroll
  for (int k = 0; k < (1 << (NB - 1)); ++k) {
    const float2 s2 = __fadd2_rn(h[k], l[k]);
    l[k] = sub2(l[k], sub2(s2, h[k]));
    h[k] = s2;
  }
}

// asynchronous global->shared copy of one element (cp.async, sm_80+): the
// gathers of a tile are all in flight at once without holding registers
template <int SZ>
__device__ __forceinline__ void cp_async_elem(void* dst, const void* src);
template <>
__device__ __forceinline__ void cp_async_elem<4>(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
template <>
__device__ __forceinline__ void cp_async_elem<8>(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Tile bits covered by the unrolled butterfly rounds (the largest tile is
// 2^15 elements in FP32 and 2^14 in 8-byte types).
constexpr int kMaxTileBits = 16;

// One butterfly round on local bits [G0, G0 + GS) of the shared-memory tile.
// G0 and GS are compile-time constants, so each of a thread's 2^GS slots is
// the thread's base slot plus a constant: j0 and i << G0 have disjoint bits,
// and spad(a | b) = spad(a) + spad(b) for disjoint a, b (no carry reaches
// bit 5).
template <class T, int G0, int GS>
__device__ __forceinline__ void smem_round(T* sm, int n, T r, int swap) {
  const int nfree = 1 << (n - GS);
  for (int f = threadIdx.x; f < nfree; f += blockDim.x) {
    const int j0 = (f & ((1 << G0) - 1)) | ((f >> G0) << (G0 + GS));
    T* b = sm + spad(j0);
    if constexpr (std::is_same<T, float>::value && GS >= 2) {
      float2 v[1 << (GS - 1)];
#pragma unroll
      for (int k = 0; k < (1 << (GS - 1)); ++k) {
        v[k].x = b[spad((2 * k) << G0)];
        v[k].y = b[spad((2 * k + 1) << G0)];
      }
      reg_bfly_f2<GS>(v, r, swap);
#pragma unroll
      for (int k = 0; k < (1 << (GS - 1)); ++k) {
        b[spad((2 * k) << G0)] = v[k].x;
        b[spad((2 * k + 1) << G0)] = v[k].y;
      }
    } else if constexpr (std::is_same<T, dfloat>::value && GS >= 2) {
      float2 h[1 << (GS - 1)], l[1 << (GS - 1)];
#pragma unroll
      for (int k = 0; k < (1 << (GS - 1)); ++k) {
        const dfloat a = b[spad((2 * k) << G0)], c = b[spad((2 * k + 1) << G0)];
        h[k] = make_float2(a.hi, c.hi);
        l[k] = make_float2(a.lo, c.lo);
      }
      reg_bfly_df2<GS>(h, l, r, swap);
#pragma unroll
      for (int k = 0; k < (1 << (GS - 1)); ++k) {
        b[spad((2 * k) << G0)] = dfloat(h[k].x, l[k].x);
        b[spad((2 * k + 1) << G0)] = dfloat(h[k].y, l[k].y);
      }
    } else {
      T v[1 << GS];
#pragma unroll
      for (int i = 0; i < (1 << GS); ++i) v[i] = b[spad(i << G0)];
      reg_bfly<T, GS>(v, r, swap);
      if constexpr (std::is_same<T, dfloat>::value) {
        // the double-float levels skip renormalisation; once per round here
#pragma unroll
        for (int i = 0; i < (1 << GS); ++i) v[i] = df_norm(v[i]);
      }
#pragma unroll
      for (int i = 0; i < (1 << GS); ++i) b[spad(i << G0)] = v[i];
    }
  }
}

// the last round when it covers fewer than KB bits (gs = 1 .. KB - 1)
template <class T, int KB, int G0, int GS = 1>
__device__ __forceinline__ void smem_round_tail(T* sm, int n, int gs, T r, int swap) {
  if constexpr (GS < KB) {
    if (gs == GS)
      smem_round<T, G0, GS>(sm, n, r, swap);
    else
      smem_round_tail<T, KB, G0, GS + 1>(sm, n, gs, r, swap);
  }
}

// butterflies on local bits [0, nbits) of the shared-memory tile, KB bits per
// round (nbits <= kMaxTileBits)
template <class T, int KB, int R = 0>
__device__ __forceinline__ void smem_rounds(T* sm, const EOArgs& A, int nbits) {
  constexpr int G0 = R * KB;
  if (G0 >= nbits) return;
  if (G0 + KB <= nbits)
    smem_round<T, G0, KB>(sm, A.n, coef_r<T>(A), A.swap);
  else
    smem_round_tail<T, KB, G0>(sm, A.n, nbits - G0, coef_r<T>(A), A.swap);
  __syncthreads();
  if constexpr ((R + 1) * KB < kMaxTileBits) smem_rounds<T, KB, R + 1>(sm, A, nbits);
}

// streaming (evict-first) loads and stores of data read or written once
template <class V>
__device__ __forceinline__ V ld_stream(const V* p) {
  if constexpr (std::is_same<V, dfloat>::value) {
    const float2 v = __ldcs(reinterpret_cast<const float2*>(p));
    return dfloat(v.x, v.y);
  } else {
    return __ldcs(p);
  }
}
template <class V>
__device__ __forceinline__ void st_stream(V* p, V v) {
  if constexpr (std::is_same<V, dfloat>::value)
    __stcs(reinterpret_cast<float2*>(p), make_float2(v.hi, v.lo));
  else
    __stcs(p, v);
}

// acc += c * v over the 16 / sizeof(T) elements of a 16-byte chunk
template <class T>
__device__ __forceinline__ void axpy16(float4& acc, const float4& v, T c);
template <>
__device__ __forceinline__ void axpy16<float>(float4& acc, const float4& v, float c) {
  acc.x = fmaf(c, v.x, acc.x);
  acc.y = fmaf(c, v.y, acc.y);
  acc.z = fmaf(c, v.z, acc.z);
  acc.w = fmaf(c, v.w, acc.w);
}
template <>
__device__ __forceinline__ void axpy16<double>(float4& acc, const float4& v, double c) {
  double2 a = *reinterpret_cast<double2*>(&acc);
  const double2 x = *reinterpret_cast<const double2*>(&v);
  a.x = fma(c, x.x, a.x);
  a.y = fma(c, x.y, a.y);
  acc = *reinterpret_cast<float4*>(&a);
}
template <>
__device__ __forceinline__ void axpy16<dfloat>(float4& acc, const float4& v, dfloat c) {
  const dfloat a0 = df_fma(c, dfloat(v.x, v.y), dfloat(acc.x, acc.y));
  const dfloat a1 = df_fma(c, dfloat(v.z, v.w), dfloat(acc.z, acc.w));
  acc = make_float4(a0.hi, a0.lo, a1.hi, a1.lo);
}

// 16-byte chunks of one CTA's exchange slot: the padded tile rounded up to
// whole 128-byte lines
__host__ __device__ __forceinline__ int64_t xchg_slot_chunks(int n, int elem) {
  const int64_t chunks = ((int64_t)((1 << n) + (1 << n) / 32) * elem) / 16;
  return (chunks + 7) & ~(int64_t)7;
}

// Combine the cluster's 2^c partial tiles (butterflies on the top c tile
// bits) in place: afterwards sm[spad(j)] holds the final value of local
// element j.  The combination is elementwise at equal positions of the
// padded tiles, so it runs over raw 16-byte chunks of the buffer (the padding
// slots carry values nobody reads).
//
// With an exchange buffer (xchg), each CTA first stores its tile to its own
// slot (CTA index order, 128-byte aligned); after a cluster barrier, whose
// release/acquire orders those stores before the partners' loads, every
// thread reads its chunks of the partners' tiles from L2 and of its own tile
// from shared memory.  A second barrier marks the partners' reads done; each
// CTA then discards its slot's lines from L2, so the buffer is never written
// back to DRAM.  Without one, the partners' tiles are read through DSMEM, and
// the write-back waits for a cluster barrier so no CTA overwrites values
// another still reads.  The arithmetic is the same either way.
template <class T, int KB>
__device__ __forceinline__ void cluster_reduce(cg::cluster_group& cl, T* sm, int rank, const EOArgs& A,
                                               float4* __restrict__ xchg) {
  const T a = A.swap ? coef_r<T>(A) : T(1), b = A.swap ? T(1) : coef_r<T>(A);
  if constexpr (std::is_same<T, double>::value) {
    // native FP64: element-wise (the chunk accumulators and FP64 temporaries
    // together would spill)
    const int p = A.p, kb = A.n - A.p;
    T acc[1 << KB];
#pragma unroll
    for (int k = 0; k < (1 << KB); ++k) acc[k] = T(0);
    cl.sync();
    for (int r = 0; r < (1 << A.c); ++r) {
      T coef = T(1);
      for (int bit = 0; bit < A.c; ++bit) coef = coef * ((((r ^ rank) >> bit) & 1) ? b : a);
      const T* src = (r == rank) ? sm : cl.map_shared_rank(sm, r);
#pragma unroll
      for (int k = 0; k < (1 << KB); ++k)
        if (k < (1 << kb)) acc[k] = acc[k] + coef * src[spad(threadIdx.x + (k << p))];
    }
    cl.sync();
#pragma unroll
    for (int k = 0; k < (1 << KB); ++k)
      if (k < (1 << kb)) sm[spad(threadIdx.x + (k << p))] = acc[k];
    __syncthreads();
    return;
  }
  constexpr int kMaxChunks = ((1 << KB) * 33 * (int)sizeof(T) + 511) / 512;  // ceil(2^KB * 33/32 * sizeof(T) / 16)
  const int nchunks = (((1 << A.n) + (1 << (A.n - 5))) * (int)sizeof(T)) / 16;
  const int nc = 1 << A.c;
  float4* dst = reinterpret_cast<float4*>(sm);
  float4 acc[kMaxChunks];
  if (xchg) {
    const int64_t slot = xchg_slot_chunks(A.n, (int)sizeof(T));
    const int64_t first = (int64_t)blockIdx.x - rank;  // the cluster's CTAs are consecutive
    float4* mine = xchg + (int64_t)blockIdx.x * slot;
#pragma unroll
    for (int k = 0; k < kMaxChunks; ++k) {
      const int q = (int)threadIdx.x + k * (int)blockDim.x;
      if (q < nchunks) __stcg(mine + q, dst[q]);
      acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    cl.sync();
    for (int r = 0; r < nc; ++r) {
      T coef = T(1);
      for (int bit = 0; bit < A.c; ++bit) coef = coef * ((((r ^ rank) >> bit) & 1) ? b : a);
      if (r == rank) {
#pragma unroll
        for (int k = 0; k < kMaxChunks; ++k) {
          const int q = (int)threadIdx.x + k * (int)blockDim.x;
          if (q < nchunks) axpy16<T>(acc[k], dst[q], coef);
        }
      } else {
        const float4* src = xchg + (first + r) * slot;
#pragma unroll
        for (int k = 0; k < kMaxChunks; ++k) {
          const int q = (int)threadIdx.x + k * (int)blockDim.x;
          if (q < nchunks) axpy16<T>(acc[k], __ldcg(src + q), coef);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < kMaxChunks; ++k) {
      const int q = (int)threadIdx.x + k * (int)blockDim.x;
      if (q < nchunks) dst[q] = acc[k];
    }
    cl.sync();  // the partners' reads of this slot are done (and the tile is complete)
    for (int64_t line = threadIdx.x; line < slot / 8; line += blockDim.x)
      asm volatile("discard.global.L2 [%0], 128;\n" ::"l"(mine + line * 8) : "memory");
    return;
  }
#pragma unroll
  for (int k = 0; k < kMaxChunks; ++k) acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  cl.sync();
  for (int r = 0; r < nc; ++r) {
    T coef = T(1);
    for (int bit = 0; bit < A.c; ++bit) coef = coef * ((((r ^ rank) >> bit) & 1) ? b : a);
    const float4* src = reinterpret_cast<const float4*>((r == rank) ? sm : cl.map_shared_rank(sm, r));
#pragma unroll
    for (int k = 0; k < kMaxChunks; ++k) {
      const int q = (int)threadIdx.x + k * (int)blockDim.x;
      if (q < nchunks) axpy16<T>(acc[k], src[q], coef);
    }
  }
  cl.sync();
#pragma unroll
  for (int k = 0; k < kMaxChunks; ++k) {
    const int q = (int)threadIdx.x + k * (int)blockDim.x;
    if (q < nchunks) dst[q] = acc[k];
  }
  // only this CTA reads its combined tile from here on
  __syncthreads();
}

// elements per batch of the output loops (independent loads in flight per thread)
constexpr int kOutBatch = 8;
// elements per chunk of the gather loops
constexpr int kGatherChunk = 16;

// pass 1: w1(t, e) = (Th_E v)[(e, o_rep(t))],  v[(e,o_rep)] = u[map1[t][P]]
// where P runs over the iteration order of e (it_e).  CTA `rank` of the
// cluster owns the e with top c bits = rank, iteration positions
// [rank*2^n, (rank+1)*2^n).  (InT: element type of u, the same size as T;
// T: arithmetic / storage type of the tile and w1)
template <class T, int KB, class InT, bool CL>
__global__ void __launch_bounds__(1024, 1) eo_pass1(EOArgs A, const InT* __restrict__ u,
                                                    const uint32_t* __restrict__ map1,
                                                    const uint16_t* __restrict__ it_e,
                                                    const uint2* __restrict__ wout, T* __restrict__ w1,
                                                    float4* __restrict__ xchg) {
  static_assert(sizeof(T) == sizeof(InT), "u and the tile share the element size");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  cg::cluster_group cl = cg::this_cluster();
  const int rank = CL ? (int)cl.block_rank() : 0;
  const int64_t tile = blockIdx.x >> A.c;
  const int n = A.n, p = A.p;
  const int kb = n - p;
  const uint32_t lmask = (1u << n) - 1u;
  const uint32_t base = (uint32_t)rank << n;
  const uint32_t* mrow = map1 + (tile << A.m);
  // gather the tile: index loads, then one asynchronous copy per element.
  // A warp's elements are one or two symmetry classes of e, whose orbits sit
  // in a few contiguous runs of u.
  // (in chunks of kGatherChunk per thread: the copies are asynchronous, so
  // the chunks overlap while holding fewer registers)
  {
#pragma unroll
    for (int c0 = 0; c0 < (1 << KB); c0 += kGatherChunk) {
      uint32_t idx[kGatherChunk];
      uint16_t ev[kGatherChunk];
#pragma unroll
      for (int i = 0; i < kGatherChunk; ++i) {
        if (c0 + i < (1 << kb)) {
          const uint32_t P = base + threadIdx.x + ((c0 + i) << p);
          idx[i] = __ldcs(mrow + P);  // read once: evict first, keep u in L2
          ev[i] = __ldg(it_e + P);
        }
      }
#pragma unroll
      for (int i = 0; i < kGatherChunk; ++i)
        if (c0 + i < (1 << kb)) cp_async_elem<sizeof(T)>(sm + spad(ev[i] & lmask), u + idx[i]);
    }
    cp_async_wait_all();
    if constexpr (!std::is_same<T, InT>::value) {
      // each thread converts the elements it copied
#pragma unroll
      for (int i = 0; i < (1 << KB); ++i) {
        if (i < (1 << kb)) {
          T* slot = sm + spad(__ldg(it_e + base + threadIdx.x + (i << p)) & lmask);
          *slot = T(*reinterpret_cast<const InT*>(slot));
        }
      }
    }
  }
  __syncthreads();
  smem_rounds<T, KB>(sm, A, n);
  if constexpr (CL) cluster_reduce<T, KB>(cl, sm, rank, A, xchg);
  // Output.  w1 is class-major: the block of e-class C holds, for each tile,
  // the |C| values of C's members, so a warp writes a few contiguous runs.
  // (the table entries of a whole batch are loaded before any is used, so
  // their loads are in flight together)
  constexpr int kOB = (1 << KB) < 12 ? (1 << KB) : 12;
  for (int k0 = 0; k0 < (1 << kb); k0 += kOB) {
    uint2 w[kOB];  // (w1 offset, it_e | class size << 16)
#pragma unroll
    for (int q = 0; q < kOB; ++q)
      if (k0 + q < (1 << kb)) w[q] = __ldg(wout + base + threadIdx.x + ((k0 + q) << p));
#pragma unroll
    for (int q = 0; q < kOB; ++q)
      if (k0 + q < (1 << kb)) st_stream(w1 + (int64_t)w[q].x + tile * (w[q].y >> 16), sm[spad(w[q].y & lmask)]);
  }
}

// Output modes of pass 2: y = val * sout32 (FP32), val * sout64 * post
// (FP64), or val * soutdf in double-float (double-float storage).
enum { kOutF32 = 0, kOutF64 = 1, kOutDF = 2 };

// pass 2: z[(e_rep, o)] = (Th_O w)[(e_rep, o)]; emit designated outputs.
// The w value at (e_rep, o) is the pass-1 value at the H-image
// (act_e(g, e_rep), o_rep) with act_o(g, o) = o_rep.  CTA `rank` owns the o
// with top c bits = rank (iteration positions of it_o as in pass 1).
// (OutT: element type of y)
template <class T, int KB, int OSC, class OutT, bool CL>
__global__ void __launch_bounds__(1024, 1) eo_pass2(EOArgs A, const T* __restrict__ w1,
                                                    const uint2* __restrict__ t2o,
                                                    const uint16_t* __restrict__ cf_e,
                                                    const uint32_t* __restrict__ erep,
                                                    const uint32_t* __restrict__ cls_start,
                                                    const uint32_t* __restrict__ cls_size,
                                                    const uint32_t* __restrict__ out_off,
                                                    const uint16_t* __restrict__ out_o,
                                                    const double* __restrict__ sout64,
                                                    const float* __restrict__ sout32,
                                                    const dfloat* __restrict__ soutdf, double post,
                                                    OutT* __restrict__ y, float4* __restrict__ xchg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  __shared__ uint32_t he[128];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = CL ? (int)cl.block_rank() : 0;
  const int64_t tile = blockIdx.x >> A.c;
  const int n = A.n, p = A.p;
  const int kb = n - p;
  const uint32_t lmask = (1u << n) - 1u;
  const uint32_t base = (uint32_t)rank << n;
  const uint32_t e_rep = erep[tile];
  // this tile's w1 block (class-major): member offsets of the H-images of e_rep
  const uint32_t hb = cls_start[tile], hs = cls_size[tile];
  for (int g = threadIdx.x; g < A.ng; g += blockDim.x)
    he[g] = hb * (uint32_t)A.n_orep + (__ldg(cf_e + act_e(g, e_rep, A.m)) - hb);
  __syncthreads();
  {
#pragma unroll
    for (int c0 = 0; c0 < (1 << KB); c0 += kGatherChunk) {
      uint32_t code[kGatherChunk];
      uint16_t ov[kGatherChunk];
#pragma unroll
      for (int i = 0; i < kGatherChunk; ++i) {
        if (c0 + i < (1 << kb)) {
          const uint32_t P = base + threadIdx.x + ((c0 + i) << p);
          const uint2 w = __ldg(t2o + P);  // (t2 code, it_o)
          code[i] = w.x;
          ov[i] = (uint16_t)w.y;
        }
      }
#pragma unroll
      for (int i = 0; i < kGatherChunk; ++i)
        if (c0 + i < (1 << kb))
          cp_async_elem<sizeof(T)>(sm + spad(ov[i] & lmask),
                                   w1 + he[code[i] & 255u] + (int64_t)(code[i] >> 8) * hs);
    }
    cp_async_wait_all();
  }
  __syncthreads();
  smem_rounds<T, KB>(sm, A, n);
  if constexpr (CL) cluster_reduce<T, KB>(cl, sm, rank, A, xchg);
  // Designated outputs of this tile.  They are ordered like it_o, so the
  // outputs whose o this CTA holds form one contiguous range: groups
  // [rank, rank + 1) * 2^(ct - c) of the tile's 2^ct output groups.
  const int64_t g0 = (tile << A.ct) + ((int64_t)rank << (A.ct - A.c));
  const uint32_t k0 = out_off[g0], k1 = out_off[g0 + (1 << (A.ct - A.c))];
  // the output scales are loaded with the o indices, a batch at a time, so
  // their loads are in flight together
  using Scale = typename std::conditional<OSC == kOutDF, dfloat, typename std::conditional<OSC == kOutF64, double, float>::type>::type;
  const Scale* __restrict__ scale = [&] {
    if constexpr (OSC == kOutDF) return soutdf;
    else if constexpr (OSC == kOutF64) return sout64;
    else return sout32;
  }();
  const uint32_t step = blockDim.x * kOutBatch;
  for (uint32_t kk = k0 + threadIdx.x; kk < k1; kk += step) {
    uint16_t ov[kOutBatch];
    Scale sc[kOutBatch];
#pragma unroll
    for (int q = 0; q < kOutBatch; ++q) {
      const uint32_t k = kk + q * blockDim.x;
      if (k < k1) {
        ov[q] = ld_stream(out_o + k);
        sc[q] = ld_stream(scale + k);
      }
    }
#pragma unroll
    for (int q = 0; q < kOutBatch; ++q) {
      const uint32_t k = kk + q * blockDim.x;
      if (k < k1) {
        const T val = sm[spad(ov[q] & lmask)];
        if constexpr (OSC == kOutDF)
          y[k] = val * sc[q];
        else if constexpr (OSC == kOutF64)
          y[k] = (OutT)((double)val * sc[q] * post);
        else
          y[k] = (OutT)(val * T(sc[q]));
      }
    }
  }
}

// ---------------------------------------------------------------- plan kernels


struct PlanDev {
  GroupDev g;
  int m;
  const uint32_t* bits;
  const uint32_t* prefix;
};

__device__ __forceinline__ uint32_t rank_of(const PlanDev& P, uint64_t c) {
  uint32_t w = (uint32_t)(c >> 5);
  return P.prefix[w] + __popc(P.bits[w] & ((1u << (c & 31)) - 1u));
}

// Designated output key of a state's orbit: the minimum of (tile << m |
// pos_o(o)) over the orbit images whose even part is an H-representative
// (pass-2 tile `tile`); pos_o is the position of o in pass 2's iteration
// order.  The layer group is H u H.tau with tau = rotation by one site, which
// maps (e, o) to (o, rotr_m(e, 1)); within a coset the images with a
// representative even part are those of the H elements taking e to its
// representative, usually one (einfo), so the key takes two lookups per coset
// instead of a walk over the whole group.
__device__ __forceinline__ uint32_t coset_key(uint32_t e, uint32_t o, int m, int ng,
                                              const uint32_t* __restrict__ einfo,
                                              const uint16_t* __restrict__ pos_o) {
  const uint32_t inf = __ldg(einfo + e);
  const uint32_t t = inf & 0xffffu, j = (inf >> 16) & 31u, nst = inf >> 24;
  const uint32_t mask = (1u << m) - 1u;
  // act_o of the decoded element: rotate right by j, reflect, flip
  uint32_t r = j ? (((o >> j) | (o << (m - j))) & mask) : o;
  if (inf & (1u << 21)) r = __brev(r) >> (32 - m);
  if (inf & (1u << 22)) r ^= mask;
  uint32_t best = (t << m) | __ldg(pos_o + r);
  if (nst > 1) {
    // e has a nontrivial stabiliser in H: the nst elements reaching its
    // representative, g0 first.  H is walked as (flip, reflection, rotation
    // j) with the rotations applied one site at a time.
    const int g0 = (int)j + m * (int)(((inf >> 21) & 1u) + 2u * ((inf >> 22) & 1u));
    const uint32_t rep = act_e(g0, e, m);
    uint32_t found = 1;
    for (int fl = 0; fl * 2 * m < ng && found < nst; ++fl)
      for (int rf = 0; rf < 2 && found < nst; ++rf) {
        uint32_t ee = e, oo = o;  // rotated right by j2
        for (int j2 = 0; j2 < m && found < nst; ++j2) {
          if (j2 + m * (rf + 2 * fl) > g0) {
            uint32_t ae = ee;
            if (rf) {
              ae = brev_m(ee, m);
              ae = ((ae << 1) | (ae >> (m - 1))) & mask;  // rotate left by one
            }
            if (fl) ae ^= mask;
            if (ae == rep) {
              uint32_t ao = rf ? brev_m(oo, m) : oo;
              if (fl) ao ^= mask;
              best = min(best, (t << m) | __ldg(pos_o + ao));
              ++found;
            }
          }
          ee = ((ee >> 1) | (ee << (m - 1))) & mask;
          oo = ((oo >> 1) | (oo << (m - 1))) & mask;
        }
      }
  }
  return best;
}

__device__ __forceinline__ uint32_t designated_key(uint32_t s, int m, int ng, const uint32_t* __restrict__ einfo,
                                                   const uint16_t* __restrict__ pos_o) {
  const uint32_t e = gather16(s), o = gather16(s >> 1);
  const uint32_t e1 = ((e >> 1) | (e << (m - 1))) & ((1u << m) - 1u);  // rotr_m(e, 1)
  return min(coset_key(e, o, m, ng, einfo, pos_o), coset_key(o, e1, m, ng, einfo, pos_o));
}

__global__ void eo_key_kernel(int m, int ng, const uint32_t* __restrict__ idx, int64_t R,
                              const uint32_t* __restrict__ einfo, const uint16_t* __restrict__ pos_o,
                              uint32_t* __restrict__ key, uint32_t* __restrict__ dbits) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < R; i += st) {
    const uint32_t best = designated_key(idx[i], m, ng, einfo, pos_o);
    key[i] = best;
    atomicOr(dbits + (best >> 5), 1u << (best & 31));
  }
}

__global__ void popc_kernel(const uint32_t* __restrict__ bits, uint32_t* __restrict__ cnt, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) cnt[i] = __popc(bits[i]);
}

__global__ void eo_perm_kernel(const uint32_t* __restrict__ key, int64_t R, const uint32_t* __restrict__ dbits,
                               const uint32_t* __restrict__ dpre, int m, const uint16_t* __restrict__ o_of_pos,
                               uint32_t* __restrict__ pi, uint32_t* __restrict__ pinv,
                               uint16_t* __restrict__ out_o) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < R; i += st) {
    uint32_t k = key[i];
    uint32_t w = k >> 5;
    uint32_t pos = dpre[w] + __popc(dbits[w] & ((1u << (k & 31)) - 1u));
    pi[pos] = (uint32_t)i;
    pinv[i] = pos;
    out_o[pos] = o_of_pos[k & ((1u << m) - 1u)];
  }
}

// map1: pi position of the orbit of (it_e[P], o_rep(t)): its minimum by a
// walk over the group, then the orbit rank (rep bitset and word prefix)
__global__ void eo_map1_kernel(PlanDev P, const uint32_t* __restrict__ olist, int n_orep,
                               const uint16_t* __restrict__ it_e, const uint32_t* __restrict__ pinv,
                               uint32_t* __restrict__ map1) {
  const int64_t total = (int64_t)n_orep << P.m;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < total; i += st) {
    uint32_t t = (uint32_t)(i >> P.m), e = it_e[i & ((1 << P.m) - 1)];
    uint32_t s = join_eo(e, olist[t]);
    uint64_t c = canon(P.g, s);
    map1[i] = pinv[rank_of(P, c)];
  }
}

__global__ void eo_scale_kernel(const uint32_t* __restrict__ pi, const double* __restrict__ tv,
                                const uint16_t* __restrict__ dup, int64_t R, double gin, double* sin64,
                                double* sout64, float* sin32, float* sout32, dfloat* sindf, dfloat* soutdf) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < R; i += st) {
    uint32_t r = pi[i];
    double t = tv[r];
    double so = (double)dup[r] * t;
    sin64[i] = t;
    sout64[i] = so;
    sin32[i] = (float)t;
    sout32[i] = (float)so;
    sindf[i] = dfloat(t * gin);
    soutdf[i] = dfloat(so);
  }
}

__global__ void eo_offsets_kernel(const uint32_t* __restrict__ dpre, const uint32_t* __restrict__ dbits,
                                  int64_t nwords, int nparts, int part_words, uint32_t* off) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nparts) return;
  if (i < nparts)
    off[i] = dpre[(int64_t)i * part_words];
  else
    off[i] = dpre[nwords - 1] + __popc(dbits[nwords - 1]);
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)num_sms() * 16));
}

}  // namespace

// Cap on the tile bits of the passes for operators created from now on
// (0: none).  A diagnostic: it lets small operators run the clustered code
// paths that otherwise only L >= 30 reaches.
static std::atomic<int> g_eo_tile_bits_cap{0};
void eo_set_tile_bits_cap(int bits) { g_eo_tile_bits_cap.store(bits < 0 ? 0 : bits); }

// Decide cluster bits so a CTA's tile part fits in shared memory.
static int cluster_bits_for(int m, size_t elem) {
  int c = 0;
  while (((size_t)(1 << (m - c)) * elem * 33 / 32) > 200 * 1024) ++c;
  const int cap = g_eo_tile_bits_cap.load();
  if (cap > 0 && m - c > cap) c = m - cap;
  return c;
}

// Bytes of exchange slots the clustered launches of a plan need (0: none;
// only clusters of 4 or more CTAs use them).
size_t eo_xchg_bytes(const EOPlan& P) {
  size_t b = 0;
  const size_t nt = (size_t)std::max(P.n_orep, P.n_erep);
  if (P.c32 >= 2) b = std::max(b, (nt << P.c32) * (size_t)xchg_slot_chunks(P.m - P.c32, 4) * 16);
  if (P.c64 >= 2) b = std::max(b, (nt << P.c64) * (size_t)xchg_slot_chunks(P.m - P.c64, 8) * 16);
  return b;
}

// Orders of the m-bit patterns used by the passes.  cls: H-class index of
// each pattern (ncls classes); ct: top bits that split a tile over a cluster.
//   iteration order: (top ct bits, class, pattern) -- a CTA of a 2^c-CTA
//     cluster (c <= ct) owns one contiguous range, and a warp's elements are
//     one or two classes;
//   class-first order: (class, top ct bits, pattern) -- each class contiguous.
// A counting sort over the (top, class) buckets, patterns ascending within.
static std::vector<uint32_t> pattern_order(const std::vector<uint32_t>& cls, uint32_t ncls, int m, int ct,
                                           bool class_first) {
  const uint32_t M = 1u << m, ntop = 1u << ct;
  const size_t nb = (size_t)ncls * ntop;
  auto bucket = [&](uint32_t x) -> size_t {
    const uint32_t top = x >> (m - ct);
    return class_first ? (size_t)cls[x] * ntop + top : (size_t)top * ncls + cls[x];
  };
  std::vector<uint32_t> start(nb + 1, 0);
  for (uint32_t x = 0; x < M; ++x) ++start[bucket(x) + 1];
  for (size_t b = 0; b < nb; ++b) start[b + 1] += start[b];
  std::vector<uint32_t> ord(M);
  for (uint32_t x = 0; x < M; ++x) ord[start[bucket(x)]++] = x;
  return ord;
}

// Host tables of the even/odd plan.  They depend on m and the spin flip only,
// so they are computed on a host thread while the orbit table is built.
struct EOHostTables {
  int m = 0, ng = 0, c32 = 0, c64 = 0, ct = 0, n_orep = 0, n_erep = 0;
  std::vector<uint32_t> olist, elist, etile, t2, wbase, cls_start, cls_size;
  // per m-bit pattern x: e-tile of its H-representative (bits 0-15), the first
  // H element g = j + m (refl + 2 flip) with act_e(g, x) = rep, decoded (j in
  // bits 16-20, refl bit 21, flip bit 22), and how many reach it (bits 24-31)
  std::vector<uint32_t> einfo;
  std::vector<uint16_t> it_e, cf_e, it_o, pos_o;
  std::vector<uint8_t> wsz;
};

std::shared_ptr<EOHostTables> eo_host_tables(int m, int flip) {
  auto H = std::make_shared<EOHostTables>();
  H->m = m;
  H->ng = 2 * m * (flip ? 2 : 1);
  const uint32_t M = 1u << m, mask = M - 1u;
  // bit reversal of m-bit patterns through a byte table
  uint8_t rev8[256];
  for (int x = 0; x < 256; ++x) {
    int r = 0;
    for (int i = 0; i < 8; ++i) r |= ((x >> i) & 1) << (7 - i);
    rev8[x] = (uint8_t)r;
  }
  auto brev = [&](uint32_t x) { return (((uint32_t)rev8[x & 255u] << 8) | rev8[(x >> 8) & 255u]) >> (16 - m); };
  auto rot1 = [&](uint32_t x) { return ((x >> 1) | (x << (m - 1))) & mask; };  // rotate right by one
  // orbit minima under H and, for odd patterns, the first H element (in the
  // order g = j + m*refl + 2m*flip of act_o) reaching it
  std::vector<uint32_t> orep(M), erep_of(M);
  std::vector<int> og(M);
  for (uint32_t o = 0; o < M; ++o) {
    uint32_t best = o, r = o;
    int bg = 0;
    for (int j = 0; j < m; ++j, r = rot1(r)) {
      const uint32_t b = brev(r);
      const uint32_t im[4] = {r, b, r ^ mask, b ^ mask};
      for (int q = 0; q < (flip ? 4 : 2); ++q) {
        const int g = j + m * q;
        if (im[q] < best || (im[q] == best && g < bg)) {
          best = im[q];
          bg = g;
        }
      }
    }
    orep[o] = best;
    og[o] = (best == o) ? 0 : bg;
  }
  for (uint32_t e = 0; e < M; ++e) {
    uint32_t best = e, r = e;
    for (int j = 0; j < m; ++j, r = rot1(r)) {
      const uint32_t b = ((brev(r) << 1) | (brev(r) >> (m - 1))) & mask;  // rotl(brev(r), 1)
      best = std::min(best, std::min(r, b));
      if (flip) best = std::min(best, std::min(r ^ mask, b ^ mask));
    }
    erep_of[e] = best;
  }
  std::vector<uint32_t> otile(M, 0xffffffffu);
  H->etile.assign(M, 0xffffffffu);
  for (uint32_t o = 0; o < M; ++o)
    if (orep[o] == o) {
      otile[o] = (uint32_t)H->olist.size();
      H->olist.push_back(o);
    }
  for (uint32_t e = 0; e < M; ++e)
    if (erep_of[e] == e) {
      H->etile[e] = (uint32_t)H->elist.size();
      H->elist.push_back(e);
    }
  H->n_orep = (int)H->olist.size();
  H->n_erep = (int)H->elist.size();
  if (H->n_erep > 0xffff) fail(TM_ERR_LIMIT, "even/odd plan: too many even tiles");
  H->einfo.resize(M);
  for (uint32_t e = 0; e < M; ++e) {
    const uint32_t rep = erep_of[e];
    int g0 = -1, cnt = 0;
    uint32_t r = e;
    // act_e(g, e) for g = j + m * q, q = reflection + 2 * flip
    for (int j = 0; j < m; ++j, r = rot1(r)) {
      const uint32_t b = ((brev(r) << 1) | (brev(r) >> (m - 1))) & mask;
      const uint32_t im[4] = {r, b, r ^ mask, b ^ mask};
      for (int q = 0; q < (flip ? 4 : 2); ++q)
        if (im[q] == rep) {
          const int g = j + m * q;
          if (g0 < 0 || g < g0) g0 = g;
          ++cnt;
        }
    }
    const uint32_t j0 = (uint32_t)(g0 % m), q0 = (uint32_t)(g0 / m);
    H->einfo[e] = H->etile[rep] | (j0 << 16) | ((q0 & 1u) << 21) | ((q0 >> 1) << 22) | ((uint32_t)cnt << 24);
  }
  H->c32 = cluster_bits_for(m, 4);
  H->c64 = cluster_bits_for(m, 8);
  const int ct = H->ct = std::max(H->c32, H->c64);
  if (ct > 2) fail(TM_ERR_LIMIT, "even/odd tile split over more than 4 CTAs");
  std::vector<uint32_t> ecls(M), ocls(M);
  for (uint32_t x = 0; x < M; ++x) {
    ecls[x] = H->etile[erep_of[x]];
    ocls[x] = otile[orep[x]];
  }
  // pass 1 walks e in iteration order and stores w1 class-major; pass 2
  // walks o in iteration order, and the designated outputs of a pass-2 tile
  // follow the same order (so a CTA's outputs are contiguous)
  const std::vector<uint32_t> e_it = pattern_order(ecls, H->n_erep, m, ct, false);
  const std::vector<uint32_t> e_cf = pattern_order(ecls, H->n_erep, m, ct, true);
  const std::vector<uint32_t> o_it = pattern_order(ocls, H->n_orep, m, ct, false);
  H->it_e.resize(M);
  H->cf_e.resize(M);
  H->it_o.resize(M);
  H->pos_o.resize(M);
  H->t2.resize(M);
  H->wbase.resize(M);
  H->wsz.resize(M);
  H->cls_start.assign(H->n_erep, M);
  H->cls_size.assign(H->n_erep, 0);
  for (uint32_t i = 0; i < M; ++i) {
    H->cf_e[e_cf[i]] = (uint16_t)i;
    H->pos_o[o_it[i]] = (uint16_t)i;
  }
  for (uint32_t x = 0; x < M; ++x) {
    H->cls_start[ecls[x]] = std::min<uint32_t>(H->cls_start[ecls[x]], H->cf_e[x]);
    H->cls_size[ecls[x]] += 1;
  }
  // w1 is class-major: element (t, e) of e-class C at
  // start(C) * n_orep + t * |C| + (cf(e) - start(C))
  for (uint32_t i = 0; i < M; ++i) {
    const uint32_t e = e_it[i], C = ecls[e];
    H->it_e[i] = (uint16_t)e;
    H->wbase[i] = H->cls_start[C] * (uint32_t)H->n_orep + (H->cf_e[e] - H->cls_start[C]);
    H->wsz[i] = (uint8_t)H->cls_size[C];
    const uint32_t o = o_it[i];
    H->it_o[i] = (uint16_t)o;
    H->t2[i] = (otile[orep[o]] << 8) | (uint32_t)og[o];
  }
  return H;
}

void build_eo_plan(Op& op, const EOHostTables* Hp) {
  std::shared_ptr<EOHostTables> own;
  if (!Hp) {
    own = eo_host_tables(op.L / 2, op.grp.flip);
    Hp = own.get();
  }
  const EOHostTables& H = *Hp;
  EOPlan& P = op.eo;
  const int L = op.L, m = L / 2;
  if (H.m != m || H.ng != 2 * m * (op.grp.flip ? 2 : 1))
    fail(TM_ERR_ARG, "even/odd host tables for another L or spin-flip setting");
  const uint32_t M = 1u << m;
  P.m = m;
  P.ng = H.ng;
  P.n_orep = H.n_orep;
  P.n_erep = H.n_erep;
  P.c32 = H.c32;
  P.c64 = H.c64;
  const int ct = H.ct;
  const std::vector<uint32_t>& olist = H.olist;
  const std::vector<uint32_t>& elist = H.elist;
  const std::vector<uint32_t>& t2 = H.t2;
  const std::vector<uint32_t>& cls_start = H.cls_start;
  const std::vector<uint32_t>& cls_size = H.cls_size;
  const std::vector<uint16_t>& h_pos_o = H.pos_o;
  const std::vector<uint16_t>& h_it_e = H.it_e;
  const std::vector<uint16_t>& h_cf_e = H.cf_e;
  const std::vector<uint16_t>& h_it_o = H.it_o;
  const std::vector<uint32_t>& h_wbase = H.wbase;
  const std::vector<uint8_t>& h_wsz = H.wsz;

  cudaStream_t s = op.stream;
  DBuf d_olist, d_einfo, d_pos_o;
  d_olist.alloc(olist.size() * 4);
  d_einfo.alloc(M * 4);
  d_pos_o.alloc(M * 2);
  P.it_e.alloc(M * 2);
  P.cls_start.alloc(cls_start.size() * 4);
  P.cls_size.alloc(cls_size.size() * 4);
  P.cf_e.alloc(M * 2);
  P.it_o.alloc(M * 2);
  P.erep.alloc(elist.size() * 4);
  TM_CK(cudaMemcpyAsync(d_olist.p, olist.data(), olist.size() * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(d_einfo.p, H.einfo.data(), M * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(d_pos_o.p, h_pos_o.data(), M * 2, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(P.it_e.p, h_it_e.data(), M * 2, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(P.cls_start.p, cls_start.data(), cls_start.size() * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(P.cls_size.p, cls_size.data(), cls_size.size() * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(P.cf_e.p, h_cf_e.data(), M * 2, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(P.it_o.p, h_it_o.data(), M * 2, cudaMemcpyHostToDevice, s));
  {
    // per-position pairs read together by the passes
    std::vector<uint32_t> wo(2 * (size_t)M), to(2 * (size_t)M);
    for (uint32_t i = 0; i < M; ++i) {
      wo[2 * i] = h_wbase[i];
      wo[2 * i + 1] = (uint32_t)h_it_e[i] | ((uint32_t)h_wsz[i] << 16);
      to[2 * i] = t2[i];
      to[2 * i + 1] = h_it_o[i];
    }
    P.wout.alloc((size_t)M * 8);
    P.t2o.alloc((size_t)M * 8);
    TM_CK(cudaMemcpyAsync(P.wout.p, wo.data(), (size_t)M * 8, cudaMemcpyHostToDevice, s));
    TM_CK(cudaMemcpyAsync(P.t2o.p, to.data(), (size_t)M * 8, cudaMemcpyHostToDevice, s));
  }
  TM_CK(cudaMemcpyAsync(P.erep.p, elist.data(), elist.size() * 4, cudaMemcpyHostToDevice, s));

  const int64_t R = op.n;
  // designated outputs -> pi
  const int64_t nkeybits = (int64_t)P.n_erep << m;
  const int64_t nwords = (nkeybits + 31) / 32;
  DBuf key, dbits, dpre;
  key.alloc(R * 4);
  dbits.alloc(nwords * 4);
  dpre.alloc(nwords * 4);
  TM_CK(cudaMemsetAsync(dbits.p, 0, nwords * 4, s));
  eo_key_kernel<<<grid_for(R), 256, 0, s>>>(m, P.ng, op.idx.as<uint32_t>(), R, d_einfo.as<uint32_t>(),
                                            d_pos_o.as<uint16_t>(), key.as<uint32_t>(), dbits.as<uint32_t>());
  TM_CKK("eo_key");
  popc_kernel<<<grid_for(nwords), 256, 0, s>>>(dbits.as<uint32_t>(), dpre.as<uint32_t>(), nwords);
  TM_CKK("popc");
  exclusive_scan_u32(dpre.as<uint32_t>(), dpre.as<uint32_t>(), nwords, s);
  op.pi.alloc(R * 4);
  op.pinv.alloc(R * 4);
  P.out_o.alloc(R * 2);
  eo_perm_kernel<<<grid_for(R), 256, 0, s>>>(key.as<uint32_t>(), R, dbits.as<uint32_t>(), dpre.as<uint32_t>(), m,
                                             P.it_o.as<uint16_t>(), op.pi.as<uint32_t>(),
                                             op.pinv.as<uint32_t>(), P.out_o.as<uint16_t>());
  TM_CKK("eo_perm");
  // designated-output offsets per group of 2^(m-ct) iteration positions
  // of each pass-2 tile
  P.ct = ct;
  const int ngroups = P.n_erep << ct;
  P.out_off.alloc((size_t)(ngroups + 1) * 4);
  eo_offsets_kernel<<<(ngroups + 1 + 255) / 256, 256, 0, s>>>(dpre.as<uint32_t>(), dbits.as<uint32_t>(), nwords,
                                                              ngroups, (int)((M >> ct) / 32),
                                                              P.out_off.as<uint32_t>());
  TM_CKK("eo_offsets");
  // map1
  const int64_t n1 = (int64_t)P.n_orep << m;
  P.map1.alloc(n1 * 4);
  PlanDev pd;
  pd.g = to_dev(op.grp);
  pd.m = m;
  pd.bits = op.ws_a.as<uint32_t>();
  pd.prefix = op.ws_b.as<uint32_t>();
  eo_map1_kernel<<<grid_for(n1), 256, 0, s>>>(pd, d_olist.as<uint32_t>(), P.n_orep, P.it_e.as<uint16_t>(),
                                              op.pinv.as<uint32_t>(), P.map1.as<uint32_t>());
  TM_CKK("eo_map1");
  // scales in pi order
  op.sin64.alloc(R * 8);
  op.sout64.alloc(R * 8);
  op.sin32.alloc(R * 4);
  op.sout32.alloc(R * 4);
  op.sindf.alloc(R * 8);
  op.soutdf.alloc(R * 8);
  // double-float input scale with the (1 + r)^-L factor of the
  // unnormalised butterflies folded in
  const double gin = std::pow(1.0 + std::exp(-2.0 * std::fabs(op.mp.betaJ)), -(double)op.L);
  eo_scale_kernel<<<grid_for(R), 256, 0, s>>>(op.pi.as<uint32_t>(), op.tvec.as<double>(), op.dup.as<uint16_t>(),
                                              R, gin, op.sin64.as<double>(), op.sout64.as<double>(),
                                              op.sin32.as<float>(), op.sout32.as<float>(), op.sindf.as<dfloat>(),
                                              op.soutdf.as<dfloat>());
  TM_CKK("eo_scale");
  TM_CK(cudaStreamSynchronize(s));
  op.has_pi = true;
  P.active = true;
}

// ------------------------------------------------------------------ launch
namespace {

// u = x * sin * gin.  gin = (1 + r)^-L keeps the magnitudes of the
// unnormalised butterflies x0 + r x1 those of the normalised operator.
template <class T>
__global__ void eo_scale_in(const T* __restrict__ x, const double* __restrict__ s64,
                            const float* __restrict__ s32, T* __restrict__ u, int64_t n, double gin) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  const float gin32 = (float)gin;
  for (; i < n; i += st) {
    if (sizeof(T) == 8)
      u[i] = (T)((double)x[i] * s64[i] * gin);
    else
      u[i] = x[i] * ((T)s32[i] * gin32);
  }
}

// input factor of the unnormalised butterflies: (1 + r)^-L, r = e^-2|K|
double eo_gin(const Op& op) {
  return std::pow(1.0 + std::exp(-2.0 * std::fabs(op.mp.betaJ)), -(double)op.L);
}

// element types around each engine: FP32 and FP64 read and write their own
// type; double-float reads and writes FP64
template <class T>
struct EoIO {
  using In = T;
  using Out = T;
};
template <>
struct EoIO<dfloat> {
  using In = double;
  using Out = double;
};

// The exchange buffer for a clustered launch of `ntiles` tiles (one slot per
// CTA), or null: the cluster combine then reads the partners' tiles through
// DSMEM.  Clusters of 4 or more CTAs exchange through L2 (at L = 32 the
// double-float passes take 4.55 + 3.99 ms that way against 5.05 + 4.62 ms
// over DSMEM); a 2-CTA cluster reads its one partner through DSMEM, which
// measured 2-3% faster than the round trip through L2.  Native FP64
// combines element by element through DSMEM.
template <class T>
float4* eo_xchg(const EOArgs& A, const EOPlan& P, int ntiles) {
  if (A.c < 2 || std::is_same<T, double>::value || !P.xchg.p) return nullptr;
  const size_t need = ((size_t)ntiles << A.c) * (size_t)xchg_slot_chunks(A.n, (int)sizeof(T)) * 16;
  return need <= P.xchg.bytes ? P.xchg.as<float4>() : nullptr;
}

template <class T, int KB>
void launch_pass1(const EOArgs& A, int ntiles, const typename EoIO<T>::In* u, const EOPlan& P, T* w1,
                  cudaStream_t s) {
  size_t shm = (size_t)((1 << A.n) + (1 << A.n) / 32 + 1) * sizeof(T);
  auto kfn = (A.c > 0) ? eo_pass1<T, KB, typename EoIO<T>::In, true> : eo_pass1<T, KB, typename EoIO<T>::In, false>;
  raise_smem_limit((const void*)kfn, shm);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(ntiles << A.c));
  cfg.blockDim = dim3(1u << A.p);
  cfg.dynamicSmemBytes = shm;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 1u << A.c;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  TM_CK(cudaLaunchKernelEx(&cfg, kfn, A, u, P.map1.as<uint32_t>(), P.it_e.as<uint16_t>(), P.wout.as<uint2>(), w1,
                           eo_xchg<T>(A, P, ntiles)));
}

template <class T, int KB, int OSC, class OutT = typename EoIO<T>::Out>
void launch_pass2(const EOArgs& A, int ntiles, const T* w1, const EOPlan& P, const double* sout64,
                  const float* sout32, const dfloat* soutdf, double post, OutT* y, cudaStream_t s) {
  size_t shm = (size_t)((1 << A.n) + (1 << A.n) / 32 + 1) * sizeof(T);
  auto kfn = (A.c > 0) ? eo_pass2<T, KB, OSC, OutT, true> : eo_pass2<T, KB, OSC, OutT, false>;
  raise_smem_limit((const void*)kfn, shm);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(ntiles << A.c));
  cfg.blockDim = dim3(1u << A.p);
  cfg.dynamicSmemBytes = shm;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 1u << A.c;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  TM_CK(cudaLaunchKernelEx(&cfg, kfn, A, w1, P.t2o.as<uint2>(), P.cf_e.as<uint16_t>(),
                           P.erep.as<uint32_t>(), P.cls_start.as<uint32_t>(), P.cls_size.as<uint32_t>(),
                           P.out_off.as<uint32_t>(), P.out_o.as<uint16_t>(), sout64, sout32, soutdf, post, y,
                           eo_xchg<T>(A, P, ntiles)));
}

template <class T>
EOArgs make_args(const Op& op, int c) {
  EOArgs A;
  A.m = op.eo.m;
  A.c = c;
  A.ct = op.eo.ct;
  A.n = A.m - c;
  if (A.n > kMaxTileBits) fail(TM_ERR_LIMIT, "even/odd tile larger than 2^16 elements");
  const int KB = (sizeof(T) == 8) ? 4 : 5;
  int kb = std::min(KB, std::max(1, A.n - 5));
  A.p = A.n - kb;
  if (A.p > 10) A.p = 10;
  A.ng = op.eo.ng;
  A.n_orep = op.eo.n_orep;
  const double K = op.mp.betaJ;
  A.r64 = std::exp(-2.0 * std::fabs(K));
  A.r32 = (float)A.r64;
  A.swap = K < 0 ? 1 : 0;
  return A;
}

template <class T, int KB>
void eo_dispatch(const Op& op, const EOArgs& A, const typename EoIO<T>::In* x, typename EoIO<T>::Out* y,
                 bool scaled32, cudaStream_t s) {
  using In = typename EoIO<T>::In;
  const EOPlan& P = op.eo;
  const int64_t R = op.n;
  In* u = static_cast<In*>(op.ws_c.p);
  T* w1 = (sizeof(T) == 8) ? static_cast<T*>(P.w1_64.p) : static_cast<T*>(P.w1_32.p);
  if (P.prof_on) TM_CK(cudaEventRecord(P.prof_ev[0], s));
  eo_scale_in<In><<<grid_for(R), 256, 0, s>>>(x, op.sin64.as<double>(), op.sin32.as<float>(), u, R,
                                               eo_gin(op));
  TM_CKK("eo_scale_in");
  if (P.prof_on) TM_CK(cudaEventRecord(P.prof_ev[1], s));
  launch_pass1<T, KB>(A, P.n_orep, u, P, w1, s);
  TM_CKK("eo_pass1");
  if (P.prof_on) TM_CK(cudaEventRecord(P.prof_ev[2], s));
  const double S = std::pow(std::exp(op.mp.betaJ) + std::exp(-op.mp.betaJ), (double)op.L);
  if (scaled32)
    launch_pass2<T, KB, kOutF32>(A, P.n_erep, w1, P, op.sout64.as<double>(), op.sout32.as<float>(), nullptr, 1.0,
                                 y, s);
  else
    launch_pass2<T, KB, kOutF64>(A, P.n_erep, w1, P, op.sout64.as<double>(), op.sout32.as<float>(), nullptr, S, y,
                                 s);
  TM_CKK("eo_pass2");
  if (P.prof_on) TM_CK(cudaEventRecord(P.prof_ev[3], s));
}

template <class T>
void matvec_eo_engine(const Op& op, const typename EoIO<T>::In* x, typename EoIO<T>::Out* y, bool scaled32,
                      cudaStream_t s) {
  const int c = (sizeof(T) == 8) ? op.eo.c64 : op.eo.c32;
  EOArgs A = make_args<T>(op, c);
  int kb = A.n - A.p;
  switch (kb) {
    case 1: eo_dispatch<T, 1>(op, A, x, y, scaled32, s); break;
    case 2: eo_dispatch<T, 2>(op, A, x, y, scaled32, s); break;
    case 3: eo_dispatch<T, 3>(op, A, x, y, scaled32, s); break;
    case 4: eo_dispatch<T, 4>(op, A, x, y, scaled32, s); break;
    default:
      if constexpr (sizeof(T) == 4)
        eo_dispatch<T, 5>(op, A, x, y, scaled32, s);
      else
        fail(TM_ERR_LIMIT, "even/odd tile too large for the 8-byte engines");
      break;
  }
}

}  // namespace

// y = T x in pi order.  scaled32: FP32 result divided by (e^K+e^-K)^L (the
// solver applies that factor in FP64).
template <class T>
void matvec_eo(const Op& op, const T* x, T* y, bool scaled32, cudaStream_t s) {
  matvec_eo_engine<T>(op, x, y, scaled32, s);
}

template void matvec_eo<float>(const Op&, const float*, float*, bool, cudaStream_t);
template void matvec_eo<double>(const Op&, const double*, double*, bool, cudaStream_t);

// FP64 in/out, double-float arithmetic (the solver's refinement products)
void matvec_eo_df(const Op& op, const double* x, double* y, cudaStream_t s) {
  matvec_eo_engine<dfloat>(op, x, y, false, s);
}

namespace {
__global__ void eo_scale_in_dd(const dfloat* __restrict__ x, const dfloat* __restrict__ sdf, dfloat* __restrict__ u,
                               int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    u[i] = x[i] * sdf[i];
}

template <int KB>
void eo_dispatch_dd(const Op& op, const EOArgs& A, const dfloat* x, dfloat* y, cudaStream_t s) {
  const EOPlan& P = op.eo;
  const int64_t R = op.n;
  dfloat* u = static_cast<dfloat*>(op.ws_c.p);
  dfloat* w1 = static_cast<dfloat*>(P.w1_64.p);
  eo_scale_in_dd<<<grid_for(R), 256, 0, s>>>(x, op.sindf.as<dfloat>(), u, R);
  TM_CKK("eo_scale_in_dd");
  const size_t shm = (size_t)((1 << A.n) + (1 << A.n) / 32 + 1) * sizeof(dfloat);
  auto k1 = (A.c > 0) ? eo_pass1<dfloat, KB, dfloat, true> : eo_pass1<dfloat, KB, dfloat, false>;
  raise_smem_limit((const void*)k1, shm);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(P.n_orep << A.c));
  cfg.blockDim = dim3(1u << A.p);
  cfg.dynamicSmemBytes = shm;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 1u << A.c;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  TM_CK(cudaLaunchKernelEx(&cfg, k1, A, (const dfloat*)u, P.map1.as<uint32_t>(), P.it_e.as<uint16_t>(),
                           P.wout.as<uint2>(), w1, eo_xchg<dfloat>(A, P, P.n_orep)));
  TM_CKK("eo_pass1_dd");
  launch_pass2<dfloat, KB, kOutDF, dfloat>(A, P.n_erep, w1, P, op.sout64.as<double>(), op.sout32.as<float>(),
                                           op.soutdf.as<dfloat>(), 1.0, y, s);
  TM_CKK("eo_pass2_dd");
}
}  // namespace

// Double-float in/out: y = T x / S with S = eo_scale32 (the FP32 products'
// scale), so values stay in the FP32 exponent range.
void matvec_eo_dd(const Op& op, const dfloat* x, dfloat* y, cudaStream_t s) {
  EOArgs A = make_args<dfloat>(op, op.eo.c64);
  switch (A.n - A.p) {
    case 1: eo_dispatch_dd<1>(op, A, x, y, s); break;
    case 2: eo_dispatch_dd<2>(op, A, x, y, s); break;
    case 3: eo_dispatch_dd<3>(op, A, x, y, s); break;
    case 4: eo_dispatch_dd<4>(op, A, x, y, s); break;
    default: fail(TM_ERR_LIMIT, "even/odd tile too large for the 8-byte engines");
  }
}

// FP64 even/odd product in pi order with caller-provided scratch: u (R
// doubles) and w1 (n_orep * 2^m doubles).  Used by the entry point whose
// scratch lives in a fixed device array.
void matvec_eo_f64_into(const Op& op, const double* x, double* y, double* u, double* w1, cudaStream_t s) {
  const EOPlan& P = op.eo;
  const int64_t R = op.n;
  EOArgs A = make_args<double>(op, P.c64);
  if (A.n - A.p > 4) fail(TM_ERR_LIMIT, "even/odd tile too large for the FP64 engine");
  eo_scale_in<double><<<grid_for(R), 256, 0, s>>>(x, op.sin64.as<double>(), op.sin32.as<float>(), u, R,
                                                   eo_gin(op));
  TM_CKK("eo_scale_in");
  const double S = std::pow(std::exp(op.mp.betaJ) + std::exp(-op.mp.betaJ), (double)op.L);
  switch (A.n - A.p) {
#define TM_EO_INTO(KBV)                                                                                      \
  case KBV:                                                                                                  \
    launch_pass1<double, KBV>(A, P.n_orep, u, P, w1, s);                                                     \
    TM_CKK("eo_pass1");                                                                                      \
    launch_pass2<double, KBV, kOutF64>(A, P.n_erep, w1, P, op.sout64.as<double>(), op.sout32.as<float>(),   \
                                       nullptr, S, y, s);                                                    \
    TM_CKK("eo_pass2");                                                                                      \
    break;
    TM_EO_INTO(1)
    TM_EO_INTO(2)
    TM_EO_INTO(3)
    TM_EO_INTO(4)
#undef TM_EO_INTO
  }
}

double eo_scale32(const Op& op) {
  return std::pow(std::exp(op.mp.betaJ) + std::exp(-op.mp.betaJ), (double)op.L);
}

}  // namespace ltm
