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
// The reference rotates the state by one (two) sites after every step, so the
// sites a step touches are always the low ones.  Undoing the rotation (a
// fixed frame: after L/KS steps the rotation is the identity) shows that step
// t is a local gate: it rewrites the aux bits and the KS sites at positions
// KS*t .. KS*t+KS-1 from the same 2^(NA+KS) values, with weights that depend on
// the next KS sites (or, at the last step, on the lastbit pass).  Here a pass
// gathers tiles of 2^12 (FP64) or 2^13 (FP32) elements whose index bits are the
// aux bits, a few contiguous low sites (coalescing) and the sites of several
// consecutive steps, applies those steps in shared memory and writes the tile
// back in place: ceil(steps / steps-per-pass) sweeps over HBM instead of one
// per step.  The first pass builds its tiles from x (the reference's sparse
// initial vector), the last pass folds aux bits and lastbit passes into y.
// Arithmetic per element is the reference's, in its order.  FP32 steps are
// scaled by the inverse of their largest row sum; the product of the scales
// is applied in FP64.  Reduced operators (XDM, ZBM) gather x through the
// state->rank map and contract the full-space result at the representatives.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>
#include <vector>

#include "tm_chain.h"
#include "tm_df.cuh"
#include "tm_internal.h"

namespace ltm {

namespace {

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)num_sms() * 32));
}

__device__ __forceinline__ int spad(int e) { return e + (e >> 5); }

__device__ __forceinline__ int64_t chain_pass_blocks_dev(const ChainPass& cp);

// the part of a tile value the fold sums: the value, or for a tangent pair
// its derivative (the tangent product's output)
__device__ __forceinline__ double fold_part(float x) { return (double)x; }
__device__ __forceinline__ double fold_part(double x) { return x; }
__device__ __forceinline__ double fold_part(dfloat x) { return (double)x; }
__device__ __forceinline__ double fold_part(tangent x) { return (double)x.d; }

// acc + a b in the chain's arithmetic: one renormalisation for double-float
// (df_fma) instead of one per multiply and add
__device__ __forceinline__ float mad_t(float a, float b, float acc) { return fmaf(a, b, acc); }
__device__ __forceinline__ double mad_t(double a, double b, double acc) { return fma(a, b, acc); }
__device__ __forceinline__ dfloat mad_t(dfloat a, dfloat b, dfloat acc) { return df_fma(a, b, acc); }
__device__ __forceinline__ tangent mad_t(tangent a, tangent b, tangent acc) { return acc + a * b; }

// Double-float values two to a lane pair (hi words in one float2, lo words
// in another), for the double-float BNNNI steps on the packed FP32 pipes.
// Each is the scalar double-float operation of tm_df.cuh lane by lane, in
// the same operation order; differences are fma(b, -1, a), and -p comes from
// the weight's negated hi word, so no operand needs a separate negation.
__device__ __forceinline__ float2 dsub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
// x * w (operator*): w = (wh, wl) with wn = -wh
__device__ __forceinline__ void df2_mul(float2 xh, float2 xl, float2 wh, float2 wl, float2 wn, float2& oh,
                                       float2& ol) {
  const float2 np = __fmul2_rn(xh, wn);  // -p
  float2 e = __ffma2_rn(xh, wh, np);
  e = __ffma2_rn(xh, wl, e);
  e = __ffma2_rn(xl, wh, e);
  oh = dsub2(e, np);                        // p + e
  ol = dsub2(e, __fadd2_rn(oh, np));        // e - (h - p)
}
// x * w + y (df_fma)
__device__ __forceinline__ void df2_fma(float2 xh, float2 xl, float2 wh, float2 wl, float2 wn, float2 yh, float2 yl,
                                       float2& oh, float2& ol) {
  const float2 np = __fmul2_rn(xh, wn);  // -p
  float2 pe = __ffma2_rn(xh, wh, np);
  pe = __ffma2_rn(xh, wl, pe);
  pe = __ffma2_rn(xl, wh, pe);
  const float2 sm = dsub2(yh, np);                     // p + y.hi
  const float2 bb = __fadd2_rn(sm, np);                // s - p
  const float2 e2 = dsub2(yh, bb);                     // y.hi - bb
  float2 se = dsub2(e2, __fadd2_rn(np, dsub2(sm, bb)));  // (p - (s - bb)) + (y.hi - bb)
  se = __fadd2_rn(se, __fadd2_rn(pe, yl));
  oh = __fadd2_rn(sm, se);
  ol = dsub2(se, dsub2(oh, sm));
}

// byte offset of the fold accumulators in chain_kernel's shared memory
__host__ __device__ __forceinline__ size_t chain_acc_offset(int tile, size_t elem) {
  return (((size_t)(tile + tile / 32 + 1) * elem) + 15) & ~(size_t)15;
}

// tile state index -> state bits: the tile's state bits are the contiguous
// runs [0, cb) and [lo, lo + nst - cb)
__device__ __forceinline__ uint64_t tile_state(uint64_t v, int cb, int lo) {
  return (v & ((1ull << cb) - 1)) | ((v >> cb) << lo);
}

__device__ __forceinline__ uint64_t dep(uint64_t v, const int* pos, int nb) {
  uint64_t g = 0;
  for (int k = 0; k < nb; ++k) g |= ((v >> k) & 1ull) << pos[k];
  return g;
}

// Initial (lastbit pass lb) value of element (aux, r): TMat/tmat.cpp:392-457
// (DNNI: aux = copy of the top site, site 0 = lb; boundary cases 5 and 9) and
// :604-612 (BNNNI: aux = copy of the two top sites, sites 0-1 = lb).
template <class T, int ZB, class IO>
__device__ __forceinline__ T chain_init(const IO* __restrict__ x, const double* __restrict__ pre,
                                        const uint32_t* __restrict__ smap, int L, int bc, uint64_t r, int aux, int lb,
                                        const AuxCoefT<T>& c) {
  auto u = [&]() -> T {
    if (smap) {
      const uint32_t q = smap[r];
      return (T)((double)x[q] * pre[q]);
    }
    return pre ? (T)((double)x[r] * pre[r]) : (T)x[r];
  };
  if (ZB) {
    if ((int)(r >> (L - 2)) == aux && (int)(r & 3) == lb) return u();
    return (T)0;
  }
  if (bc == 0) {
    if ((int)(r >> (L - 1)) == aux && (int)(r & 1) == lb) return u();
    return (T)0;
  }
  if (bc == 5) return aux == 0 ? u() * c.b2[r & 1] * c.b2[r >> (L - 1)] : (T)0;
  return aux == 1 ? u() * c.b2[(r & 1) ^ 1] * c.b2[r >> (L - 1)] : (T)0;  // bc 9
}

// One pass of steps over tiles in shared memory.
//   ZB = 0: DNNI, NA = 1 aux bit, one site per step (permute_mult_T1 /
//           _last, TMat/tmat.cpp:344-376); L steps.
//   ZB = 1: diagonal BNNNI, NA = 2, two sites per step (TMat/tmat.cpp:521-588,
//           dir = optdirection); L/2 steps.
// P: the nlb*2^L*2^NA buffer (in place).  first: tiles built from x; last:
// y[r] = postc * post[r] * sum_{lb, aux} (one CTA loops the lastbit passes).
// (the body of one block: `blk` is its index within the pass's grid)
template <class T, int ZB, class IO>
__device__ __forceinline__ void chain_block(T* __restrict__ P, const IO* __restrict__ x,
                                            const double* __restrict__ pre, const uint32_t* __restrict__ smap,
                                            IO* __restrict__ y, const double* __restrict__ post, double postc, int L,
                                            int bc, int dir, const AuxCoefT<T>& c, const ChainPass& cp, uint64_t blk) {
  constexpr int NA = ZB ? 2 : 1, KS = ZB ? 2 : 1, GB = NA + KS;  // group bits
  extern __shared__ unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int tile = 1 << (NA + cp.nst);
  const int nsteps = ZB ? L / 2 : L;
  // FP64 fold accumulators after the padded tile, at a 16-byte boundary
  // (the FP32 tile's padded size is not a multiple of 8 bytes)
  double* acc = reinterpret_cast<double*>(smraw + chain_acc_offset(tile, sizeof(T)));
  // Step coefficients, functions of the control bits only.  The step's
  // matrix factorises as out(a', s') = z_f[s'] u[a'][s'] sum_q w[s'][q]
  // in(q, a'): w and u (the step normalisation folded into u) are the same
  // for every group and sit in shared memory, read as broadcast rows; only
  // z depends on the group's control bits f and is formed in registers.
  //   BNNNI dir 0: w = b1[sr^al] b2[sr^ar] b2[sl^al], u = b1[sr^pl] b3[sr^pr] b3[sl^pl],
  //                z = b2[sr^fr] b2[sl^fl];
  //   BNNNI dir 1: w = b2[sr^ar] b2[sl^al], u = b1[sl^pr] b3[sr^pr] b3[sl^pl],
  //                z = b1[sl^fr] b2[sr^fr] b2[sl^fl];
  //   DNNI:        w = b2[s^q], u = b1[s^a], z = b2[nb^s].
  // (TMat/tmat.cpp:344-376 and 521-588 form the same products per element.)
  constexpr int NS = 1 << KS;
  __shared__ __align__(16) T wrow[16];  // [s'][q]
  __shared__ __align__(16) T urow[16];  // [s'][a']
  if (ZB) {
    for (int k = threadIdx.x; k < 16; k += blockDim.x) {
      const int sv = k >> 2, q = k & 3, sl = sv >> 1, sr = sv & 1, al = q >> 1, ar = q & 1;
      wrow[k] = !dir ? c.b1[sr ^ al] * c.b2[sr ^ ar] * c.b2[sl ^ al] : c.b2[sr ^ ar] * c.b2[sl ^ al];
      const int pl = q >> 1, pr = q & 1;  // here q is a' = (pl, pr)
      urow[k] = (!dir ? c.b1[sr ^ pl] * c.b3[sr ^ pr] * c.b3[sl ^ pl] : c.b1[sl ^ pr] * c.b3[sr ^ pr] * c.b3[sl ^ pl]) *
                c.g;
    }
  } else {
    for (int k = threadIdx.x; k < 4; k += blockDim.x) {
      const int sv = k >> 1, q = k & 1;
      wrow[k] = c.b2[sv ^ q];
      urow[k] = c.b1[sv ^ q] * c.g;  // q is a here
    }
  }
  // native FP64 (bound by the FP64 pipe): z_f[s'] u[a'][s'] for all four f
  // from a table, one multiply per output fewer
  constexpr bool kZuTable = ZB && std::is_same<T, double>::value;
  __shared__ __align__(16) T zutab[kZuTable ? 64 : 1];
  if constexpr (kZuTable) {
    for (int k = threadIdx.x; k < 64; k += blockDim.x) {
      const int f = k >> 4, sv = (k >> 2) & 3, aux = k & 3;
      const int fl = f >> 1, fr = f & 1, sl = sv >> 1, sr = sv & 1, pl = aux >> 1, pr = aux & 1;
      T z = c.b2[sr ^ fr] * c.b2[sl ^ fl];
      if (dir) z = z * c.b1[sl ^ fr];
      const T u = (!dir ? c.b1[sr ^ pl] * c.b3[sr ^ pr] * c.b3[sl ^ pl] : c.b1[sl ^ pr] * c.b3[sr ^ pr] * c.b3[sl ^ pl]) * c.g;
      zutab[k] = z * u;
    }
  }
  // double-float BNNNI: the steps run on packed lanes (aux pairs); z_f u
  // for all four f and the weights, split into hi / lo planes (the weights
  // duplicated across the two lanes, with the negated hi word)
  constexpr bool kPacked = ZB && std::is_same<T, dfloat>::value;
  __shared__ __align__(16) float zuh[kPacked ? 64 : 1], zul[kPacked ? 64 : 1];
  __shared__ __align__(16) float2 wph[kPacked ? 16 : 1], wpl[kPacked ? 16 : 1], wpn[kPacked ? 16 : 1];
  if constexpr (kPacked) {
    // (from the coefficients, as urow and wrow are formed: those rows are
    // written by other threads and read only after the tile barrier)
    for (int k = threadIdx.x; k < 64; k += blockDim.x) {
      const int f = k >> 4, sv = (k >> 2) & 3, aux = k & 3;
      const int fl = f >> 1, fr = f & 1, sl = sv >> 1, sr = sv & 1, pl = aux >> 1, pr = aux & 1;
      const T u = (!dir ? c.b1[sr ^ pl] * c.b3[sr ^ pr] * c.b3[sl ^ pl] : c.b1[sl ^ pr] * c.b3[sr ^ pr] * c.b3[sl ^ pl]) *
                  c.g;
      T z = c.b2[sr ^ fr] * c.b2[sl ^ fl];
      if (dir) z = z * c.b1[sl ^ fr];
      const T zu = u * z;
      zuh[k] = zu.hi;
      zul[k] = zu.lo;
    }
    for (int k = threadIdx.x; k < 16; k += blockDim.x) {
      const int sv = k >> 2, q = k & 3, sl = sv >> 1, sr = sv & 1, al = q >> 1, ar = q & 1;
      const T w = !dir ? c.b1[sr ^ al] * c.b2[sr ^ ar] * c.b2[sl ^ al] : c.b2[sr ^ ar] * c.b2[sl ^ al];
      wph[k] = make_float2(w.hi, w.hi);
      wpl[k] = make_float2(w.lo, w.lo);
      wpn[k] = make_float2(-w.hi, -w.hi);
    }
  }
  // the factors z selects from, in registers (no indexed access)
  const T b1_0 = c.b1[0], b1_1 = c.b1[1], b2_0 = c.b2[0], b2_1 = c.b2[1];
  // outer index: state bits, then (unless last) the lastbit pass
  const uint64_t ob = blk & ((1ull << cp.no) - 1);
  const int lb_outer = (int)(blk >> cp.no);
  const uint64_t rbase = dep(ob, cp.opos, cp.no);
  const int site0 = KS * cp.t0;  // lowest site of the pass's steps
  const int nloop = cp.last ? cp.nlb : 1;
  if (cp.last)
    for (int e = threadIdx.x; e < (tile >> NA); e += blockDim.x) acc[e] = 0.0;
  // The aux bits and the cb low sites are contiguous in HBM, so a pass with
  // 2^(NA + cb) >= VEC elements per run moves whole 16-byte chunks (VEC
  // consecutive tile elements sit in consecutive padded slots: VEC divides 32).
  constexpr int VEC = 16 / (int)sizeof(T);
  const bool vec_io = (1 << (NA + cp.jbit0)) >= VEC;
  for (int li = 0; li < nloop; ++li) {
    const int lb = cp.last ? li : lb_outer;
    // load / build the tile
    if (!cp.first && vec_io) {
      for (int e = threadIdx.x * VEC; e < tile; e += blockDim.x * VEC) {
        const uint64_t r = rbase | tile_state((uint64_t)(e >> NA), cp.jbit0, site0);
        const uint64_t at = (((uint64_t)lb << L | r) << NA) | (uint64_t)(e & ((1 << NA) - 1));
        const uint4 raw = __ldcs(reinterpret_cast<const uint4*>(P + at));
        const T* v = reinterpret_cast<const T*>(&raw);
        T* dst = sm + spad(e);
#pragma unroll
        for (int k = 0; k < VEC; ++k) dst[k] = v[k];
      }
    } else {
      for (int e = threadIdx.x; e < tile; e += blockDim.x) {
        const int aux = e & ((1 << NA) - 1);
        const uint64_t r = rbase | tile_state((uint64_t)(e >> NA), cp.jbit0, site0);
        T v;
        if (cp.first)
          v = chain_init<T, ZB, IO>(x, pre, smap, L, bc, r, aux, lb, c);
        else
          v = P[(((uint64_t)lb << L | r) << NA) | (uint64_t)aux];
        sm[spad(e)] = v;
      }
    }
    __syncthreads();
    for (int j = 0; j < cp.T; ++j) {
      const int t = cp.t0 + j;
      const int sb = NA + cp.jbit0 + KS * j;  // tile bit of the step's lowest site
      const bool lastst = (t == nsteps - 1);
      const int groups = tile >> GB;
      // Slot of (group base, aux q, step sites sp): spad(ebase) + q +
      // spad(sp << sb), since spad(a | b) = spad(a) + spad(b) for disjoint
      // a, b and q < 4 never reaches bit 5 of an aux-aligned base.
      const int o1 = spad(1 << sb), o2 = ZB ? spad(2 << sb) : 0, o3 = ZB ? spad(3 << sb) : 0;
      // The control sites (the next step's sites) are tile bits [sb + KS,
      // sb + 2 KS) unless this is the pass's last step; then they are outer
      // bits of the block, or the lastbit pass at the product's last step.
      const bool ctl_in_tile = (j + 1 < cp.T);
      const int ctl_outer = lastst ? (ZB ? lb : (bc == 0 ? lb : 0))
                                   : (int)((rbase >> (KS * t + KS)) & (uint64_t)((1 << KS) - 1));
      for (int gi = threadIdx.x; gi < groups; gi += blockDim.x) {
        // tile index of the group base: insert zeros at [0, NA) and [sb, sb+KS)
        const int lo = gi & ((1 << (sb - NA)) - 1);
        const int hi = gi >> (sb - NA);
        const int ebase = (hi << (sb + KS)) | (lo << NA);
        const int ctl = ctl_in_tile ? ((ebase >> (sb + KS)) & ((1 << KS) - 1)) : ctl_outer;
        T* b0 = sm + spad(ebase);
        // an offset the compiler cannot see through: the coefficient rows are
        // re-read (broadcast) per group instead of held in registers across
        // the loop, which would leave too few for the group's values
        int z0 = 0;
        asm volatile("" : "+r"(z0));
        const T* wr = wrow + z0;
        const T* ur = urow + z0;
        if (!ZB) {
          // DNNI: out(a, s) = b1[s^a] b2[nb^s] (b2[s] in(0, a) + b2[s^1] in(1, a)),
          // in(q, s') = value with aux q and site t = s'
          const int nb = ctl;
          T* b1p = b0 + o1;
          T in[2][2];
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            in[q][0] = b0[q];
            in[q][1] = b1p[q];
          }
#pragma unroll
          for (int sv = 0; sv < 2; ++sv) {
            const T z = (nb ^ sv) ? b2_1 : b2_0;
            const T w0 = wr[sv * 2], w1 = wr[sv * 2 + 1];
            T* bo = sv ? b1p : b0;
#pragma unroll
            for (int a = 0; a < 2; ++a) bo[a] = (ur[sv * 2 + a] * z) * mad_t(w1, in[1][a], w0 * in[0][a]);
          }
        } else {
          // BNNNI: out((pl,pr), (sl,sr)) = z_f[s'] u[a'][s'] sum_q w[s'][q] in(q, a')
          const int fl = ctl >> 1, fr = ctl & 1;
          T* const bp[4] = {b0, b0 + o1, b0 + o2, b0 + o3};
          if constexpr (kPacked) {
            // lanes: a' = 2 pp and 2 pp + 1
            float2 ih[4][2], il[4][2];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
              for (int pp = 0; pp < 2; ++pp) {
                const float* e0 = reinterpret_cast<const float*>(bp[2 * pp] + q);
                const float* e1 = reinterpret_cast<const float*>(bp[2 * pp + 1] + q);
                ih[q][pp] = make_float2(e0[0], e1[0]);
                il[q][pp] = make_float2(e0[1], e1[1]);
              }
#pragma unroll
            for (int sv = 0; sv < NS; ++sv) {
              const int kw = sv * 4 + z0;
#pragma unroll
              for (int pp = 0; pp < 2; ++pp) {
                float2 dh, dl;
                df2_mul(ih[0][pp], il[0][pp], wph[kw], wpl[kw], wpn[kw], dh, dl);
#pragma unroll
                for (int q = 1; q < 4; ++q)
                  df2_fma(ih[q][pp], il[q][pp], wph[kw + q], wpl[kw + q], wpn[kw + q], dh, dl, dh, dl);
                const int kz = ctl * 16 + sv * 4 + 2 * pp + z0;
                const float2 zh = *reinterpret_cast<const float2*>(zuh + kz);
                const float2 zl = *reinterpret_cast<const float2*>(zul + kz);
                // zu * d (operator* with zu first): the d operand is the one negated
                float2 oh, ol;
                df2_mul(zh, zl, dh, dl, make_float2(-dh.x, -dh.y), oh, ol);
                float* o0 = reinterpret_cast<float*>(bp[sv] + 2 * pp);
                o0[0] = oh.x;
                o0[1] = ol.x;
                o0[2] = oh.y;
                o0[3] = ol.y;
              }
            }
            continue;
          }
          T in[4][4];
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int sp = 0; sp < 4; ++sp) in[q][sp] = bp[sp][q];
          // every input is read before any output is written, so each output
          // is stored as soon as it is formed (fewer live registers)
#pragma unroll
          for (int sv = 0; sv < NS; ++sv) {
            const int sl = sv >> 1, sr = sv & 1;
            const T w0 = wr[sv * 4], w1 = wr[sv * 4 + 1], w2 = wr[sv * 4 + 2], w3 = wr[sv * 4 + 3];
            if constexpr (kZuTable) {
              const T* zu = zutab + ctl * 16 + sv * 4 + z0;
#pragma unroll
              for (int aux = 0; aux < 4; ++aux) {
                T d = in[0][aux] * w0;
                d = mad_t(in[1][aux], w1, d);
                d = mad_t(in[2][aux], w2, d);
                d = mad_t(in[3][aux], w3, d);
                bp[sv][aux] = zu[aux] * d;
              }
            } else {
              T z = ((sr ^ fr) ? b2_1 : b2_0) * ((sl ^ fl) ? b2_1 : b2_0);
              if (dir) z = z * ((sl ^ fr) ? b1_1 : b1_0);
#pragma unroll
              for (int aux = 0; aux < 4; ++aux) {
                T d = in[0][aux] * w0;
                d = mad_t(in[1][aux], w1, d);
                d = mad_t(in[2][aux], w2, d);
                d = mad_t(in[3][aux], w3, d);
                bp[sv][aux] = (ur[sv * 4 + aux] * z) * d;
              }
            }
          }
        }
      }
      __syncthreads();
    }
    if (cp.last) {
      for (int e = threadIdx.x; e < (tile >> NA); e += blockDim.x) {
        double a = acc[e];
#pragma unroll
        for (int aux = 0; aux < (1 << NA); ++aux) a += fold_part(sm[spad((e << NA) | aux)]);
        acc[e] = a;
      }
    } else if (vec_io) {
      for (int e = threadIdx.x * VEC; e < tile; e += blockDim.x * VEC) {
        const uint64_t r = rbase | tile_state((uint64_t)(e >> NA), cp.jbit0, site0);
        uint4 raw;
        T* v = reinterpret_cast<T*>(&raw);
        const T* src = sm + spad(e);
#pragma unroll
        for (int k = 0; k < VEC; ++k) v[k] = src[k];
        const uint64_t at = (((uint64_t)lb << L | r) << NA) | (uint64_t)(e & ((1 << NA) - 1));
        __stcs(reinterpret_cast<uint4*>(P + at), raw);
      }
    } else {
      for (int e = threadIdx.x; e < tile; e += blockDim.x) {
        const uint64_t r = rbase | tile_state((uint64_t)(e >> NA), cp.jbit0, site0);
        P[(((uint64_t)lb << L | r) << NA) | (uint64_t)(e & ((1 << NA) - 1))] = sm[spad(e)];
      }
    }
    __syncthreads();
  }
  if (cp.last) {
    for (int e = threadIdx.x; e < (tile >> NA); e += blockDim.x) {
      const uint64_t r = rbase | tile_state((uint64_t)e, cp.jbit0, site0);
      double v = acc[e];
      if (post) v *= post[r];
      y[r] = (IO)(v * postc);
    }
  }
}

template <class T, int ZB, class IO>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 ? 4 : (sizeof(T) == 8 ? 3 : 2))) chain_kernel(T* __restrict__ P, const IO* __restrict__ x,
                                                    const double* __restrict__ pre, const uint32_t* __restrict__ smap,
                                                    IO* __restrict__ y, const double* __restrict__ post, double postc,
                                                    int L, int bc, int dir, AuxCoefT<T> c, ChainPass cp) {
  chain_block<T, ZB, IO>(P, x, pre, smap, y, post, postc, L, bc, dir, c, cp, blockIdx.x);
}

// ------------------------------------------------------------------ reduced contract
template <class T>
__global__ void red_contract(const T* __restrict__ z, const uint32_t* __restrict__ idx, const uint16_t* __restrict__ dup,
                             const double* __restrict__ tv, double post, T* __restrict__ y, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) y[i] = (T)((double)z[idx[i]] * post * (double)dup[i] * tv[i]);
}

__device__ __forceinline__ int64_t chain_pass_blocks_dev(const ChainPass& cp) {
  return (int64_t)(cp.last ? 1 : cp.nlb) << cp.no;
}

// ------------------------------------------------------------------ batched product
// One pass over every batch member's tiles: a block takes its member from the
// per-block member map, then runs the same tile body as chain_kernel on
// kBatchTiles consecutive tiles of that member's geometry (copied to shared
// memory).  km[i] = (Krylov column the member extends, product mode).
template <class T, int ZB, class IO, int MODE>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 ? 4 : (sizeof(T) == 8 ? 3 : 2)))
    chain_batch_kernel(const ChainInst* __restrict__ inst, const int2* __restrict__ km, const int64_t* __restrict__ start,
                       const int* __restrict__ bmem, int pass, int theta) {
  __shared__ ChainPass cps;
  const int s_i = bmem[blockIdx.x];  // the member of this block
  const ChainInst& I = inst[s_i];
  const int64_t blk = (int64_t)blockIdx.x - start[s_i];
  const int np = (sizeof(T) == 4) ? I.np4 : (sizeof(T) == 8 ? I.np8 : I.np16);
  const int2 kmi = km[s_i];
  if (kmi.y != MODE || pass >= np) return;  // uniform over the block
  const int j = kmi.x;
  {
    const int* src = reinterpret_cast<const int*>((sizeof(T) == 4) ? &I.p4[pass]
                                                  : (sizeof(T) == 8 ? &I.p8[pass] : &I.p16[pass]));
    int* dst = reinterpret_cast<int*>(&cps);
    for (int q = threadIdx.x; q < (int)(sizeof(ChainPass) / sizeof(int)); q += blockDim.x) dst[q] = src[q];
  }
  __syncthreads();
  const int64_t ntiles = chain_pass_blocks_dev(cps);
  const IO* x = (MODE == kModeF32) ? reinterpret_cast<const IO*>(I.x32)
                                   : reinterpret_cast<const IO*>(I.V + (int64_t)j * I.ldv);
  const AuxCoefT<T>* c;
  if constexpr (MODE == kModeF32)
    c = reinterpret_cast<const AuxCoefT<T>*>(&I.c32);
  else if constexpr (MODE == kModeDF)
    c = reinterpret_cast<const AuxCoefT<T>*>(&I.cdf);
  else if constexpr (MODE == kModeTangent)
    c = reinterpret_cast<const AuxCoefT<T>*>(&I.ctan[theta]);
  else
    c = reinterpret_cast<const AuxCoefT<T>*>(&I.c64);
  for (int q = 0; q < kBatchTiles; ++q) {
    const int64_t tile = blk * kBatchTiles + q;
    if (tile >= ntiles) break;  // uniform over the block
    if (q) __syncthreads();     // the previous tile's last reads of shared memory
    chain_block<T, ZB, IO>(reinterpret_cast<T*>(I.P), x, I.tvec, I.smap, reinterpret_cast<IO*>(I.fold), nullptr, 1.0,
                           I.L, I.bc, I.dir, *c, cps, (uint64_t)tile);
  }
}

// w[k] = fold[idx[k]] * gs * dup[k] * tvec[k] (reduced) or fold[k] * gs * nf *
// tvec[k] (full), per member; kSweepRows rows per block
template <class IO, int MODE>
__global__ void __launch_bounds__(256) contract_batch_kernel(const ChainInst* __restrict__ inst,
                                                             const int2* __restrict__ km,
                                                             const int64_t* __restrict__ rstart,
                                                             const int* __restrict__ rmem) {
  const int s_i = rmem[blockIdx.x];  // the member of this row block
  const ChainInst& I = inst[s_i];
  const int2 kmi = km[s_i];
  if (kmi.y != MODE) return;
  const int64_t r0 = ((int64_t)blockIdx.x - rstart[s_i]) * kSweepRows;
  const int64_t r1 = min(r0 + (int64_t)kSweepRows, I.n);
  const double gs = (MODE == kModeF32) ? I.gs32 : (MODE == kModeF64 ? I.gs64 : I.gsdf);  // tangent steps as DF
  const IO* z = reinterpret_cast<const IO*>(I.fold);
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const double f = I.idx ? (double)z[I.idx[r]] * (double)I.dup[r] : (double)z[r] * I.nf;
    I.w[r] = f * gs * I.tvec[r];
  }
}

}  // namespace

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

// Batch members keep no product buffers of their own: the batch owns them.
static thread_local bool g_batch_member = false;
BatchMemberScope::BatchMemberScope() : prev(g_batch_member) { g_batch_member = true; }
BatchMemberScope::~BatchMemberScope() { g_batch_member = prev; }

void build_aux(Op& op) {
  const int L = op.L;
  const int64_t N = 1ll << L;
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  if (zb && L % 2) fail(TM_ERR_ARG, "diagonal BNNNI operators need an even width");
  if (g_batch_member) return;
  // one in-place pass buffer of nlb * 2^NA * 2^L elements (FP64 size)
  const int64_t per = zb ? 16 * N : 4 * N;
  op.ws_a.alloc((size_t)per * 8);
  if (op.kind == K_XDM || op.kind == K_ZBM) op.xp.alloc((size_t)N * 8);  // full-space result before contraction
}

// ------------------------------------------------------------------ autotuner inputs
namespace {
__global__ void tune_fill_kernel(double* v, int64_t n, uint64_t seed) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) {
    uint64_t z = seed + 0x9e3779b97f4a7c15ull * (uint64_t)(i + 1);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    v[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
}
__global__ void tune_f32_kernel(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) y[i] = (float)x[i];
}
}  // namespace

void fill_uniform_dev(double* v, int64_t n, uint64_t seed, cudaStream_t s) {
  tune_fill_kernel<<<grid_for(n), 256, 0, s>>>(v, n, seed);
  TM_CKK("tune_fill");
}
void to_f32_dev(const double* x, float* y, int64_t n, cudaStream_t s) {
  tune_f32_kernel<<<grid_for(n), 256, 0, s>>>(x, y, n);
  TM_CKK("tune_f32");
}

// ------------------------------------------------------------------ pass plans and tuning
// Tile bits and threads per block of the chain passes, per (element size,
// carried bits, width).  Defaults: 2^13-element tiles for 4-byte elements and
// 2^12 for 8-byte ones (32 KB either way), 256 threads, except where the
// built-in table of measured choices has an entry; tm_chain_autotune and
// tm_chain_set_tuning override entries at run time.
namespace {
struct ChainTune {
  int tile_bits = 0, threads = 0;
};
std::mutex g_tune_mu;
ChainTune g_tune[2][2][33];  // [elem 4/8][zb][L]
}  // namespace

// Choices of the autotuner (python -m latttmat_gb300.autotune) measured on a
// GB300 for the diagonal BNNNI widths of the 256-point parameter sweep:
// {L, tile bits, threads} for 4-byte and for 8-byte elements.
struct TunedEntry {
  int L, tb4, th4, tb8, th8;
};
constexpr TunedEntry kTunedBNNNI[] = {
    {16, 11, 128, 11, 128}, {18, 13, 256, 13, 256}, {20, 11, 128, 11, 128},
    {22, 13, 128, 13, 128}, {24, 12, 128, 12, 128},
};

void chain_tuning(int L, size_t elem, bool zb, int& tile_bits, int& threads) {
  if (elem >= 16) {  // tangent pairs (adjoint): 32 KB tiles, fewer threads
    tile_bits = 11;
    threads = 128;
    return;
  }
  tile_bits = (elem == 8) ? 12 : 13;
  threads = 256;
  if (L < 0 || L > 32) return;
  if (zb)
    for (const TunedEntry& t : kTunedBNNNI)
      if (t.L == L) {
        tile_bits = (elem == 8) ? t.tb8 : t.tb4;
        threads = (elem == 8) ? t.th8 : t.th4;
      }
  std::lock_guard<std::mutex> lock(g_tune_mu);
  const ChainTune& t = g_tune[elem == 8][zb ? 1 : 0][L];
  if (t.tile_bits) tile_bits = t.tile_bits;
  if (t.threads) threads = t.threads;
}

void chain_set_tuning(int L, size_t elem, bool zb, int tile_bits, int threads) {
  if (L < 0 || L > 32) fail(TM_ERR_ARG, "width out of range");
  if (tile_bits && (tile_bits < 10 || tile_bits > (elem == 8 ? 13 : 14))) fail(TM_ERR_ARG, "tile bits out of range");
  if (threads && threads != 64 && threads != 128 && threads != 256) fail(TM_ERR_ARG, "threads must be 64, 128 or 256");
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune[elem == 8][zb ? 1 : 0][L] = ChainTune{tile_bits, threads};
}

// The passes of one product: the first holds up to cap0 steps (its sites
// start at 0), the others up to cap1 (they carry a few contiguous low sites
// for coalescing); the steps are spread evenly over the passes needed.
std::vector<ChainPass> chain_plan(int L, bool zb, int nlb, int tile_bits) {
  const int NA = zb ? 2 : 1, KS = zb ? 2 : 1;
  const int nsteps = zb ? L / 2 : L;
  const int cbn = zb ? 2 : 3;
  const int cap0 = std::max(1, (tile_bits - NA) / KS), cap1 = std::max(1, (tile_bits - NA - cbn) / KS);
  const int npass = (nsteps <= cap0) ? 1 : 1 + (nsteps - cap0 + cap1 - 1) / cap1;
  std::vector<ChainPass> out;
  int t0 = 0, pass = 0;
  while (t0 < nsteps) {
    // tile state bits: contiguous low sites for coalescing (none when the
    // steps start at site 0), then the sites of this pass's steps
    const int cb = (t0 == 0) ? 0 : std::min(KS * t0, cbn);
    const int left = npass - pass;
    const int even = (nsteps - t0 + left - 1) / left;
    const int T_ = std::max(1, std::min(nsteps - t0, std::min(even, t0 == 0 ? cap0 : cap1)));
    ++pass;
    ChainPass cp{};
    std::vector<int> sp;
    for (int k = 0; k < cb; ++k) sp.push_back(k);
    for (int k = 0; k < KS * T_; ++k) sp.push_back(KS * t0 + k);
    cp.nst = (int)sp.size();
    for (int k = 0; k < cp.nst; ++k) cp.spos[k] = sp[k];
    uint64_t used = 0;
    for (int k : sp) used |= 1ull << k;
    cp.no = 0;
    for (int b = 0; b < L; ++b)
      if (!((used >> b) & 1ull)) cp.opos[cp.no++] = b;
    cp.t0 = t0;
    cp.T = T_;
    cp.jbit0 = cb;
    cp.first = (t0 == 0);
    cp.last = (t0 + T_ >= nsteps);
    cp.nlb = nlb;
    out.push_back(cp);
    t0 += T_;
  }
  return out;
}

// blocks of one pass and its dynamic shared memory
int64_t chain_pass_blocks(const ChainPass& cp) { return (int64_t)(cp.last ? 1 : cp.nlb) << cp.no; }
size_t chain_pass_smem(const ChainPass& cp, bool zb, size_t elem) {
  const int NA = zb ? 2 : 1;
  const int tile = 1 << (NA + cp.nst);
  return chain_acc_offset(tile, elem) + (cp.last ? (size_t)(tile >> NA) * 8 : 0);
}

// y = T x (or T^T x for transposed views); scaled: FP32 result divided by the
// returned factor.
// T: arithmetic and pass-buffer type (float, double, or dfloat: FP64-accurate
// products on the FP32 pipes); IO: element type of x and y.
template <class T>
T coef_with_derivative(double v, double d) {
  if constexpr (std::is_same<T, tangent>::value)
    return tangent(v, d);
  else
    return (T)v;
}

template <class T, class IO = T>
double matvec_aux_dir(const Op& op, const IO* x, IO* y, bool scaled, int dir, cudaStream_t s,
                      const AuxCoef* dcoef = nullptr, void* pass_buf = nullptr) {
  const int L = op.L;
  const bool reduced = (op.kind == K_XDM || op.kind == K_ZBM);
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  AuxCoef c64 = coef_of(op);
  const double gb = step_bound(op, c64, dir);
  // FP32 and double-float steps (tangent pairs included) are normalised
  // (FP32 exponent range)
  const bool norm = (sizeof(T) == 4) || std::is_same<T, dfloat>::value || std::is_same<T, tangent>::value;
  AuxCoefT<T> c;
  for (int k = 0; k < 2; ++k) {
    c.b1[k] = coef_with_derivative<T>(c64.b1[k], dcoef ? dcoef->b1[k] : 0.0);
    c.b2[k] = coef_with_derivative<T>(c64.b2[k], dcoef ? dcoef->b2[k] : 0.0);
    c.b3[k] = coef_with_derivative<T>(c64.b3[k], dcoef ? dcoef->b3[k] : 0.0);
  }
  c.g = norm ? (T)(1.0 / gb) : (T)1;
  const int nsteps = zb ? L / 2 : L;
  const double gscale = norm ? std::pow(gb, (double)nsteps) : 1.0;
  const double sf = scaled ? 1.0 : gscale;
  const int bc = zb ? 0 : op.boundary;
  const int nlb = zb ? 4 : (bc == 0 ? 2 : 1);
  int tile_bits = 0, threads = 0;
  chain_tuning(L, sizeof(T), zb, tile_bits, threads);
  T* P = pass_buf ? static_cast<T*>(pass_buf) : op.ws_a.as<T>();
  const uint32_t* smap = reduced ? op.smap.as<uint32_t>() : nullptr;
  IO* fold_out = reduced ? op.xp.as<IO>() : y;
  const double postc = zb ? sf : (reduced ? sf : op.normfactor * sf);
  const double* post = reduced ? nullptr : op.tvec.as<double>();
  for (const ChainPass& cp : chain_plan(L, zb, nlb, tile_bits)) {
    const int64_t nblocks = chain_pass_blocks(cp);
    const size_t shm = chain_pass_smem(cp, zb, sizeof(T));
    if (zb) {
      raise_smem_limit((const void*)chain_kernel<T, 1, IO>, shm);
      chain_kernel<T, 1, IO><<<(unsigned)nblocks, threads, shm, s>>>(P, x, op.tvec.as<double>(), smap, fold_out, post,
                                                                postc, L, bc, dir, c, cp);
    } else {
      raise_smem_limit((const void*)chain_kernel<T, 0, IO>, shm);
      chain_kernel<T, 0, IO><<<(unsigned)nblocks, threads, shm, s>>>(P, x, op.tvec.as<double>(), smap, fold_out, post,
                                                                postc, L, bc, dir, c, cp);
    }
    TM_CKK("aux_chain");
  }
  if (reduced) {
    red_contract<IO><<<grid_for(op.n), 256, 0, s>>>(fold_out, op.idx.as<uint32_t>(), op.dup.as<uint16_t>(),
                                                   op.tvec.as<double>(), 1.0, y, op.n);
    TM_CKK("red_contract");
  }
  return scaled ? gscale : 1.0;
}

// ------------------------------------------------------------------ batch members
void chain_inst_fill(const Op& op, int dir, ChainInst& rec, int tb4, int tb8) {
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  const bool reduced = (op.kind == K_XDM || op.kind == K_ZBM);
  const int L = op.L;
  rec.L = L;
  rec.zb = zb;
  rec.bc = zb ? 0 : op.boundary;
  rec.dir = dir;
  rec.nlb = zb ? 4 : (rec.bc == 0 ? 2 : 1);
  rec.n = op.n;
  // full DNNI applies the normfactor at the output; the BNNNI Tvec holds it
  rec.nf = (reduced || zb) ? 1.0 : op.normfactor;
  const AuxCoef c = coef_of(op);
  const double gb = step_bound(op, c, dir);
  const int nsteps = zb ? L / 2 : L;
  for (int q = 0; q < 2; ++q) {
    rec.c32.b1[q] = (float)c.b1[q];
    rec.c32.b2[q] = (float)c.b2[q];
    rec.c32.b3[q] = (float)c.b3[q];
    rec.cdf.b1[q] = dfloat(c.b1[q]);
    rec.cdf.b2[q] = dfloat(c.b2[q]);
    rec.cdf.b3[q] = dfloat(c.b3[q]);
    rec.c64.b1[q] = c.b1[q];
    rec.c64.b2[q] = c.b2[q];
    rec.c64.b3[q] = c.b3[q];
  }
  rec.c32.g = (float)(1.0 / gb);
  rec.cdf.g = dfloat(1.0 / gb);
  rec.c64.g = 1.0;
  rec.gs32 = rec.gsdf = std::pow(gb, (double)nsteps);
  rec.gs64 = 1.0;
  int th = 0;
  if (tb4 <= 0) chain_tuning(L, 4, zb, tb4, th);
  if (tb8 <= 0) chain_tuning(L, 8, zb, tb8, th);
  int tb16 = 0;
  chain_tuning(L, 16, zb, tb16, th);
  const std::vector<ChainPass> p16 = chain_plan(L, zb, rec.nlb, tb16);
  if ((int)p16.size() > kChainMaxPass) fail(TM_ERR_LIMIT, "too many chain passes");
  rec.np16 = (int)p16.size();
  for (int q = 0; q < rec.np16; ++q) rec.p16[q] = p16[q];
  for (int t = 0; t < 3; ++t) {
    const AuxCoef db = aux_coef_derivative(op.mp.betaJ, op.mp.kappa, op.mp.kappa2, t);
    for (int q = 0; q < 2; ++q) {
      rec.ctan[t].b1[q] = tangent(c.b1[q], db.b1[q]);
      rec.ctan[t].b2[q] = tangent(c.b2[q], db.b2[q]);
      rec.ctan[t].b3[q] = tangent(c.b3[q], db.b3[q]);
    }
    rec.ctan[t].g = tangent(1.0 / gb);  // a constant: no derivative
  }
  rec.kind = op.kind;
  rec.bj = op.mp.betaJ;
  rec.kap = op.mp.kappa;
  rec.kap2 = op.mp.kappa2;
  rec.h = op.mp.h;
  const std::vector<ChainPass> p4 = chain_plan(L, zb, rec.nlb, tb4), p8 = chain_plan(L, zb, rec.nlb, tb8);
  if ((int)p4.size() > kChainMaxPass || (int)p8.size() > kChainMaxPass) fail(TM_ERR_LIMIT, "too many chain passes");
  rec.np4 = (int)p4.size();
  rec.np8 = (int)p8.size();
  for (int q = 0; q < rec.np4; ++q) rec.p4[q] = p4[q];
  for (int q = 0; q < rec.np8; ++q) rec.p8[q] = p8[q];
  rec.smap = reduced ? op.smap.as<uint32_t>() : nullptr;
  rec.tvec = op.tvec.as<double>();
  rec.idx = reduced ? op.idx.as<uint32_t>() : nullptr;
  rec.dup = reduced ? op.dup.as<uint16_t>() : nullptr;
}

namespace {
template <class T, int ZB, class IO, int MODE>
void launch_batch_pass(const ChainInst* inst, const int2* km, const int64_t* start, const int* bmem, int pass,
                       int64_t nblk, int threads, size_t smem, cudaStream_t s, int theta) {
  raise_smem_limit((const void*)chain_batch_kernel<T, ZB, IO, MODE>, smem);
  chain_batch_kernel<T, ZB, IO, MODE><<<(unsigned)nblk, threads, smem, s>>>(inst, km, start, bmem, pass, theta);
  TM_CKK("chain_batch");
}

template <int ZB, int MODE>
int batch_product_mode(const ChainBatch& B, const int2* km, const ChainBatch::Plan& P, cudaStream_t s, int theta) {
  int launches = 0;
  for (int p = 0; p < P.np; ++p) {
    if (P.nblk[p] == 0) continue;
    const int64_t* st = P.start + (size_t)p * (B.count + 1);
    const int* bm = P.bmem + P.boff[p];
    if constexpr (MODE == kModeF32)
      launch_batch_pass<float, ZB, float, MODE>(B.inst, km, st, bm, p, P.nblk[p], P.threads, P.smem, s, theta);
    else if constexpr (MODE == kModeDF)
      launch_batch_pass<dfloat, ZB, double, MODE>(B.inst, km, st, bm, p, P.nblk[p], P.threads, P.smem, s, theta);
    else if constexpr (MODE == kModeTangent)
      launch_batch_pass<tangent, ZB, double, MODE>(B.inst, km, st, bm, p, P.nblk[p], P.threads, P.smem, s, theta);
    else
      launch_batch_pass<double, ZB, double, MODE>(B.inst, km, st, bm, p, P.nblk[p], P.threads, P.smem, s, theta);
    ++launches;
  }
  if constexpr (MODE == kModeF32)
    contract_batch_kernel<float, MODE><<<(unsigned)B.nrblk, 256, 0, s>>>(B.inst, km, B.rstart, B.rmem);
  else
    contract_batch_kernel<double, MODE><<<(unsigned)B.nrblk, 256, 0, s>>>(B.inst, km, B.rstart, B.rmem);
  TM_CKK("contract_batch");
  return launches + 1;
}
}  // namespace

int chain_batch_product(const ChainBatch& B, const int2* km, int mode, cudaStream_t s, int theta) {
  if (B.zb) {
    if (mode == kModeF32) return batch_product_mode<1, kModeF32>(B, km, B.p4, s, theta);
    if (mode == kModeDF) return batch_product_mode<1, kModeDF>(B, km, B.p8, s, theta);
    if (mode == kModeTangent) return batch_product_mode<1, kModeTangent>(B, km, B.p16, s, theta);
    return batch_product_mode<1, kModeF64>(B, km, B.p8, s, theta);
  }
  if (mode == kModeF32) return batch_product_mode<0, kModeF32>(B, km, B.p4, s, theta);
  if (mode == kModeDF) return batch_product_mode<0, kModeDF>(B, km, B.p8, s, theta);
  if (mode == kModeTangent) return batch_product_mode<0, kModeTangent>(B, km, B.p16, s, theta);
  return batch_product_mode<0, kModeF64>(B, km, B.p8, s, theta);
}

// ------------------------------------------------------------------ autotuner
// Time the operator's product (FP32, or the 8-byte double-float engine) over
// the tile sizes and block sizes the chain kernels take, CUDA events on the
// operator's stream, and keep the fastest for this (element size, carried
// bits, width) in the tuning table.  Results do not depend on the choice
// (same arithmetic per element, in the same order).
void chain_autotune(const Op& op0, tm_dtype dt, int& best_tb, int& best_th, double& best_ms) {
  const Op& op = op0.parent ? *op0.parent : op0;
  if (op.kind != K_ZBT && op.kind != K_ZBM && op.kind != K_XDT && op.kind != K_XDM)
    fail(TM_ERR_UNSUPPORTED, "the autotuner covers the aux-bit operators (models B and D)");
  if (!op.ws_a.p) fail(TM_ERR_ARG, "operator has no product buffers (a sweep member)");
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  const size_t elem = (dt == TM_F32) ? 4 : 8;
  cudaStream_t s = op.stream;
  AllocStream guard(s);
  DBuf x, y, x32, y32;
  x.alloc((size_t)op.n * 8);
  y.alloc((size_t)op.n * 8);
  x32.alloc((size_t)op.n * 4);
  y32.alloc((size_t)op.n * 4);
  fill_uniform_dev(x.as<double>(), op.n, 7, s);
  to_f32_dev(x.as<double>(), x32.as<float>(), op.n, s);
  int tb0 = 0, th0 = 0;
  chain_tuning(op.L, elem, zb, tb0, th0);
  const int tbs[4] = {11, 12, 13, 14};
  const int ths[2] = {128, 256};
  cudaEvent_t e0, e1;
  TM_CK(cudaEventCreate(&e0));
  TM_CK(cudaEventCreate(&e1));
  best_ms = 1e30;
  best_tb = tb0;
  best_th = th0;
  try {
    for (int tb : tbs) {
      if (tb > (elem == 8 ? 13 : 14)) continue;
      for (int th : ths) {
        chain_set_tuning(op.L, elem, zb, tb, th);
        auto run = [&]() {
          if (elem == 4)
            matvec_aux_dir<float>(op, x32.as<float>(), y32.as<float>(), true, 0, s);
          else
            matvec_aux_dir<dfloat, double>(op, x.as<double>(), y.as<double>(), false, 0, s);
        };
        run();
        TM_CK(cudaEventRecord(e0, s));
        for (int r = 0; r < 3; ++r) run();
        TM_CK(cudaEventRecord(e1, s));
        TM_CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        TM_CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms / 3.0 < best_ms) {
          best_ms = ms / 3.0;
          best_tb = tb;
          best_th = th;
        }
      }
    }
  } catch (...) {
    chain_set_tuning(op.L, elem, zb, tb0 == ((elem == 8) ? 12 : 13) ? 0 : tb0, th0 == 256 ? 0 : th0);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  chain_set_tuning(op.L, elem, zb, best_tb, best_th);
}

template <class T>
double matvec_aux(const Op& op, const T* x, T* y, bool scaled, cudaStream_t s) {
  const Op& base = op.parent ? *op.parent : op;
  return matvec_aux_dir<T>(base, x, y, scaled, op.transposed ? 1 : 0, s);
}

template double matvec_aux<float>(const Op&, const float*, float*, bool, cudaStream_t);
template double matvec_aux<double>(const Op&, const double*, double*, bool, cudaStream_t);

// Tangent product of the adjoint: y = D_out (dC/dtheta) D_in x, the chain
// steps differentiated with respect to one parameter whose effect on the step
// factors b1, b2, b3 is `db` (the Boltzmann weights Tvec held fixed), FP64.
void matvec_aux_tangent(const Op& op, const double* x, double* y, const AuxCoef& db, int dir, cudaStream_t s) {
  // the pass buffer at 16 bytes per element (the operator's holds 8)
  const bool zb = (op.kind == K_ZBT || op.kind == K_ZBM);
  const int64_t per = (zb ? 16ll : 4ll) << op.L;
  AllocStream guard(s);
  DBuf P;
  P.alloc((size_t)per * sizeof(tangent));
  matvec_aux_dir<tangent, double>(op, x, y, false, dir, s, &db, P.p);
}

// FP64-accurate product in double-float arithmetic (the solver's refinement
// products for the aux-bit operators)
void matvec_aux_df(const Op& op, const double* x, double* y, cudaStream_t s) {
  const Op& base = op.parent ? *op.parent : op;
  matvec_aux_dir<dfloat, double>(base, x, y, false, op.transposed ? 1 : 0, s);
}

}  // namespace ltm
