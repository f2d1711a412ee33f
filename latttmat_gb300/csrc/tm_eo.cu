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
// Work and HBM traffic are about 2^(L+1)/|H| elements instead of 2^L * L.  The
// reduced vector is kept in "pi order" (pass-2 tile order) so the output
// stores are contiguous; pi maps back to the reference's idxlist order.
//
// A tile of 2^m elements is split over a cluster of 2^c CTAs (FP32 m=16: two
// CTAs x 2^15 elements in 135 KB of shared memory).  The butterflies on the
// top c tile bits combine the CTAs' shared memory through DSMEM.  Inside a CTA
// each thread owns 2^KB elements in registers: KB butterfly levels per round,
// with a padded shared-memory transpose between rounds.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
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
  int ng;               // H elements
  int64_t n_orep;       // pass-1 tiles (row length of the transposed w1)
  float a32, b32;       // normalised butterfly coefficients
  double a64, b64;
};

__device__ __forceinline__ int spad(int e) { return e + (e >> 5); }

template <class T>
__device__ __forceinline__ T ca(const EOArgs& A);
template <>
__device__ __forceinline__ float ca<float>(const EOArgs& A) { return A.a32; }
template <>
__device__ __forceinline__ double ca<double>(const EOArgs& A) { return A.a64; }
template <class T>
__device__ __forceinline__ T cb(const EOArgs& A);
template <>
__device__ __forceinline__ float cb<float>(const EOArgs& A) { return A.b32; }
template <>
__device__ __forceinline__ double cb<double>(const EOArgs& A) { return A.b64; }
template <>
__device__ __forceinline__ dfloat ca<dfloat>(const EOArgs& A) { return dfloat(A.a64); }
template <>
__device__ __forceinline__ dfloat cb<dfloat>(const EOArgs& A) { return dfloat(A.b64); }

// in-register butterflies over the 2^NB elements held by one thread
template <class T, int NB>
__device__ __forceinline__ void reg_bfly(T (&v)[1 << NB], int nb, T a, T b) {
#pragma unroll
  for (int lv = 0; lv < NB; ++lv) {
    if (lv < nb) {
#pragma unroll
      for (int i = 0; i < (1 << NB); ++i) {
        if (!(i & (1 << lv))) {
          T x0 = v[i], x1 = v[i | (1 << lv)];
          v[i] = a * x0 + b * x1;
          v[i | (1 << lv)] = b * x0 + a * x1;
        }
      }
    }
  }
}

// butterflies on local bits [0, p) of the shared-memory tile, KB bits per round
template <class T, int KB>
__device__ __forceinline__ void smem_rounds(T* sm, const EOArgs& A) {
  const T a = ca<T>(A), b = cb<T>(A);
  const int n = A.n, p = A.p;
  for (int g0 = 0; g0 < p; g0 += KB) {
    const int gs = min(KB, p - g0);
    const int nfree = 1 << (n - gs);
    for (int f = threadIdx.x; f < nfree; f += blockDim.x) {
      int j0 = (f & ((1 << g0) - 1)) | ((f >> g0) << (g0 + gs));
      T v[1 << KB];
#pragma unroll
      for (int i = 0; i < (1 << KB); ++i)
        if (i < (1 << gs)) v[i] = sm[spad(j0 | (i << g0))];
      reg_bfly<T, KB>(v, gs, a, b);
#pragma unroll
      for (int i = 0; i < (1 << KB); ++i)
        if (i < (1 << gs)) sm[spad(j0 | (i << g0))] = v[i];
    }
    __syncthreads();
  }
}

// combine the cluster's 2^c partial tiles for local element j (top c bits)
template <class T>
__device__ __forceinline__ T cluster_combine(cg::cluster_group& cl, T* sm, int rank, int j,
                                             const EOArgs& A) {
  const T a = ca<T>(A), b = cb<T>(A);
  T acc = 0;
  const int nc = 1 << A.c;
  for (int r = 0; r < nc; ++r) {
    T coef = 1;
    for (int bit = 0; bit < A.c; ++bit) coef *= (((r ^ rank) >> bit) & 1) ? b : a;
    const T* src = (r == rank) ? sm : cl.map_shared_rank(sm, r);
    acc += coef * src[spad(j)];
  }
  return acc;
}

// pass 1: w1[t][e] = (Th_E v)[(e, o_rep(t))],  v[(e,o_rep)] = u[map1[t][e]]
// (InT: element type of u; T: arithmetic / storage type of the tile and w1)
template <class T, int KB, class InT>
__global__ void __launch_bounds__(1024, 1) eo_pass1(EOArgs A, const InT* __restrict__ u,
                                                    const uint32_t* __restrict__ map1,
                                                    const uint32_t* __restrict__ colmap,
                                                    T* __restrict__ w1) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (A.c > 0) ? (int)cl.block_rank() : 0;
  const int64_t tile = blockIdx.x >> A.c;
  const int n = A.n, p = A.p;
  const int kb = n - p;
  const uint32_t* mrow = map1 + (tile << A.m) + ((int64_t)rank << n);
  // round A: gather straight into registers; register bits are local bits [p, n)
  {
    T v[1 << KB];
#pragma unroll
    for (int i = 0; i < (1 << KB); ++i) {
      if (i < (1 << kb)) {
        int j = threadIdx.x + (i << p);
        v[i] = T(u[__ldg(mrow + j)]);
      }
    }
    reg_bfly<T, KB>(v, kb, ca<T>(A), cb<T>(A));
#pragma unroll
    for (int i = 0; i < (1 << KB); ++i)
      if (i < (1 << kb)) sm[spad(threadIdx.x + (i << p))] = v[i];
  }
  __syncthreads();
  smem_rounds<T, KB>(sm, A);
  // Output.  w1 is stored transposed: e goes to row colmap[e], column
  // `tile`.  The column writes of concurrently running tiles fill adjacent
  // words of each row, which L2 merges into full sectors.
  T* wcol = w1 + tile;
  if (A.c > 0) cl.sync();
  for (int j = threadIdx.x; j < (1 << n); j += blockDim.x) {
    T val = (A.c == 0) ? sm[spad(j)] : cluster_combine<T>(cl, sm, rank, j, A);
    uint32_t row = __ldg(colmap + (((uint32_t)rank << n) | (uint32_t)j));
    wcol[(int64_t)row * A.n_orep] = val;
  }
  if (A.c > 0) cl.sync();
}

// pass 2: z[(e_rep, o)] = (Th_O w)[(e_rep, o)]; emit designated outputs
// (OutT: element type of y)
template <class T, int KB, bool F64SCALE, class OutT>
__global__ void __launch_bounds__(1024, 1) eo_pass2(EOArgs A, const T* __restrict__ w1,
                                                    const uint32_t* __restrict__ t2,
                                                    const uint32_t* __restrict__ erep,
                                                    const uint32_t* __restrict__ colmap,
                                                    const uint32_t* __restrict__ out_off,
                                                    const uint16_t* __restrict__ out_o,
                                                    const double* __restrict__ sout64,
                                                    const float* __restrict__ sout32, double post,
                                                    OutT* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  __shared__ uint32_t he[128];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (A.c > 0) ? (int)cl.block_rank() : 0;
  const int64_t tile = blockIdx.x >> A.c;
  const int n = A.n, p = A.p;
  const int kb = n - p;
  const uint32_t e_rep = erep[tile];
  // w1 rows of this tile's H-class (one contiguous block of rows)
  for (int g = threadIdx.x; g < A.ng; g += blockDim.x) he[g] = __ldg(colmap + act_e(g, e_rep, A.m));
  __syncthreads();
  {
    T v[1 << KB];
#pragma unroll
    for (int i = 0; i < (1 << KB); ++i) {
      if (i < (1 << kb)) {
        int j = threadIdx.x + (i << p);
        uint32_t o = ((uint32_t)rank << n) | (uint32_t)j;
        uint32_t code = __ldg(t2 + o);
        v[i] = w1[(int64_t)he[code & 255u] * A.n_orep + (code >> 8)];
      }
    }
    reg_bfly<T, KB>(v, kb, ca<T>(A), cb<T>(A));
#pragma unroll
    for (int i = 0; i < (1 << KB); ++i)
      if (i < (1 << kb)) sm[spad(threadIdx.x + (i << p))] = v[i];
  }
  __syncthreads();
  smem_rounds<T, KB>(sm, A);
  const int part = (int)(tile << A.c) + rank;
  const uint32_t k0 = out_off[part], k1 = out_off[part + 1];
  const int lmask = (1 << n) - 1;
  if (A.c > 0) cl.sync();
  for (uint32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    int j = out_o[k] & lmask;
    T val = (A.c == 0) ? sm[spad(j)] : cluster_combine<T>(cl, sm, rank, j, A);
    if (F64SCALE)
      y[k] = (OutT)((double)val * sout64[k] * post);
    else
      y[k] = (OutT)(val * T(sout32[k]));
  }
  if (A.c > 0) cl.sync();
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

// designated output key per representative: min over orbit images whose even
// part is an H-representative of (tile << m | o)
__global__ void eo_key_kernel(PlanDev P, const uint32_t* __restrict__ idx, int64_t R,
                              const uint32_t* __restrict__ e_tile, uint32_t* __restrict__ key,
                              uint32_t* __restrict__ dbits) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < R; i += st) {
    uint64_t s = idx[i];
    uint32_t best = 0xffffffffu;
    for_each_image(P.g, s, [&](uint64_t im) {
      uint32_t e = gather16((uint32_t)im), o = gather16((uint32_t)(im >> 1));
      uint32_t t = e_tile[e];
      if (t != 0xffffffffu) {
        uint32_t k = (t << P.m) | o;
        if (k < best) best = k;
      }
      return true;
    });
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
                               const uint32_t* __restrict__ dpre, int m, uint32_t* __restrict__ pi,
                               uint32_t* __restrict__ pinv, uint16_t* __restrict__ out_o) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < R; i += st) {
    uint32_t k = key[i];
    uint32_t w = k >> 5;
    uint32_t pos = dpre[w] + __popc(dbits[w] & ((1u << (k & 31)) - 1u));
    pi[pos] = (uint32_t)i;
    pinv[i] = pos;
    out_o[pos] = (uint16_t)(k & ((1u << m) - 1u));
  }
}

__global__ void eo_map1_kernel(PlanDev P, const uint32_t* __restrict__ olist, int n_orep,
                               const uint32_t* __restrict__ pinv, uint32_t* __restrict__ map1) {
  const int64_t total = (int64_t)n_orep << P.m;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < total; i += st) {
    uint32_t t = (uint32_t)(i >> P.m), e = (uint32_t)(i & ((1 << P.m) - 1));
    uint32_t s = join_eo(e, olist[t]);
    uint64_t c = canon(P.g, s);
    map1[i] = pinv[rank_of(P, c)];
  }
}

__global__ void eo_scale_kernel(const uint32_t* __restrict__ pi, const double* __restrict__ tv,
                                const uint16_t* __restrict__ dup, int64_t R, double* sin64, double* sout64,
                                float* sin32, float* sout32) {
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

// Decide cluster bits so a CTA's tile part fits in shared memory.
static int cluster_bits_for(int m, size_t elem) {
  int c = 0;
  while (((size_t)(1 << (m - c)) * elem * 33 / 32) > 200 * 1024) ++c;
  return c;
}

void build_eo_plan(Op& op) {
  EOPlan& P = op.eo;
  const int L = op.L, m = L / 2;
  P.m = m;
  const int flip = op.grp.flip;
  P.ng = 2 * m * (flip ? 2 : 1);
  const uint32_t M = 1u << m;
  // host tables over m-bit patterns
  std::vector<uint32_t> orep(M), erep_of(M);
  std::vector<int> og(M);
  for (uint32_t o = 0; o < M; ++o) {
    uint32_t best = o;
    int bg = 0;
    for (int g = 0; g < P.ng; ++g) {
      uint32_t im = act_o(g, o, m);
      if (im < best) {
        best = im;
        bg = g;
      }
    }
    orep[o] = best;
    og[o] = bg;
  }
  std::vector<uint32_t> olist, elist;
  std::vector<uint32_t> otile(M, 0xffffffffu), etile(M, 0xffffffffu);
  for (uint32_t o = 0; o < M; ++o)
    if (orep[o] == o) {
      otile[o] = (uint32_t)olist.size();
      olist.push_back(o);
    }
  for (uint32_t e = 0; e < M; ++e) {
    uint32_t best = e;
    for (int g = 0; g < P.ng; ++g) best = std::min(best, act_e(g, e, m));
    if (best == e) {
      etile[e] = (uint32_t)elist.size();
      elist.push_back(e);
    }
  }
  std::vector<uint32_t> t2(M);
  for (uint32_t o = 0; o < M; ++o) t2[o] = (otile[orep[o]] << 8) | (uint32_t)og[o];
  // w1 row of each even pattern e.  Rows in e order: pass 1's column writes
  // then walk the rows in order (consecutive threads, consecutive rows), and
  // pass 2 reads the |class| rows of its tile's H-class.  (Grouping each
  // H-class into contiguous rows was measured slower: 2.48 against 1.99 ms for
  // pass 1 at L=32, pass 2 unchanged.)
  std::vector<uint32_t> colmap(M);
  for (uint32_t e = 0; e < M; ++e) colmap[e] = e;
  P.n_orep = (int)olist.size();
  P.n_erep = (int)elist.size();
  P.c32 = cluster_bits_for(m, 4);
  P.c64 = cluster_bits_for(m, 8);

  cudaStream_t s = op.stream;
  DBuf d_olist, d_etile;
  d_olist.alloc(olist.size() * 4);
  d_etile.alloc(M * 4);
  P.t2.alloc(M * 4);
  P.erep.alloc(elist.size() * 4);
  P.colmap.alloc(M * 4);
  TM_CK(cudaMemcpyAsync(P.colmap.p, colmap.data(), M * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(d_olist.p, olist.data(), olist.size() * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(d_etile.p, etile.data(), M * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(P.t2.p, t2.data(), M * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaMemcpyAsync(P.erep.p, elist.data(), elist.size() * 4, cudaMemcpyHostToDevice, s));

  PlanDev pd;
  pd.g = to_dev(op.grp);
  pd.m = m;
  pd.bits = op.ws_a.as<uint32_t>();
  pd.prefix = op.ws_b.as<uint32_t>();
  const int64_t R = op.n;
  // designated outputs -> pi
  const int64_t nkeybits = (int64_t)P.n_erep << m;
  const int64_t nwords = (nkeybits + 31) / 32;
  DBuf key, dbits, dpre;
  key.alloc(R * 4);
  dbits.alloc(nwords * 4);
  dpre.alloc(nwords * 4);
  TM_CK(cudaMemsetAsync(dbits.p, 0, nwords * 4, s));
  eo_key_kernel<<<grid_for(R), 256, 0, s>>>(pd, op.idx.as<uint32_t>(), R, d_etile.as<uint32_t>(),
                                            key.as<uint32_t>(), dbits.as<uint32_t>());
  TM_CKK("eo_key");
  popc_kernel<<<grid_for(nwords), 256, 0, s>>>(dbits.as<uint32_t>(), dpre.as<uint32_t>(), nwords);
  TM_CKK("popc");
  exclusive_scan_u32(dpre.as<uint32_t>(), dpre.as<uint32_t>(), nwords, s);
  op.pi.alloc(R * 4);
  op.pinv.alloc(R * 4);
  P.out_o.alloc(R * 2);
  eo_perm_kernel<<<grid_for(R), 256, 0, s>>>(key.as<uint32_t>(), R, dbits.as<uint32_t>(),
                                             dpre.as<uint32_t>(), m, op.pi.as<uint32_t>(),
                                             op.pinv.as<uint32_t>(), P.out_o.as<uint16_t>());
  TM_CKK("eo_perm");
  // per-part output offsets for both cluster splits
  auto offsets = [&](int c, DBuf& dst) {
    int nparts = P.n_erep << c;
    int part_bits = m - c;
    int part_words = (1 << part_bits) / 32;
    dst.alloc((size_t)(nparts + 1) * 4);
    eo_offsets_kernel<<<(nparts + 1 + 255) / 256, 256, 0, s>>>(dpre.as<uint32_t>(), dbits.as<uint32_t>(),
                                                               nwords, nparts, part_words, dst.as<uint32_t>());
    TM_CKK("eo_offsets");
  };
  offsets(P.c64, P.out_off);
  offsets(P.c32, P.out_off32);
  // map1
  const int64_t n1 = (int64_t)P.n_orep << m;
  P.map1.alloc(n1 * 4);
  eo_map1_kernel<<<grid_for(n1), 256, 0, s>>>(pd, d_olist.as<uint32_t>(), P.n_orep, op.pinv.as<uint32_t>(),
                                              P.map1.as<uint32_t>());
  TM_CKK("eo_map1");
  // scales in pi order
  op.sin64.alloc(R * 8);
  op.sout64.alloc(R * 8);
  op.sin32.alloc(R * 4);
  op.sout32.alloc(R * 4);
  eo_scale_kernel<<<grid_for(R), 256, 0, s>>>(op.pi.as<uint32_t>(), op.tvec.as<double>(), op.dup.as<uint16_t>(),
                                              R, op.sin64.as<double>(), op.sout64.as<double>(),
                                              op.sin32.as<float>(), op.sout32.as<float>());
  TM_CKK("eo_scale");
  TM_CK(cudaStreamSynchronize(s));
  op.has_pi = true;
  P.active = true;
}

// ------------------------------------------------------------------ launch
namespace {

template <class T>
__global__ void eo_scale_in(const T* __restrict__ x, const double* __restrict__ s64,
                            const float* __restrict__ s32, T* __restrict__ u, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) {
    if (sizeof(T) == 8)
      u[i] = (T)((double)x[i] * s64[i]);
    else
      u[i] = x[i] * (T)s32[i];
  }
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

template <class T, int KB>
void launch_pass1(const EOArgs& A, int ntiles, const typename EoIO<T>::In* u, const uint32_t* map1,
                  const uint32_t* colmap, T* w1, cudaStream_t s) {
  size_t shm = (size_t)((1 << A.n) + (1 << A.n) / 32 + 1) * sizeof(T);
  auto kfn = eo_pass1<T, KB, typename EoIO<T>::In>;
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
  TM_CK(cudaLaunchKernelEx(&cfg, kfn, A, u, map1, colmap, w1));
}

template <class T, int KB, bool F64S>
void launch_pass2(const EOArgs& A, int ntiles, const T* w1, const EOPlan& P, const uint32_t* off,
                  const double* sout64, const float* sout32, double post, typename EoIO<T>::Out* y,
                  cudaStream_t s) {
  size_t shm = (size_t)((1 << A.n) + (1 << A.n) / 32 + 1) * sizeof(T);
  auto kfn = eo_pass2<T, KB, F64S, typename EoIO<T>::Out>;
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
  TM_CK(cudaLaunchKernelEx(&cfg, kfn, A, w1, P.t2.as<uint32_t>(), P.erep.as<uint32_t>(),
                           P.colmap.as<uint32_t>(), off, P.out_o.as<uint16_t>(), sout64, sout32, post, y));
}

template <class T>
EOArgs make_args(const Op& op, int c) {
  EOArgs A;
  A.m = op.eo.m;
  A.c = c;
  A.n = A.m - c;
  const int KB = (sizeof(T) == 8) ? 4 : 5;
  int kb = std::min(KB, std::max(1, A.n - 5));
  A.p = A.n - kb;
  if (A.p > 10) A.p = 10;
  A.ng = op.eo.ng;
  A.n_orep = op.eo.n_orep;
  const double K = op.mp.betaJ;
  double ea = std::exp(K), eb = std::exp(-K);
  A.a64 = ea / (ea + eb);
  A.b64 = eb / (ea + eb);
  A.a32 = (float)A.a64;
  A.b32 = (float)A.b64;
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
  eo_scale_in<In><<<grid_for(R), 256, 0, s>>>(x, op.sin64.as<double>(), op.sin32.as<float>(), u, R);
  TM_CKK("eo_scale_in");
  if (P.prof_on) TM_CK(cudaEventRecord(P.prof_ev[1], s));
  launch_pass1<T, KB>(A, P.n_orep, u, P.map1.as<uint32_t>(), P.colmap.as<uint32_t>(), w1, s);
  TM_CKK("eo_pass1");
  if (P.prof_on) TM_CK(cudaEventRecord(P.prof_ev[2], s));
  const uint32_t* off = (sizeof(T) == 8) ? P.out_off.as<uint32_t>() : P.out_off32.as<uint32_t>();
  const double S = std::pow(std::exp(op.mp.betaJ) + std::exp(-op.mp.betaJ), (double)op.L);
  if (scaled32)
    launch_pass2<T, KB, false>(A, P.n_erep, w1, P, off, op.sout64.as<double>(), op.sout32.as<float>(), 1.0, y, s);
  else
    launch_pass2<T, KB, true>(A, P.n_erep, w1, P, off, op.sout64.as<double>(), op.sout32.as<float>(), S, y, s);
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

// FP64 even/odd product in pi order with caller-provided scratch: u (R
// doubles) and w1 (n_orep * 2^m doubles).  Used by the entry point whose
// scratch lives in a fixed device array.
void matvec_eo_f64_into(const Op& op, const double* x, double* y, double* u, double* w1, cudaStream_t s) {
  const EOPlan& P = op.eo;
  const int64_t R = op.n;
  EOArgs A = make_args<double>(op, P.c64);
  if (A.n - A.p > 4) fail(TM_ERR_LIMIT, "even/odd tile too large for the FP64 engine");
  eo_scale_in<double><<<grid_for(R), 256, 0, s>>>(x, op.sin64.as<double>(), op.sin32.as<float>(), u, R);
  TM_CKK("eo_scale_in");
  const double S = std::pow(std::exp(op.mp.betaJ) + std::exp(-op.mp.betaJ), (double)op.L);
  switch (A.n - A.p) {
#define TM_EO_INTO(KBV)                                                                                      \
  case KBV:                                                                                                  \
    launch_pass1<double, KBV>(A, P.n_orep, u, P.map1.as<uint32_t>(), P.colmap.as<uint32_t>(), w1, s);       \
    TM_CKK("eo_pass1");                                                                                      \
    launch_pass2<double, KBV, true>(A, P.n_erep, w1, P, P.out_off.as<uint32_t>(), op.sout64.as<double>(),    \
                                    op.sout32.as<float>(), S, y, s);                                        \
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
