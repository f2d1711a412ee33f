// Orbit tables, state->representative rank maps and Boltzmann-weight vectors,
// all built on the GPU.
//
//  * rep bitset: one bit per state, set iff the state is its orbit's minimum
//    (warp ballot over 32 consecutive states);
//  * exclusive prefix of per-word popcounts -> rank of any representative;
//  * compaction -> idxlist (ascending, u32) and duplist (orbit sizes, u16),
//    bit-exact with the reference's serial scans (see tm_group.cuh);
//  * Tvec per operator, restating each reference genTvec.
#include <cmath>
#include <cstdio>
#include <vector>

#include "tm_group.cuh"
#include "tm_internal.h"

namespace ltm {

// ------------------------------------------------------------------ scan
namespace {
constexpr int SCAN_T = 1024;
constexpr int SCAN_E = 4;
constexpr int SCAN_CHUNK = SCAN_T * SCAN_E;

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t block_total;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
    uint32_t z = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) z += y;
    }
    warp_sums[lane] = z - w;
    if (lane == 31) block_total = z;
  }
  __syncthreads();
  uint32_t res = warp_sums[wid] + x - v;
  if (total) *total = block_total;
  __syncthreads();
  return res;
}

__global__ void scan_reduce_kernel(const uint32_t* in, uint32_t* part, int64_t n) {
  int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
  uint32_t s = 0;
  for (int e = 0; e < SCAN_E; ++e) {
    int64_t i = base + (int64_t)e * SCAN_T + threadIdx.x;
    if (i < n) s += in[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ uint32_t ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t t = ws[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

__global__ void scan_down_kernel(const uint32_t* in, uint32_t* out, const uint32_t* part, int64_t n) {
  int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK + (int64_t)threadIdx.x * SCAN_E;
  uint32_t v[SCAN_E];
  uint32_t loc = 0;
  for (int e = 0; e < SCAN_E; ++e) {
    int64_t i = base + e;
    v[e] = (i < n) ? in[i] : 0;
    loc += v[e];
  }
  uint32_t off = block_excl_scan(loc, nullptr) + (part ? part[blockIdx.x] : 0);
  for (int e = 0; e < SCAN_E; ++e) {
    int64_t i = base + e;
    if (i < n) out[i] = off;
    off += v[e];
  }
}
}  // namespace

int exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t s) {
  if (n <= 0) return 0;
  int64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if (nb == 1) {
    scan_down_kernel<<<1, SCAN_T, 0, s>>>(in, out, nullptr, n);
    TM_CKK("scan_down");
    return 0;
  }
  DBuf part, partx;
  part.alloc(nb * sizeof(uint32_t));
  partx.alloc(nb * sizeof(uint32_t));
  scan_reduce_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(in, part.as<uint32_t>(), n);
  TM_CKK("scan_reduce");
  exclusive_scan_u32(part.as<uint32_t>(), partx.as<uint32_t>(), nb, s);
  scan_down_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(in, out, partx.as<uint32_t>(), n);
  TM_CKK("scan_down");
  TM_CK(cudaStreamSynchronize(s));  // temporaries are released on return
  return 0;
}

uint32_t read_u32(const uint32_t* dptr, cudaStream_t s) {
  uint32_t v = 0;
  TM_CK(cudaMemcpyAsync(&v, dptr, sizeof(v), cudaMemcpyDeviceToHost, s));
  TM_CK(cudaStreamSynchronize(s));
  return v;
}

// ------------------------------------------------------------------ orbit table
namespace {

__global__ void rep_bits_kernel(GroupDev g, uint64_t nstate, uint32_t* bits, uint32_t* cnt,
                                int64_t nwords) {
  const int lane = threadIdx.x & 31;
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp; w < nwords; w += nwarps) {
    uint64_t s = (uint64_t)w * 32 + lane;
    bool rep = (s < nstate) && is_rep(g, s);
    uint32_t word = __ballot_sync(0xffffffffu, rep);
    if (lane == 0) {
      bits[w] = word;
      cnt[w] = __popc(word);
    }
  }
}

// Representative bitset for the periodic X-2D group, L <= 32.  A warp takes
// 32 consecutive words, lane j screening word j with word_rejected_x2d32; in
// each surviving word every lane tests its own state, first against the
// necessary condition, then exactly (lane_rep_x2d32).  Lane j stores word j,
// so the stores coalesce.
__global__ void rep_bits_x2d32_kernel(int L, int flip, uint64_t nstate, uint32_t* bits, uint32_t* cnt,
                                      int64_t nwords) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w0 = warp * 32; w0 < nwords; w0 += nwarps * 32) {
    const int nw = (int)((nwords - w0 < 32) ? nwords - w0 : 32);
    uint32_t todo = __ballot_sync(0xffffffffu, lane < nw && !word_rejected_x2d32((uint64_t)(w0 + lane), L, flip));
    uint32_t mine = 0;
    while (todo) {
      const int j = __ffs(todo) - 1;
      todo &= todo - 1;
      const int64_t w = w0 + j;
      const uint64_t s = (uint64_t)w * 32 + lane;
      int fix;
      const bool rep = s < nstate && rep_candidate_x2d32((uint32_t)s, L, flip) &&
                       lane_rep_x2d32((uint32_t)s, L, flip, &fix);
      const uint32_t word = __ballot_sync(0xffffffffu, rep);
      if (lane == j) mine = word;
    }
    if (lane < nw) {
      bits[w0 + lane] = mine;
      cnt[w0 + lane] = __popc(mine);
    }
  }
}

// Compaction with orbit sizes (X-2D periodic, L <= 32).  A warp loads 32
// words and their prefixes at once, then takes the non-empty words one by
// one, a lane per representative: lane b computes its state's stabiliser
// count and stores at the word's offset plus its rank within the word.
__global__ void compact_x2d32_kernel(int L, int flip, const uint32_t* bits, const uint32_t* prefix,
                                     int64_t nwords, uint32_t* idx, uint16_t* dup) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int order = 2 * L * (flip ? 2 : 1);
  for (int64_t w0 = warp * 32; w0 < nwords; w0 += nwarps * 32) {
    const int64_t wl = w0 + lane;
    const uint32_t word = (wl < nwords) ? bits[wl] : 0u;
    const uint32_t pos = (wl < nwords) ? prefix[wl] : 0u;
    uint32_t nz = __ballot_sync(0xffffffffu, word != 0);
    while (nz) {
      const int src = __ffs(nz) - 1;
      nz &= nz - 1;
      const uint32_t wd = __shfl_sync(0xffffffffu, word, src);
      const uint32_t p = __shfl_sync(0xffffffffu, pos, src);
      if ((wd >> lane) & 1u) {
        const uint32_t s = (uint32_t)((w0 + src) * 32) + (uint32_t)lane;
        int fix = 1;
        lane_rep_x2d32(s, L, flip, &fix);
        const uint32_t at = p + __popc(wd & ((1u << lane) - 1u));
        idx[at] = s;
        dup[at] = (uint16_t)(order / fix);
      }
    }
  }
}

__global__ void compact_kernel(GroupDev g, const uint32_t* bits, const uint32_t* prefix,
                               int64_t nwords, uint32_t* idx, uint16_t* dup) {
  const int lane = threadIdx.x & 31;
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp; w < nwords; w += nwarps) {
    uint32_t word = bits[w];
    if (!word) continue;
    if ((word >> lane) & 1u) {
      uint64_t s = (uint64_t)w * 32 + lane;
      uint32_t pos = prefix[w] + __popc(word & ((1u << lane) - 1u));
      idx[pos] = (uint32_t)s;
      dup[pos] = (uint16_t)orbit_size(g, s);
    }
  }
}

__global__ void state_map_kernel(GroupDev g, uint64_t nstate, const uint32_t* bits,
                                 const uint32_t* prefix, uint32_t* smap) {
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = tid; s < (int64_t)nstate; s += nth) {
    uint64_t c = canon(g, (uint64_t)s);
    uint32_t w = (uint32_t)(c >> 5);
    smap[s] = prefix[w] + __popc(bits[w] & ((1u << (c & 31)) - 1u));
  }
}

}  // namespace

int GroupDesc::order() const { return group_order(to_dev(*this)); }

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    TM_CK(cudaGetDevice(&dev));
    TM_CK(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  }
  return n;
}

// Builds op.idx / op.dup, and keeps the rank structure (rep bitset + word
// prefix) in ws_a / ws_b for the map builders that follow.
void build_orbit_table(Op& op) {
  GroupDev g = to_dev(op.grp);
  const uint64_t nstate = 1ull << (op.grp.nbits ? op.grp.nbits : op.L);
  const int64_t nwords = (int64_t)((nstate + 31) / 32);
  op.ws_a.alloc(nwords * sizeof(uint32_t));  // bits
  op.ws_b.alloc(nwords * sizeof(uint32_t));  // counts -> prefix
  uint32_t* bits = op.ws_a.as<uint32_t>();
  uint32_t* pre = op.ws_b.as<uint32_t>();
  const int threads = 256;
  int64_t want = (nwords * 32 + threads - 1) / threads;
  int blocks = (int)std::min<int64_t>(want, (int64_t)num_sms() * 64);
  const bool x2d32 = g.kind == G_X2D && g.periodic && g.L <= 32 && !op.grp.nbits;
  if (x2d32)
    rep_bits_x2d32_kernel<<<blocks, threads, 0, op.stream>>>(g.L, g.flip, nstate, bits, pre, nwords);
  else
    rep_bits_kernel<<<blocks, threads, 0, op.stream>>>(g, nstate, bits, pre, nwords);
  TM_CKK("rep_bits");
  uint32_t last_cnt = 0, last_bits = 0;
  TM_CK(cudaMemcpyAsync(&last_bits, bits + nwords - 1, 4, cudaMemcpyDeviceToHost, op.stream));
  exclusive_scan_u32(pre, pre, nwords, op.stream);
  uint32_t last_pre = read_u32(pre + nwords - 1, op.stream);
  last_cnt = __builtin_popcount(last_bits);
  const int64_t R = (int64_t)last_pre + last_cnt;
  op.n = R;
  op.idx.alloc(R * sizeof(uint32_t));
  op.dup.alloc(R * sizeof(uint16_t));
  if (x2d32)
    compact_x2d32_kernel<<<blocks, threads, 0, op.stream>>>(g.L, g.flip, bits, pre, nwords, op.idx.as<uint32_t>(),
                                                            op.dup.as<uint16_t>());
  else
    compact_kernel<<<blocks, threads, 0, op.stream>>>(g, bits, pre, nwords, op.idx.as<uint32_t>(),
                                                      op.dup.as<uint16_t>());
  TM_CKK("compact");
  TM_CK(cudaStreamSynchronize(op.stream));
}

// state -> rank map for operators built without one (the even/odd plan frees
// its rank structure): rebuild the representative bitset and prefix in
// temporaries, then map every state.
void ensure_state_map(Op& op) {
  if (op.smap.p) return;
  if (op.L > 30) fail(TM_ERR_LIMIT, "full-space state map limited to L <= 30");
  GroupDev g = to_dev(op.grp);
  const uint64_t nstate = 1ull << op.L;
  const int64_t nwords = (int64_t)((nstate + 31) / 32);
  DBuf bits, pre;
  bits.alloc(nwords * 4);
  pre.alloc(nwords * 4);
  int blocks = (int)std::min<int64_t>((nwords * 32 + 255) / 256, (int64_t)num_sms() * 64);
  if (g.kind == G_X2D && g.periodic && g.L <= 32 && !op.grp.nbits)
    rep_bits_x2d32_kernel<<<blocks, 256, 0, op.stream>>>(g.L, g.flip, nstate, bits.as<uint32_t>(),
                                                        pre.as<uint32_t>(), nwords);
  else
    rep_bits_kernel<<<blocks, 256, 0, op.stream>>>(g, nstate, bits.as<uint32_t>(), pre.as<uint32_t>(), nwords);
  TM_CKK("rep_bits");
  exclusive_scan_u32(pre.as<uint32_t>(), pre.as<uint32_t>(), nwords, op.stream);
  op.smap.alloc(nstate * sizeof(uint32_t));
  int mb = (int)std::min<int64_t>((int64_t)(nstate + 255) / 256, (int64_t)num_sms() * 32);
  state_map_kernel<<<mb, 256, 0, op.stream>>>(g, nstate, bits.as<uint32_t>(), pre.as<uint32_t>(),
                                              op.smap.as<uint32_t>());
  TM_CKK("state_map");
  TM_CK(cudaStreamSynchronize(op.stream));
}

void build_state_map(Op& op) {
  GroupDev g = to_dev(op.grp);
  const uint64_t nstate = 1ull << op.L;
  op.smap.alloc(nstate * sizeof(uint32_t));
  int blocks = (int)std::min<int64_t>((int64_t)(nstate + 255) / 256, (int64_t)num_sms() * 32);
  state_map_kernel<<<blocks, 256, 0, op.stream>>>(g, nstate, op.ws_a.as<uint32_t>(),
                                                  op.ws_b.as<uint32_t>(), op.smap.as<uint32_t>());
  TM_CKK("state_map");
  TM_CK(cudaStreamSynchronize(op.stream));
}

// ------------------------------------------------------------------ Tvec
namespace {

struct TvecParams {
  int kind, L, size1, size2, boundary;
  double betaJ, kappa, kappa2, h, nfexp, halfnf;
};

// XATMatVecProd2D::genTvec (TMat/tmat.hpp:208-310) evaluated at betaJ/2.
__device__ double tv_xat(const TvecParams& p, uint64_t s) {
  const int L = p.L;
  const double hb = 0.5 * p.betaJ;
  const double J1 = -hb, J2 = hb * p.kappa, hJ = -hb * p.h;
  const uint64_t mask = (1ull << L) - 1;
  int n1, n2, n0 = popc64(s);
  int ns1 = L, ns2 = L;
  uint64_t a, b;
  switch (p.boundary) {
    case 0:
      n1 = popc64(s ^ rotr(s, L, 1));
      n2 = popc64(s ^ rotr(s, L, 2));
      break;
    case 1:
      n1 = popc64((s & (mask >> 1)) ^ (s >> 1));
      n2 = popc64((s & (mask >> 2)) ^ (s >> 2));
      ns1 = L - 1;
      ns2 = L - 2;
      break;
    case 5:
    case 9:
      a = (s << 1) | (p.boundary == 9 ? 1ull : 0ull);
      b = s >> 1;
      n1 = popc64(s ^ a);
      n2 = popc64((a & mask) ^ b);
      ns1 = L + 1;
      break;
    default:  // 13, 17
      a = (s << 1) | (p.boundary == 17 ? 1ull : 0ull);
      b = (s << 2) | (p.boundary == 17 ? 3ull : 0ull);
      n1 = popc64(s ^ a);
      n2 = popc64(s ^ b);
      ns1 = L + 1;
      ns2 = L + 2;
      break;
  }
  double bz1 = J1 * (2.0 * n1 - ns1);
  double bz2 = J2 * (2.0 * n2 - ns2);
  double bz0 = hJ * (2.0 * n0 - L);
  return exp(bz1 + bz2 + bz0);
}

// XDTMatVecProd2D::genTvec (TMat/tmat.hpp:437-504) evaluated at betaJ/2.
__device__ double tv_xdt(const TvecParams& p, uint64_t s) {
  const int L = p.L;
  const double hb = 0.5 * p.betaJ;
  const double J1 = -hb, hJ = -hb * p.h;
  const uint64_t nst = 1ull << L;
  int n1, ns1 = L, n0 = popc64(s);
  switch (p.boundary) {
    case 0: n1 = popc64(s ^ rotr(s, L, 1)); break;
    case 1: n1 = popc64((s & ((nst - 1) >> 1)) ^ (s >> 1)); ns1 = L - 1; break;
    case 5: n1 = popc64((s << 1) ^ s); ns1 = L + 1; break;
    default: n1 = popc64(((s << 1) | 1ull) ^ s); ns1 = L + 1; break;  // 9
  }
  double bz1 = J1 * (2.0 * n1 - ns1);
  double bz0 = hJ * (2.0 * n0 - L);
  return exp(bz1 + bz0);
}

// ZBTMatVecProd2D::genTvec (TMat/tmat.hpp:537-556) at betaJ/2, times the
// half normfactor (TMat/tmat.cpp:512-517).
__device__ double tv_zbt(const TvecParams& p, uint64_t s) {
  const int L = p.L;
  const double hb = 0.5 * p.betaJ;
  const double J1 = -hb, J3 = p.kappa2 * hb, hJ = -hb * p.h;
  int n1 = popc64(s ^ rotr(s, L, 1)), n2 = popc64(s ^ rotr(s, L, 2)), n0 = popc64(s);
  double bz1 = J1 * (2.0 * n1 - L), bz2 = J3 * (2.0 * n2 - L), bz0 = hJ * (2.0 * n0 - L);
  return exp(bz1 + bz2 + bz0) * p.halfnf;
}

// XAMMatVecProd2D::genTvec (TMat/tmatreduce.cpp:367-404), without the
// 1/sqrt(dup) factor.
__device__ double tv_xam(const TvecParams& p, uint64_t s) {
  const int L = p.L;
  const double hb = 0.5 * p.betaJ;
  const double J1 = -hb, J2 = hb * p.kappa, hJ = -hb * p.h, Jn = hb * p.nfexp;
  const uint64_t mask = (1ull << L) - 1;
  int n1, n2;
  if (!p.boundary) {
    n1 = popc64(s ^ rotr(s, L, 1));
    n2 = popc64(s ^ rotr(s, L, 2));
  } else {
    n1 = popc64((s & (mask >> 1)) ^ (s >> 1));
    n2 = popc64((s & (mask >> 2)) ^ (s >> 2));
  }
  int n0 = popc64(s);
  double bz = J1 * (2 * n1 - L) + J2 * (2 * n2 - L) + hJ * (2 * n0 - L) + Jn;
  return exp(bz);
}

// XDMMatVecProd2D::genTvec (TMat/tmatreduce.cpp:1367-1400) without 1/sqrt(dup).
__device__ double tv_xdm(const TvecParams& p, uint64_t s) {
  const int L = p.L;
  const double hb = 0.5 * p.betaJ;
  const double J1 = -hb, hJ = -hb * p.h, Jn = hb * p.nfexp;
  int n1 = popc64(s ^ rotr(s, L, 1)), n0 = popc64(s);
  double bz = J1 * (2 * n1 - L) + hJ * (2 * n0 - L) + Jn;
  return exp(bz);
}

// ZBMMatVecProd2D::genTvec (TMat/tmatreduce.cpp:1813-1855) without 1/sqrt(dup).
__device__ double tv_zbm(const TvecParams& p, uint64_t s) {
  const int L = p.L;
  const double hb = 0.5 * p.betaJ;
  const double J1 = -hb, J3 = hb * p.kappa2, hJ = -hb * p.h, Jn = hb * p.nfexp;
  int n1 = popc64(s ^ rotr(s, L, 1)), n2 = popc64(s ^ rotr(s, L, 2)), n0 = popc64(s);
  double bz1 = J1 * (2.0 * n1 - L), bz2 = J3 * (2.0 * n2 - L), bz0 = hJ * (2.0 * n0 - L);
  return exp(bz1 + bz2 + bz0 + Jn);
}

// XAMMatVecProd3D::genTvec (TMat/tmat3d.cpp:179-201) without 1/sqrt(dup).
__device__ double tv_xam3(const TvecParams& p, uint64_t s) {
  const int L = p.L, s1 = p.size1, s2 = p.size2;
  const double hb = 0.5 * p.betaJ;
  const double J1 = -hb, J2 = hb * p.kappa, hJ = -hb * p.h, Jn = hb * p.nfexp;
  int n1a = popc64(s ^ rshift3d(s, s1, s2, 1));
  int n1b = popc64(s ^ dshift3d(s, s1, s2, 1));
  int n2 = popc64(s ^ rshift3d(s, s1, s2, 2));
  int n0 = popc64(s);
  double bz = 2 * J1 * (n1a + n1b - L) + J2 * (2 * n2 - L) + hJ * (2 * n0 - L) + Jn;
  return exp(bz);
}

__device__ double tv_eval(const TvecParams& p, uint64_t s) {
  switch (p.kind) {
    case K_XAT: return tv_xat(p, s);
    case K_XDT: return tv_xdt(p, s);
    case K_ZBT: return tv_zbt(p, s);
    case K_XAM: return tv_xam(p, s);
    case K_XDM: return tv_xdm(p, s);
    case K_ZBM: return tv_zbm(p, s);
    case K_XAM3: return tv_xam3(p, s);
  }
  return 0.0;
}

__global__ void tvec_full_kernel(TvecParams p, int64_t n, double* tv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) tv[i] = tv_eval(p, (uint64_t)i);
}

// Reduced x-ANNNI weights from a table over the bond counts: tv_xam's
// exponent takes (L+1)^3 values (n1, n2, n0 in [0, L]), so its exponentials
// are evaluated once on the host with the same expression.
// tab[(cell) * ndiv + k] = exp(...) / sqrt(d_k) over the bond-count cells
// (n1, n2, n0) and the divisors d_k of the group order (every orbit size is
// one), divided on the host in the same double arithmetic; divk[d] = k.  The
// FP64 square root and division per representative would cost more than the
// rest of the kernel on GB300's FP64 pipe.
__global__ void tvec_xam_tab_kernel(int L, int boundary, int64_t n, const uint32_t* __restrict__ idx,
                                    const uint16_t* __restrict__ dup, const double* __restrict__ tab,
                                    const uint8_t* __restrict__ divk, int ndiv, double* __restrict__ tv) {
  const uint64_t mask = (1ull << L) - 1;
  const int w = L + 1;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) {
    const uint64_t s = idx[i];
    int n1, n2;
    if (!boundary) {
      n1 = popc64(s ^ rotr(s, L, 1));
      n2 = popc64(s ^ rotr(s, L, 2));
    } else {
      n1 = popc64((s & (mask >> 1)) ^ (s >> 1));
      n2 = popc64((s & (mask >> 2)) ^ (s >> 2));
    }
    const int n0 = popc64(s);
    tv[i] = __ldg(tab + (((int64_t)n1 * w + n2) * w + n0) * ndiv + __ldg(divk + dup[i]));
  }
}

__global__ void tvec_red_kernel(TvecParams p, int64_t n, const uint32_t* idx, const uint16_t* dup,
                                double* tv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) tv[i] = tv_eval(p, (uint64_t)idx[i]) / sqrt((double)dup[i]);
}

}  // namespace

void build_tvec(Op& op) {
  TvecParams p;
  p.kind = op.kind;
  p.L = op.L;
  p.size1 = op.size1;
  p.size2 = op.size2;
  p.boundary = op.boundary;
  p.betaJ = op.mp.betaJ;
  p.kappa = op.mp.kappa;
  p.kappa2 = op.mp.kappa2;
  p.h = op.mp.h;
  p.nfexp = op.nfexp;
  p.halfnf = std::exp(0.5 * op.mp.betaJ * op.nfexp);
  const bool reduced = (op.kind == K_XAM || op.kind == K_XDM || op.kind == K_ZBM || op.kind == K_XAM3);
  const int64_t n = reduced ? op.n : (int64_t)op.nstate;
  op.tvec.alloc(n * sizeof(double));
  int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 16);
  if (blocks < 1) blocks = 1;
  DBuf tab, divk;  // freed after the synchronisation below
  if (reduced && op.kind == K_XAM && op.L <= 32) {
    // tv_xam's exponentials over all bond counts, same expression
    const int L = op.L, w = L + 1;
    const double hb = 0.5 * p.betaJ;
    const double J1 = -hb, J2 = hb * p.kappa, hJ = -hb * p.h, Jn = hb * p.nfexp;
    // orbit sizes divide the group order
    const int G = op.grp.order();
    std::vector<int> divs;
    for (int d = 1; d <= G; ++d)
      if (G % d == 0) divs.push_back(d);
    const int ndiv = (int)divs.size();
    std::vector<uint8_t> K((size_t)G + 1, 0);
    for (int k = 0; k < ndiv; ++k) K[divs[k]] = (uint8_t)k;
    std::vector<double> T((size_t)w * w * w * ndiv);
    for (int n1 = 0; n1 <= L; ++n1)
      for (int n2 = 0; n2 <= L; ++n2)
        for (int n0 = 0; n0 <= L; ++n0) {
          const double e = std::exp(J1 * (2 * n1 - L) + J2 * (2 * n2 - L) + hJ * (2 * n0 - L) + Jn);
          for (int k = 0; k < ndiv; ++k)
            T[(((size_t)n1 * w + n2) * w + n0) * ndiv + k] = e / std::sqrt((double)divs[k]);
        }
    tab.alloc(T.size() * 8);
    divk.alloc(K.size());
    TM_CK(cudaMemcpyAsync(tab.p, T.data(), T.size() * 8, cudaMemcpyHostToDevice, op.stream));
    TM_CK(cudaMemcpyAsync(divk.p, K.data(), K.size(), cudaMemcpyHostToDevice, op.stream));
    tvec_xam_tab_kernel<<<blocks, 256, 0, op.stream>>>(L, p.boundary, n, op.idx.as<uint32_t>(),
                                                       op.dup.as<uint16_t>(), tab.as<double>(),
                                                       divk.as<uint8_t>(), ndiv, op.tvec.as<double>());
  } else if (reduced) {
    tvec_red_kernel<<<blocks, 256, 0, op.stream>>>(p, n, op.idx.as<uint32_t>(), op.dup.as<uint16_t>(),
                                                   op.tvec.as<double>());
  } else {
    tvec_full_kernel<<<blocks, 256, 0, op.stream>>>(p, n, op.tvec.as<double>());
  }
  TM_CKK("tvec");
  TM_CK(cudaStreamSynchronize(op.stream));
}

}  // namespace ltm
