// Configuration planting (the reference's DumpConfig) on the device.
//
// The reference samples equilibrium layer sequences from the leading
// eigenvector q of a transfer matrix (DumpConfig/dumpconfig.cpp:88-136 for
// the full x-ANNNI TM, DumpConfig/dumpreduce.cpp:47-122 for the reduced one,
// DumpConfig/dumpreduce.cpp:516-591 for the reduced DNNI one):
//   start:  a state with probability q_a^2 (cumulative sums, upper_bound on
//           rand * total);
//   step:   the next state with probability  T(a', a) q_a'  (the column of
//           T at the current state, cumulative, upper_bound again); for the
//           reduced TM the column is T_red e_qa (one perform_op per cache
//           miss of a 20-entry LRU cache), and the layer state inside the
//           chosen orbit is drawn with weights exp(crossintr(ra, member)).
// The chains are independent except for the one random stream they draw
// from in order (chain 0's draws, then chain 1's, ...), and each step draws a
// fixed number of values, so every chain's draws are known in advance.  Here
// all chains advance together:
//   - the random stream is drawn once on the host, in the reference's order,
//     with the reference's generator (std::mt19937 seeded like
//     MyUtility::setseed, std::uniform_real_distribution<double>);
//   - one kernel launch per step computes every chain's column (one block per
//     chain), its cumulative sums and the upper_bound of its draw; the full
//     TM column is analytic, the reduced x-ANNNI column comes straight from
//     its definition T_red[b, a] = dup_b Tvec_b Tvec_a sum_{s in orbit(a)}
//     Th(idx_b, s), with Th(s', s) = e^{K (L - 2 popcount(s' ^ s))} from a
//     table of L + 1 values (no cache is needed: a column costs one pass);
//     the reduced DNNI column is the operator's own FP64 product of the unit
//     vector, as the reference forms it (one product per chain and step);
//   - the two-layer parallel TM (YAT2DDumpConfig::dump,
//     DumpConfig/dumpconfig.cpp:171-219) walks pairs of layers (ra, rb) ->
//     (rb, rc): its column over rc is analytic, weighted by the right
//     eigenvector at (rc, rb), and its start is drawn from |r| |l|; the
//     reduced two-layer TMs (YAM2DDumpConfig / YBM2DDumpConfig::dump,
//     DumpConfig/dumpreduce.cpp:156-256) take their columns from the
//     operator's products and draw the layer pair inside the chosen orbit
//     among the members that continue the chain (low layer = rb);
//   - for the full TM the chains run all their steps in one launch; for the
//     reduced TM the host draws the state inside the chosen orbit, with the
//     orbit enumerated in the reference's order (getEqvStates inserts into a
//     std::unordered_set and lists it, TMat/tmatreduce.cpp:615-657).
// Sampling decisions compare cumulative sums; sums formed in a different
// order differ in the last bits, which changes a decision only for a draw
// within ~1e-16 of a boundary.
#include <algorithm>
#include <cmath>
#include <random>
#include <unordered_set>
#include <vector>

#include "tm_internal.h"

namespace ltm {

namespace {

constexpr int kDumpThreads = 512;

struct DumpArgs {
  int L, n_is_full;         // width; 1: full TM (column over all 2^L states)
  int64_t n;                // column length (2^L or R)
  int nchain, length;
  int draws_per_chain, draw_stride;  // draws used per chain, draws per step
  double bj, kap, hj;       // betaJ, -kappa betaJ, h betaJ (the reference's interacton[])
  const double* vec;        // |q| (the sampling weights' eigenvector)
  const double* draws;      // [nchain][draws_per_chain]
  const double* thtab;      // e^{K (L - 2 d)}, d = 0..L
  const uint32_t* idx;      // reduced: representatives
  const uint16_t* dup;
  const double* tvec;
  const uint32_t* orb;      // reduced: orbit members of each chain's current rep [nchain][orb_cap]
  const int* orb_n;
  int orb_cap;
  const double* ycol;       // reduced DNNI: [nchain][n] the chains' current columns T e_a
  double* pref;             // [nchain][n] cumulative sums (scratch)
  int64_t* cur;             // [nchain] current state (full) or rep index (reduced)
  uint64_t* states;         // full: [nchain][length] states
};

__device__ __forceinline__ int popc64(uint64_t x) { return __popcll(x); }

__device__ __forceinline__ uint64_t rot_r(uint64_t s, int L, int k) {
  const uint64_t mask = (L == 64) ? ~0ull : ((1ull << L) - 1);
  return ((s >> k) | (s << (L - k))) & mask;
}

// selfintr(ra) of the full x-ANNNI dump (DumpConfig/dumpconfig.cpp:69-77)
__device__ __forceinline__ double selfintr(const DumpArgs& A, uint64_t ra) {
  const int L = A.L;
  double t = A.hj * (L - 2.0 * popc64(ra));
  t += A.bj * (L - 2.0 * popc64(ra ^ rot_r(ra, L, 1)));
  t += A.kap * (L - 2.0 * popc64(ra ^ rot_r(ra, L, 2)));
  return t;
}

// column value i of chain c's current column
__device__ __forceinline__ double column(const DumpArgs& A, int c, uint64_t a, int64_t i, double intr1) {
  if (A.n_is_full) {
    // exp(selfintr(a) + crossintr(a, i)) q_i  (crossintr = betaJ (L - 2 popcount(a ^ i)))
    return exp(intr1 + A.bj * (A.L - 2.0 * popc64(a ^ (uint64_t)i))) * A.vec[i];
  }
  if (A.ycol) return A.ycol[(int64_t)c * A.n + i] * A.vec[i];  // (T e_a)_i q_i
  // T_red[i, a] q_i
  const uint32_t si = A.idx[i];
  const uint32_t* orb = A.orb + (int64_t)c * A.orb_cap;
  const int no = A.orb_n[c];
  double acc = 0.0;
  for (int k = 0; k < no; ++k) acc += A.thtab[popc64(si ^ orb[k])];
  return (double)A.dup[i] * A.tvec[i] * A.tvec[a] * acc * A.vec[i];
}

// One column of chain c: cumulative sums into pref, then the upper_bound of
// draw * total.  Returns the index (the same in every thread).
__device__ int64_t column_sample(const DumpArgs& A, int c, uint64_t a, double draw) {
  __shared__ double warp_sums[kDumpThreads / 32];
  __shared__ double carry;
  __shared__ int64_t found;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  double* pref = A.pref + (int64_t)c * A.n;
  const double intr1 = A.n_is_full ? selfintr(A, a) : 0.0;
  if (tid == 0) carry = 0.0;
  __syncthreads();
  for (int64_t base = 0; base < A.n; base += blockDim.x) {
    const int64_t i = base + tid;
    double v = (i < A.n) ? column(A, c, a, i, intr1) : 0.0;
    // inclusive scan within the warp, then across warps
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[wid] = v;
    __syncthreads();
    if (wid == 0) {
      double w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0.0;
      for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      if (lane < (int)(blockDim.x >> 5)) warp_sums[lane] = w;  // inclusive prefix of warp totals
    }
    __syncthreads();
    const double before = carry + (wid > 0 ? warp_sums[wid - 1] : 0.0);
    if (i < A.n) pref[i] = before + v;
    __syncthreads();
    if (tid == blockDim.x - 1) carry = before + v;
    __syncthreads();
  }
  if (tid == 0) {
    const double target = draw * pref[A.n - 1];
    // upper_bound: first i with pref[i] > target
    int64_t lo = 0, hi = A.n;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (pref[mid] <= target)
        lo = mid + 1;
      else
        hi = mid;
    }
    found = lo < A.n ? lo : A.n - 1;
  }
  __syncthreads();
  return found;
}

// Full TM: every step of chain blockIdx.x in one launch.
__global__ void __launch_bounds__(kDumpThreads) dump_full_kernel(DumpArgs A) {
  const int c = blockIdx.x;
  int64_t a = A.cur[c];
  const double* d = A.draws + (int64_t)c * A.draws_per_chain;
  for (int rq = 1; rq < A.length; ++rq) {
    a = column_sample(A, c, (uint64_t)a, d[1 + (rq - 1) * A.draw_stride]);
    if (threadIdx.x == 0) A.states[(int64_t)c * A.length + rq] = (uint64_t)a;
  }
  if (threadIdx.x == 0) A.cur[c] = a;
}

// Two-layer parallel TM (YAT): every step of chain blockIdx.x in one launch.
// State = rb << L | ra; the column over rc is exp(selfintr(ra, rb) +
// crossintr(ra, rc)) r[rc << L | rb], with selfintr = field + NN in the layer
// + NN to the partner layer and crossintr = -kappa betaJ (L - 2 popcount(ra ^
// rc)) (DumpConfig/dumpconfig.cpp:146-168).  Records ra0, the rb of every
// step and the last rc: length + 1 layers.
__device__ __forceinline__ double yat_column(const DumpArgs& A, uint64_t ra, uint64_t rb, int64_t rc, double intr1) {
  return exp(intr1 + A.kap * (A.L - 2.0 * popc64(ra ^ (uint64_t)rc))) * A.vec[((uint64_t)rc << A.L) | rb];
}

__global__ void __launch_bounds__(kDumpThreads) dump_yat_kernel(DumpArgs A) {
  __shared__ double warp_sums[kDumpThreads / 32];
  __shared__ double carry;
  __shared__ int64_t found;
  const int c = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint64_t mask = (1ull << A.L) - 1;
  const int64_t ncol = (int64_t)1 << A.L;
  double* pref = A.pref + (int64_t)c * ncol;
  uint64_t cur = (uint64_t)A.cur[c];
  const double* d = A.draws + (int64_t)c * A.draws_per_chain;
  if (tid == 0) A.states[(int64_t)c * (A.length + 1)] = cur & mask;
  for (int rq = 1; rq < A.length; ++rq) {
    const uint64_t ra = cur & mask, rb = cur >> A.L;
    if (tid == 0) A.states[(int64_t)c * (A.length + 1) + rq] = rb;
    const int L = A.L;
    double intr1 = A.hj * (L - 2.0 * popc64(ra));
    intr1 += A.bj * (L - 2.0 * popc64(ra ^ rot_r(ra, L, 1)));
    intr1 += A.bj * (L - 2.0 * popc64(ra ^ rb));
    if (tid == 0) carry = 0.0;
    __syncthreads();
    for (int64_t base = 0; base < ncol; base += blockDim.x) {
      const int64_t i = base + tid;
      double v = (i < ncol) ? yat_column(A, ra, rb, i, intr1) : 0.0;
      for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
      }
      if (lane == 31) warp_sums[wid] = v;
      __syncthreads();
      if (wid == 0) {
        double w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0.0;
        for (int o = 1; o < 32; o <<= 1) {
          const double t = __shfl_up_sync(0xffffffffu, w, o);
          if (lane >= o) w += t;
        }
        if (lane < (int)(blockDim.x >> 5)) warp_sums[lane] = w;
      }
      __syncthreads();
      const double before = carry + (wid > 0 ? warp_sums[wid - 1] : 0.0);
      if (i < ncol) pref[i] = before + v;
      __syncthreads();
      if (tid == blockDim.x - 1) carry = before + v;
      __syncthreads();
    }
    if (tid == 0) {
      const double target = d[1 + (rq - 1) * A.draw_stride] * pref[ncol - 1];
      int64_t lo = 0, hi = ncol;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (pref[mid] <= target)
          lo = mid + 1;
        else
          hi = mid;
      }
      found = lo < ncol ? lo : ncol - 1;
    }
    __syncthreads();
    cur = ((uint64_t)found << A.L) | rb;
    __syncthreads();
  }
  if (tid == 0) A.states[(int64_t)c * (A.length + 1) + A.length] = cur >> A.L;
}

// Reduced TM: step rq of every chain (the rep index of the next orbit).
__global__ void __launch_bounds__(kDumpThreads) dump_reduced_kernel(DumpArgs A, int rq) {
  const int c = blockIdx.x;
  const int64_t qa = A.cur[c];
  const double draw = A.draws[(int64_t)c * A.draws_per_chain + 1 + (rq - 1) * A.draw_stride];
  const int64_t q = column_sample(A, c, (uint64_t)qa, draw);
  if (threadIdx.x == 0) A.cur[c] = q;
}

// The orbit of a representative in the order the reference lists it:
// XAMMatVecProd2D::getEqvStates (periodic), TMat/tmatreduce.cpp:615-643 --
// rotations of the state (with their flips), then rotations of its bit
// reversal, inserted into a std::unordered_set and read back in its order.
std::vector<uint64_t> eqv_states(uint64_t s, int L, bool flip) {
  std::unordered_set<uint64_t> res;
  const uint64_t mask = (1ull << L) - 1;
  auto rot1 = [&](uint64_t x) { return (x >> 1) | ((x & 1ull) << (L - 1)); };
  auto brev = [&](uint64_t x) {
    uint64_t r = 0;
    for (int i = 0; i < L; ++i) r |= ((x >> i) & 1ull) << (L - 1 - i);
    return r;
  };
  for (uint64_t nx = s; res.find(nx) == res.end(); nx = rot1(nx)) {
    res.insert(nx);
    if (flip) res.insert(~nx & mask);
  }
  for (uint64_t nx = brev(s); res.find(nx) == res.end(); nx = rot1(nx)) {
    res.insert(nx);
    if (flip) res.insert(~nx & mask);
  }
  return std::vector<uint64_t>(res.begin(), res.end());
}

__global__ void unit_vector_kernel(double* __restrict__ x, int64_t n, int64_t at) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = (i == at) ? 1.0 : 0.0;
}

// The orbit of a two-layer state in the order the reference lists it:
// YAMMatVecProd2D::getEqvStates, TMat/tmatreduce.cpp:911-943 -- the joint
// rotations of both layers, then those of the bit-reversed pair, then (with
// the spin flip) the same for the flipped pair, inserted into a
// std::unordered_set and read back in its order.
std::vector<uint64_t> eqv_states_2layer(uint64_t s, int L, bool flip) {
  std::unordered_set<uint64_t> res;
  const uint64_t lm = (1ull << L) - 1, mask = (1ull << (2 * L)) - 1;
  auto rot1 = [&](uint64_t x) { return (x >> 1) | ((x & 1ull) << (L - 1)); };
  auto brev = [&](uint64_t x) {
    uint64_t r = 0;
    for (int i = 0; i < L; ++i) r |= ((x >> i) & 1ull) << (L - 1 - i);
    return r;
  };
  auto scan = [&](uint64_t st) {
    uint64_t hi = st >> L, lo = st & lm;
    for (uint64_t nx = st; res.find(nx) == res.end();) {
      res.insert(nx);
      hi = rot1(hi);
      lo = rot1(lo);
      nx = hi << L | lo;
    }
  };
  scan(s);
  scan(brev(s >> L) << L | brev(s & lm));
  if (flip) {
    const uint64_t f = ~s & mask;
    scan(f);
    scan(brev(f >> L) << L | brev(f & lm));
  }
  return std::vector<uint64_t>(res.begin(), res.end());
}

}  // namespace

// y = T x in the reference's vector order (tm_capi.cu)
void matvec_ref_order(const Op& op, const void* x, void* y, tm_dtype dt, cudaStream_t s);

void dump_configs(const Op& op0, const double* vec_h, const double* vecl_h, int nchain, int length, uint32_t seed,
                  uint64_t* out) {
  const Op& op = op0.parent ? *op0.parent : op0;
  const bool full = (op.kind == K_XAT && op.boundary == 0);
  const bool red = (op.kind == K_XAM && op.grp.periodic);
  const bool red_dnni = (op.kind == K_XDM && op.grp.periodic);
  const bool yat = (op.kind == K_YAT && op.boundary == 0);
  const bool red2 = (op.kind == K_YAM);  // YAM (A/6) and YBM (B/6): periodic only
  const bool two_layer = yat || red2;
  if (!full && !red && !red_dnni && !two_layer)
    fail(TM_ERR_UNSUPPORTED,
         "configuration planting covers the periodic x-ANNNI perpendicular TMs (A/1, A/5), the reduced DNNI "
         "one (D/5) and the two-layer parallel TMs (A/2, A/6, B/6): the reference's finished DumpConfig dumpers");
  if (two_layer && !vecl_h) fail(TM_ERR_ARG, "the two-layer TMs plant from their right and left eigenvectors");
  if (!two_layer && vecl_h) fail(TM_ERR_UNSUPPORTED, "left/right planting is for the two-layer parallel TMs");
  if (nchain < 1 || length < 1) fail(TM_ERR_ARG, "nconfig and length must be >= 1");
  const int L = op.L;
  const int64_t n = op.n;
  if (full && L > 24) fail(TM_ERR_LIMIT, "full-TM planting supports L <= 24");
  cudaStream_t s = op.stream;
  AllocStream guard(s);
  // sampling weights: |q| as the reference reads its vector file
  // (DumpConfig/dumpconfig.hpp:56-77), start weights q^2 summed in order
  // (|r| |l| for the two-layer TM, DumpConfig/dumpconfig.cpp:45-56)
  std::vector<double> vabs(n), qmargin(n);
  double acc = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    vabs[i] = std::fabs(vec_h[i]);
    acc += vabs[i] * (two_layer ? std::fabs(vecl_h[i]) : vabs[i]);
    qmargin[i] = acc;
  }
  // the random stream, in the reference's order
  std::mt19937 rg(seed);
  std::uniform_real_distribution<> rrand;
  const int stride = (full || yat) ? 1 : 2;
  const int per = 1 + stride * (length - 1);
  std::vector<double> draws((size_t)nchain * per);
  for (double& d : draws) d = rrand(rg);
  // start states
  std::vector<int64_t> cur(nchain);
  for (int c = 0; c < nchain; ++c) {
    const double t = draws[(size_t)c * per] * qmargin.back();
    cur[c] = std::upper_bound(qmargin.begin(), qmargin.end(), t) - qmargin.begin();
    if (cur[c] >= n) cur[c] = n - 1;
  }
  const double bj = op.mp.betaJ;
  std::vector<double> th(L + 1);
  for (int d = 0; d <= L; ++d) th[d] = std::exp(bj * (L - 2.0 * d));
  DBuf dvec, ddraw, dth, dpref, dcur, dstates, dorb, dorbn;
  auto up = [&](DBuf& b, const void* src, size_t bytes) {
    b.alloc(bytes);
    TM_CK(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, s));
  };
  up(dvec, vabs.data(), n * 8);
  up(ddraw, draws.data(), draws.size() * 8);
  up(dth, th.data(), th.size() * 8);
  up(dcur, cur.data(), cur.size() * 8);
  dpref.alloc((size_t)nchain * (yat ? ((int64_t)1 << L) : n) * 8);
  DumpArgs A{};
  A.L = L;
  A.n_is_full = full;
  A.n = n;
  A.nchain = nchain;
  A.length = length;
  A.draws_per_chain = per;
  A.draw_stride = stride;
  A.bj = bj;
  A.kap = -op.mp.kappa * bj;
  A.hj = op.mp.h * bj;
  A.vec = dvec.as<double>();
  A.draws = ddraw.as<double>();
  A.thtab = dth.as<double>();
  A.pref = dpref.as<double>();
  A.cur = dcur.as<int64_t>();
  if (yat) {
    dstates.alloc((size_t)nchain * (length + 1) * 8);
    A.states = dstates.as<uint64_t>();
    dump_yat_kernel<<<nchain, kDumpThreads, 0, s>>>(A);
    TM_CKK("dump_yat");
    TM_CK(cudaMemcpyAsync(out, dstates.p, (size_t)nchain * (length + 1) * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    return;
  }
  if (full) {
    std::vector<uint64_t> st0((size_t)nchain * length, 0);
    for (int c = 0; c < nchain; ++c) st0[(size_t)c * length] = (uint64_t)cur[c];
    up(dstates, st0.data(), st0.size() * 8);
    A.states = dstates.as<uint64_t>();
    dump_full_kernel<<<nchain, kDumpThreads, 0, s>>>(A);
    TM_CKK("dump_full");
    TM_CK(cudaMemcpyAsync(out, dstates.p, st0.size() * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    return;
  }
  // reduced: representatives on the host for the orbit draws
  std::vector<uint32_t> idx_h(n);
  TM_CK(cudaMemcpyAsync(idx_h.data(), op.idx.p, n * 4, cudaMemcpyDeviceToHost, s));
  TM_CK(cudaStreamSynchronize(s));
  const bool flip = red2 ? (op.censym != 0) : (op.grp.flip != 0);
  const bool by_product = red_dnni || red2;  // columns from the operator's own products
  const int cap = 4 * L;
  std::vector<uint32_t> orb((size_t)nchain * cap);
  std::vector<int> orbn(nchain);
  dorb.alloc(orb.size() * 4);
  dorbn.alloc(orbn.size() * 4);
  A.idx = op.idx.as<uint32_t>();
  A.dup = op.dup.as<uint16_t>();
  A.tvec = op.tvec.as<double>();
  DBuf dycol, dunit;
  if (by_product) {
    dycol.alloc((size_t)nchain * n * 8);
    dunit.alloc((size_t)n * 8);
    A.ycol = dycol.as<double>();
  }
  A.orb = dorb.as<uint32_t>();
  A.orb_n = dorbn.as<int>();
  A.orb_cap = cap;
  // ra: the chain's current layer state (a layer pair for the two-layer
  // TMs, whose dumpers record its low layer at the start of every step and
  // once more at the end)
  const uint64_t lmask = (1ull << L) - 1;
  std::vector<uint64_t> ra(nchain);
  for (int c = 0; c < nchain; ++c) {
    ra[c] = idx_h[cur[c]];
    if (!red2) out[(size_t)c * length] = ra[c];
  }
  for (int rq = 1; rq < length; ++rq) {
    if (red2)
      for (int c = 0; c < nchain; ++c) out[(size_t)c * length + rq - 1] = ra[c] & lmask;
    if (!by_product) {
      // the current orbits (for the analytic column sums)
      for (int c = 0; c < nchain; ++c) {
        const std::vector<uint64_t> m = eqv_states(idx_h[cur[c]], L, flip);
        orbn[c] = (int)m.size();
        for (size_t k = 0; k < m.size(); ++k) orb[(size_t)c * cap + k] = (uint32_t)m[k];
      }
      TM_CK(cudaMemcpyAsync(dorb.p, orb.data(), orb.size() * 4, cudaMemcpyHostToDevice, s));
      TM_CK(cudaMemcpyAsync(dorbn.p, orbn.data(), orbn.size() * 4, cudaMemcpyHostToDevice, s));
    }
    if (by_product) {
      // the current columns T e_a, one FP64 product per chain
      const int g = (int)std::min<int64_t>((n + 255) / 256, 1024);
      for (int c = 0; c < nchain; ++c) {
        unit_vector_kernel<<<g, 256, 0, s>>>(dunit.as<double>(), n, cur[c]);
        TM_CKK("unit_vector");
        matvec_ref_order(op, dunit.p, dycol.as<double>() + (int64_t)c * n, TM_F64, s);
      }
    }
    dump_reduced_kernel<<<nchain, kDumpThreads, 0, s>>>(A, rq);
    TM_CKK("dump_reduced");
    TM_CK(cudaMemcpyAsync(cur.data(), dcur.p, cur.size() * 8, cudaMemcpyDeviceToHost, s));
    TM_CK(cudaStreamSynchronize(s));
    // the layer state inside the chosen orbit, weights exp(crossintr(ra, e))
    // in the reference's member order (DumpConfig/dumpreduce.cpp:97-111;
    // the DNNI cross interaction adds the two diagonals,
    // DumpConfig/dumpreduce.cpp:509-514)
    auto rotr1 = [&](uint64_t x) { return (x >> 1) | ((x & 1ull) << (L - 1)); };
    auto rotl1 = [&](uint64_t x) { return ((x << 1) & lmask) | (x >> (L - 1)); };
    auto cross = [&](uint64_t a, uint64_t b) {
      double v = bj * (L - 2.0 * __builtin_popcountll(a ^ b));
      if (red_dnni)
        v += A.kap * (L - 2.0 * __builtin_popcountll(a ^ rotr1(b))) +
             A.kap * (L - 2.0 * __builtin_popcountll(a ^ rotl1(b)));
      return v;
    };
    for (int c = 0; c < nchain; ++c) {
      const std::vector<uint64_t> eq =
          red2 ? eqv_states_2layer(idx_h[cur[c]], L, flip) : eqv_states(idx_h[cur[c]], L, flip);
      std::vector<double> qcond(eq.size());
      double t = 0.0;
      for (size_t k = 0; k < eq.size(); ++k) {
        if (!red2) {
          t += std::exp(cross(ra[c], eq[k]));
        } else if ((eq[k] & lmask) == (ra[c] >> L)) {
          // members whose low layer continues the chain (rb), weight
          // exp(crossintr(ra, rc)), crossintr = -kappa betaJ (L - 2 popcount)
          // (DumpConfig/dumpreduce.cpp:152-155, 236-244)
          t += std::exp(A.kap * (L - 2.0 * __builtin_popcountll((ra[c] & lmask) ^ (eq[k] >> L))));
        }
        qcond[k] = t;
      }
      const double target = draws[(size_t)c * per + 1 + (rq - 1) * stride + 1] * qcond.back();
      size_t k = std::upper_bound(qcond.begin(), qcond.end(), target) - qcond.begin();
      if (k >= eq.size()) k = eq.size() - 1;
      ra[c] = eq[k];
      if (!red2) out[(size_t)c * length + rq] = ra[c];
    }
  }
  if (red2)
    for (int c = 0; c < nchain; ++c) out[(size_t)c * length + length - 1] = ra[c] & lmask;
}

}  // namespace ltm

using namespace ltm;

extern "C" tm_status tm_dump_configs(const tm_op* op, const double* vec_host, int nconfig, int length, uint32_t seed,
                                     uint64_t* states_out) {
  try {
    if (!op || !vec_host || !states_out) fail(TM_ERR_ARG, "null argument");
    dump_configs(*op->impl, vec_host, nullptr, nconfig, length, seed, states_out);
  } catch (const Failure& f) {
    set_error(f.msg);
    return f.code;
  } catch (const std::exception& e) {
    set_error(e.what());
    return TM_ERR_CUDA;
  }
  return TM_OK;
}

extern "C" tm_status tm_dump_configs_lr(const tm_op* op, const double* vecr_host, const double* vecl_host, int nconfig,
                                        int length, uint32_t seed, uint64_t* states_out) {
  try {
    if (!op || !vecr_host || !vecl_host || !states_out) fail(TM_ERR_ARG, "null argument");
    dump_configs(*op->impl, vecr_host, vecl_host, nconfig, length, seed, states_out);
  } catch (const Failure& f) {
    set_error(f.msg);
    return f.code;
  } catch (const std::exception& e) {
    set_error(e.what());
    return TM_ERR_CUDA;
  }
  return TM_OK;
}
