// Two-layer parallel transfer matrices: the y-direction TMs, whose state is a
// pair of adjacent layers (2L spins; the reference index puts one layer in the
// high L bits and the other in the low L bits).
//
//   YATMatVecProd2D / _T (TMat/tmat.cpp:106-242): L shift-and-mix steps on one
//     layer amount to the Kronecker factor (x)_i [[e^-Kk, e^Kk], [e^Kk, e^-Kk]]
//     on that layer's L bits, then a layer swap and the dense NN-only x-ANNNI
//     weight as a diagonal: y = nf * Tvec .* swap(K_high x); the transpose is
//     y = nf * swap(K_low (Tvec .* x)).
//   Y2ATMatVecProd2D (TMat/tmat.cpp:245-315): the L steps of permute_mult_T1
//     apply one 4x4 matrix to every bit pair (i, L+i); y = nf * Tv^(1/2) .*
//     P4 (Tv^(1/2) .* x).  The reference's get_t_instance is the operator itself.
//   YAMMatVecProd2D / _T, YBMMatVecProd2D (TMat/tmatreduce.cpp:661-1021):
//     representatives are grouped by their left (high) layer l; one CTA per
//     group fills the right-layer vector at g(r) for every g in the stabiliser
//     of l, applies the Kronecker factor on the L right bits in shared memory
//     and writes each representative's entry to its layer-swapped orbit.
//
// The full forms run as shared-memory tile passes over HBM: a pass gathers a
// tile of 2^nt states whose index bits are chosen per pass (a few contiguous
// low bits for coalescing plus the bits being mixed), applies the factor for
// those bits, and writes the tile back.  FP64 throughout (these operators are
// at most 4^14 states).
#include <algorithm>
#include <cmath>
#include <vector>

#include "tm_bits.cuh"
#include "tm_group.cuh"
#include "tm_internal.h"

namespace ltm {

namespace {

constexpr int kMaxTileBits = 12;  // 4096 doubles = 32 KB per tile

__device__ __forceinline__ int spad(int e) { return e + (e >> 5); }

struct Mat4 {
  double c[16];
};

struct TileMap {
  int nt;        // tile bits
  int pos[16];   // tile bit k -> state bit pos[k]
  int no;        // outer bits
  int opos[32];  // outer bit j -> state bit opos[j]
};

__device__ __forceinline__ uint64_t deposit(uint64_t v, const int* pos, int nb) {
  uint64_t g = 0;
  for (int k = 0; k < nb; ++k) g |= ((v >> k) & 1ull) << pos[k];
  return g;
}

// One tile pass.  MODE 0: Kronecker [[w0, w1], [w1, w0]] on tile bits
// [k0, nt).  MODE 1: the 4x4 matrix m4 (row-major, p = low + 2*high) on the
// tile bit pairs (k0 + j, k0 + np + j), j < np.  pre / post_sc: optional
// per-state input / output weights; post: output scale.
template <int MODE>
__global__ void __launch_bounds__(512) tile_kernel(const double* __restrict__ x, double* __restrict__ y, TileMap tm,
                                                   int k0, int np, double w0, double w1, Mat4 m4,
                                                   const double* __restrict__ pre,
                                                   const double* __restrict__ post_sc, double post) {
  extern __shared__ double sm[];
  const int tile = 1 << tm.nt;
  const uint64_t base = deposit((uint64_t)blockIdx.x, tm.opos, tm.no);
  for (int e = threadIdx.x; e < tile; e += blockDim.x) {
    const uint64_t g = base | deposit((uint64_t)e, tm.pos, tm.nt);
    double v = x[g];
    if (pre) v *= pre[g];
    sm[spad(e)] = v;
  }
  __syncthreads();
  if (MODE == 0) {
    for (int k = k0; k < tm.nt; ++k) {
      const int lowm = (1 << k) - 1;
      for (int p = threadIdx.x; p < (tile >> 1); p += blockDim.x) {
        const int e0 = ((p & ~lowm) << 1) | (p & lowm), e1 = e0 | (1 << k);
        const double a = sm[spad(e0)], b = sm[spad(e1)];
        sm[spad(e0)] = w0 * a + w1 * b;
        sm[spad(e1)] = w1 * a + w0 * b;
      }
      __syncthreads();
    }
  } else {
    for (int j = 0; j < np; ++j) {
      const int ba = k0 + j, bb = k0 + np + j;  // ba < bb
      const int ma = 1 << ba, mb = 1 << bb;
      for (int q = threadIdx.x; q < (tile >> 2); q += blockDim.x) {
        // insert zeros at bits ba and bb
        int e = q;
        e = ((e >> ba) << (ba + 1)) | (e & (ma - 1));
        e = ((e >> bb) << (bb + 1)) | (e & (mb - 1));
        double in[4], out[4];
        in[0] = sm[spad(e)];
        in[1] = sm[spad(e | ma)];
        in[2] = sm[spad(e | mb)];
        in[3] = sm[spad(e | ma | mb)];
#pragma unroll
        for (int p = 0; p < 4; ++p)
          out[p] = m4.c[p * 4 + 0] * in[0] + m4.c[p * 4 + 1] * in[1] + m4.c[p * 4 + 2] * in[2] +
                   m4.c[p * 4 + 3] * in[3];
        sm[spad(e)] = out[0];
        sm[spad(e | ma)] = out[1];
        sm[spad(e | mb)] = out[2];
        sm[spad(e | ma | mb)] = out[3];
      }
      __syncthreads();
    }
  }
  for (int e = threadIdx.x; e < tile; e += blockDim.x) {
    const uint64_t g = base | deposit((uint64_t)e, tm.pos, tm.nt);
    double v = sm[spad(e)] * post;
    if (post_sc) v *= post_sc[g];
    y[g] = v;
  }
}

// y[h*N + l] = post * sc[h*N + l] * v[l*N + h]  (layer swap, N = 2^L)
__global__ void swap_scale_kernel(const double* __restrict__ v, double* __restrict__ y, int L,
                                  const double* __restrict__ sc, double post) {
  __shared__ double tile[32][33];
  const int64_t N = 1ll << L;
  const int T = blockDim.x;
  const int64_t bx = (int64_t)blockIdx.x * T, by = (int64_t)blockIdx.y * T;
  for (int r = threadIdx.y; r < T; r += blockDim.y) tile[r][threadIdx.x] = v[(by + r) * N + bx + threadIdx.x];
  __syncthreads();
  for (int r = threadIdx.y; r < T; r += blockDim.y) {
    const int64_t o = (bx + r) * N + by + threadIdx.x;
    double val = tile[threadIdx.x][r] * post;
    if (sc) val *= sc[o];
    y[o] = val;
  }
}

// --- Tvec of the full forms
// YATMatVecProd2D::genTvec (TMat/tmat.hpp:361-366, TMat/tmat.cpp:668-684):
// entry (row = low layer, col = high layer) of the dense NN-only x-ANNNI TM
__global__ void yat_tvec_kernel(double* __restrict__ tv, int L, double bj, double h) {
  const int64_t n = 1ll << (2 * L);
  const uint64_t lm = (1ull << L) - 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t row = (uint64_t)i & lm, col = (uint64_t)i >> L;
    const int n1 = popc64(row ^ rotr(row, L, 1)), n0 = popc64(row), nx = popc64(row ^ col);
    tv[i] = exp(-bj * (2 * n1 - L) - bj * h * (2 * n0 - L) - bj * (2 * nx - L));
  }
}

// Y2ATMatVecProd2D::genTvec (TMat/tmat.hpp:396-414) at betaJ/2: Tv^(1/2)
__global__ void y2at_tvec_kernel(double* __restrict__ tv, int L, double bj, double h) {
  const int64_t n = 1ll << (2 * L);
  const uint64_t lm = (1ull << L) - 1;
  const double J1 = -0.5 * bj, hJ = -0.5 * bj * h;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = (uint64_t)i & lm, hi = (uint64_t)i >> L;
    const int n1 = popc64(lo ^ rotr(lo, L, 1)), n2 = popc64(hi ^ rotr(hi, L, 1)), n0 = popc64(lo ^ hi);
    const int fa = 2 * (n1 + n2 + n0) - 3 * L, fb = 2 * (popc64((uint64_t)i) - L);
    tv[i] = exp(J1 * fa + hJ * fb);
  }
}

// YAMMatVecProd2D::genTvec / genTvec1 (TMat/tmatreduce.cpp:725-797)
__global__ void yam_tvec_kernel(const uint32_t* __restrict__ idx, const uint16_t* __restrict__ dup,
                                double* __restrict__ tv, int64_t n, int L, int ltype, double bj, double k,
                                double k2, double h, double nfe) {
  const uint64_t lm = (1ull << L) - 1;
  const double hb = 0.5 * bj, J1 = -hb, hJ = -hb * h, Jn = hb * nfe, k1J = hb * k, k2J = hb * k2;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = idx[r], l = s >> L, rt = s & lm;
    const int n1 = popc64(l ^ rotr(l, L, 1)), n2 = popc64(l ^ rt), n0 = popc64(l);
    double bz = J1 * (2 * (n1 + n2 - L)) + hJ * (2 * n0 - L) + Jn;
    if (ltype) {
      const int b1 = popc64(l ^ rotr(l, L, 2)), d1 = popc64(l ^ rotr(rt, L, 1)), d2 = popc64(l ^ rotl(rt, L, 1));
      bz += k1J * (2 * b1 - L) + k2J * (2 * (d1 + d2 - L));
    }
    tv[r] = exp(bz) / sqrt((double)dup[r]);
  }
}

// swp[r] = rank of the orbit holding the layer-swapped states of orbit r
__global__ void yswap_kernel(GroupDev g, const uint32_t* __restrict__ idx, int64_t n,
                             const uint32_t* __restrict__ bits, const uint32_t* __restrict__ prefix,
                             uint32_t* __restrict__ swp) {
  const int L = g.L;
  const uint64_t lm = (1ull << L) - 1;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = idx[r];
    const uint64_t c = canon(g, (s & lm) << L | (s >> L));
    const uint32_t w = (uint32_t)(c >> 5);
    swp[r] = prefix[w] + __popc(bits[w] & ((1u << (c & 31)) - 1u));
  }
}

// one layer under group element gi of the two-layer group (translation,
// reflection, flip), the same element acting on both layers
__device__ __forceinline__ uint32_t layer_act(uint32_t x, int L, int gi) {
  const uint32_t lm = (1u << L) - 1;
  const int sh = gi % L, rf = (gi / L) & 1, f = gi / (2 * L);
  uint64_t v = x;
  if (rf) v = brev(v, L);
  if (f) v = ~v & lm;
  return (uint32_t)rotr(v, L, sh);
}

// YAMMatVecProd2D::perform_op (TMat/tmatreduce.cpp:827-876), transposed:
// YAMMatVecProd2D_T::perform_op (:953-1016).  One CTA per left-layer block.
__global__ void __launch_bounds__(512) yam_block_kernel(const double* __restrict__ x, double* __restrict__ y,
                                                        const uint32_t* __restrict__ idx,
                                                        const uint16_t* __restrict__ dup,
                                                        const double* __restrict__ tv,
                                                        const uint32_t* __restrict__ swp,
                                                        const uint32_t* __restrict__ bstart, int L, int ng,
                                                        int transposed, double w0, double w1) {
  extern __shared__ double tmp[];
  __shared__ int stab[64];
  __shared__ int nstab;
  const uint32_t r0 = bstart[blockIdx.x], r1 = bstart[blockIdx.x + 1];
  const uint32_t lm = (1u << L) - 1;
  const uint32_t l = idx[r0] >> L;
  if (threadIdx.x == 0) nstab = 0;
  __syncthreads();
  if ((int)threadIdx.x < ng && layer_act(l, L, threadIdx.x) == l) stab[atomicAdd(&nstab, 1)] = threadIdx.x;
  __syncthreads();
  const int ns = nstab;
  for (uint32_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const uint32_t src = transposed ? swp[r] : r;
    const double v = tv[src] * x[src];
    const uint32_t rt = idx[r] & lm;
    for (int q = 0; q < ns; ++q) tmp[spad((int)layer_act(rt, L, stab[q]))] = v;
  }
  __syncthreads();
  const int half = 1 << (L - 1);
  for (int b = 0; b < L; ++b) {
    const int lowm = (1 << b) - 1;
    for (int p = threadIdx.x; p < half; p += blockDim.x) {
      const int e0 = ((p & ~lowm) << 1) | (p & lowm), e1 = e0 | (1 << b);
      const double a = tmp[spad(e0)], c = tmp[spad(e1)];
      tmp[spad(e0)] = w0 * a + w1 * c;
      tmp[spad(e1)] = w1 * a + w0 * c;
    }
    __syncthreads();
  }
  for (uint32_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const uint32_t dst = transposed ? r : swp[r];
    y[dst] = tv[dst] * (double)dup[dst] * tmp[spad((int)(idx[r] & lm))];
  }
}

int grid_n(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 16));
}

// tile map: tile bits = `tb` (in order), outer bits = all others below nbits
TileMap make_map(const std::vector<int>& tb, int nbits) {
  TileMap m{};
  m.nt = (int)tb.size();
  uint64_t used = 0;
  for (int k = 0; k < m.nt; ++k) {
    m.pos[k] = tb[k];
    used |= 1ull << tb[k];
  }
  m.no = 0;
  for (int b = 0; b < nbits; ++b)
    if (!((used >> b) & 1ull)) m.opos[m.no++] = b;
  return m;
}

template <int MODE>
void launch_tile(const double* x, double* y, const TileMap& m, int k0, int np, double w0, double w1, const Mat4& m4,
                 const double* pre, const double* post_sc, double post, cudaStream_t s) {
  const int tile = 1 << m.nt;
  const size_t shm = (size_t)(tile + tile / 32 + 1) * sizeof(double);
  const int threads = std::min(512, std::max(32, tile / 4));
  tile_kernel<MODE><<<(unsigned)(1u << m.no), threads, shm, s>>>(x, y, m, k0, np, w0, w1, m4, pre, post_sc, post);
  TM_CKK("two_layer_tile");
}

// Kronecker [[w0, w1], [w1, w0]] over state bits [lo, hi) of a 2L-bit vector
void kron_range(const double* x, double* y, int nbits, int lo, int hi, double w0, double w1, const double* pre,
                const double* post_sc, double post, cudaStream_t s) {
  const Mat4 none{};
  int b = lo;
  bool first = true;
  const double* src = x;
  while (b < hi) {
    const int cb = (b == 0) ? 0 : std::min(5, b);  // contiguous low bits for coalescing
    const int nb = std::min(hi - b, kMaxTileBits - cb);
    std::vector<int> tb;
    for (int k = 0; k < cb; ++k) tb.push_back(k);
    for (int k = 0; k < nb; ++k) tb.push_back(b + k);
    const bool last = (b + nb >= hi);
    launch_tile<0>(src, y, make_map(tb, nbits), cb, 0, w0, w1, none, first ? pre : nullptr,
                   last ? post_sc : nullptr, last ? post : 1.0, s);
    src = y;
    first = false;
    b += nb;
  }
}

}  // namespace

void build_two_layer(Op& op) {
  const int L = op.L;
  if (L > 14) fail(TM_ERR_LIMIT, "two-layer operators support L <= 14 (4^L states)");
  const double bj = op.mp.betaJ, k = op.mp.kappa, k2 = op.mp.kappa2, h = op.mp.h;
  op.nstate = 1ll << (2 * L);
  cudaStream_t s = op.stream;
  if (op.kind == K_YAT || op.kind == K_Y2AT) {
    op.n = op.nstate;
    op.tvec.alloc((size_t)op.n * 8);
    op.ws_a.alloc((size_t)op.n * 8);
    if (op.kind == K_YAT)
      yat_tvec_kernel<<<grid_n(op.n), 256, 0, s>>>(op.tvec.as<double>(), L, bj, h);
    else
      y2at_tvec_kernel<<<grid_n(op.n), 256, 0, s>>>(op.tvec.as<double>(), L, bj, h);
    TM_CKK("two_layer_tvec");
    TM_CK(cudaStreamSynchronize(s));
    return;
  }
  // reduced: orbits of the two-layer group
  op.grp.kind = G_Y2D;
  op.grp.L = L;
  op.grp.nbits = 2 * L;
  op.grp.periodic = 1;
  op.grp.flip = op.censym;
  build_orbit_table(op);
  const int64_t R = op.n;
  GroupDev g = to_dev(op.grp);
  op.swp.alloc((size_t)R * 4);
  yswap_kernel<<<grid_n(R), 256, 0, s>>>(g, op.idx.as<uint32_t>(), R, op.ws_a.as<uint32_t>(),
                                         op.ws_b.as<uint32_t>(), op.swp.as<uint32_t>());
  TM_CKK("two_layer_swap");
  op.tvec.alloc((size_t)R * 8);
  yam_tvec_kernel<<<grid_n(R), 256, 0, s>>>(op.idx.as<uint32_t>(), op.dup.as<uint16_t>(), op.tvec.as<double>(), R,
                                            L, op.ltype, bj, k, k2, h, op.nfexp);
  TM_CKK("two_layer_tvec");
  // blocks of representatives sharing the left (high) layer
  std::vector<uint32_t> idx((size_t)R), starts;
  TM_CK(cudaMemcpyAsync(idx.data(), op.idx.p, (size_t)R * 4, cudaMemcpyDeviceToHost, s));
  TM_CK(cudaStreamSynchronize(s));
  for (int64_t r = 0; r < R; ++r)
    if (r == 0 || (idx[r] >> L) != (idx[r - 1] >> L)) starts.push_back((uint32_t)r);
  starts.push_back((uint32_t)R);
  op.nblocks = (int)starts.size() - 1;
  op.bstart.alloc(starts.size() * 4);
  TM_CK(cudaMemcpyAsync(op.bstart.p, starts.data(), starts.size() * 4, cudaMemcpyHostToDevice, s));
  TM_CK(cudaStreamSynchronize(s));
  op.ws_a.release();
  op.ws_b.release();
}

void matvec_two_layer(const Op& op, const double* x, double* y, cudaStream_t s) {
  const Op& b = op.parent ? *op.parent : op;
  const bool tr = op.transposed;
  const int L = b.L;
  const double bj = b.mp.betaJ, k = b.mp.kappa;
  if (b.kind == K_YAT) {
    // bzwj2 = e^{-+K kappa} (TMat/tmat.cpp:110-113)
    const double w0 = std::exp(-bj * k), w1 = 1.0 / w0;
    double* v = b.ws_a.as<double>();
    const int T = std::min(32, 1 << L);
    const dim3 grid((1u << L) / T, (1u << L) / T), blk(T, std::min(T, 8));
    if (!tr) {
      kron_range(x, v, 2 * L, L, 2 * L, w0, w1, nullptr, nullptr, 1.0, s);
      swap_scale_kernel<<<grid, blk, 0, s>>>(v, y, L, b.tvec.as<double>(), b.normfactor);
    } else {
      kron_range(x, v, 2 * L, 0, L, w0, w1, b.tvec.as<double>(), nullptr, 1.0, s);
      swap_scale_kernel<<<grid, blk, 0, s>>>(v, y, L, nullptr, b.normfactor);
    }
    TM_CKK("two_layer_swap_scale");
  } else if (b.kind == K_Y2AT) {
    // bzwj1 = e^{+-K}, bzwj2 = e^{-+2K kappa} (TMat/tmat.cpp:247-253); the 4x4
    // matrix on a bit pair with p = low + 2*high, j = low ^ high:
    //   out(p) = w1[j] (w2[0] in(p) + in(p^2)) + w1[j^1] (w2[1] in(p^3) + in(p^1))
    const double e1[2] = {std::exp(bj), std::exp(-bj)};
    const double e2[2] = {std::exp(-2.0 * bj * k), std::exp(2.0 * bj * k)};
    Mat4 m4{};
    for (int p = 0; p < 4; ++p) {
      const int j = (p & 1) ^ (p >> 1);
      m4.c[p * 4 + p] += e1[j] * e2[0];
      m4.c[p * 4 + (p ^ 2)] += e1[j];
      m4.c[p * 4 + (p ^ 3)] += e1[j ^ 1] * e2[1];
      m4.c[p * 4 + (p ^ 1)] += e1[j ^ 1];
    }
    int lo = 0;
    const double* src = x;
    while (lo < L) {
      const int cb = (lo == 0) ? 0 : std::min(3, lo);
      const int np = std::min(L - lo, (kMaxTileBits - cb) / 2);
      std::vector<int> tb;
      for (int q = 0; q < cb; ++q) tb.push_back(q);
      for (int q = 0; q < np; ++q) tb.push_back(lo + q);
      for (int q = 0; q < np; ++q) tb.push_back(L + lo + q);
      const bool first = (lo == 0), last = (lo + np >= L);
      launch_tile<1>(src, y, make_map(tb, 2 * L), cb, np, 0.0, 0.0, m4, first ? b.tvec.as<double>() : nullptr,
                     last ? b.tvec.as<double>() : nullptr, last ? b.normfactor : 1.0, s);
      src = y;
      lo += np;
    }
  } else if (b.kind == K_YAM) {
    const double w0 = std::exp(-bj * k), w1 = 1.0 / w0;
    const size_t shm = (size_t)((1 << L) + (1 << L) / 32 + 1) * sizeof(double);
    raise_smem_limit((const void*)yam_block_kernel, shm);
    const int ng = 2 * L * (b.censym ? 2 : 1);
    yam_block_kernel<<<(unsigned)b.nblocks, 512, shm, s>>>(x, y, b.idx.as<uint32_t>(), b.dup.as<uint16_t>(),
                                                           b.tvec.as<double>(), b.swp.as<uint32_t>(),
                                                           b.bstart.as<uint32_t>(), L, ng, tr ? 1 : 0, w0, w1);
    TM_CKK("two_layer_block");
  } else {
    fail(TM_ERR_ARG, "not a two-layer operator");
  }
}

}  // namespace ltm
