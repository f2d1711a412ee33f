// Parameter sweeps of aux-bit operators (diagonal BNNNI, DNNI) solved as one
// batch on the device.
//
// The reference runs one parameter point per tmat invocation (TMat/main.cpp,
// TMat/pfunc.cpp:16-106): build the operator, solve with Spectra, write the
// outputs.  A sweep over (betaJ, kappa, kappa2, h, L) points is that run
// repeated.  Here every point of a sweep is a member of one batch:
//   - an instance table in device memory (ChainInst, tm_chain.h) holds each
//     member's pass geometry, Boltzmann factors and buffers, whatever its
//     width;
//   - each chain pass is ONE launch over the tiles of every member (a block
//     takes its member from a per-block member map); so are the contraction
//     and the Krylov vector kernels (row chunks of kSweepRows);
//   - every step, each active member extends its Arnoldi basis by one column
//     (member i at its own column j_i, km[i] on the device), so members
//     restart independently and none waits for another's cycle;
//   - one step of all members is captured once in a CUDA graph and replayed;
//   - after each step the host takes the projected matrices back; a member
//     whose basis is full gets its small projected problem solved (the
//     Krylov-Schur restart of tm_arnoldi.cu, tm_krylov.h) and its kept basis
//     rotated in before the next step; converged members go idle;
//   - members are grouped into waves whose buffers fit a share of the free
//     device memory; a wave holds members of any mix of widths, all with the
//     tile size tuned for its widest member.
// Mixed precision as in tm_arnoldi.cu: FP32 products until the Ritz residuals
// reach the FP32 floor, then FP64-accurate (double-float) products from the
// combined wanted Ritz vectors until the tolerance is met.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "tm_blas.cuh"
#include "tm_chain.h"
#include "tm_internal.h"
#include "tm_krylov.h"

namespace ltm {

void note_launches(int64_t n);

namespace {

constexpr int kSweepMaxM = 24;  // largest Krylov subspace of a sweep member
// per-member small values (doubles): CGS coefficients, |w|^2, projected matrix
constexpr int kScH1 = 0, kScH2 = 32, kScN = 64, kScH = 72;
constexpr int kScStride = kScH + (kSweepMaxM + 1) * (kSweepMaxM + 1) + 7;  // 704

// the member and row range of a row-chunk block
struct RowBlock {
  int i;
  int64_t r0, r1;
};

// (rmem: the member of every row block, stored after the prefix rstart[count + 1])
__device__ __forceinline__ RowBlock row_block(const ChainInst* __restrict__ inst, const int64_t* __restrict__ rstart,
                                              int count) {
  const int* rmem = reinterpret_cast<const int*>(rstart + count + 1);
  RowBlock rb;
  rb.i = rmem[blockIdx.x];
  rb.r0 = ((int64_t)blockIdx.x - rstart[rb.i]) * kSweepRows;
  rb.r1 = min(rb.r0 + (int64_t)kSweepRows, inst[rb.i].n);
  return rb;
}

// km[i] = (column j the member extends this step, product mode or idle)
__device__ __forceinline__ bool step_on(int2 km) { return km.y != kModeIdle; }

// x32 = (float) V[:, j] for the members in the FP32 phase
__global__ void __launch_bounds__(256) sw_to_f32(const ChainInst* __restrict__ inst, const int2* __restrict__ km,
                                                 const int64_t* __restrict__ rstart, int count) {
  const RowBlock rb = row_block(inst, rstart, count);
  const int2 k = km[rb.i];
  if (k.y != kModeF32) return;
  const ChainInst& I = inst[rb.i];
  const double* v = I.V + (int64_t)k.x * I.ldv;
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) I.x32[r] = (float)v[r];
}

// partial dots of w against columns 0..j: one warp per column, lanes over rows
__global__ void __launch_bounds__(256) sw_mdot(const ChainInst* __restrict__ inst, const int2* __restrict__ km,
                                               const int64_t* __restrict__ rstart, int count,
                                               double* __restrict__ part) {
  const RowBlock rb = row_block(inst, rstart, count);
  const int2 k = km[rb.i];
  if (!step_on(k)) return;
  const int j = k.x;
  const ChainInst& I = inst[rb.i];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int c = warp; c <= j; c += nw) {
    const double* __restrict__ v = I.V + (int64_t)c * I.ldv;
    double acc = 0.0;
    for (int64_t r = rb.r0 + lane; r < rb.r1; r += 32) acc = fma(v[r], I.w[r], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) part[(int64_t)blockIdx.x * kSweepMaxM + c] = acc;
  }
}

// partial |w|^2 (slot 0)
__global__ void __launch_bounds__(256) sw_nrm(const ChainInst* __restrict__ inst, const int2* __restrict__ km,
                                              const int64_t* __restrict__ rstart, int count,
                                              double* __restrict__ part) {
  const RowBlock rb = row_block(inst, rstart, count);
  if (!step_on(km[rb.i])) return;
  const ChainInst& I = inst[rb.i];
  double acc = 0.0;
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) acc = fma(I.w[r], I.w[r], acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    part[(int64_t)blockIdx.x * kSweepMaxM] = t;
  }
}

// sum the row-chunk partials of each member into sc[off + c], c <= j (one
// block per member, one thread per column; fixed order, so deterministic)
__global__ void sw_reduce(const ChainInst* __restrict__ inst, const int2* __restrict__ km,
                          const int64_t* __restrict__ rstart, const double* __restrict__ part, int off) {
  const int i = blockIdx.x, c = threadIdx.x;
  const int2 k = km[i];
  if (!step_on(k) || c > k.x) return;
  double acc = 0.0;
  for (int64_t b = rstart[i]; b < rstart[i + 1]; ++b) acc += part[b * kSweepMaxM + c];
  inst[i].sc[off + c] = acc;
}

// w -= V[:, 0..j] h, h = sc[off .. off + j]
__global__ void __launch_bounds__(256) sw_maxpy(const ChainInst* __restrict__ inst, const int2* __restrict__ km,
                                                const int64_t* __restrict__ rstart, int count, int off) {
  const RowBlock rb = row_block(inst, rstart, count);
  const int2 k = km[rb.i];
  if (!step_on(k)) return;
  const int j = k.x;
  const ChainInst& I = inst[rb.i];
  __shared__ double hs[kSweepMaxM];
  if (threadIdx.x <= j) hs[threadIdx.x] = I.sc[off + threadIdx.x];
  __syncthreads();
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) {
    double acc = I.w[r];
    for (int c = 0; c <= j; ++c) acc = fma(-I.V[(int64_t)c * I.ldv + r], hs[c], acc);
    I.w[r] = acc;
  }
}

// |w|^2 from the partials; column j of the projected matrix:
// H[0..j, j] = h1 + h2, H[j+1, j] = |w|
__global__ void sw_hcol(const ChainInst* __restrict__ inst, const int2* __restrict__ km,
                        const int64_t* __restrict__ rstart, int m, const double* __restrict__ part) {
  const int i = blockIdx.x, c = threadIdx.x;
  const int2 k = km[i];
  if (!step_on(k)) return;
  const int j = k.x;
  double* sc = inst[i].sc;
  double* H = sc + kScH;
  const int ld = m + 1;
  if (c == 0) {
    double acc = 0.0;
    for (int64_t b = rstart[i]; b < rstart[i + 1]; ++b) acc += part[b * kSweepMaxM];
    sc[kScN] = acc;
    H[(j + 1) + j * ld] = sqrt(acc);
  }
  if (c <= j) H[c + j * ld] = sc[kScH1 + c] + sc[kScH2 + c];
}

// V[:, j+1] = w / |w| (zero column on a breakdown: the residual is then 0)
__global__ void __launch_bounds__(256) sw_normalize(const ChainInst* __restrict__ inst, const int2* __restrict__ km,
                                                    const int64_t* __restrict__ rstart, int count) {
  const RowBlock rb = row_block(inst, rstart, count);
  const int2 k = km[rb.i];
  if (!step_on(k)) return;
  const int j = k.x;
  const ChainInst& I = inst[rb.i];
  const double nsq = I.sc[kScN];
  const double f = nsq > 0.0 ? 1.0 / sqrt(nsq) : 0.0;
  double* v = I.V + (int64_t)(j + 1) * I.ldv;
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) v[r] = I.w[r] * f;
}

// Restart / new start vector of the members with rot[i].x > 0:
// V[:, 0..k) = V[:, 0..m) W_i (W_i m x k column-major at Wall + i*m*m) and,
// when rot[i].y, V[:, k] = V[:, m].  Each thread holds one row's m values, so
// the columns are rewritten in place.
__global__ void __launch_bounds__(256) sw_rotate(const ChainInst* __restrict__ inst, const int64_t* __restrict__ rstart,
                                                 int count, int m, const double* __restrict__ Wall,
                                                 const int2* __restrict__ rot) {
  const RowBlock rb = row_block(inst, rstart, count);
  const int2 rp = rot[rb.i];
  if (rp.x <= 0) return;
  const ChainInst& I = inst[rb.i];
  __shared__ double Ws[kSweepMaxM * kSweepMaxM];
  for (int q = threadIdx.x; q < m * rp.x; q += blockDim.x) Ws[q] = Wall[(int64_t)rb.i * m * m + q];
  __syncthreads();
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) {
    double v[kSweepMaxM];
#pragma unroll
    for (int q = 0; q < kSweepMaxM; ++q)
      if (q < m) v[q] = I.V[(int64_t)q * I.ldv + r];
    for (int c = 0; c < rp.x; ++c) {
      double acc = 0.0;
      // zero coefficients are skipped: after a mid-cycle stop the columns
      // past the member's last step may never have been written
#pragma unroll
      for (int q = 0; q < kSweepMaxM; ++q)
        if (q < m && Ws[c * m + q] != 0.0) acc = fma(v[q], Ws[c * m + q], acc);
      I.V[(int64_t)c * I.ldv + r] = acc;
    }
    if (rp.y) I.V[(int64_t)rp.x * I.ldv + r] = I.V[(int64_t)m * I.ldv + r];
  }
}

// |V[:, 0]|^2 partials and scaling, for members with flag[i] set
__global__ void __launch_bounds__(256) sw_col0_nrm(const ChainInst* __restrict__ inst, const int64_t* __restrict__ rstart,
                                                   int count, const int* __restrict__ flag, double* __restrict__ part) {
  const RowBlock rb = row_block(inst, rstart, count);
  if (!flag[rb.i]) return;
  const ChainInst& I = inst[rb.i];
  double acc = 0.0;
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) acc = fma(I.V[r], I.V[r], acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    part[(int64_t)blockIdx.x * kSweepMaxM] = t;
  }
}

__global__ void __launch_bounds__(256) sw_col0_scale(const ChainInst* __restrict__ inst,
                                                     const int64_t* __restrict__ rstart, int count,
                                                     const int* __restrict__ flag, const double* __restrict__ part) {
  const RowBlock rb = row_block(inst, rstart, count);
  if (!flag[rb.i]) return;
  const ChainInst& I = inst[rb.i];
  __shared__ double f;
  if (threadIdx.x == 0) {
    double acc = 0.0;
    for (int64_t b = rstart[rb.i]; b < rstart[rb.i + 1]; ++b) acc += part[b * kSweepMaxM];
    f = acc > 0.0 ? 1.0 / sqrt(acc) : 0.0;
  }
  __syncthreads();
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) I.V[r] *= f;
}

// y_i = w_i (the product-only entry point), for members in `mode`
__global__ void __launch_bounds__(256) sw_copy_out(const ChainInst* __restrict__ inst, const int64_t* __restrict__ rstart,
                                                   int count, double* const* __restrict__ y) {
  const RowBlock rb = row_block(inst, rstart, count);
  const ChainInst& I = inst[rb.i];
  double* yi = y[rb.i];
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) yi[r] = I.w[r];
}

__global__ void __launch_bounds__(256) sw_copy_in(const ChainInst* __restrict__ inst, const int64_t* __restrict__ rstart,
                                                  int count, const double* const* __restrict__ x) {
  const RowBlock rb = row_block(inst, rstart, count);
  const ChainInst& I = inst[rb.i];
  const double* xi = x[rb.i];
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) I.V[r] = xi[r];
}

// V[:, col] = x_i (the gradient's right and left vectors)
__global__ void __launch_bounds__(256) sw_copy_col(const ChainInst* __restrict__ inst,
                                                  const int64_t* __restrict__ rstart, int count, int col,
                                                  const double* const* __restrict__ x) {
  const RowBlock rb = row_block(inst, rstart, count);
  const ChainInst& I = inst[rb.i];
  const double* xi = x[rb.i];
  double* v = I.V + (int64_t)col * I.ldv;
  for (int64_t r = rb.r0 + threadIdx.x; r < rb.r1; r += blockDim.x) v[r] = xi[r];
}

// Partial sums of the adjoint's weight term over each member's rows, with
// r = V[:, 0] and l = V[:, 1]: slots 0..3 sum l r g_t (g = d ln Tvec/d theta),
// slot 4 sums l r; slot 5 sums l w (w = the last tangent product) when dot_w.
__global__ void __launch_bounds__(256) sw_grad_sums(const ChainInst* __restrict__ inst,
                                                   const int64_t* __restrict__ rstart, int count, int dot_w,
                                                   double* __restrict__ part) {
  const RowBlock rb = row_block(inst, rstart, count);
  const ChainInst& I = inst[rb.i];
  const double* r = I.V;
  const double* l = I.V + I.ldv;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t i = rb.r0 + threadIdx.x; i < rb.r1; i += blockDim.x) {
    if (dot_w) {
      acc[5] += l[i] * I.w[i];
      continue;
    }
    const uint64_t st = I.idx ? (uint64_t)I.idx[i] : (uint64_t)i;
    double g[4];
    aux_tvec_grad(I.kind, I.L, I.bc, I.bj, I.kap2, I.h, st, g);
    const double lr = l[i] * r[i];
    for (int t = 0; t < 4; ++t) acc[t] += lr * g[t];
    acc[4] += lr;
  }
  __shared__ double sh[6][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < 6; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[threadIdx.x][q];
    part[(int64_t)blockIdx.x * kSweepMaxM + threadIdx.x] = t;
  }
}

// out[i * 8 + c] = sum of member i's row-block partials in slot c (c < 6)
__global__ void sw_sum_slots(const int64_t* __restrict__ rstart, const double* __restrict__ part,
                             double* __restrict__ out) {
  const int i = blockIdx.x, c = threadIdx.x;
  if (c >= 6) return;
  double acc = 0.0;
  for (int64_t b = rstart[i]; b < rstart[i + 1]; ++b) acc += part[b * kSweepMaxM + c];
  out[(int64_t)i * 8 + c] = acc;
}

// ------------------------------------------------------------------ host side
struct OpDeleter {
  void operator()(Op* o) const {
    if (!o) return;
    cudaStream_t st = o->stream;
    delete o;
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  }
};

// Solve state of one member.
struct Member {
  std::unique_ptr<Op, OpDeleter> op;
  int phase = kModeIdle;  // product mode of the current steps
  int j = 0;              // column extended by the next step (kept columns after a restart)
  bool done = false;
  tm_status status = TM_OK;
  std::string msg;
  double best = 1e300;
  int stall = 0, cycles = 0;
  tm_eigs_info info{};
  std::vector<std::complex<double>> vals;
};

}  // namespace

struct Sweep {
  char model;
  int dim, axialdir, ec;
  std::vector<Member> mem;
  cudaStream_t s = nullptr;
  int zb = 0;
  size_t budget_override = 0;  // bytes of member buffers per wave (0: from free memory)
  int dir = 0;                 // 1: the members' transposes (left eigenvectors)
  // diagnostics of the last solve: waves, steps, seconds building waves, in
  // steps (device work, host-timed), in host restarts
  double stats[5] = {0, 0, 0, 0, 0};

  ~Sweep() {
    mem.clear();
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  }

  // device memory one member needs in a wave (basis of m+1 columns)
  size_t member_bytes(const Op& o, int m, size_t elem = 8) const {
    const int64_t N = 1ll << o.L;
    const int64_t per = zb ? 16 * N : 4 * N;
    return (size_t)per * elem + (size_t)N * 8 + (size_t)(m + 1) * o.n * 8 + (size_t)o.n * 12 + kScStride * 8 + 4096;
  }

  std::vector<std::pair<int, int>> waves(int m, size_t elem = 8) const {
    size_t budget = budget_override;
    if (!budget) {
      size_t fr = 0, tot = 0;
      TM_CK(cudaMemGetInfo(&fr, &tot));
      budget = (size_t)(0.6 * (double)fr);
    }
    std::vector<std::pair<int, int>> w;
    int a = 0;
    size_t used = 0;
    for (int i = 0; i < (int)mem.size(); ++i) {
      const size_t b = member_bytes(*mem[i].op, m, elem);
      if (i > a && used + b > budget) {
        w.push_back({a, i});
        a = i;
        used = 0;
      }
      used += b;
    }
    if (a < (int)mem.size()) w.push_back({a, (int)mem.size()});
    return w;
  }
};

namespace {

// Buffers and device tables of one wave of members [a, b).
struct Wave {
  Sweep& sw;
  int a, b, count, m;
  std::vector<std::unique_ptr<DBuf>> bufs;
  DBuf inst, kmd, start4, start8, start16, bmem4, bmem8, bmem16, rstart, part, sc, Wall, rot, flag, yptr;
  std::vector<ChainInst> host;
  ChainBatch B;
  DBuf slots;  // per-member sums of the adjoint (8 doubles each)
  int np4max = 0, np8max = 0, np16max = 0, threads4 = 256, threads8 = 256;
  size_t smem4 = 0, smem8 = 0, smem16 = 0;
  int64_t nrblk = 0;
  std::map<int, cudaGraphExec_t> graphs;  // one step, by the product modes present
  std::map<int, int64_t> graph_kernels;

  Wave(Sweep& s_, int a_, int b_, int m_, bool tangent_bufs = false)
      : sw(s_), a(a_), b(b_), count(b_ - a_), m(m_) {
    cudaStream_t s = sw.s;
    host.resize(count);
    // one tile size and block size per element size for the whole wave: the
    // tuned choice at the widest member (most of the work), so every block
    // of a launch gets the shared memory it uses
    int Lmax = 0;
    for (int q = 0; q < count; ++q) Lmax = std::max(Lmax, sw.mem[a + q].op->L);
    int tb4 = 0, tb8 = 0;
    chain_tuning(Lmax, 4, sw.zb, tb4, threads4);
    chain_tuning(Lmax, 8, sw.zb, tb8, threads8);
    for (int q = 0; q < count; ++q) {
      const Op& o = *sw.mem[a + q].op;
      ChainInst& I = host[q];
      std::memset(&I, 0, sizeof(I));
      chain_inst_fill(o, sw.dir, I, tb4, tb8);
      const int64_t N = 1ll << o.L;
      auto mk = [&](size_t bytes) {
        bufs.emplace_back(new DBuf());
        bufs.back()->alloc(bytes);
        return bufs.back()->p;
      };
      I.P = mk((size_t)(sw.zb ? 16 * N : 4 * N) * (tangent_bufs ? 16 : 8));
      I.fold = mk((size_t)N * 8);
      I.ldv = (o.n + 1) & ~(int64_t)1;
      I.V = static_cast<double*>(mk((size_t)(m + 1) * I.ldv * 8));
      I.w = static_cast<double*>(mk((size_t)o.n * 8));
      I.x32 = static_cast<float*>(mk((size_t)o.n * 4));
      np4max = std::max(np4max, I.np4);
      np8max = std::max(np8max, I.np8);
      for (int p = 0; p < I.np4; ++p) smem4 = std::max(smem4, chain_pass_smem(I.p4[p], sw.zb, 4));
      for (int p = 0; p < I.np8; ++p) smem8 = std::max(smem8, chain_pass_smem(I.p8[p], sw.zb, 8));
      np16max = std::max(np16max, I.np16);
      for (int p = 0; p < I.np16; ++p) smem16 = std::max(smem16, chain_pass_smem(I.p16[p], sw.zb, 16));
    }
    sc.alloc((size_t)count * kScStride * 8);
    TM_CK(cudaMemsetAsync(sc.p, 0, sc.bytes, s));
    for (int q = 0; q < count; ++q) host[q].sc = sc.as<double>() + (size_t)q * kScStride;
    // block prefixes per pass (kBatchTiles tiles per block) and the member of
    // every block
    auto plan_tables = [&](int four, int npmax, std::vector<int64_t>& st, std::vector<int>& bm,
                           std::vector<int64_t>& nblk, std::vector<int64_t>& boff) {
      st.assign((size_t)std::max(npmax, 1) * (count + 1), 0);
      nblk.assign(std::max(npmax, 1), 0);
      boff.assign(std::max(npmax, 1), 0);
      bm.clear();
      for (int p = 0; p < npmax; ++p) {
        boff[p] = (int64_t)bm.size();
        for (int q = 0; q < count; ++q) {
          const int np = four == 4 ? host[q].np4 : (four == 8 ? host[q].np8 : host[q].np16);
          const ChainPass* pp = four == 4 ? host[q].p4 : (four == 8 ? host[q].p8 : host[q].p16);
          const int64_t nb = p < np ? (chain_pass_blocks(pp[p]) + kBatchTiles - 1) / kBatchTiles : 0;
          st[(size_t)p * (count + 1) + q + 1] = st[(size_t)p * (count + 1) + q] + nb;
          bm.insert(bm.end(), (size_t)nb, q);
        }
        nblk[p] = st[(size_t)p * (count + 1) + count];
        if (nblk[p] >= (1ll << 31)) fail(TM_ERR_LIMIT, "sweep wave too large for one launch");
      }
    };
    std::vector<int64_t> s4, s8, s16;
    std::vector<int> bm4, bm8, bm16;
    plan_tables(4, np4max, s4, bm4, B.p4.nblk, B.p4.boff);
    plan_tables(8, np8max, s8, bm8, B.p8.nblk, B.p8.boff);
    if (tangent_bufs) plan_tables(16, np16max, s16, bm16, B.p16.nblk, B.p16.boff);
    std::vector<int64_t> rst(count + 1, 0);
    for (int q = 0; q < count; ++q) rst[q + 1] = rst[q] + (host[q].n + kSweepRows - 1) / kSweepRows;
    nrblk = rst[count];
    // row prefix followed by the member of every row block (one buffer)
    std::vector<int64_t> rtab(rst);
    std::vector<int> rm;
    for (int q = 0; q < count; ++q) rm.insert(rm.end(), (size_t)(rst[q + 1] - rst[q]), q);
    rtab.resize(rst.size() + (rm.size() * 4 + 7) / 8, 0);
    std::memcpy(rtab.data() + rst.size(), rm.data(), rm.size() * 4);
    auto up = [&](DBuf& d, const void* src, size_t bytes) {
      d.alloc(bytes);
      TM_CK(cudaMemcpyAsync(d.p, src, bytes, cudaMemcpyHostToDevice, s));
    };
    up(inst, host.data(), sizeof(ChainInst) * count);
    up(start4, s4.data(), s4.size() * 8);
    up(start8, s8.data(), s8.size() * 8);
    up(bmem4, bm4.data(), std::max<size_t>(bm4.size(), 1) * 4);
    up(bmem8, bm8.data(), std::max<size_t>(bm8.size(), 1) * 4);
    if (tangent_bufs) {
      up(start16, s16.data(), s16.size() * 8);
      up(bmem16, bm16.data(), std::max<size_t>(bm16.size(), 1) * 4);
      int tb16 = 0;
      chain_tuning(Lmax, 16, sw.zb, tb16, B.p16.threads);
      B.p16.np = np16max;
      B.p16.smem = smem16;
      B.p16.start = start16.as<int64_t>();
      B.p16.bmem = bmem16.as<int>();
    }
    up(rstart, rtab.data(), rtab.size() * 8);
    B.inst = inst.as<ChainInst>();
    B.count = count;
    B.zb = sw.zb;
    B.p4.np = np4max;
    B.p4.threads = threads4;
    B.p4.smem = smem4;
    B.p4.start = start4.as<int64_t>();
    B.p4.bmem = bmem4.as<int>();
    B.p8.np = np8max;
    B.p8.threads = threads8;
    B.p8.smem = smem8;
    B.p8.start = start8.as<int64_t>();
    B.p8.bmem = bmem8.as<int>();
    B.rstart = rstart.as<int64_t>();
    B.rmem = reinterpret_cast<const int*>(rstart.as<int64_t>() + count + 1);
    B.nrblk = nrblk;
    kmd.alloc((size_t)count * sizeof(int2));
    part.alloc((size_t)nrblk * kSweepMaxM * 8 + 64);
    Wall.alloc((size_t)count * m * m * 8);
    rot.alloc((size_t)count * sizeof(int2));
    flag.alloc((size_t)count * sizeof(int));
    yptr.alloc((size_t)count * sizeof(void*));
    slots.alloc((size_t)count * 8 * 8);
    // synchronise here: the host vectors above must outlive the copies
    TM_CK(cudaStreamSynchronize(s));
  }

  ~Wave() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
  }

  const ChainInst* I() const { return inst.as<ChainInst>(); }
  const int2* km() const { return kmd.as<int2>(); }

  int product(int mode, int theta = 0) {
    int nl = 0;
    if (mode == kModeF32) {
      sw_to_f32<<<(unsigned)nrblk, 256, 0, sw.s>>>(I(), km(), rstart.as<int64_t>(), count);
      TM_CKK("sw_to_f32");
      ++nl;
    }
    nl += chain_batch_product(B, km(), mode, sw.s, theta);
    return nl;
  }

  // one Arnoldi step of every member taking part (each at its own column)
  void step(bool f32_phase, bool df_phase, bool f64_phase) {
    cudaStream_t s = sw.s;
    const int64_t* rs = rstart.as<int64_t>();
    double* pt = part.as<double>();
    if (f32_phase) product(kModeF32);
    if (df_phase) product(kModeDF);
    if (f64_phase) product(kModeF64);
    for (int pass = 0; pass < 2; ++pass) {
      const int off = pass ? kScH2 : kScH1;
      sw_mdot<<<(unsigned)nrblk, 256, 0, s>>>(I(), km(), rs, count, pt);
      TM_CKK("sw_mdot");
      sw_reduce<<<count, 32, 0, s>>>(I(), km(), rs, pt, off);
      TM_CKK("sw_reduce");
      sw_maxpy<<<(unsigned)nrblk, 256, 0, s>>>(I(), km(), rs, count, off);
      TM_CKK("sw_maxpy");
    }
    sw_nrm<<<(unsigned)nrblk, 256, 0, s>>>(I(), km(), rs, count, pt);
    TM_CKK("sw_nrm");
    sw_hcol<<<count, 32, 0, s>>>(I(), km(), rs, m, pt);
    TM_CKK("sw_hcol");
    sw_normalize<<<(unsigned)nrblk, 256, 0, s>>>(I(), km(), rs, count);
    TM_CKK("sw_normalize");
  }

  // one step of every member, as a CUDA graph captured on first use per set
  // of product modes present
  void run_step(bool f32_phase, bool df_phase, bool f64_phase) {
    const int key = (f32_phase << 0) | (df_phase << 1) | (f64_phase << 2);
    auto it = graphs.find(key);
    if (it == graphs.end()) {
      const int64_t l0 = tm_launch_count();
      cudaGraph_t g;
      TM_CK(cudaStreamBeginCapture(sw.s, cudaStreamCaptureModeThreadLocal));
      try {
        step(f32_phase, df_phase, f64_phase);
      } catch (...) {
        cudaStreamEndCapture(sw.s, &g);
        throw;
      }
      TM_CK(cudaStreamEndCapture(sw.s, &g));
      cudaGraphExec_t ex;
      TM_CK(cudaGraphInstantiate(&ex, g, 0));
      TM_CK(cudaGraphDestroy(g));
      graph_kernels[key] = tm_launch_count() - l0;
      it = graphs.emplace(key, ex).first;
      // the kernels were counted when captured; count them per replay instead
      note_launches(-graph_kernels[key]);
    }
    TM_CK(cudaGraphLaunch(it->second, sw.s));
    note_launches(graph_kernels[key]);
  }

  // normalise V[:, 0] of the flagged members
  void normalize_starts(const std::vector<int>& fl) {
    TM_CK(cudaMemcpyAsync(flag.p, fl.data(), fl.size() * sizeof(int), cudaMemcpyHostToDevice, sw.s));
    sw_col0_nrm<<<(unsigned)nrblk, 256, 0, sw.s>>>(I(), rstart.as<int64_t>(), count, flag.as<int>(), part.as<double>());
    TM_CKK("sw_col0_nrm");
    sw_col0_scale<<<(unsigned)nrblk, 256, 0, sw.s>>>(I(), rstart.as<int64_t>(), count, flag.as<int>(),
                                                      part.as<double>());
    TM_CKK("sw_col0_scale");
  }
};

}  // namespace

// Solve every member: nev wanted eigenvalues to tol (relative), mode
// TM_EIGS_F64 or TM_EIGS_MIXED.
// vec_out (host pointers per member, or null): each member's leading
// eigenvector (real, unit norm), taken when the member converges.
void sweep_solve(Sweep& sw, int nev, int ncv, double tol, int mode, double* const* vec_out = nullptr) {
  if (nev < 1) fail(TM_ERR_ARG, "nev must be >= 1");
  int64_t nmin = INT64_MAX;
  for (auto& mb : sw.mem) nmin = std::min(nmin, mb.op->n);
  // ncv 0: the reference's suggested_nev rule, but at least 12 columns --
  // members restart less often, and over the 256-point B/7 sweep a 12-column
  // subspace took 15% fewer products than the 7 columns the rule gives at nev=2
  int m = ncv > 0 ? ncv : std::max((nev > 4) ? 2 * nev + 1 : 2 * nev + 3, 12);
  m = std::max(m, 2 * nev + 2);
  m = std::min<int64_t>(m, nmin - 1);
  if (m > kSweepMaxM - 1) fail(TM_ERR_LIMIT, "sweep subspace larger than 23");
  if (m < nev + 2) fail(TM_ERR_ARG, "operators too small for the requested eigenvalues");
  if (tol <= 0) tol = 1e-10;
  const double tol32 = std::max(tol, 3e-7);
  const int first_phase = (mode == TM_EIGS_MIXED) ? kModeF32 : kModeF64;
  const int final_phase = (mode == TM_EIGS_MIXED) ? kModeDF : kModeF64;
  const int max_cycles = (mode == TM_EIGS_MIXED) ? 200 : 300;
  for (double& v : sw.stats) v = 0.0;
  using clk = std::chrono::steady_clock;
  auto since = [](clk::time_point t) { return std::chrono::duration<double>(clk::now() - t).count(); };
  for (auto& wv : sw.waves(m)) {
    AllocStream guard(sw.s);
    const auto tw = clk::now();
    Wave W(sw, wv.first, wv.second, m);
    sw.stats[0] += 1;
    sw.stats[2] += since(tw);
    const int count = W.count;
    const auto t0 = clk::now();
    std::vector<int2> kmh(count);
    std::vector<int> fl(count, 1);
    for (int q = 0; q < count; ++q) {
      Member& mb = sw.mem[W.a + q];
      mb.phase = first_phase;
      mb.j = 0;
      mb.done = false;
      mb.info = tm_eigs_info{};
      mb.info.ncv = m;
      fill_uniform(W.host[q].V, mb.op->n, 0, sw.s);  // start vector uniform(0,1), seed 0
    }
    W.normalize_starts(fl);
    std::vector<double> sch((size_t)count * kScStride, 0.0), Wh((size_t)count * m * m, 0.0);
    std::vector<int2> roth(count);
    while (true) {
      bool ph[4] = {false, false, false, false};
      bool any = false;
      for (int q = 0; q < count; ++q) {
        Member& mb = sw.mem[W.a + q];
        const bool on = !mb.done && mb.status == TM_OK;
        kmh[q] = make_int2(mb.j, on ? mb.phase : kModeIdle);
        if (on) {
          any = true;
          ph[mb.phase] = true;
        }
      }
      if (!any) break;  // every member finished
      const auto ts = clk::now();
      TM_CK(cudaMemcpyAsync(W.kmd.p, kmh.data(), count * sizeof(int2), cudaMemcpyHostToDevice, sw.s));
      W.run_step(ph[kModeF32], ph[kModeDF], ph[kModeF64]);
      TM_CK(cudaMemcpyAsync(sch.data(), W.sc.p, sch.size() * 8, cudaMemcpyDeviceToHost, sw.s));
      TM_CK(cudaStreamSynchronize(sw.s));
      sw.stats[1] += 1;
      sw.stats[3] += since(ts);
      const auto th = clk::now();
      bool any_rot = false, any_start = false;
      std::vector<int> extract;
      for (int q = 0; q < count; ++q) {
        roth[q] = make_int2(0, 0);
        fl[q] = 0;
        Member& mb = sw.mem[W.a + q];
        if (kmh[q].y == kModeIdle) continue;
        mb.info.matvecs += 1;
        if (mb.phase != kModeF32) mb.info.matvecs_f64 += 1;
        double* Hh = sch.data() + (size_t)q * kScStride + kScH;
        if (++mb.j < m) {
          // Once the basis holds a few vectors, test the pairs after every
          // step (a Rayleigh-Ritz of the first j columns): a member in its
          // final phase stops at the first step that converges it, and one in
          // the FP32 phase moves on to the final phase as soon as it reaches
          // the FP32 floor.
          const int jc = mb.j;
          if (mb.cycles == 0 && mb.phase != final_phase) continue;  // the FP32 phase's first cycle runs whole
          if (jc < std::min(m - 1, nev + 4)) continue;
          try {
            std::vector<double> Hj((size_t)(jc + 1) * jc);
            for (int c = 0; c < jc; ++c)
              for (int i = 0; i <= jc; ++i) Hj[i + (size_t)c * (jc + 1)] = Hh[i + (size_t)c * (m + 1)];
            const Ritz R = krylov_project(Hj.data(), jc, nev);
            const bool f32 = (mb.phase != final_phase);
            const double ref = std::max(std::abs(R.theta[0]), 1e-300);
            bool ok = true;
            double mr = 0.0;
            for (int i = 0; i < nev; ++i) {
              const double ai = std::max(std::abs(R.theta[i]), 1e-300);
              if (!(R.resid[i] <= (f32 ? tol32 * ref : tol * ai))) ok = false;
              mr = std::max(mr, R.resid[i] / ai);
            }
            if (!ok) continue;
            double* Wq = Wh.data() + (size_t)q * m * m;
            if (f32) {
              // restart the final phase from the wanted Ritz vectors' real
              // parts (as at the end of a cycle)
              for (int i = 0; i < m; ++i) {
                double acc = 0.0;
                if (i < jc)
                  for (int c = 0; c < nev; ++c) acc += R.y[c][i].real();
                Wq[i] = acc;
              }
              roth[q] = make_int2(1, 0);
              fl[q] = 1;
              std::fill(Hh, Hh + (m + 1) * (m + 1), 0.0);
              mb.phase = final_phase;
              mb.j = 0;
              mb.cycles = 0;
              any_rot = any_start = true;
              continue;
            }
            mb.done = true;
            mb.info.nconv = nev;
            mb.info.max_resid = mr;
            mb.vals.assign(R.theta.begin(), R.theta.begin() + nev);
            if (vec_out && vec_out[W.a + q]) {
              const std::vector<std::complex<double>>& y0 = R.y[0];
              int kmax = 0;
              for (int i = 1; i < jc; ++i)
                if (std::abs(y0[i]) > std::abs(y0[kmax])) kmax = i;
              const std::complex<double> ph = std::conj(y0[kmax]) / std::max(std::abs(y0[kmax]), 1e-300);
              for (int i = 0; i < m; ++i) Wq[i] = (i < jc) ? (y0[i] * ph).real() : 0.0;
              roth[q] = make_int2(1, 0);
              fl[q] = 1;
              any_rot = any_start = true;
              extract.push_back(q);
            }
          } catch (const Failure& f) {
            mb.status = f.code;
            mb.msg = f.msg;
          }
          continue;
        }
        // end of this member's cycle: project, test, restart
        ++mb.cycles;
        try {
          const int kvec = krylov_kvec(m, nev);
          Ritz R = krylov_project(Hh, m, kvec);
          const double ref = std::abs(R.theta[0]);
          const bool f32 = (mb.phase == kModeF32);
          bool ok = true;
          int nconv = 0;
          double worst = 0.0;
          for (int i = 0; i < nev; ++i) {
            const double lim = f32 ? tol32 * ref : tol * std::max(std::abs(R.theta[i]), 1e-300);
            worst = std::max(worst, R.resid[i] / std::max(ref, 1e-300));
            if (R.resid[i] <= lim)
              ++nconv;
            else
              ok = false;
          }
          bool to_final = false;
          if (f32) {
            if (ok) {
              to_final = true;
            } else if (worst < 0.7 * mb.best) {
              mb.best = worst;
              mb.stall = 0;
            } else if (++mb.stall >= 3 && worst < 1e-4) {
              to_final = true;
            }
          } else if (ok) {
            mb.done = true;
            mb.info.nconv = nev;
            double mr = 0;
            for (int i = 0; i < nev; ++i) mr = std::max(mr, R.resid[i] / std::max(std::abs(R.theta[i]), 1e-300));
            mb.info.max_resid = mr;
            mb.vals.assign(R.theta.begin(), R.theta.begin() + nev);
            if (vec_out && vec_out[W.a + q]) {
              // the leading Ritz vector V y0 into column 0, y0 turned so its
              // largest component is real positive (the vector is real)
              const std::vector<std::complex<double>>& y0 = R.y[0];
              int kmax = 0;
              for (int i = 1; i < m; ++i)
                if (std::abs(y0[i]) > std::abs(y0[kmax])) kmax = i;
              const std::complex<double> ph = std::conj(y0[kmax]) / std::max(std::abs(y0[kmax]), 1e-300);
              double* Wq = Wh.data() + (size_t)q * m * m;
              for (int i = 0; i < m; ++i) Wq[i] = (y0[i] * ph).real();
              roth[q] = make_int2(1, 0);
              fl[q] = 1;
              any_rot = any_start = true;
              extract.push_back(q);
            }
            continue;
          }
          if (mb.cycles >= max_cycles) {
            mb.status = TM_ERR_NOCONV;
            mb.msg = "sweep member did not converge";
            mb.vals.assign(R.theta.begin(), R.theta.begin() + nev);
            continue;
          }
          double* Wq = Wh.data() + (size_t)q * m * m;
          if (to_final) {
            // restart from the sum of the wanted Ritz vectors' real parts with
            // FP64-accurate products (the FP32 phase's projection is only FP32
            // accurate, so it is rebuilt)
            for (int i = 0; i < m; ++i) {
              double acc = 0.0;
              for (int c = 0; c < nev; ++c) acc += R.y[c][i].real();
              Wq[i] = acc;
            }
            roth[q] = make_int2(1, 0);
            fl[q] = 1;
            std::fill(Hh, Hh + (m + 1) * (m + 1), 0.0);
            mb.phase = final_phase;
            mb.j = 0;
            mb.cycles = 0;
            any_start = true;
          } else {
            std::vector<double> Wm;
            int knew = krylov_basis(R, m, krylov_keep(m, nev, nconv, kvec), Wm);
            if (knew >= m - 1) knew = m - 2;
            std::copy(Wm.begin(), Wm.begin() + (size_t)m * knew, Wq);
            std::vector<double> Hn;
            krylov_restart_h(Hh, m, Wm, knew, R.beta, Hn);
            std::copy(Hn.begin(), Hn.end(), Hh);
            roth[q] = make_int2(knew, 1);
            mb.j = knew;
            ++mb.info.restarts;
          }
          any_rot = true;
        } catch (const Failure& f) {
          mb.status = f.code;
          mb.msg = f.msg;
        }
      }
      if (any_rot) {
        TM_CK(cudaMemcpyAsync(W.Wall.p, Wh.data(), Wh.size() * 8, cudaMemcpyHostToDevice, sw.s));
        TM_CK(cudaMemcpyAsync(W.rot.p, roth.data(), count * sizeof(int2), cudaMemcpyHostToDevice, sw.s));
        TM_CK(cudaMemcpyAsync(W.sc.p, sch.data(), sch.size() * 8, cudaMemcpyHostToDevice, sw.s));
        sw_rotate<<<(unsigned)W.nrblk, 256, 0, sw.s>>>(W.I(), W.rstart.as<int64_t>(), count, m, W.Wall.as<double>(),
                                                       W.rot.as<int2>());
        TM_CKK("sw_rotate");
        if (any_start) W.normalize_starts(fl);
        for (int q : extract)
          TM_CK(cudaMemcpyAsync(vec_out[W.a + q], W.host[q].V, (size_t)W.host[q].n * 8, cudaMemcpyDeviceToHost,
                                sw.s));
      }
      sw.stats[4] += since(th);
    }
    TM_CK(cudaStreamSynchronize(sw.s));
    const double secs = since(t0);
    for (int q = 0; q < count; ++q) sw.mem[W.a + q].info.seconds = secs;
  }
}

// y_i = T_i x_i for every member (device FP64 vectors; FP32 computed and
// widened, or double-float / FP64), one launch per pass over all members.
void sweep_product(Sweep& sw, const double* const* x, double* const* y, tm_dtype dt) {
  const int mode = (dt == TM_F32) ? kModeF32 : (dt == TM_F64_DF ? kModeDF : kModeF64);
  for (auto& wv : sw.waves(1)) {
    AllocStream guard(sw.s);
    Wave W(sw, wv.first, wv.second, 1);
    const int count = W.count;
    std::vector<int2> kmh(count, make_int2(0, mode));
    TM_CK(cudaMemcpyAsync(W.kmd.p, kmh.data(), count * sizeof(int2), cudaMemcpyHostToDevice, sw.s));
    TM_CK(cudaMemcpyAsync(W.yptr.p, x + W.a, count * sizeof(void*), cudaMemcpyHostToDevice, sw.s));
    sw_copy_in<<<(unsigned)W.nrblk, 256, 0, sw.s>>>(W.I(), W.rstart.as<int64_t>(), count,
                                                    W.yptr.as<const double* const>());
    TM_CKK("sw_copy_in");
    W.product(mode);
    TM_CK(cudaStreamSynchronize(sw.s));  // the pointer table is rewritten below
    TM_CK(cudaMemcpyAsync(W.yptr.p, y + W.a, count * sizeof(void*), cudaMemcpyHostToDevice, sw.s));
    sw_copy_out<<<(unsigned)W.nrblk, 256, 0, sw.s>>>(W.I(), W.rstart.as<int64_t>(), count, W.yptr.as<double* const>());
    TM_CKK("sw_copy_out");
    TM_CK(cudaStreamSynchronize(sw.s));
    for (int q = 0; q < count; ++q) sw.mem[W.a + q].op->matvecs++;
  }
}

// d ln(lambda_i)/d(betaJ, kappa, kappa2, h) of every member, from its right
// and left leading eigenvectors (host) and its internal eigenvalue: the
// Boltzmann-weight term 2 <g>_{lr} from one batched reduction, and the chain
// term <l, D_out (dC) D_in r> / (lambda <l, r>) from batched tangent
// products, one per parameter the step factors depend on (the same formula
// as tm_grad for one operator).
void sweep_grad(Sweep& sw, const double* const* qr, const double* const* ql, const double* lam, double* grad) {
  for (auto& wv : sw.waves(1, 16)) {
    AllocStream guard(sw.s);
    Wave W(sw, wv.first, wv.second, 1, true);
    const int count = W.count;
    auto copy_col = [&](int col, const double* const* src) {
      TM_CK(cudaMemcpyAsync(W.yptr.p, src + W.a, count * sizeof(void*), cudaMemcpyHostToDevice, sw.s));
      sw_copy_col<<<(unsigned)W.nrblk, 256, 0, sw.s>>>(W.I(), W.rstart.as<int64_t>(), count, col,
                                                       W.yptr.as<const double* const>());
      TM_CKK("sw_copy_col");
      TM_CK(cudaStreamSynchronize(sw.s));  // the pointer table is rewritten next
    };
    copy_col(0, qr);
    copy_col(1, ql ? ql : qr);
    std::vector<double> sums((size_t)count * 8);
    auto slot_sums = [&](int dot_w) {
      sw_grad_sums<<<(unsigned)W.nrblk, 256, 0, sw.s>>>(W.I(), W.rstart.as<int64_t>(), count, dot_w,
                                                        W.part.as<double>());
      TM_CKK("sw_grad_sums");
      sw_sum_slots<<<count, 32, 0, sw.s>>>(W.rstart.as<int64_t>(), W.part.as<double>(), W.slots.as<double>());
      TM_CKK("sw_sum_slots");
      TM_CK(cudaMemcpyAsync(sums.data(), W.slots.p, sums.size() * 8, cudaMemcpyDeviceToHost, sw.s));
      TM_CK(cudaStreamSynchronize(sw.s));
    };
    slot_sums(0);
    std::vector<double> wsum(count);
    for (int q = 0; q < count; ++q) {
      wsum[q] = sums[(size_t)q * 8 + 4];
      for (int t = 0; t < 4; ++t) grad[(size_t)(W.a + q) * 4 + t] = 2.0 * sums[(size_t)q * 8 + t] / wsum[q];
    }
    for (int t = 0; t < 3; ++t) {
      if (t == 2 && !sw.zb) break;  // DNNI steps do not depend on kappa2
      std::vector<int2> kmh(count, make_int2(0, kModeTangent));
      TM_CK(cudaMemcpyAsync(W.kmd.p, kmh.data(), count * sizeof(int2), cudaMemcpyHostToDevice, sw.s));
      W.product(kModeTangent, t);
      slot_sums(1);
      for (int q = 0; q < count; ++q)
        grad[(size_t)(W.a + q) * 4 + t] += sums[(size_t)q * 8 + 5] / (lam[W.a + q] * wsum[q]);
    }
  }
}

bool sweep_supported(const Op& o) { return o.kind == K_ZBM || o.kind == K_ZBT || o.kind == K_XDM || o.kind == K_XDT; }

Sweep* sweep_create(const tm_params* params, int count, char model, int dim, int axialdir, int ec) {
  if (!params || count < 1) fail(TM_ERR_ARG, "a sweep needs at least one parameter point");
  std::unique_ptr<Sweep> sw(new Sweep());
  sw->model = model;
  sw->dim = dim;
  sw->axialdir = axialdir;
  sw->ec = ec;
  TM_CK(cudaStreamCreateWithFlags(&sw->s, cudaStreamNonBlocking));
  sw->mem.resize(count);
  {
    BatchMemberScope scope;
    for (int i = 0; i < count; ++i) {
      sw->mem[i].op.reset(create_op(&params[i], model, dim, axialdir, ec));
      if (!sweep_supported(*sw->mem[i].op))
        fail(TM_ERR_UNSUPPORTED, "sweeps cover the aux-bit operators (models B and D)");
    }
  }
  sw->zb = (sw->mem[0].op->kind == K_ZBM || sw->mem[0].op->kind == K_ZBT);
  TM_CK(cudaDeviceSynchronize());  // tables were built on the members' own streams
  return sw.release();
}

}  // namespace ltm

using namespace ltm;

struct tm_sweep {
  ltm::Sweep* impl;
};

#define SW_BEGIN try {
#define SW_END                           \
  }                                      \
  catch (const Failure& f) {             \
    set_error(f.msg);                    \
    return f.code;                       \
  }                                      \
  catch (const std::exception& e) {      \
    set_error(e.what());                 \
    return TM_ERR_CUDA;                  \
  }                                      \
  return TM_OK;

extern "C" {

tm_status tm_sweep_create(const tm_params* params, int count, char model, int dim, int axialdir, int extend_cond,
                          tm_sweep** out) {
  SW_BEGIN
  if (!out) fail(TM_ERR_ARG, "null output");
  *out = nullptr;
  Sweep* s = sweep_create(params, count, model, dim, axialdir, extend_cond);
  *out = new tm_sweep{s};
  SW_END
}

tm_status tm_sweep_destroy(tm_sweep* sw) {
  SW_BEGIN
  if (!sw) return TM_OK;
  delete sw->impl;
  delete sw;
  SW_END
}

int tm_sweep_count(const tm_sweep* sw) { return sw ? (int)sw->impl->mem.size() : -1; }

int64_t tm_sweep_rows(const tm_sweep* sw, int i) {
  if (!sw || i < 0 || i >= (int)sw->impl->mem.size()) return -1;
  return sw->impl->mem[i].op->n;
}

double tm_sweep_normfactor(const tm_sweep* sw, int i) {
  if (!sw || i < 0 || i >= (int)sw->impl->mem.size()) return 0.0;
  return sw->impl->mem[i].op->normfactor;
}

tm_status tm_sweep_set_wave_bytes(tm_sweep* sw, size_t bytes) {
  SW_BEGIN
  if (!sw) fail(TM_ERR_ARG, "null sweep");
  sw->impl->budget_override = bytes;
  SW_END
}

tm_status tm_sweep_set_transpose(tm_sweep* sw, int transpose) {
  SW_BEGIN
  if (!sw) fail(TM_ERR_ARG, "null sweep");
  sw->impl->dir = transpose ? 1 : 0;
  SW_END
}

tm_status tm_sweep_grad(tm_sweep* sw, const double* const* qr_host, const double* const* ql_host,
                        const double* lambda_internal, double* grad4) {
  SW_BEGIN
  if (!sw || !qr_host || !lambda_internal || !grad4) fail(TM_ERR_ARG, "null argument");
  if (sw->impl->dir) fail(TM_ERR_ARG, "gradients are taken on the sweep of the operators, not of their transposes");
  for (auto& mb : sw->impl->mem)
    if (!mb.op->symmetric && !ql_host) fail(TM_ERR_ARG, "general operators need the left eigenvectors");
  for (int i = 0; i < (int)sw->impl->mem.size(); ++i)
    if (!(lambda_internal[i] != 0.0) || !std::isfinite(lambda_internal[i]))
      fail(TM_ERR_ARG, "eigenvalues must be finite and nonzero");
  sweep_grad(*sw->impl, qr_host, ql_host, lambda_internal, grad4);
  SW_END
}

int tm_sweep_stats(const tm_sweep* sw, double* out, int cap) {
  if (!sw || !out) return 0;
  int n = 0;
  for (; n < cap && n < 5; ++n) out[n] = sw->impl->stats[n];
  return n;
}

tm_status tm_sweep_perform_op_dev(tm_sweep* sw, const double* const* x_dev, double* const* y_dev, tm_dtype dtype) {
  SW_BEGIN
  if (!sw || !x_dev || !y_dev) fail(TM_ERR_ARG, "null argument");
  if (dtype != TM_F32 && dtype != TM_F64 && dtype != TM_F64_DF) fail(TM_ERR_ARG, "bad dtype");
  sweep_product(*sw->impl, x_dev, y_dev, dtype);
  SW_END
}

static tm_status sweep_eigs_impl(tm_sweep* sw, int nev, int ncv, double tol, int mode, double* vals_re,
                                 double* vals_im, double* const* vec0, tm_eigs_info* infos, tm_status* status);

tm_status tm_sweep_eigs(tm_sweep* sw, int nev, int ncv, double tol, int mode, double* vals_re, double* vals_im,
                        tm_eigs_info* infos, tm_status* status) {
  return sweep_eigs_impl(sw, nev, ncv, tol, mode, vals_re, vals_im, nullptr, infos, status);
}

tm_status tm_sweep_eigs_vec(tm_sweep* sw, int nev, int ncv, double tol, int mode, double* vals_re, double* vals_im,
                            double* const* vec0_host, tm_eigs_info* infos, tm_status* status) {
  return sweep_eigs_impl(sw, nev, ncv, tol, mode, vals_re, vals_im, vec0_host, infos, status);
}

static tm_status sweep_eigs_impl(tm_sweep* sw, int nev, int ncv, double tol, int mode, double* vals_re,
                                 double* vals_im, double* const* vec0, tm_eigs_info* infos, tm_status* status) {
  SW_BEGIN
  if (!sw || !vals_re || !vals_im) fail(TM_ERR_ARG, "null argument");
  if (mode != TM_EIGS_F64 && mode != TM_EIGS_MIXED) fail(TM_ERR_ARG, "bad mode");
  Sweep& s = *sw->impl;
  for (auto& mb : s.mem) {
    mb.status = TM_OK;
    mb.msg.clear();
    mb.vals.clear();
    mb.best = 1e300;
    mb.stall = 0;
    mb.cycles = 0;
  }
  sweep_solve(s, nev, ncv, tol, mode, vec0);
  tm_status first = TM_OK;
  for (int i = 0; i < (int)s.mem.size(); ++i) {
    Member& mb = s.mem[i];
    const double nf = mb.op->normfactor;
    for (int c = 0; c < nev; ++c) {
      const std::complex<double> z = c < (int)mb.vals.size() ? mb.vals[c] : std::complex<double>(0.0, 0.0);
      vals_re[(size_t)i * nev + c] = z.real() / nf;
      vals_im[(size_t)i * nev + c] = z.imag() / nf;
    }
    mb.op->matvecs += mb.info.matvecs;
    if (infos) infos[i] = mb.info;
    if (status) status[i] = mb.status;
    if (mb.status != TM_OK && first == TM_OK) {
      first = mb.status;
      set_error("sweep member " + std::to_string(i) + ": " + mb.msg);
    }
  }
  return first;
  SW_END
}

tm_status tm_chain_autotune(const tm_op* op, tm_dtype dtype, int* tile_bits, int* threads, double* ms) {
  SW_BEGIN
  if (!op) fail(TM_ERR_ARG, "null operator");
  if (dtype != TM_F32 && dtype != TM_F64_DF) fail(TM_ERR_ARG, "the autotuner times TM_F32 or TM_F64_DF products");
  int tb = 0, th = 0;
  double t = 0;
  chain_autotune(*op->impl, dtype, tb, th, t);
  if (tile_bits) *tile_bits = tb;
  if (threads) *threads = th;
  if (ms) *ms = t;
  SW_END
}

tm_status tm_chain_set_tuning(char model, int L, tm_dtype dtype, int tile_bits, int threads) {
  SW_BEGIN
  if (model != 'B' && model != 'D') fail(TM_ERR_ARG, "model must be B or D");
  chain_set_tuning(L, dtype == TM_F32 ? 4 : 8, model == 'B', tile_bits, threads);
  SW_END
}

}  // extern "C"
