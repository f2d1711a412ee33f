// Eigenvector observables as fused weighted reductions on the GPU.
//
// Restates the reference's moments / phys_extend loops (TMat/tmatphys.cpp:13-135,
// TMat/tmatreduce.cpp:565-613, 882-909, 1261-1320, 1748-1775,
// TMat/tmat3d.cpp:137-163): for each basis state s with weight w = ql*qr
// (q^2 for symmetric operators), accumulate w*M^k (M = 2*popcount(s) - L),
// sum w, w*nnode, w*nnode^2 and the DNNI stripe magnetisations.
#include <cmath>
#include <vector>

#include "tm_internal.h"

namespace ltm {
namespace {

constexpr int NS = 11;

__global__ void obs_kernel(const double* __restrict__ ql, const double* __restrict__ qr, int sym,
                           const uint32_t* __restrict__ idx, int64_t n, int L, int open_bc, int lshift,
                           double* __restrict__ part) {
  double acc[NS];
  for (int k = 0; k < NS; ++k) acc[k] = 0.0;
  const uint64_t mask = (1ull << L) - 1;
  const uint64_t stripflip = 0xaaaaaaaaaaaaaaaaull;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += st) {
    // two-layer states: one layer's spins (lshift selects it)
    uint64_t s = ((idx ? (uint64_t)idx[i] : (uint64_t)i) >> lshift) & mask;
    double w = sym ? ql[i] * ql[i] : ql[i] * qr[i];
    double m = (double)(2 * popc64(s) - L);
    double mk = m;
    for (int k = 0; k < 4; ++k) {
      acc[k] += mk * w;
      mk *= m;
    }
    acc[4] += w;
    double nn = (double)nnode(s, L, open_bc);
    acc[5] += nn * w;
    acc[6] += nn * nn * w;
    double dm = (double)(2 * popc64((s ^ stripflip) & mask) - L);
    acc[7] += fabs(dm) * w;
    acc[8] += fabs(m) * w;
    acc[9] += dm * dm * w;
    acc[10] += m * m * w;
  }
  __shared__ double sh[NS][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < NS; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < NS) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[threadIdx.x][q];
    part[(int64_t)blockIdx.x * NS + threadIdx.x] = t;
  }
}

}  // namespace

void observables(const Op& op, const double* ql, const double* qr, double* sums) {
  const int64_t n = op.n;
  cudaStream_t s = op.stream;
  DBuf dl, dr, part;
  dl.alloc((size_t)n * 8);
  TM_CK(cudaMemcpyAsync(dl.p, ql, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  const double* qrd = dl.as<double>();
  if (!op.symmetric && qr != ql) {
    dr.alloc((size_t)n * 8);
    TM_CK(cudaMemcpyAsync(dr.p, qr, (size_t)n * 8, cudaMemcpyHostToDevice, s));
    qrd = dr.as<double>();
  }
  int nb = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 4));
  part.alloc((size_t)nb * NS * 8);
  const bool reduced =
      (op.kind == K_XAM || op.kind == K_XDM || op.kind == K_ZBM || op.kind == K_XAM3 || op.kind == K_YAM);
  // GenMatPhys::moments takes the low layer of the full two-layer state
  // (TMat/tmatphys.cpp:71-98), YAMMatVecProd2D::moments the left (high) layer
  // of the representative (TMat/tmatreduce.cpp:878-905)
  const int lshift = (op.kind == K_YAM) ? op.L : 0;
  // nnode boundary: the MatPhys boundary_cond each reference class passes
  // (XAT: its boundary case; XAM: extend_cond & 1; XDT, XDM: 0)
  int open_bc = 0;
  if (op.kind == K_XAT) open_bc = op.boundary != 0;
  if (op.kind == K_XAM) open_bc = op.boundary != 0;
  obs_kernel<<<nb, 256, 0, s>>>(dl.as<double>(), qrd, op.symmetric, reduced ? op.idx.as<uint32_t>() : nullptr,
                                n, op.L, open_bc, lshift, part.as<double>());
  TM_CKK("obs");
  std::vector<double> h((size_t)nb * NS);
  TM_CK(cudaMemcpyAsync(h.data(), part.p, h.size() * 8, cudaMemcpyDeviceToHost, s));
  TM_CK(cudaStreamSynchronize(s));
  for (int k = 0; k < NS; ++k) {
    double t = 0.0;
    for (int b = 0; b < nb; ++b) t += h[(size_t)b * NS + k];
    sums[k] = t;
  }
}

}  // namespace ltm
