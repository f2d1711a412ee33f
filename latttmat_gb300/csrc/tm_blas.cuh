// Device vector kernels for the Krylov solvers: fused multi-vector dot
// products and updates over a column-major basis V (leading dimension ldv).
// Each entry point runs 16-byte vector forms when every column it touches
// starts on a 16-byte boundary, and element-wise forms otherwise.
#pragma once
#include "tm_df.cuh"
#include "tm_internal.h"
#include "tm_stage.cuh"

namespace ltm {

// h[k] = sum_i V[k][i] * w[i], k < nv  (two-stage reduction)
void mdot(const double* V, int64_t ldv, int nv, const double* w, int64_t n, double* h_dev,
          double* part, cudaStream_t s);
// h[k] = sum_i V[k][i] * scale * (double)w32[i]  (FP32 right-hand side)
void mdot32(const double* V, int64_t ldv, int nv, const float* w32, double scale, int64_t n,
            double* h_dev, double* part, cudaStream_t s);
// w[i] -= sum_k V[k][i] * h[k]; optionally also accumulates hsum[k] += h[k]
void maxpy(const double* V, int64_t ldv, int nv, const double* h_dev, double* w, int64_t n,
           cudaStream_t s);
// w = scale * (double) w32, then w -= V h  (fused first CGS update)
void maxpy32(const double* V, int64_t ldv, int nv, const double* h_dev, const float* w32, double scale,
             double* w, int64_t n, cudaStream_t s);
// out = ||w||^2 on device
void nrm2sq(const double* w, int64_t n, double* out_dev, double* part, cudaStream_t s);
// v = w / sqrt(*nsq_dev); also writes v32 = (float)v when v32 != nullptr
void normalize(const double* w, const double* nsq_dev, double* v, float* v32, int64_t n, cudaStream_t s);
// X[:, 0..k) = V[:, 0..m) * Y[0..m, 0..k)  in place, row-wise (Y on device, column-major m x k)
void basis_rotate(double* V, int64_t ldv, int m, const double* Y_dev, int k, int64_t n, cudaStream_t s);
// out[:, 0..k) = V[:, 0..m) * Y[0..m, 0..k)  (out-of-place; out columns spaced ldo)
void basis_combine(const double* V, int64_t ldv, int m, const double* Y_dev, int k, double* out, int64_t ldo,
                   int64_t n, cudaStream_t s);
// out = (float) in
void to_f32(const double* in, float* out, int64_t n, cudaStream_t s);
// out = a*x + b*y
void axpby(double a, const double* x, double b, const double* y, double* out, int64_t n, cudaStream_t s);
// uniform(0,1) start vector from splitmix64(seed ^ index)
void fill_uniform(double* v, int64_t n, uint64_t seed, cudaStream_t s);
// count of non-finite entries (device counter)
void count_nonfinite(const double* v, int64_t n, unsigned int* cnt_dev, cudaStream_t s);

// Leading dimension of a Krylov basis of length-n columns: columns start on
// 256-byte boundaries, so the 16-byte vector forms of the kernels apply.
inline int64_t col_ld(int64_t n) { return (n + 63) & ~(int64_t)63; }

// ---- FP32-basis Krylov kernels (nv <= 16): FP32 data, per-thread FP32
// partial sums, FP64 block/global reductions.
constexpr int NV32 = 16;
// h[k] = sum_i V[k][i] w[i]
void mdot_f32(const float* V, int64_t ldv, int nv, const float* w, int64_t n, double* h, double* part,
              cudaStream_t s);
// Reduction kernels run at most kRedBlocksPerSM blocks of 256 threads per SM;
// their partial-sum buffers need red_part_bytes(values per block).
constexpr int kRedBlocksPerSM = 8;
size_t red_part_bytes(int width);

// Block forms over up to 8 FP32 vectors at once (one sweep over V serves all
// of them).  H is column-major with leading dimension ldh: H[k + j*ldh] =
// V[k] . W[j]; part needs mdot_block_part_bytes().
constexpr int kMaxBlockW = 8;
struct F32Cols {
  const float* c[kMaxBlockW];
};
struct F32ColsMut {
  float* c[kMaxBlockW];
};
void mdot_block_f32(const float* V, int64_t ldv, int nv, const F32Cols& W, int nw, int64_t n, double* H,
                    int64_t ldh, double* part, cudaStream_t s);
// W[j] -= sum_k V[k] H[k + j*ldh]
void maxpy_block_f32(const float* V, int64_t ldv, int nv, const double* H, int64_t ldh, const F32ColsMut& W, int nw,
                     int64_t n, cudaStream_t s);
size_t mdot_block_part_bytes();
// H[k + j*ldh] = V[k] . W[j] with FP64 columns V and up to 4 FP32 vectors W,
// in FP64 (the FP32 values are exact in FP64)
void mdot64_block(const double* V, int64_t ldv, int nv, const F32Cols& W, int nw, int64_t n, double* H,
                  int64_t ldh, double* part, cudaStream_t s);
// w -= V h (FP32 data and arithmetic), any nv (chunks of NV32)
void maxpy_f32(const float* V, int64_t ldv, int nv, const double* h, float* w, int64_t n, cudaStream_t s);
// wout = win - V h ; h2[k] = sum_i V[k][i] wout[i]   (one pass)
void axpy_dot_f32(const float* V, int64_t ldv, int nv, const double* h, const float* win, float* wout, int64_t n,
                  double* h2, double* part, cudaStream_t s);
// w -= V h (in place) ; nsq = ||w||^2   (one pass)
void axpy_nrm_f32(const float* V, int64_t ldv, int nv, const double* h, float* w, int64_t n, double* nsq,
                  double* part, cudaStream_t s);
// v = w / sqrt(*nsq)
void normalize_f32(const float* w, const double* nsq, float* v, int64_t n, cudaStream_t s);
// V[:, 0..k) = V[:, 0..m) Y in place (FP32 storage), m <= 32
void rotate_f32(float* V, int64_t ldv, int m, const double* Y, int k, int64_t n, cudaStream_t s);
// out64[:, 0..k) = V32[:, 0..m) Y  (FP64 accumulation), m <= 32
void combine_f32_f64(const float* V, int64_t ldv, int m, const double* Y, int k, double* out, int64_t ldo, int64_t n,
                     cudaStream_t s);
// out[:, c] = V Y[:, c] with FP32 data and arithmetic (m <= 32)
void combine_f32(const float* V, int64_t ldv, int m, const double* Y, int k, float* out, int64_t ldo, int64_t n,
                 cudaStream_t s);
// uniform(0,1) FP32 start vector
void fill_uniform_f32(float* v, int64_t n, uint64_t seed, cudaStream_t s);
// ||w||^2 of an FP32 vector (FP64 result on device)
void nrm2sq_f32(const float* w, int64_t n, double* out, double* part, cudaStream_t s);

// ---- double-float vectors ((hi, lo) FP32 pairs, 8 bytes per element;
// columns 16-byte aligned, leading dimension even).  Dot products return
// FP64; part needs dd_part_bytes(8).
size_t dd_part_bytes(int width);
// h[k] = V[k] . w, k < nv <= 8
void mdot_dd(const dfloat* V, int64_t ldv, int nv, const dfloat* w, int64_t n, double* h, double* part,
             cudaStream_t s);
// w -= V h  (nv <= 8, h FP64 on the device)
void maxpy_dd(const dfloat* V, int64_t ldv, int nv, const double* h, dfloat* w, int64_t n, cudaStream_t s);
// *out = ||w||^2
void nrm2sq_dd(const dfloat* w, int64_t n, double* out, double* part, cudaStream_t s);
// out = a x + b y  (b = 0: y unused; out may alias x)
void axpby_dd(double a, const dfloat* x, double b, const dfloat* y, dfloat* out, int64_t n, cudaStream_t s);
// w /= sqrt(*nsq)
void normalize_dd(dfloat* w, const double* nsq, int64_t n, cudaStream_t s);
// out[:, c] = V32[:, 0..m) Y[:, c], c < k <= 8, in double-float (Y FP64 on the device)
void combine_f32_dd(const float* V, int64_t ldv, int m, const double* Y, int k, dfloat* out, int64_t ldo, int64_t n,
                    cudaStream_t s);
// H[k + j*ldh] = V[k] . W[j]: V double-float columns, up to 4 FP32 vectors W
void mdot_dd_block(const dfloat* V, int64_t ldv, int nv, const F32Cols& W, int nw, int64_t n, double* H, int64_t ldh,
                   double* part, cudaStream_t s);
// G[i + j*nx] = V[i] . V[j] for i < nx <= 4, j < ny <= 8 (the first nx of
// ny contiguous double-float columns against all of them) in one sweep
void mdot_dd_gram(const dfloat* V, int64_t ldv, int nx, int ny, int64_t n, double* G, double* part, cudaStream_t s);
// V[:, c] = sum_j V[:, j] Y[c*k + j], c < k <= 4, in place (Y FP64 on the device)
void combine_dd_inplace(dfloat* V, int64_t ldv, int k, const double* Y, int64_t n, cudaStream_t s);
// conversions: out = fl32(x); out = x * scale (FP64); out = x * scale (double-float)
void df_to_f32(const dfloat* x, float* out, int64_t n, cudaStream_t s);
void df_to_f64(const dfloat* x, double scale, double* out, int64_t n, cudaStream_t s);
void f64_to_df(const double* x, double scale, dfloat* out, int64_t n, cudaStream_t s);

// small dense symmetric eigenproblem on device (one warp, cyclic Jacobi, m <= 48):
// A (m x m column-major, symmetric) -> eigenvalues w[m], eigenvectors Z (m x m, column-major)
// (lda = leading dimension of A)
void small_symeig(const double* A_dev, int m, double* w_dev, double* Z_dev, cudaStream_t s, int lda);

}  // namespace ltm
