// Shared-memory staging of column chunks by bulk copies (cp.async.bulk,
// global -> shared) tracked by one mbarrier per stage.
//
// The Krylov sweeps read many long columns at once (a 16-column FP32 basis at
// L = 32 is 2.1 GB).  Streamed through registers, each thread holds one
// vector of every column, so wide sweeps run out of registers before they
// have enough bytes in flight: the 16-column update-and-dot kernel held one
// 256-thread block per SM and reached 3.0 TB/s.  Staged, one thread posts
// every column's chunk as a single bulk copy, the stages keep 130-200 KB per
// SM in flight whatever the column count, and the same sweep reaches
// 6.3 TB/s.
//
// A CTA walks chunks c = blockIdx.x, blockIdx.x + gridDim.x, ... < nch.
// Stage s holds chunk j (the CTA's j-th) when j % nstage == s; its barrier
// completes phase j / nstage when the chunk's bytes have landed.  After the
// whole CTA has consumed a stage, thread 0 refills it with the chunk nstage
// further on.  Every wait is bounded: on a timeout the CTA records it in the
// error word, waits (bounded again) for its copies still in flight and
// returns.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace ltm {

constexpr int kStageMax = 8;            // stages per CTA
constexpr int kStageWaitLimit = 1 << 22;  // try_wait rounds before a stage wait gives up
// dynamic shared memory the staged kernels may fill with stages
constexpr int kStageBytes = 220 * 1024;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

// one arrival that also announces `bytes` of copies to come
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* b, uint32_t parity) {
  for (int it = 0; it < kStageWaitLimit; ++it)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}

// Runs the CTA's chunks through `nstage` stages.  issue(c, s, bar) runs on
// thread 0: it posts chunk c's copies into stage s and arms bar with their
// byte count (mbar_arrive_expect_tx before the copies).  consume(c, s) runs
// on every thread once chunk c is in stage s.  Returns false after a timed
// out wait (the error word set, the copies in flight drained).
template <class Issue, class Consume>
__device__ __forceinline__ bool staged_sweep(uint64_t* full, int nstage, int64_t nch, int* err, Issue&& issue,
                                             Consume&& consume) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < nstage; ++s) mbar_init(&full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int j = 0; j < nstage; ++j) {
      const int64_t c = blockIdx.x + (int64_t)j * gridDim.x;
      if (c < nch) issue(c, j, &full[j]);
    }
  }
  __syncthreads();
  int j = 0;
  for (int64_t c = blockIdx.x; c < nch; c += gridDim.x, ++j) {
    const int s = j % nstage;
    const bool ok = mbar_wait_bounded(&full[s], (uint32_t)((j / nstage) & 1));
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(err, 1);
        for (int q = 0; q < nstage; ++q) {
          const int jq = j + q;
          if (blockIdx.x + (int64_t)jq * gridDim.x < nch)
            mbar_wait_bounded(&full[jq % nstage], (uint32_t)((jq / nstage) & 1));
        }
      }
      return false;
    }
    consume(c, s);
    __syncthreads();  // every thread is done with stage s
    if (threadIdx.x == 0) {
      const int64_t c2 = c + (int64_t)nstage * gridDim.x;
      if (c2 < nch) issue(c2, s, &full[s]);
    }
  }
  return true;
}

// Host side: the device error word of the staged kernels (one per device,
// zeroed at first use), and a check that raises TM_ERR_CUDA, and clears the
// word, if a stage wait timed out since the last check.
int* stage_err_word();
void stage_err_check(cudaStream_t s);
// stages of `chunk_bytes` bytes (all columns of one chunk) that fit kStageBytes, 2..kStageMax
int stage_count(int64_t chunk_bytes);

}  // namespace ltm
