// Parameter sweeps: many independent operators solved together.
//
// The reference runs one parameter point per tmat invocation (TMat/main.cpp,
// TMat/pfunc.cpp:16-106): build the operator, solve, write the outputs.  A
// sweep over (betaJ, kappa, h, L) points is that loop run many times.
//
// Aux-bit operators (models B and D) run as one device batch (tm_sweep.cu):
// every chain pass is one launch over all points' tiles, and every point
// extends its Arnoldi basis by one column per step (one CUDA graph per step),
// restarting on its own.  The other operator
// families run on a pool of host threads, each building, solving and
// releasing one operator at a time on that operator's own CUDA stream, so the
// kernels of different points overlap on the GPU.  Device memory is
// allocated stream-ordered, so one point's frees do not stall the others.
#include <algorithm>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "tm_internal.h"

using namespace ltm;

extern "C" tm_status tm_eigs_batch(const tm_params* params, int count, char model, int dim, int axialdir,
                                   int extend_cond, int nev, double tol, int mode, int nthreads, double* vals_re,
                                   double* vals_im, tm_eigs_info* infos, tm_status* status) {
  if (!params || count < 0 || nev < 1 || !vals_re || !vals_im) {
    set_error("tm_eigs_batch: bad argument");
    return TM_ERR_ARG;
  }
  if (count == 0) return TM_OK;
  const bool aux = (model == 'B' && (axialdir == 3 || axialdir == 7)) ||
                   (model == 'D' && dim == 2 &&
                    (axialdir == 1 || axialdir == 2 || axialdir == 5 || axialdir == 6 || axialdir == 17 ||
                     axialdir == 18));
  if (aux) {
    tm_sweep* sw = nullptr;
    tm_status c = tm_sweep_create(params, count, model, dim, axialdir, extend_cond, &sw);
    if (c != TM_OK) {
      if (status)
        for (int i = 0; i < count; ++i) status[i] = c;
      return c;
    }
    c = tm_sweep_eigs(sw, nev, 0, tol, mode, vals_re, vals_im, infos, status);
    const std::string err = tm_last_error();
    tm_sweep_destroy(sw);
    if (c != TM_OK) set_error(err);
    return c;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    set_error("tm_eigs_batch: no CUDA device");
    return TM_ERR_CUDA;
  }
  if (nthreads <= 0) nthreads = 16;
  nthreads = std::min(nthreads, count);
  std::atomic<int> next{0};
  std::vector<tm_status> st(count, TM_OK);
  std::vector<std::string> msg(count);
  auto worker = [&]() {
    cudaSetDevice(dev);
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= count) break;
      tm_op* op = nullptr;
      tm_status c = tm_create(&params[i], model, dim, axialdir, extend_cond, &op);
      if (c == TM_OK)
        c = tm_eigs(op, nev, 0, tol, 0, mode, vals_re + (size_t)i * nev, vals_im + (size_t)i * nev, nullptr,
                    nullptr, infos ? &infos[i] : nullptr);
      if (c != TM_OK) msg[i] = tm_last_error();
      if (op) tm_destroy(op);
      st[i] = c;
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
  tm_status first = TM_OK;
  for (int i = 0; i < count; ++i) {
    if (status) status[i] = st[i];
    if (st[i] != TM_OK && first == TM_OK) {
      first = st[i];
      set_error("instance " + std::to_string(i) + ": " + msg[i]);
    }
  }
  return first;
}
