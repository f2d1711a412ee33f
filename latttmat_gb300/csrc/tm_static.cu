// FP64 reduced x-ANNNI product that allocates nothing.
//
// Some callers cannot call cudaMalloc at the moment they need a product.
// One example is a host framework whose device memory belongs to its own
// caching allocator: a raw allocation there bypasses the framework's
// accounting and can fail once the pool holds the device. Another is a
// latency-critical loop that must not stall: cudaMalloc and cudaFree may
// synchronise the device. The regular entry points allocate their scratch
// when an operator is built. This one instead keeps its scratch in one
// file-scope device array of fixed size, reserved when the library is loaded
// and held by every GPU that loads it until the process exits. It performs
// no allocation of any kind per call.
//
// Scratch layout (doubles): x in pi order [R] | y in pi order [R] | scaled
// input u [R] | pass-1 intermediate w1 [n_orep * 2^m].  The kernels overwrite
// every element they read later, so nothing needs clearing between calls.
// The array is shared: calls that overlap on the GPU (on different streams,
// or from different threads) race on it, so callers must serialise them.
#include <mutex>

#include "tm_internal.h"

namespace ltm {

void matvec_eo_f64_into(const Op& op, const double* x, double* y, double* u, double* w1, cudaStream_t s);

namespace {

constexpr size_t kStaticScratchDoubles = size_t(1) << 21;  // 16 MiB

__device__ __align__(256) double g_static_scratch[kStaticScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_static_scratch on device `dev`, which must be the
// current device (looked up once per device, with that device current, and
// cached).
double* scratch_for_device(int dev) {
  if (dev < 0 || dev >= kMaxDevices) fail(TM_ERR_LIMIT, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    TM_CK(cudaGetSymbolAddress(&p, g_static_scratch));
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  return g_scratch_ptr[dev];
}

}  // namespace

size_t static_scratch_doubles() { return kStaticScratchDoubles; }

void perform_op_static(const Op& op, const double* x, double* y, cudaStream_t s) {
  const Op& b = op.parent ? *op.parent : op;
  if (!b.eo.active)
    fail(TM_ERR_UNSUPPORTED,
         "the fixed-scratch product covers reduced x-ANNNI operators on the even/odd path (periodic, even L >= 12)");
  const size_t R = (size_t)b.n;
  const size_t w1n = (size_t)b.eo.n_orep << b.eo.m;
  const size_t need = 3 * R + w1n;
  if (need > kStaticScratchDoubles) {
    char buf[200];
    snprintf(buf, sizeof(buf),
             "operator needs %zu doubles of scratch; the fixed scratch holds %zu (16 MiB, about L <= 24)", need,
             kStaticScratchDoubles);
    fail(TM_ERR_LIMIT, buf);
  }
  // the operator's tables live on b.device; the scratch and the launches must
  // be on that device too
  int dev = 0;
  TM_CK(cudaGetDevice(&dev));
  if (dev != b.device) {
    char buf[160];
    snprintf(buf, sizeof(buf), "the operator was created on device %d but device %d is current", b.device, dev);
    fail(TM_ERR_ARG, buf);
  }
  double* base = scratch_for_device(dev);
  double* xp = base;
  double* yp = xp + R;
  double* u = yp + R;
  double* w1 = u + R;
  const uint32_t* pi = b.pi.as<uint32_t>();
  gather_f64(x, pi, xp, (int64_t)R, s);
  matvec_eo_f64_into(b, xp, yp, u, w1, s);
  scatter_f64(yp, pi, y, (int64_t)R, s);
  const_cast<Op&>(op).matvecs++;
}

}  // namespace ltm

using namespace ltm;

extern "C" tm_status tm_perform_op_dev_noalloc(const tm_op* op, const double* x_dev, double* y_dev, void* stream) {
  try {
    if (!op || !x_dev || !y_dev) fail(TM_ERR_ARG, "null argument");
    const Op& o = *op->impl;
    const Op& b = o.parent ? *o.parent : o;
    cudaStream_t s = stream ? (cudaStream_t)stream : b.stream;
    perform_op_static(o, x_dev, y_dev, s);
    TM_CK(cudaGetLastError());
  } catch (const Failure& f) {
    set_error(f.msg);
    return f.code;
  } catch (const std::exception& e) {
    set_error(e.what());
    return TM_ERR_CUDA;
  }
  return TM_OK;
}
