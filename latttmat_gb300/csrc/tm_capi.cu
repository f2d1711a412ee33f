// C ABI of liblatttmat_gb300: operator construction (the dispatch of
// TMat/pfunc.cpp:16-106), matvec entry points, orbit tables, observables and
// the eigensolver front end.
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <future>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "tm_blas.cuh"
#include "tm_internal.h"

namespace ltm {

// ------------------------------------------------------------------ errors
static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
void fail(tm_status code, const std::string& msg) { throw Failure{code, msg}; }
void check_cuda(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    char buf[512];
    snprintf(buf, sizeof(buf), "CUDA error %s (%d) in %s at %s:%d", cudaGetErrorString(e), (int)e, what, file, line);
    throw Failure{e == cudaErrorMemoryAllocation ? TM_ERR_NOMEM : TM_ERR_CUDA, buf};
  }
}

static std::atomic<int64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
// kernels replayed inside a CUDA graph (or taken back when counted at capture)
void note_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// The attribute belongs to the current device, so the cache is kept per
// (device, kernel).
void raise_smem_limit(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::unordered_map<const void*, size_t> cur[64];
  int dev = 0;
  TM_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) fail(TM_ERR_LIMIT, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  size_t& c = cur[dev][kernel];
  if (bytes <= c) return;
  TM_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  c = bytes;
}

static thread_local cudaStream_t g_alloc_stream = nullptr;
AllocStream::AllocStream(cudaStream_t s) : prev(g_alloc_stream) { g_alloc_stream = s; }
AllocStream::~AllocStream() { g_alloc_stream = prev; }

// The device's default memory pool backs the stream-ordered buffers.  It
// keeps freed memory for reuse (release threshold raised once per device), so
// repeated solves do not map and unmap tens of GB each time; an allocation
// that fails trims the pool and retries once.
static void pool_setup(int dev) {
  static std::mutex mu;
  static bool done[64] = {false};
  std::lock_guard<std::mutex> lock(mu);
  if (dev < 0 || dev >= 64 || done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev] = true;
}

static std::atomic<int64_t> g_allocs{0};

void DBuf::alloc(size_t b) {
  release();
  if (b == 0) b = 16;
  g_allocs.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e;
  if (g_alloc_stream) {
    int dev = 0;
    cudaGetDevice(&dev);
    pool_setup(dev);
    e = cudaMallocAsync(&p, b, g_alloc_stream);
    if (e == cudaErrorMemoryAllocation) {
      (void)cudaGetLastError();
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        cudaStreamSynchronize(g_alloc_stream);
        cudaMemPoolTrimTo(pool, 0);
      }
      e = cudaMallocAsync(&p, b, g_alloc_stream);
    }
    st = g_alloc_stream;
  } else {
    e = cudaMalloc(&p, b);
    st = nullptr;
  }
  if (e != cudaSuccess) {
    p = nullptr;
    (void)cudaGetLastError();
    char buf[160];
    snprintf(buf, sizeof(buf), "device allocation of %zu bytes failed (%s)", b, cudaGetErrorString(e));
    throw Failure{TM_ERR_NOMEM, buf};
  }
  bytes = b;
}
void DBuf::release() {
  if (p) {
    if (st)
      cudaFreeAsync(p, st);
    else
      cudaFree(p);
  }
  p = nullptr;
  st = nullptr;
  bytes = 0;
}

// ------------------------------------------------------------------ dispatch
template <class T>
double matvec_bfly(const Op& op, const T* x, T* y, bool scaled, cudaStream_t s);
template <class T>
void matvec_eo(const Op& op, const T* x, T* y, bool scaled32, cudaStream_t s);
double eo_scale32(const Op& op);
template <class T>
double matvec_aux(const Op& op, const T* x, T* y, bool scaled, cudaStream_t s);
tm_status lanczos_solve(const Op& op, int nev, int ncv, double tol, uint64_t seed, int mode, double* vals,
                        double* vecs_host, tm_eigs_info* info_out);
void observables(const Op& op, const double* ql, const double* qr, double* sums /* 12 */);
void adjoint_grad(const Op& op, const double* qr_h, const double* ql_h, double lam, double grad[4]);
tm_status arnoldi_solve(const Op& op, int nev, int ncv, double tol, uint64_t seed, int mode,
                        std::vector<std::complex<double>>& vals, std::vector<double>* vr, std::vector<double>* vi,
                        tm_eigs_info* info_out);

static bool is_reduced(int kind) {
  return kind == K_XAM || kind == K_XDM || kind == K_ZBM || kind == K_XAM3 || kind == K_YAM;
}
static bool bfly_core(int kind) { return kind == K_XAT || kind == K_XAM || kind == K_XAM3; }

void matvec_eo_df(const Op& op, const double* x, double* y, cudaStream_t s);
void matvec_aux_df(const Op& op, const double* x, double* y, cudaStream_t s);
double apply_internal(const Op& op, const double* x, double* y, const float* x32, float* y32, bool f32,
                      cudaStream_t s);

// FP64-accurate product for the solver's refinement steps: double-float
// arithmetic on the FP32 pipes for the even/odd and aux-bit operators (GB300's
// FP64 rate is a small fraction of its FP32 rate), native FP64 otherwise.
void apply_refine(const Op& op, const double* x, double* y, cudaStream_t s) {
  const Op& base = op.parent ? *op.parent : op;
  if (base.eo.active) {
    matvec_eo_df(base, x, y, s);
    const_cast<Op&>(op).matvecs++;
  } else if (base.kind == K_XDT || base.kind == K_XDM || base.kind == K_ZBT || base.kind == K_ZBM) {
    matvec_aux_df(op, x, y, s);
    const_cast<Op&>(op).matvecs++;
  } else {
    apply_internal(op, x, y, nullptr, nullptr, false, s);
  }
}

void matvec_eo_dd(const Op& op, const dfloat* x, dfloat* y, cudaStream_t s);

// y = A x / S in double-float storage, FP64-accurate: the even/odd engine
// reads and writes double-float directly (its output scale is S); other
// operators go through FP64 storage around apply_refine.
void apply_refine_dd(const Op& op, const dfloat* x, dfloat* y, double S, cudaStream_t s) {
  const Op& base = op.parent ? *op.parent : op;
  if (base.eo.active && S == eo_scale32(base)) {
    matvec_eo_dd(base, x, y, s);
    const_cast<Op&>(op).matvecs++;
    return;
  }
  const int64_t n = base.n;
  DBuf x64, y64;
  x64.alloc((size_t)n * 8);
  y64.alloc((size_t)n * 8);
  df_to_f64(x, 1.0, x64.as<double>(), n, s);
  apply_refine(op, x64.as<double>(), y64.as<double>(), s);
  f64_to_df(y64.as<double>(), 1.0 / S, y, n, s);
}

double apply_internal(const Op& op, const double* x, double* y, const float* x32, float* y32, bool f32,
                      cudaStream_t s) {
  const Op& base = op.parent ? *op.parent : op;
  double S = 1.0;
  if (base.eo.active) {
    if (f32) {
      matvec_eo<float>(base, x32, y32, true, s);
      S = eo_scale32(base);
    } else {
      matvec_eo<double>(base, x, y, false, s);
    }
  } else if (is_two_layer(base.kind)) {
    if (f32) fail(TM_ERR_UNSUPPORTED, "two-layer operators run in FP64 only");
    matvec_two_layer(op, x, y, s);
  } else if (bfly_core(base.kind)) {
    S = f32 ? matvec_bfly<float>(base, x32, y32, true, s) : matvec_bfly<double>(base, x, y, false, s);
  } else {
    S = f32 ? matvec_aux<float>(op, x32, y32, true, s) : matvec_aux<double>(op, x, y, false, s);
  }
  const_cast<Op&>(op).matvecs++;
  return S;
}

// public matvec in the reference's vector order (dt = FP64 or FP32)
void matvec_ref_order(const Op& op, const void* x, void* y, tm_dtype dt, cudaStream_t s) {
  const Op& base = op.parent ? *op.parent : op;
  const int64_t n = base.n;
  const bool aux_df = base.kind == K_XDT || base.kind == K_XDM || base.kind == K_ZBT || base.kind == K_ZBM;
  // TM_F64_DF: FP64 values in double-float arithmetic where an engine for it
  // exists (even/odd and aux-bit operators), native FP64 otherwise
  if (dt == TM_F64_DF && !base.eo.active && !aux_df) dt = TM_F64;
  if (is_two_layer(base.kind)) {
    if (dt != TM_F64) fail(TM_ERR_UNSUPPORTED, "two-layer operators run in FP64 only");
    matvec_two_layer(op, (const double*)x, (double*)y, s);
  } else if (dt == TM_F64_DF && !base.has_pi) {
    if (base.eo.active)
      matvec_eo_df(base, (const double*)x, (double*)y, s);
    else
      matvec_aux_df(op, (const double*)x, (double*)y, s);
  } else if (!base.has_pi) {
    if (dt == TM_F64) {
      if (base.eo.active) {
        matvec_eo<double>(base, (const double*)x, (double*)y, false, s);
      } else if (bfly_core(base.kind)) {
        matvec_bfly<double>(base, (const double*)x, (double*)y, false, s);
      } else {
        matvec_aux<double>(op, (const double*)x, (double*)y, false, s);
      }
    } else {
      if (bfly_core(base.kind))
        matvec_bfly<float>(base, (const float*)x, (float*)y, false, s);
      else
        matvec_aux<float>(op, (const float*)x, (float*)y, false, s);
    }
  } else {
    const uint32_t* pi = base.pi.as<uint32_t>();
    if (dt != TM_F32) {
      gather_f64((const double*)x, pi, base.xp.as<double>(), n, s);
      if (dt == TM_F64_DF)
        matvec_eo_df(base, base.xp.as<double>(), base.yp.as<double>(), s);
      else
        matvec_eo<double>(base, base.xp.as<double>(), base.yp.as<double>(), false, s);
      scatter_f64(base.yp.as<double>(), pi, (double*)y, n, s);
    } else {
      gather_f32((const float*)x, pi, base.xp.as<float>(), n, s);
      matvec_eo<float>(base, base.xp.as<float>(), base.yp.as<float>(), false, s);
      scatter_f32(base.yp.as<float>(), pi, (float*)y, n, s);
    }
  }
  const_cast<Op&>(op).matvecs++;
}

// ------------------------------------------------------------------ build
static void set_normfactor(Op& op) {
  const double bj = op.mp.betaJ, k = op.mp.kappa, k2 = op.mp.kappa2;
  const int L = op.L;
  switch (op.kind) {
    case K_XAT:  // TMat/tmat.cpp:48-55
      op.normfactor = (k < 0.5) ? std::exp(L * bj * (k - 2.0)) : std::exp(-L * bj * (k + 1.0));
      break;
    case K_XAM:  // TMat/tmatreduce.cpp:349-359
      op.nfexp = (k < 0.5) ? L * (k - 2.0) : -L * (k + 1.0);
      op.normfactor = std::exp(bj * op.nfexp);
      break;
    case K_XDT:  // TMat/tmat.cpp:333-340
      op.normfactor = (k < 0.5) ? std::exp(L * bj * 2.0 * (k - 1.0)) : std::exp(-L * bj * 2.0 * k);
      break;
    case K_XDM:  // TMat/tmatreduce.cpp:1036-1046
      op.nfexp = (k < 0.5) ? L * 2.0 * (k - 1.0) : -L * 2.0 * k;
      op.normfactor = std::exp(bj * op.nfexp);
      break;
    case K_ZBT:
    case K_ZBM: {  // TMat/tmat.cpp:491-513, TMat/tmatreduce.cpp:1425-1447
      if (k + k2 < 0.5)
        op.nfexp = L * 2.0 * (k + k2 - 1.0);
      else if (k < 0.5 && k2 - k < 0.5)
        op.nfexp = -L;
      else if (k2 < 2 * k)
        op.nfexp = -L * 2.0 * k;
      else
        op.nfexp = L * 2.0 * (k - k2);
      if (op.kind == K_ZBT) {
        double half = std::exp(0.5 * bj * op.nfexp);
        op.normfactor = half * half;
      } else {
        op.normfactor = std::exp(bj * op.nfexp);
      }
      break;
    }
    case K_XAM3:  // TMat/tmat3d.cpp:117-127
      op.nfexp = (k < 0.5) ? L * (k - 3.0) : -L * (k + 2.0);
      op.normfactor = std::exp(bj * op.nfexp);
      break;
    case K_YAT:  // TMat/tmat.cpp:186-193
      op.normfactor = (k < 0.5) ? std::exp(L * bj * (k - 2.0)) : std::exp(-L * bj * (k + 1.0));
      break;
    case K_Y2AT:  // TMat/tmat.cpp:256-263
      op.normfactor = (k < 0.5) ? std::exp(2 * L * bj * (k - 2.0)) : std::exp(-2 * L * bj * (k + 1.0));
      break;
    case K_YAM:  // TMat/tmatreduce.cpp:683-717
      if (!op.ltype)
        op.nfexp = (k < 0.5) ? L * (k - 2.0) : -L * (k + 1.0);
      else if (k + k2 < 0.5)
        op.nfexp = L * 2.0 * (k + k2 - 1.0);
      else if (k < 0.5 && k2 - k < 0.5)
        op.nfexp = -L;
      else if (k2 < 2 * k)
        op.nfexp = -L * 2.0 * k;
      else
        op.nfexp = L * 2.0 * (k - k2);
      op.normfactor = std::exp(bj * op.nfexp);
      break;
  }
}

void build_aux(Op& op);  // aux-bit cores (DNNI, diagonal BNNNI)

static void build_op(Op& op) {
  set_normfactor(op);
  if (is_two_layer(op.kind)) {
    build_two_layer(op);
    return;
  }
  op.nstate = 1ll << op.L;
  if (is_reduced(op.kind)) {
    const bool eo_ok = (op.kind == K_XAM) && op.grp.periodic && (op.L % 2 == 0) && op.L >= 12 && op.L <= 32;
    // the even/odd plan's host tables depend on L and the flip only: build
    // them on a host thread while the GPU builds the orbit table
    std::future<std::shared_ptr<EOHostTables>> eo_host;
    if (eo_ok) eo_host = std::async(std::launch::async, eo_host_tables, op.L / 2, op.grp.flip);
    build_orbit_table(op);
    build_tvec(op);
    if (eo_ok) {
      build_eo_plan(op, eo_host.get().get());
      op.ws_a.release();
      op.ws_b.release();
      op.ws_c.alloc((size_t)op.n * 8);
      op.eo.w1_32.alloc(((size_t)op.eo.n_orep << op.eo.m) * 4);
      op.eo.w1_64.alloc(((size_t)op.eo.n_orep << op.eo.m) * 8);
      if (const size_t xb = eo_xchg_bytes(op.eo)) op.eo.xchg.alloc(xb);
      op.xp.alloc((size_t)op.n * 8);
      op.yp.alloc((size_t)op.n * 8);
    } else {
      if (op.L > 30) fail(TM_ERR_LIMIT, "generic reduced path supports L <= 30");
      build_state_map(op);
      op.ws_a.release();
      op.ws_b.release();
      op.ws_c.alloc((size_t)op.n * 8);
      if (bfly_core(op.kind)) op.ws_a.alloc((size_t)op.nstate * 8);
    }
  } else {
    if (op.L > 30) fail(TM_ERR_LIMIT, "full operators support L <= 30");
    op.n = op.nstate;
    build_tvec(op);
  }
  if (!bfly_core(op.kind)) build_aux(op);
}

Op* create_op(const tm_params* p, char model, int dim, int axialdir, int ec) {
  if (!p) fail(TM_ERR_ARG, "null params");
  if (dim != 2 && dim != 3) fail(TM_ERR_ARG, "dim must be 2 or 3");
  if (model != 'A' && model != 'B' && model != 'D') fail(TM_ERR_ARG, "model must be A, B or D");
  if (!std::isfinite(p->betaJ) || !std::isfinite(p->kappa) || !std::isfinite(p->kappa2) || !std::isfinite(p->h))
    fail(TM_ERR_NONFINITE, "non-finite model parameter");
  std::unique_ptr<Op> op(new Op());
  op->model = model;
  op->dim = dim;
  op->axialdir = axialdir;
  op->extend_cond = ec;
  op->mp = *p;
  TM_CK(cudaGetDevice(&op->device));
  if (dim == 2) {
    op->L = p->size;
  } else {
    op->size1 = p->size >> 16;
    op->size2 = p->size & 0xffff;
    op->L = op->size1 * op->size2;
  }
  if (op->L < 4) fail(TM_ERR_ARG, "size must be >= 4 (TMat/read_input.cpp:84-89)");
  if (op->L > 32) fail(TM_ERR_LIMIT, "layer size above 32 spins is not supported");
  auto reduced_x2d = [&](int kind, int boundary, int censym) {
    op->kind = kind;
    op->boundary = boundary;
    op->censym = censym;
    op->grp.kind = G_X2D;
    op->grp.L = op->L;
    op->grp.periodic = !boundary;
    op->grp.flip = censym;
  };
  const bool h0 = (p->h == 0.0);
  if (model == 'A' && dim == 2) {
    switch (axialdir) {
      case 1: op->kind = K_XAT; op->boundary = 0; break;
      case 9: op->kind = K_XAT; op->boundary = 1; break;
      case 17: case 18: op->kind = K_XAT; op->boundary = (axialdir & 1) ? 5 : 9; break;
      case 19: case 20: op->kind = K_XAT; op->boundary = (axialdir & 1) ? 13 : 17; break;
      case 5: reduced_x2d(K_XAM, ec & 1, h0 && !(ec & 2)); break;
      case 13: reduced_x2d(K_XAM, 1, h0 && !(ec & 2)); break;
      case 0: op->kind = K_Y2AT; op->symmetric = 0; break;
      case 2: op->kind = K_YAT; op->symmetric = 0; break;
      case 6: op->kind = K_YAM; op->symmetric = 0; op->censym = h0 && !(ec & 2); break;
      default: fail(TM_ERR_UNSUPPORTED, "model A dim 2 axialdir " + std::to_string(axialdir) + " not provided");
    }
  } else if (model == 'A' && dim == 3) {
    if (axialdir != 1) fail(TM_ERR_UNSUPPORTED, "model A dim 3 supports axialdir 1 only (TMat/pfunc.cpp:63-74)");
    op->kind = K_XAM3;
    op->censym = h0;  // TMat/tmat3d.cpp:105: flip reduction whenever h == 0
    op->grp.kind = G_X3D;
    op->grp.L = op->L;
    op->grp.size1 = op->size1;
    op->grp.size2 = op->size2;
    op->grp.periodic = 1;
    op->grp.flip = op->censym;
    op->grp.rotate = (p->kappa == 0.0 && op->size1 == op->size2);
  } else if (model == 'D') {
    switch (axialdir) {
      case 1: case 2: op->kind = K_XDT; op->boundary = 0; break;
      case 17: case 18: op->kind = K_XDT; op->boundary = (axialdir & 1) ? 5 : 9; break;
      case 5: case 6: reduced_x2d(K_XDM, 0, h0 && !(ec & 2)); break;
      default: fail(TM_ERR_UNSUPPORTED, "model D axialdir " + std::to_string(axialdir) + " not provided");
    }
  } else if (model == 'B') {
    switch (axialdir) {
      case 3: op->kind = K_ZBT; op->symmetric = 0; break;
      case 7:
        op->kind = K_ZBM;
        op->symmetric = 0;
        op->censym = h0 && !(ec & 2);
        op->grp.kind = G_Z2D;
        op->grp.L = op->L;
        op->grp.periodic = 1;
        op->grp.flip = op->censym;
        break;
      case 6:  // YBMMatVecProd2D = YAMMatVecProd2D(extend_cond | 16) (TMat/tmatreduce.cpp:1018-1021)
        op->kind = K_YAM;
        op->ltype = 1;
        op->symmetric = 0;
        op->censym = h0 && !(ec & 2);
        break;
      default: fail(TM_ERR_UNSUPPORTED, "model B axialdir " + std::to_string(axialdir) + " not provided");
    }
  }
  if (dim == 2 && op->kind == K_XAM3) fail(TM_ERR_ARG, "internal dispatch error");
  TM_CK(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
  AllocStream guard(op->stream);
  build_op(*op);
  return op.release();
}

}  // namespace ltm

using namespace ltm;

#define TM_API_BEGIN try {
#define TM_API_END                       \
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

const char* tm_last_error(void) { return g_err.c_str(); }
const char* tm_version(void) { return "latttmat_gb300 0.1 (sm_103a)"; }

tm_status tm_create(const tm_params* p, char model, int dim, int axialdir, int extend_cond, tm_op** out) {
  TM_API_BEGIN
  if (!out) fail(TM_ERR_ARG, "null output handle");
  *out = nullptr;
  Op* op = create_op(p, model, dim, axialdir, extend_cond);
  tm_op* h = new tm_op;
  h->impl = op;
  *out = h;
  TM_API_END
}

tm_status tm_transpose(const tm_op* op, tm_op** out) {
  TM_API_BEGIN
  if (!op || !out) fail(TM_ERR_ARG, "null handle");
  const Op& b = *op->impl;
  Op* v = new Op();
  v->model = b.model;
  v->dim = b.dim;
  v->axialdir = b.axialdir;
  v->extend_cond = b.extend_cond;
  v->mp = b.mp;
  v->kind = b.kind;
  v->L = b.L;
  v->size1 = b.size1;
  v->size2 = b.size2;
  v->n = b.n;
  v->nstate = b.nstate;
  v->normfactor = b.normfactor;
  v->symmetric = b.symmetric;
  v->is_view = true;
  v->transposed = b.symmetric ? false : !b.transposed;
  v->parent = b.parent ? b.parent : &b;
  v->stream = b.stream;
  v->has_pi = b.has_pi;
  tm_op* h = new tm_op;
  h->impl = v;
  *out = h;
  TM_API_END
}

tm_status tm_destroy(tm_op* op) {
  TM_API_BEGIN
  if (!op) return TM_OK;
  Op* o = op->impl;
  // buffers are freed in order on the operator's stream, then the stream goes
  cudaStream_t st = (o && !o->is_view) ? o->stream : nullptr;
  delete o;
  delete op;
  if (st) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  TM_API_END
}

int64_t tm_rows(const tm_op* op) { return op ? op->impl->n : -1; }
int64_t tm_cols(const tm_op* op) { return op ? op->impl->n : -1; }
double tm_normfactor(const tm_op* op) { return op ? op->impl->normfactor : NAN; }
int tm_layer_size(const tm_op* op) { return op ? op->impl->L : -1; }
int tm_is_symmetric(const tm_op* op) { return op ? op->impl->symmetric : -1; }
int tm_suggested_ncv(const tm_op* op, int nev) { return nev > 4 ? 2 * nev + 1 : 2 * nev + 3; }
int64_t tm_matvec_count(const tm_op* op) { return op ? op->impl->matvecs : -1; }

tm_status tm_perform_op(const tm_op* op, const double* x, double* y) {
  TM_API_BEGIN
  if (!op || !x || !y) fail(TM_ERR_ARG, "null argument");
  Op& o = *op->impl;
  const Op& b = o.parent ? *o.parent : o;
  const int64_t n = b.n;
  Op& bm = const_cast<Op&>(b);
  if (!bm.hx.p) {
    bm.hx.alloc((size_t)n * 8);
    bm.hy.alloc((size_t)n * 8);
  }
  TM_CK(cudaMemcpyAsync(bm.hx.p, x, (size_t)n * 8, cudaMemcpyHostToDevice, b.stream));
  matvec_ref_order(o, bm.hx.p, bm.hy.p, TM_F64, b.stream);
  TM_CK(cudaMemcpyAsync(y, bm.hy.p, (size_t)n * 8, cudaMemcpyDeviceToHost, b.stream));
  TM_CK(cudaStreamSynchronize(b.stream));
  TM_API_END
}

tm_status tm_perform_op_dev(const tm_op* op, const void* x, void* y, tm_dtype dt, void* stream) {
  TM_API_BEGIN
  if (!op || !x || !y) fail(TM_ERR_ARG, "null argument");
  if (dt != TM_F64 && dt != TM_F32 && dt != TM_F64_DF) fail(TM_ERR_ARG, "unknown dtype");
  Op& o = *op->impl;
  const Op& b = o.parent ? *o.parent : o;
  cudaStream_t s = stream ? (cudaStream_t)stream : b.stream;
  matvec_ref_order(o, x, y, dt, s);
  TM_CK(cudaGetLastError());
  TM_API_END
}

tm_status tm_orbit_table(const tm_op* op, uint64_t* idx, uint16_t* dup, int64_t cap, int64_t* n) {
  TM_API_BEGIN
  if (!op) fail(TM_ERR_ARG, "null handle");
  const Op& b = op->impl->parent ? *op->impl->parent : *op->impl;
  if (!is_reduced(b.kind)) fail(TM_ERR_UNSUPPORTED, "full operators have no orbit table");
  if (n) *n = b.n;
  if (idx || dup) {
    if (cap < b.n) fail(TM_ERR_ARG, "capacity smaller than the table");
    std::vector<uint32_t> tmp((size_t)b.n);
    if (idx) {
      TM_CK(cudaMemcpy(tmp.data(), b.idx.p, (size_t)b.n * 4, cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < b.n; ++i) idx[i] = tmp[i];
    }
    if (dup) TM_CK(cudaMemcpy(dup, b.dup.p, (size_t)b.n * 2, cudaMemcpyDeviceToHost));
  }
  TM_API_END
}

tm_status tm_eigs(const tm_op* op, int nev, int ncv, double tol, uint64_t seed, int mode, double* vals_re,
                  double* vals_im, double* vecs, double* vecl, tm_eigs_info* info) {
  TM_API_BEGIN
  if (!op || !vals_re) fail(TM_ERR_ARG, "null argument");
  if (mode != TM_EIGS_F64 && mode != TM_EIGS_MIXED) fail(TM_ERR_ARG, "unknown mode");
  const Op& o = *op->impl;
  const Op& b = o.parent ? *o.parent : o;
  AllocStream guard(b.stream);
  if (is_two_layer(b.kind)) mode = TM_EIGS_F64;  // FP64 products only
  tm_status st = TM_OK;
  if (!b.symmetric) {
    // general operator (TMat/pfunc.hpp:84-98 GenEigsSolver path)
    std::vector<std::complex<double>> cv;
    std::vector<double> xr, xi;
    st = arnoldi_solve(o, nev, ncv, tol, seed, mode, cv, vecs ? &xr : nullptr, vecs ? &xi : nullptr, info);
    for (int i = 0; i < nev; ++i) {
      vals_re[i] = cv[i].real() / b.normfactor;
      if (vals_im) vals_im[i] = cv[i].imag() / b.normfactor;
    }
    if (vecs) {
      for (int c = 0; c < nev; ++c)
        for (int64_t k = 0; k < b.n; ++k) {
          vecs[2 * ((size_t)c * b.n + k)] = xr[(size_t)c * b.n + k];
          vecs[2 * ((size_t)c * b.n + k) + 1] = xi[(size_t)c * b.n + k];
        }
    }
    if (vecl) {
      // left eigenvector: leading eigenvector of the transpose, nev=1, ncv=7
      // (TMat/pfunc.hpp:51-54), real part written out (TMat/pfunc.hpp:159-164)
      Op tv;
      tv.kind = b.kind;
      tv.L = b.L;
      tv.n = b.n;
      tv.symmetric = 0;
      tv.is_view = true;
      tv.transposed = !o.transposed;
      tv.parent = &b;
      tv.stream = b.stream;
      std::vector<std::complex<double>> lv;
      std::vector<double> lr, li;
      tm_eigs_info linfo{};
      tm_status lst = arnoldi_solve(tv, 1, 7, tol, seed + 1, mode, lv, &lr, &li, &linfo);
      if (info) {
        info->matvecs += linfo.matvecs;
        info->matvecs_f64 += linfo.matvecs_f64;
      }
      for (int64_t k = 0; k < b.n; ++k) vecl[k] = lr[k];
      if (lst != TM_OK) fail(lst, "left eigenvector solve did not converge");
    }
  } else {
    std::vector<double> th(nev);
    // vectors come back in the reference's order (lanczos_solve scatters
    // pi-ordered operators on the device)
    st = lanczos_solve(b, nev, ncv, tol, seed, mode, th.data(), vecs, info);
    for (int i = 0; i < nev; ++i) {
      vals_re[i] = th[i] / b.normfactor;
      if (vals_im) vals_im[i] = 0.0;
    }
    if (vecl) {
      // symmetric operators have no separate left vector (TMat/pfunc.hpp:33-44)
      fail(TM_ERR_NOTRANSPOSE, "symmetric operators have no separate left eigenvector");
    }
  }
  if (st != TM_OK) fail(st, "eigensolver did not converge");
  TM_API_END
}

tm_status tm_moments(const tm_op* op, const double* ql, const double* qr, double out4[4], int* ref_status) {
  TM_API_BEGIN
  if (!op || !ql || !qr || !out4) fail(TM_ERR_ARG, "null argument");
  const Op& b = op->impl->parent ? *op->impl->parent : *op->impl;
  AllocStream guard(b.stream);
  double sums[12];
  observables(b, ql, qr, sums);
  // sums: 0..3 = sum w m^k, 4 = sum w, 5 = sum w nnode, 6 = sum w nnode^2, 7..10 DNNI stripes
  const int L = b.L;
  if (b.kind == K_Y2AT) {
    // Y2ATMatVecProd2D::moments is not implemented there (TMat/tmat.cpp:309-314)
    for (int k = 0; k < 4; ++k) out4[k] = 0.0;
    if (ref_status) *ref_status = -1;
  } else if (b.symmetric) {
    for (int k = 0; k < 4; ++k) out4[k] = sums[k] / L;
    if (ref_status) *ref_status = 0;
  } else {
    for (int k = 0; k < 4; ++k) out4[k] = sums[k] / (L * sums[4]);
    if (ref_status) *ref_status = (b.kind == K_ZBM) ? -1 : 0;  // TMat/tmatreduce.cpp:1774
  }
  TM_API_END
}

tm_status tm_phys_extend(const tm_op* op, const double* ql, const double* qr, double* out, int cap, int* nout,
                         int* ref_status) {
  TM_API_BEGIN
  if (!op || !ql || !qr) fail(TM_ERR_ARG, "null argument");
  const Op& b = op->impl->parent ? *op->impl->parent : *op->impl;
  AllocStream guard(b.stream);
  double sums[12];
  int cnt = 0, st = 0;
  std::vector<double> r;
  if (b.kind == K_XAT || b.kind == K_XDT || b.kind == K_XAM) {
    observables(b, ql, qr, sums);
    r = {sums[5], sums[6]};
  } else if (b.kind == K_XDM) {
    observables(b, ql, qr, sums);
    const double L = b.L;
    r = {sums[7] / L, sums[8] / L, sums[9] / (L * L), sums[10] / (L * L)};
  } else if (b.kind == K_XAM3) {
    r = {NAN, NAN};
    st = -1;  // TMat/tmat3d.cpp:165-177
  } else if (b.kind == K_ZBM) {
    st = -1;  // TMat/tmatreduce.cpp:1777-1781
  } else {
    st = 0;  // GenMatPhys: nothing (TMat/tmatphys.cpp:100-106)
  }
  cnt = (int)r.size();
  for (int i = 0; i < cnt && i < cap; ++i) out[i] = r[i];
  if (nout) *nout = cnt;
  if (ref_status) *ref_status = st;
  TM_API_END
}

int64_t tm_launch_count(void) { return g_launches.load(); }

int64_t tm_alloc_count(void) { return ltm::g_allocs.load(); }

void tm_debug_set_eo_tile_bits(int bits) { ltm::eo_set_tile_bits_cap(bits); }

tm_status tm_profile_matvec(const tm_op* op, tm_dtype dt, int iters, double* ms_out, int cap, int* nstages) {
  TM_API_BEGIN
  if (!op || !ms_out || iters < 1) fail(TM_ERR_ARG, "bad argument");
  const Op& o = *op->impl;
  const Op& b = o.parent ? *o.parent : o;
  cudaStream_t s = b.stream;
  AllocStream guard(s);
  DBuf x, y, x32, y32;
  x.alloc((size_t)b.n * 8);
  y.alloc((size_t)b.n * 8);
  TM_CK(cudaMemsetAsync(x.p, 0, (size_t)b.n * 8, s));
  const bool f32 = (dt == TM_F32);
  if (f32) {
    x32.alloc((size_t)b.n * 4);
    y32.alloc((size_t)b.n * 4);
    TM_CK(cudaMemsetAsync(x32.p, 0, (size_t)b.n * 4, s));
  }
  if (dt != TM_F64 && dt != TM_F32 && dt != TM_F64_DF) fail(TM_ERR_ARG, "unknown dtype");
  const bool df = (dt == TM_F64_DF);
  auto run = [&]() {
    if (df)
      apply_refine(o, x.as<double>(), y.as<double>(), s);
    else
      apply_internal(o, x.as<double>(), y.as<double>(), x32.as<float>(), y32.as<float>(), f32, s);
  };
  run();  // warm-up
  TM_CK(cudaStreamSynchronize(s));
  int ns = 1;
  std::vector<double> acc(3, 0.0);
  EOPlan& P = const_cast<EOPlan&>(b.eo);
  if (b.eo.active) {
    ns = 3;
    for (int k = 0; k < 4; ++k) TM_CK(cudaEventCreate(&P.prof_ev[k]));
    P.prof_on = true;
    for (int it = 0; it < iters; ++it) {
      run();
      TM_CK(cudaStreamSynchronize(s));
      for (int k = 0; k < 3; ++k) {
        float ms = 0.f;
        TM_CK(cudaEventElapsedTime(&ms, P.prof_ev[k], P.prof_ev[k + 1]));
        acc[k] += ms;
      }
    }
    P.prof_on = false;
    for (int k = 0; k < 4; ++k) {
      cudaEventDestroy(P.prof_ev[k]);
      P.prof_ev[k] = nullptr;
    }
  } else {
    cudaEvent_t e0, e1;
    TM_CK(cudaEventCreate(&e0));
    TM_CK(cudaEventCreate(&e1));
    TM_CK(cudaEventRecord(e0, s));
    for (int it = 0; it < iters; ++it) run();
    TM_CK(cudaEventRecord(e1, s));
    TM_CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    TM_CK(cudaEventElapsedTime(&ms, e0, e1));
    acc[0] = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  for (int k = 0; k < ns && k < cap; ++k) ms_out[k] = acc[k] / iters;
  if (nstages) *nstages = ns;
  TM_API_END
}

tm_status tm_grad(const tm_op* op, const double* qr, const double* ql, double lambda_internal, double grad4[4]) {
  TM_API_BEGIN
  if (!op || !qr || !grad4) fail(TM_ERR_ARG, "null argument");
  if (!(lambda_internal != 0.0) || !std::isfinite(lambda_internal)) fail(TM_ERR_ARG, "eigenvalue must be finite, nonzero");
  const Op& b = op->impl->parent ? *op->impl->parent : *op->impl;
  AllocStream guard(b.stream);
  if (!b.symmetric && !ql) fail(TM_ERR_ARG, "general operators need the left eigenvector");
  adjoint_grad(b, qr, b.symmetric ? nullptr : ql, lambda_internal, grad4);
  TM_API_END
}

}  // extern "C"
