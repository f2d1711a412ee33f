// Internal declarations of liblatttmat_gb300: operator state, device tables,
// error plumbing and the kernel entry points each .cu file provides.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/latttmat.h"
#include "tm_bits.cuh"

namespace ltm {

// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
struct Failure {
  tm_status code;
  std::string msg;
};
[[noreturn]] void fail(tm_status code, const std::string& msg);
void check_cuda(cudaError_t e, const char* what, const char* file, int line);
#define TM_CK(call) ::ltm::check_cuda((call), #call, __FILE__, __LINE__)
// after every kernel launch: error check + launch counter
void note_launch();
#define TM_CKK(what) (::ltm::note_launch(), ::ltm::check_cuda(cudaGetLastError(), what, __FILE__, __LINE__))

// ---------------------------------------------------------------- memory
// Owning device buffer (freed in the destructor).
// Device buffer.  Allocation is stream-ordered (cudaMallocAsync on the
// stream an AllocStream guard set for the calling thread) when a guard is
// active, so that freeing does not synchronise the device while other
// operators' solves run concurrently; the buffer is then freed on the same
// stream.  Without a guard it is a plain cudaMalloc.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t st = nullptr;
  DBuf() {}
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void alloc(size_t b);
  void release();
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

// Sets the allocation stream of DBuf::alloc for the calling thread while in
// scope (every use of such a buffer must be ordered after its allocation on
// that stream, and its last use before the free that ends the scope).
struct AllocStream {
  cudaStream_t prev;
  explicit AllocStream(cudaStream_t s);
  ~AllocStream();
};

// ---------------------------------------------------------------- kinds
enum Kind {
  K_XAT = 0,   // XATMatVecProd2D: full x-ANNNI (TMat/tmat.cpp:39-102)
  K_XAM = 1,   // XAMMatVecProd2D: reduced x-ANNNI (TMat/tmatreduce.cpp:338-563)
  K_XDT = 2,   // XDTMatVecProd2D: full DNNI (TMat/tmat.cpp:322-476)
  K_XDM = 3,   // XDMMatVecProd2D: reduced DNNI (TMat/tmatreduce.cpp:1024-1400)
  K_ZBT = 4,   // ZBTMatVecProd2D: full diagonal BNNNI (TMat/tmat.cpp:480-662)
  K_ZBM = 5,   // ZBMMatVecProd2D: reduced diagonal BNNNI (TMat/tmatreduce.cpp:1403-1868)
  K_XAM3 = 6,  // XAMMatVecProd3D: reduced 3D ANNNI (TMat/tmat3d.cpp:102-340)
  K_YAT = 7,   // YATMatVecProd2D (+_T): full two-layer y-ANNNI (TMat/tmat.cpp:106-242)
  K_Y2AT = 8,  // Y2ATMatVecProd2D: full two-layer y2-ANNNI (TMat/tmat.cpp:245-315)
  K_YAM = 9,   // YAMMatVecProd2D (+_T) / YBMMatVecProd2D: reduced two-layer (TMat/tmatreduce.cpp:661-1021)
};

inline bool is_two_layer(int kind) { return kind == K_YAT || kind == K_Y2AT || kind == K_YAM; }

// Orbit-group families (which symmetry group the reduced basis uses)
enum GroupKind { G_NONE = 0, G_X2D = 1, G_Z2D = 2, G_X3D = 3, G_Y2D = 4 };

// Parameters of the group acting on L-bit states
struct GroupDesc {
  int kind = G_NONE;
  int L = 0;
  int size1 = 0, size2 = 0;  // 3D layer shape
  int periodic = 1;          // 0: open boundary (X/Z: identity + reflection only)
  int flip = 0;              // spin-flip (censym) included
  int rotate = 0;            // 3D 90-degree rotation included
  int nbits = 0;             // state bits when not L (two-layer states: 2L)
  int order() const;         // number of enumerated group elements
};

// Even/odd two-pass plan for x-ANNNI reduced operators (periodic, even L).
struct EOPlan {
  bool active = false;
  int m = 0;          // bits per pass (L/2)
  int c32 = 0, c64 = 0;  // cluster bits for the FP32 / FP64 passes
  int ct = 0;         // top bits grouping the iteration orders: max(c32, c64)
  int n_orep = 0;     // pass-1 tiles
  int n_erep = 0;     // pass-2 tiles
  int ng = 0;         // H elements enumerated
  DBuf map1;          // u32 [n_orep][2^m]: pi-index of the orbit of (it_e[P], o_rep)
  DBuf it_e;          // u16 [2^m]: e at each pass-1 iteration position P
  DBuf cls_start, cls_size;  // u32 [n_erep]: class-first start and size of each e-class
  DBuf wout;          // uint2 [2^m]: (w1 offset of (tile 0, it_e[P]), it_e[P] | e-class size << 16)
  DBuf t2o;           // uint2 [2^m]: ((o-tile << 8) | H element g, it_o[P]) per pass-2 position
  DBuf cf_e;          // u16 [2^m]: class-first position of each e
  DBuf it_o;          // u16 [2^m]: o at each pass-2 iteration position
  DBuf erep;          // u32 [n_erep]: e representative of each pass-2 tile
  DBuf out_off;       // u32 [n_erep*2^ct+1]: designated-output offsets per tile and top-ct-bit group
  DBuf out_o;         // u16 [R]: o of each designated output (pi order)
  DBuf w1_32, w1_64;  // pass-1 intermediates
  DBuf xchg;          // cluster-combine exchange slots (one per CTA of a clustered launch), or empty
  cudaEvent_t prof_ev[4] = {nullptr, nullptr, nullptr, nullptr};  // stage timing (diagnostics)
  bool prof_on = false;
};

struct Op {
  // identity
  char model = 'A';
  int dim = 2, axialdir = 1, extend_cond = 0;
  tm_params mp{};
  int kind = K_XAT;
  int L = 0;            // spin bits per layer
  int size1 = 0, size2 = 0;
  int boundary = 0;     // genTvec boundary case (0,1,5,9,13,17)
  int censym = 0;
  int symmetric = 1;
  int64_t nstate = 0;   // 2^L
  int64_t n = 0;        // rows == cols
  double normfactor = 1.0;
  double nfexp = 0.0;   // normfactor = exp(betaJ * nfexp)
  int device = 0;
  cudaStream_t stream = nullptr;
  bool is_view = false;   // transpose / symmetric view: does not own tables
  bool transposed = false;
  const Op* parent = nullptr;
  int64_t matvecs = 0;

  // reduced-basis tables (reference order)
  GroupDesc grp;
  DBuf idx;        // u32 [n] ascending representatives
  DBuf dup;        // u16 [n] orbit sizes
  DBuf tvec;       // f64 [n or nstate]: the operator's Tvec (Tv^(1/2) [* nf^(1/2)] / sqrt(dup))
  // generic reduced path: state -> rank map
  DBuf smap;       // u32 [nstate]
  // pi order (internal vector order): pi[k] = reference index; identity if empty
  bool has_pi = false;
  DBuf pi, pinv;   // u32 [n]
  DBuf sin64, sout64;  // f64 [n] input/output scales in pi order
  DBuf sin32, sout32;  // f32 copies
  DBuf sindf, soutdf;  // double-float [n]: input scale times (1 + r)^-L, output scale
  EOPlan eo;

  // workspace
  DBuf ws_a, ws_b, ws_c;  // full-space scratch
  DBuf hx, hy;            // device copies for host-vector matvecs
  DBuf xp, yp;            // permuted vectors for the reference-order entry
  double scale32 = 1.0;   // FP32 matvec output scale (applied in FP64)

  // two-layer operators
  int ltype = 0;          // 1: YBMMatVecProd2D (all-frustrated layer Tvec)
  DBuf swp;               // u32 [n]: index of the layer-swapped orbit
  DBuf bstart;            // u32 [nblocks+1]: representative blocks sharing the left layer
  int nblocks = 0;
};

// ---------------------------------------------------------------- builders
void build_group(Op& op);
void build_orbit_table(Op& op);          // idx, dup (reference order)
void build_tvec(Op& op);                 // Tvec for the operator
void build_state_map(Op& op);            // smap for the generic reduced path
struct EOHostTables;                     // host-side even/odd plan tables (tm_eo.cu)
std::shared_ptr<EOHostTables> eo_host_tables(int m, int flip);
void build_eo_plan(Op& op, const EOHostTables* host = nullptr);  // even/odd plan for K_XAM
size_t eo_xchg_bytes(const EOPlan& P);
void eo_set_tile_bits_cap(int bits);
void build_two_layer(Op& op);            // tables of K_YAT / K_Y2AT / K_YAM
// y = T x (or T^T x for a transposed view) of a two-layer operator, FP64
void matvec_two_layer(const Op& op, const double* x, double* y, cudaStream_t s);

// ---------------------------------------------------------------- matvec
// y = T x in the operator's internal order (pi order when has_pi), on stream.
void matvec_internal(const Op& op, const void* x, void* y, tm_dtype dt, cudaStream_t s);
// reference-order wrappers
void matvec_ref_order(const Op& op, const void* x, void* y, tm_dtype dt, cudaStream_t s);

// full-space cores (T applied to a full 2^L vector, in place where possible)
void full_apply(const Op& op, const void* xin, void* out, tm_dtype dt, cudaStream_t s, int transpose);

// ---------------------------------------------------------------- helpers
// Raise a kernel's dynamic shared-memory limit to at least `bytes`.  The
// limit is per-kernel process state: it only ever grows here, so concurrent
// host threads launching the same kernel with different tile sizes never see
// a limit below what their launch needs.
void raise_smem_limit(const void* kernel, size_t bytes);
int exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t s);  // returns 0
uint32_t read_u32(const uint32_t* dptr, cudaStream_t s);
int num_sms();

// permutation helpers
void gather_f64(const double* src, const uint32_t* idx, double* dst, int64_t n, cudaStream_t s);
// dst[c*n + i] = src[c*lds + idx[i]], c < nvec (dst may be device-mapped host memory)
void gather_cols_f64(const double* src, int64_t lds, const uint32_t* idx, double* dst, int64_t n, int nvec,
                     cudaStream_t s);
void scatter_f64(const double* src, const uint32_t* idx, double* dst, int64_t n, cudaStream_t s);
void gather_f32(const float* src, const uint32_t* idx, float* dst, int64_t n, cudaStream_t s);
void scatter_f32(const float* src, const uint32_t* idx, float* dst, int64_t n, cudaStream_t s);

}  // namespace ltm

struct tm_op {
  ltm::Op* impl;
};
