// Aux-bit chain products (DNNI, diagonal BNNNI): pass geometry, coefficients
// and the per-instance records of the batched product that a parameter sweep
// runs (tm_aux.cu implements them, tm_sweep.cu drives the batch).
#pragma once
#include <cmath>
#include <vector>

#include "tm_df.cuh"
#include "tm_internal.h"

namespace ltm {

struct AuxCoef {
  double b1[2], b2[2], b3[2];
};

template <class T>
struct AuxCoefT {
  T b1[2], b2[2], b3[2];
  T g;  // step normalisation (multiply)
};

// Geometry of one pass.  Element index in HBM: ((lb << L | r) << NA) | aux.
// Tile index e: bits [0, NA) aux, then tile state bits k -> state position
// spos[k]; the outer index (blockIdx) deposits into opos[] (state bits) and,
// when the lastbit pass is outer, into lb.
struct ChainPass {
  int nst;         // tile state bits
  int spos[16];
  int no;          // outer state bits
  int opos[32];
  int t0, T;       // steps [t0, t0 + T)
  int jbit0;       // tile state bit of step t0's lowest site
  int first, last; // build from x / fold into y
  int nlb;         // lastbit passes (DNNI 2 or 1, BNNNI 4)
};

constexpr int kChainMaxPass = 8;
constexpr int kBatchTiles = 4;  // tiles of one member per block of a batched pass

// Product modes of a batch member in one step.
enum { kModeIdle = 0, kModeF32 = 1, kModeDF = 2, kModeF64 = 3, kModeTangent = 4 };

// One operator of a batched product, in device memory.  The batch kernels
// find their member from a per-block member map and skip members whose
// product mode (km[i].y, set per step) differs from the launch's; km[i].x is
// the Krylov column the member extends this step.
struct ChainInst {
  ChainPass p4[kChainMaxPass];   // passes of the 4-byte (FP32) plan
  ChainPass p8[kChainMaxPass];   // passes of the 8-byte (FP64, double-float) plan
  ChainPass p16[kChainMaxPass];  // passes of the 16-byte (tangent pair) plan
  int np4, np8, np16;
  int L, bc, dir, zb, nlb, kind;
  double bj, kap, kap2, h;       // model parameters (the adjoint's weight derivatives)
  int64_t n;                    // rows
  AuxCoefT<float> c32;
  AuxCoefT<dfloat> cdf;
  AuxCoefT<double> c64;
  AuxCoefT<tangent> ctan[3];    // FP64 factors with their derivative by betaJ, kappa, kappa2
  double gs32, gsdf, gs64;      // output factors undoing the step normalisation
  double nf;                    // normfactor (full operators)
  const uint32_t* smap;         // state -> rank (reduced) or null
  const double* tvec;
  const uint32_t* idx;          // reduced: representatives (null for full operators)
  const uint16_t* dup;
  void* P;                      // pass buffer (8-byte elements, 16-byte for tangent products)
  void* fold;                   // fold output, 2^L (8-byte) elements
  double* V;                    // Krylov basis: column c at V + c * ldv
  int64_t ldv;
  float* x32;                   // FP32 product input
  double* w;                    // product output and CGS work vector
  double* sc;                   // small per-instance values (kSweepScal doubles)
};

// d(exponent of Tvec)/d(betaJ, kappa, kappa2, h) of the aux-bit operators
// at state s, without the normfactor term (it cancels against the division
// of the reported eigenvalue): diagonal BNNNI (ZBTMatVecProd2D::genTvec,
// TMat/tmat.hpp:537-556): -bJ/2 (2 n1 - L) + bJ k2/2 (2 n2 - L) -
// bJ h/2 (2 n0 - L); DNNI (XDTMatVecProd2D::genTvec, TMat/tmat.hpp:437-504):
// -bJ/2 (2 n1 - ns1) - bJ h/2 (2 n0 - L), n1 and ns1 per boundary case.
TM_HD void aux_tvec_grad(int kind, int L, int boundary, double bj, double k2, double h, uint64_t s,
                                double g[4]) {
  const uint64_t mask = (1ull << L) - 1;
  const int n0 = popc64(s);
  g[0] = g[1] = g[2] = g[3] = 0.0;
  if (kind == K_ZBT || kind == K_ZBM) {
    const int n1 = popc64(s ^ rotr(s, L, 1)), n2 = popc64(s ^ rotr(s, L, 2));
    g[0] = -0.5 * (2.0 * n1 - L) + 0.5 * k2 * (2.0 * n2 - L) - 0.5 * h * (2.0 * n0 - L);
    g[2] = 0.5 * bj * (2.0 * n2 - L);
  } else {
    int n1, ns1 = L;
    switch (boundary) {
      case 0: n1 = popc64(s ^ rotr(s, L, 1)); break;
      case 1: n1 = popc64((s & (mask >> 1)) ^ (s >> 1)); ns1 = L - 1; break;
      case 5: n1 = popc64((s << 1) ^ s); ns1 = L + 1; break;
      default: n1 = popc64(((s << 1) | 1ull) ^ s); ns1 = L + 1; break;  // 9
    }
    g[0] = -0.5 * (2.0 * n1 - ns1) - 0.5 * h * (2.0 * n0 - L);
  }
  g[3] = -0.5 * bj * (2.0 * n0 - L);
}

// Derivatives of the step factors b1 = e^{+-bJ}, b2 = e^{-+bJ k},
// b3 = e^{-+bJ k2} with respect to parameter t (0 betaJ, 1 kappa, 2 kappa2).
inline AuxCoef aux_coef_derivative(double bj, double k, double k2, int t) {
  const double e1 = std::exp(bj), e2 = std::exp(-bj * k), e3 = std::exp(-bj * k2);
  AuxCoef db{};
  if (t == 0) {
    db.b1[0] = e1;
    db.b1[1] = -1.0 / e1;
    db.b2[0] = -k * e2;
    db.b2[1] = k / e2;
    db.b3[0] = -k2 * e3;
    db.b3[1] = k2 / e3;
  } else if (t == 1) {
    db.b2[0] = -bj * e2;
    db.b2[1] = bj / e2;
  } else if (t == 2) {
    db.b3[0] = -bj * e3;
    db.b3[1] = bj / e3;
  }
  return db;
}

// Coefficients and scales of an operator's product in the three arithmetics.
AuxCoef coef_of(const Op& op);
double step_bound(const Op& op, const AuxCoef& c, int dir);
void chain_tuning(int L, size_t elem, bool zb, int& tile_bits, int& threads);
void chain_set_tuning(int L, size_t elem, bool zb, int tile_bits, int threads);
std::vector<ChainPass> chain_plan(int L, bool zb, int nlb, int tile_bits);
int64_t chain_pass_blocks(const ChainPass& cp);
size_t chain_pass_smem(const ChainPass& cp, bool zb, size_t elem);

// Fill the geometry and coefficients of `rec` for operator `op` (an aux-bit
// operator; dir 1 for its transpose), with tiles of 2^tb4 (4-byte) and 2^tb8
// (8-byte) elements (0: the tuning table's choice for the width).
void chain_inst_fill(const Op& op, int dir, ChainInst& rec, int tb4 = 0, int tb8 = 0);

// Device tables of a batched product over `count` members.
struct ChainBatch {
  const ChainInst* inst = nullptr;
  int count = 0, zb = 0;
  // per plan (4-byte, 8-byte): passes, block prefix [pass][count+1] (blocks of
  // kBatchTiles tiles), the member of every block (per pass, from boff[p]),
  // blocks per pass, threads per block and dynamic shared memory
  struct Plan {
    int np = 0, threads = 256;
    size_t smem = 0;
    const int64_t* start = nullptr;
    const int* bmem = nullptr;
    std::vector<int64_t> nblk, boff;
  } p4, p8, p16;
  const int64_t* rstart = nullptr;  // row-chunk prefix [count+1] (kSweepRows rows per block)
  const int* rmem = nullptr;        // the member of every row block
  int64_t nrblk = 0;
};

// Batched product of every member in `mode` (input: column km[i].x of its
// basis, or its x32 in FP32): one launch per pass over all members' tiles,
// then one contraction launch into each w.  In kModeTangent the product is
// the chain's derivative by parameter `theta` (0 betaJ, 1 kappa, 2 kappa2)
// between the fixed Boltzmann weights.  Returns the launches issued.
int chain_batch_product(const ChainBatch& B, const int2* km, int mode, cudaStream_t s, int theta = 0);

constexpr int kSweepRows = 4096;  // rows per block of the batched row kernels

// While in scope on the calling thread, operators built by create_op keep no
// aux-bit product buffers (the batch that owns them provides its own).
struct BatchMemberScope {
  bool prev;
  BatchMemberScope();
  ~BatchMemberScope();
};

// Measure the operator's product over the chain kernels' tile and block sizes
// and keep the fastest in the tuning table (tm_aux.cu).
void chain_autotune(const Op& op, tm_dtype dt, int& tile_bits, int& threads, double& ms);

// Operator construction as tm_create does it (throws Failure).
Op* create_op(const tm_params* p, char model, int dim, int axialdir, int ec);

}  // namespace ltm
