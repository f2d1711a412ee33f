// Aux-bit chain products (DNNI, diagonal BNNNI): pass geometry, coefficients
// and the per-instance records of the batched product that a parameter sweep
// runs (tm_aux.cu implements them, tm_sweep.cu drives the batch).
#pragma once
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
enum { kModeIdle = 0, kModeF32 = 1, kModeDF = 2, kModeF64 = 3 };

// One operator of a batched product, in device memory.  The batch kernels
// find their member from a per-block member map and skip members whose
// product mode (km[i].y, set per step) differs from the launch's; km[i].x is
// the Krylov column the member extends this step.
struct ChainInst {
  ChainPass p4[kChainMaxPass];  // passes of the 4-byte (FP32) plan
  ChainPass p8[kChainMaxPass];  // passes of the 8-byte (FP64, double-float) plan
  int np4, np8;
  int L, bc, dir, zb, nlb;
  int64_t n;                    // rows
  AuxCoefT<float> c32;
  AuxCoefT<dfloat> cdf;
  AuxCoefT<double> c64;
  double gs32, gsdf, gs64;      // output factors undoing the step normalisation
  double nf;                    // normfactor (full operators)
  const uint32_t* smap;         // state -> rank (reduced) or null
  const double* tvec;
  const uint32_t* idx;          // reduced: representatives (null for full operators)
  const uint16_t* dup;
  void* P;                      // pass buffer (8-byte elements)
  void* fold;                   // fold output, 2^L (8-byte) elements
  double* V;                    // Krylov basis: column c at V + c * ldv
  int64_t ldv;
  float* x32;                   // FP32 product input
  double* w;                    // product output and CGS work vector
  double* sc;                   // small per-instance values (kSweepScal doubles)
};

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
  } p4, p8;
  const int64_t* rstart = nullptr;  // row-chunk prefix [count+1] (kSweepRows rows per block)
  const int* rmem = nullptr;        // the member of every row block
  int64_t nrblk = 0;
};

// Batched product of every member in `mode` (input: column km[i].x of its
// basis, or its x32 in FP32): one launch per pass over all members' tiles,
// then one contraction launch into each w.  Returns the launches issued.
int chain_batch_product(const ChainBatch& B, const int2* km, int mode, cudaStream_t s);

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
