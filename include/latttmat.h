/*
 * latttmat.h -- C ABI of the GB300 transfer-matrix library (liblatttmat_gb300.so).
 *
 * A tm_op is one transfer-matrix operator, the GPU counterpart of one of the
 * reference's MatVecProd classes.  Its tables live in HBM.  Each entry point
 * names the reference interface it replaces (file:line in LattTMat).
 *
 * Conventions
 *  - Every call returns a tm_status (0 = TM_OK).  No C++ exception crosses
 *    this boundary.  tm_last_error() returns a message for the calling thread's
 *    last failure.
 *  - Buffers are owned by the caller.  Each argument says whether it is a host
 *    or a device pointer.  Host vectors are FP64, as in the reference's
 *    perform_op(const double*, double*).
 *  - Vector order is the reference's: full operators index states 0..2^L-1.
 *    Reduced operators index orbit representatives in ascending state order,
 *    the reference's idxlist order.
 *  - Operators are thread-compatible, not thread-safe: one call at a time per
 *    tm_op.  The reference op is not reentrant either; its matvec counter is
 *    a non-atomic static (TMat/utility.hpp:191-199).
 */
#ifndef LATTTMAT_GB300_H
#define LATTTMAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tm_op tm_op;
typedef int tm_status;

enum {
  TM_OK = 0,
  TM_ERR_ARG = 1,         /* invalid argument (reference: assert / int error codes) */
  TM_ERR_UNSUPPORTED = 2, /* model/dim/axialdir not provided (reference: assert(false), TMat/pfunc.cpp:59) */
  TM_ERR_CUDA = 3,        /* CUDA runtime failure */
  TM_ERR_NOMEM = 4,       /* device allocation failed */
  TM_ERR_NOCONV = 5,      /* eigensolver did not converge (reference: TMat/pfunc.hpp:110-114) */
  TM_ERR_NONFINITE = 6,   /* NaN/Inf detected in an input or iterate */
  TM_ERR_NOTRANSPOSE = 7, /* operator has no transpose form */
  TM_ERR_LIMIT = 8        /* size outside an entry point's stated maximum */
};

/* TM_F64_DF: FP64 values computed in double-float (FP32 pair) arithmetic,
 * the solver's refinement product: FP64 accuracy (relative error ~1e-14 per
 * product) on the FP32 pipes, for the even/odd x-ANNNI and aux-bit (DNNI,
 * BNNNI) operators; other operators compute it in native FP64. */
typedef enum { TM_F64 = 0, TM_F32 = 1, TM_F64_DF = 2 } tm_dtype;

/* Model parameters; mirrors MParameter (TMat/commondef.hpp:18-24).  For dim=3
 * `size` is packed as (size1 << 16) | size2, as TMat/read_input.cpp:41 does. */
typedef struct {
  double betaJ;
  double kappa;
  double kappa2;
  double h;
  int size;
} tm_params;

/* Eigensolver precision modes for tm_eigs. */
enum {
  TM_EIGS_F64 = 0,   /* every matvec in FP64 */
  TM_EIGS_MIXED = 1  /* FP32 matvec bulk + FP64 Rayleigh-Ritz refinement and residual check */
};

/* Diagnostics returned by tm_eigs. */
typedef struct {
  int nconv;          /* converged eigenvalues (Spectra compute() return value) */
  int matvecs;        /* total operator applications (reference: OpCounter) */
  int matvecs_f64;    /* of which FP64 */
  int restarts;       /* restart cycles */
  int ncv;            /* subspace size used */
  double max_resid;   /* max relative residual ||T v - lambda v|| / |lambda| of the returned pairs (FP64) */
  double seconds;     /* wall time inside tm_eigs */
  /* mixed mode only: the FP64-accurate refinement of the FP32 phase */
  int refine_rounds;    /* Rayleigh-Ritz rounds */
  int refine_checks;    /* verifications with FP64-accurate products */
  int refine_outcome;   /* 0 not run, 1 accepted on the certified estimate, 2 accepted after a
                           verification, 3 not accepted (FP64 Lanczos continued) */
  double refine_est;    /* last estimated max relative residual */
  double refine_true;   /* last verified max relative residual (0 if none) */
  /* mixed mode only: split of the solve (host clock, stream synchronised) */
  int matvecs_phase1;     /* FP32 products of the FP32 Lanczos phase */
  double seconds_phase1;  /* FP32 Lanczos phase */
  double seconds_refine;  /* refinement, including its FP64-accurate products */
} tm_eigs_info;

/* ---- operator lifetime ------------------------------------------------- */

/* Build an operator.  Replaces the constructors dispatched by pfunc
 * (TMat/pfunc.cpp:16-106): model 'A','B','D'; dim 2 or 3; axialdir as in the
 * reference; extend_cond as the reference constructors take it (bit 0 open
 * boundary, bit 1 disables the spin-flip reduction, TMat/tmatreduce.cpp:338-341).
 * The reference driver passes extend_cond = (neigs > 1 ? 2 : 0) for reduced
 * operators (TMat/pfunc.cpp:22).  Orbit tables and Boltzmann weights are built
 * on the GPU.  Uses the current CUDA device. */
tm_status tm_create(const tm_params* p, char model, int dim, int axialdir, int extend_cond,
                    tm_op** out);

/* Transpose operator T^T, sharing the parent's tables (the parent must outlive
 * it).  Replaces get_t_instance() (e.g. TMat/tmatreduce.hpp:195-196,
 * TMat/tmat.hpp:534-535).  Symmetric operators return a view of themselves. */
tm_status tm_transpose(const tm_op* op, tm_op** out);

/* Release an operator and its device memory. */
tm_status tm_destroy(tm_op* op);

/* ---- Spectra operator concept (TMat/tmat.hpp:82-120) ------------------- */

int64_t tm_rows(const tm_op* op);          /* MatVecProd::rows() */
int64_t tm_cols(const tm_op* op);          /* MatVecProd::cols() */
double tm_normfactor(const tm_op* op);     /* MatVecProd::getnormfactor(); eigenvalues are lambda/normfactor */
int tm_layer_size(const tm_op* op);        /* MatVecProd2D/3D::getLayerSize() */
int tm_is_symmetric(const tm_op* op);      /* 1 if Scalar=double (SymEigsSolver path), 0 if general */
int tm_suggested_ncv(const tm_op* op, int nev); /* MatVecProd::suggested_nev (TMat/tmat.hpp:88) */
int64_t tm_matvec_count(const tm_op* op);  /* OpCounter::get() (TMat/utility.hpp:191-199), per operator */

/* y = T x on host FP64 buffers of length cols(); drop-in for perform_op
 * (TMat/tmat.hpp:89).  Copies in, computes in FP64 on the GPU, copies out. */
tm_status tm_perform_op(const tm_op* op, const double* x_host, double* y_host);

/* y = T x on device buffers (dtype TM_F64, TM_F32 or TM_F64_DF; length
 * cols()), on the given CUDA stream (cudaStream_t, or NULL for the library's
 * stream).  TM_F64_DF buffers hold doubles.  Asynchronous with respect to the
 * host. */
tm_status tm_perform_op_dev(const tm_op* op, const void* x_dev, void* y_dev, tm_dtype dtype,
                            void* stream);

/* No counterpart in the reference.  FP64 y = T x on device buffers, like
 * tm_perform_op_dev with TM_F64, but allocating nothing: no cudaMalloc,
 * cudaFree or allocating library call.  It is meant for callers that cannot
 * allocate device memory when they need a product: code running inside a
 * host framework whose caching allocator owns the device memory, or a
 * latency-bound loop where an allocation's implicit synchronisation would
 * stall other streams.  The scratch is one fixed 16 MiB device array built
 * into the library (2^21 doubles; every GPU that loads the library holds it
 * until the process exits).
 *
 * Covers the reduced x-ANNNI operators on the even/odd path (model 'A',
 * reduced, periodic, even L >= 12).  An operator needs 3*rows + n_orep*2^(L/2)
 * doubles of scratch, which fits up to L = 24; larger operators return
 * TM_ERR_LIMIT, other operators TM_ERR_UNSUPPORTED.
 *
 * The first call on a device looks up that device's address of the array
 * (with the device current), so make the first call on each device before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * (different streams, or different host threads) race on it and must be
 * serialised by the caller.  Each call overwrites every scratch element it
 * reads, so nothing is carried over from the previous call. */
tm_status tm_perform_op_dev_noalloc(const tm_op* op, const double* x_dev, double* y_dev, void* stream);

/* Orbit table of a reduced operator: ascending representatives (idxlist) and
 * orbit sizes (duplist), bit-exact with genX2DDuplist / genZ2DDuplist /
 * genX3DDuplist (TMat/tmatreduce.cpp:19-111, 242-334; TMat/tmat3d.cpp:17-98).
 * Host buffers of capacity `cap`; *n receives the table length.  Either
 * buffer may be NULL to query the length only.  Full operators return
 * TM_ERR_UNSUPPORTED. */
tm_status tm_orbit_table(const tm_op* op, uint64_t* idx_host, uint16_t* dup_host, int64_t cap,
                         int64_t* n);

/* ---- eigensolver (replaces pfunc_inner, TMat/pfunc.hpp:79-202) ---------- */

/* Largest-magnitude eigenpairs on the GPU: thick-restart Lanczos for symmetric
 * operators, Krylov-Schur Arnoldi for general ones.  FP64 Gram-Schmidt and
 * Rayleigh-Ritz on the device.
 *   nev       wanted eigenvalues (reference `neigs`)
 *   ncv       subspace size (0 = tm_suggested_ncv; in TM_EIGS_MIXED mode on a
 *             symmetric operator at least 16, which costs fewer products)
 *   tol       relative residual tolerance
 *   seed      start vector uniform(0,1) from splitmix64(seed)
 *   mode      TM_EIGS_F64 or TM_EIGS_MIXED
 *   vals_re/vals_im  host, nev each: eigenvalues / normfactor, in descending
 *             magnitude (vals_im may be NULL for symmetric operators)
 *   vecs      host or NULL: right eigenvectors, column-major rows x nev.
 *             FP64 for symmetric operators; complex128 (re,im interleaved)
 *             for general ones.
 *   vecl      host or NULL: general operators only, the leading left
 *             eigenvector (real part, length rows), from a second solve on the
 *             transpose as getlefteigvec does (TMat/pfunc.hpp:47-68)
 *   info      host or NULL: diagnostics */
tm_status tm_eigs(const tm_op* op, int nev, int ncv, double tol, uint64_t seed, int mode,
                  double* vals_re, double* vals_im, double* vecs, double* vecl, tm_eigs_info* info);

/* Parameter sweep: solve `count` independent operators (params[i], and the
 * same model/dim/axialdir/extend_cond for all; widths may differ).  Replaces
 * running the reference tmat once per parameter point (TMat/main.cpp,
 * TMat/pfunc.cpp:16-106).  Aux-bit operators (models B and D) are solved as
 * one device batch (tm_sweep_create + tm_sweep_eigs); other families by a pool
 * of `nthreads` host threads (0 = 16), each point on its own CUDA stream with
 * tm_eigs (ncv = tm_suggested_ncv, seed 0).  vals_re/vals_im: host, count*nev;
 * infos: host count or NULL; status: host count or NULL, per-instance codes.
 * Returns TM_OK if every instance succeeded, else the first failing code
 * (message names the instance). */
tm_status tm_eigs_batch(const tm_params* params, int count, char model, int dim, int axialdir,
                        int extend_cond, int nev, double tol, int mode, int nthreads, double* vals_re,
                        double* vals_im, tm_eigs_info* infos, tm_status* status);

/* ---- batched sweeps of aux-bit operators (no reference counterpart) ----- */

/* A sweep: `count` operators of one aux-bit family (model 'B' axialdir 3 or 7,
 * model 'D' axialdir 1, 2, 5, 6, 17 or 18; params[i] per point, widths may
 * differ) solved as one batch on the device.  The reference builds one
 * operator per tmat run (TMat/pfunc.cpp:16-106).  Here each chain pass of the
 * product is one launch over every member's tiles (an instance table in
 * device memory), every member extends its Arnoldi basis by one column per
 * step (one CUDA graph per step) and restarts on its own, and members are processed in waves that fit
 * the free device memory (tm_sweep_set_wave_bytes overrides the share). */
typedef struct tm_sweep tm_sweep;
tm_status tm_sweep_create(const tm_params* params, int count, char model, int dim, int axialdir,
                          int extend_cond, tm_sweep** out);
tm_status tm_sweep_destroy(tm_sweep* sweep);
int tm_sweep_count(const tm_sweep* sweep);
int64_t tm_sweep_rows(const tm_sweep* sweep, int i);        /* rows of member i */
double tm_sweep_normfactor(const tm_sweep* sweep, int i);   /* normfactor of member i */
tm_status tm_sweep_set_wave_bytes(tm_sweep* sweep, size_t bytes);  /* 0: 60% of free memory */
/* Diagnostics of the last tm_sweep_eigs: {waves, steps, seconds building the
 * waves, seconds in steps (device work, host-timed), seconds in host
 * restarts}; returns the count written (<= cap). */
int tm_sweep_stats(const tm_sweep* sweep, double* out, int cap);

/* y_i = T_i x_i for every member: host arrays of `count` device pointers to
 * FP64 vectors (length tm_sweep_rows(i)); dtype TM_F64, TM_F64_DF or TM_F32
 * (computed in FP32, returned widened).  Synchronous. */
tm_status tm_sweep_perform_op_dev(tm_sweep* sweep, const double* const* x_dev, double* const* y_dev,
                                  tm_dtype dtype);

/* Largest-magnitude eigenvalues of every member (Arnoldi; ncv 0 = the
 * reference's suggested_nev rule with at least 12 columns; start vector
 * uniform(0,1), seed 0).
 * vals_re/vals_im: host, count*nev, eigenvalues / normfactor in descending
 * magnitude; infos, status: host arrays of count or NULL.  Returns TM_OK or
 * the first failing member's code. */
tm_status tm_sweep_eigs(tm_sweep* sweep, int nev, int ncv, double tol, int mode, double* vals_re,
                        double* vals_im, tm_eigs_info* infos, tm_status* status);

/* As tm_sweep_eigs, and each member's leading eigenvector (real, unit norm)
 * into vec0_host[i] (host, tm_sweep_rows(i) doubles; NULL entries skip a
 * member), taken from the member's converged Ritz vector on the device. */
tm_status tm_sweep_eigs_vec(tm_sweep* sweep, int nev, int ncv, double tol, int mode, double* vals_re,
                            double* vals_im, double* const* vec0_host, tm_eigs_info* infos, tm_status* status);

/* transpose 1: the sweep's solves and products use the members' transposes
 * T^T (their eigenvectors are the left eigenvectors of T, as the reference's
 * getlefteigvec takes them from get_t_instance, TMat/pfunc.hpp:47-68). */
tm_status tm_sweep_set_transpose(tm_sweep* sweep, int transpose);

/* Batched adjoint (no reference counterpart): grad4[4 i + t] = d ln(lambda_i)
 * / d(betaJ, kappa, kappa2, h)_t of every member's reported eigenvalue, from
 * its right and left eigenvectors (host arrays of device-independent host
 * pointers, tm_sweep_rows(i) doubles each; ql_host NULL for symmetric
 * operators) and its internal eigenvalue (reported eigenvalue times
 * normfactor).  The Boltzmann-weight term is one batched reduction over all
 * members; the chain term is one batched tangent product per parameter (one
 * launch per pass over every member), as tm_grad computes for one operator. */
tm_status tm_sweep_grad(tm_sweep* sweep, const double* const* qr_host, const double* const* ql_host,
                        const double* lambda_internal, double* grad4);

/* Autotuner of the aux-bit chain kernels (no reference counterpart): times
 * the operator's product (TM_F32 or TM_F64_DF) over 2^11..2^14-element tiles
 * and 128 or 256 threads per block, keeps the fastest for this model, width
 * and element size in the process-wide tuning table (used by tm_perform_op*,
 * tm_eigs and sweeps), and returns it with its time per product. */
tm_status tm_chain_autotune(const tm_op* op, tm_dtype dtype, int* tile_bits, int* threads, double* ms);
/* Sets one entry of the tuning table (tile_bits 0 / threads 0: the default). */
tm_status tm_chain_set_tuning(char model, int L, tm_dtype dtype, int tile_bits, int threads);

/* ---- configuration planting (replaces DumpConfig) ----------------------- */

/* Plant `nconfig` layer sequences of `length` layers from the leading
 * eigenvector of a periodic x-ANNNI perpendicular TM (model 'A', axialdir 1:
 * XAT2DDumpConfig::dump, DumpConfig/dumpconfig.cpp:88-136; axialdir 5:
 * XAM2DDumpConfig::dump, DumpConfig/dumpreduce.cpp:47-122) or of the reduced
 * DNNI one (model 'D', axialdir 5: XDM2DDumpConfig::dump,
 * DumpConfig/dumpreduce.cpp:516-591).  vec_host: the
 * eigenvector as tm_eigs returns it (length rows; its absolute values are
 * used, as the reference reads X_vec.dat).  seed: the seed of the
 * reference's generator (std::mt19937 + uniform_real_distribution, as
 * MyUtility::setseed; its random stream is consumed in the reference's
 * order, so the same seed plants the same configurations).  states_out:
 * host, nconfig * length layer states (bit i = site i; the reference writes
 * each as a line of L digits, bit 0 first, to <prefix>_config_<k>.dat).
 * All chains advance together on the device: one launch per step computes
 * every chain's transfer-matrix column, cumulative sums and draw. */
tm_status tm_dump_configs(const tm_op* op, const double* vec_host, int nconfig, int length, uint32_t seed,
                          uint64_t* states_out);
/* The same for the two-layer parallel TMs, which plant from their right and
 * left leading eigenvectors (start weights |r| |l|, steps weighted by |r|; the
 * reference reads both files, GenDumpConfig::initq): the full one (model 'A',
 * axialdir 2: YAT2DDumpConfig::dump, DumpConfig/dumpconfig.cpp:171-219;
 * states_out holds nconfig * (length + 1) layers, as the reference writes
 * them: the first layer, the partner layer of every step, the last layer) and
 * the reduced ones (model 'A' axialdir 6 and model 'B' axialdir 6:
 * YAM2DDumpConfig / YBM2DDumpConfig::dump, DumpConfig/dumpreduce.cpp:156-256;
 * nconfig * length layers).  Other operators return TM_ERR_UNSUPPORTED here
 * (tm_dump_configs plants from their one vector). */
tm_status tm_dump_configs_lr(const tm_op* op, const double* vecr_host, const double* vecl_host, int nconfig,
                             int length, uint32_t seed, uint64_t* states_out);

/* ---- observables ------------------------------------------------------- */

/* Magnetisation moments <M^k>/L, k=1..4 (TMat/tmatphys.cpp:13-38, 71-98,
 * reduced overrides TMat/tmatreduce.cpp:565-591, 882-909, 1261-1287,
 * 1748-1775; TMat/tmat3d.cpp:137-163), from host eigenvectors ql, qr of
 * length rows (ql may equal qr).  Returns the reference's status in *ref_status. */
tm_status tm_moments(const tm_op* op, const double* ql_host, const double* qr_host, double out4[4],
                     int* ref_status);

/* Extended observables (phys_extend): <n_node>, <n_node^2> for X operators
 * (TMat/tmatphys.cpp:40-59, TMat/tmatreduce.cpp:593-613), the four stripe /
 * magnetisation averages for reduced DNNI (TMat/tmatreduce.cpp:1289-1320).
 * *nout receives the count written (<= cap); *ref_status the reference's
 * return status. */
tm_status tm_phys_extend(const tm_op* op, const double* ql_host, const double* qr_host, double* out,
                         int cap, int* nout, int* ref_status);

/* ---- adjoint (no reference counterpart) -------------------------------- */

/* d ln(lambda)/d(betaJ, kappa, kappa2, h) of the eigenvalue whose right
 * eigenvector is qr (and left eigenvector ql, NULL for symmetric operators),
 * for the x-ANNNI (model A, 2D and 3D), DNNI (model D) and diagonal BNNNI
 * (model B, axialdir 3 and 7) operators; the two-layer operators return
 * TM_ERR_UNSUPPORTED.
 * host FP64 vectors of length rows.  lambda_internal is the operator's own
 * eigenvalue (reported eigenvalue times normfactor).  The result includes the
 * -d ln(normfactor) term, so it is the derivative of the reported eigenvalue. */
tm_status tm_grad(const tm_op* op, const double* qr_host, const double* ql_host,
                  double lambda_internal, double grad4[4]);

/* ---- diagnostics (no reference counterpart) ---------------------------- */

/* Time the operator's matvec stages with CUDA events on the operator's
 * stream, averaged over `iters` products in the internal vector order
 * (dtype TM_F32, TM_F64 or TM_F64_DF).  For the even/odd reduced x-ANNNI product the
 * stages are {input scaling, pass 1, pass 2}; other operators report one
 * stage {whole product}.  ms_out receives up to `cap` per-launch averages;
 * *nstages the count. */
tm_status tm_profile_matvec(const tm_op* op, tm_dtype dtype, int iters, double* ms_out, int cap, int* nstages);

/* Number of CUDA kernels this library has launched since load (all ops). */
int64_t tm_launch_count(void);

/* Number of device allocations this library has requested since load (every
 * device buffer of operators, solvers and products goes through one
 * allocator).  A diagnostic: tests use it to show that an entry point
 * allocates nothing. */
int64_t tm_alloc_count(void);

/* Caps the tile size of the even/odd x-ANNNI passes at 2^bits elements for
 * operators created afterwards (0 removes the cap).  Operators whose tiles
 * exceed the cap split them over thread-block clusters, as those with
 * L >= 30 always do; the cap makes those code paths reachable at small L,
 * for tests.  Results are the same up to rounding. */
void tm_debug_set_eo_tile_bits(int bits);

/* ---- misc -------------------------------------------------------------- */

const char* tm_last_error(void);
const char* tm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* LATTTMAT_GB300_H */
