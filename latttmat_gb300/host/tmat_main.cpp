// tmat -- GB300 drop-in for the reference's `tmat` driver (TMat/main.cpp:31-65,
// TMat/pfunc.cpp:16-106, TMat/pfunc.hpp:79-202).
//
//   tmat [input.dat] [--mixed] [--parse-only]
//
// Reads the same positional input file, builds the operator on the GPU
// through the C ABI, solves for `neigs` largest-magnitude eigenvalues and
// writes <out>_val.dat, <out>_vec.dat, <out>_vecl.dat, <out>_phys.dat in the
// reference formats.  Default: every matvec in FP64, residual tolerance 1e-10
// (the reference's solver default), so vectors and observables match the
// reference.  --mixed: FP32 matvec bulk with FP64 refinement; eigenvalues to
// 1e-10 relative, eigenvectors to FP32-level accuracy.
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <iostream>
#include <vector>

#include "latttmat.h"
#include "latttmat.hpp"
#include "read_input.hpp"
#include "tmat_io.hpp"

using latttmat::ReadInput;

// extend_cond the reference driver passes for each reduced operator
// (TMat/pfunc.cpp:22-99: multieigs = neigs>1 ? 2 : 0; axialdir 13 adds the
// open-boundary bit)
static int driver_extend_cond(const ReadInput& in) {
  const int multieigs = in.neigs > 1 ? 2 : 0;
  if (in.model == 'A' && in.dim == 2 && in.axialdir == 13) return multieigs | 1;
  return multieigs;
}

static int pfunc(const ReadInput& in, int mode, int64_t* opcount) {
  tm_params p{in.betaJ, in.kappa, in.kappa2, in.h, in.size};
  tm_op* op = nullptr;
  tm_status st = tm_create(&p, in.model, in.dim, in.axialdir, driver_extend_cond(in), &op);
  if (st != TM_OK) {
    std::cout << "Function yet implemented" << std::endl;
    std::cerr << tm_last_error() << std::endl;
    return -1;
  }
  const int64_t n = tm_rows(op);
  const bool sym = tm_is_symmetric(op) == 1;
  const double nf = tm_normfactor(op);
  int nev = in.neigs;
  if (nev >= n) nev = (int)n - 1;
  std::vector<double> vr(nev), vi(nev);
  std::vector<double> vecs(sym ? (size_t)nev * n : (size_t)2 * nev * n);
  tm_eigs_info info{};
  st = tm_eigs(op, nev, 0, 1e-10, 0, mode, vr.data(), vi.data(), vecs.data(), nullptr, &info);
  if (info.nconv == 0) {
    std::cerr << "Number of converged eigenvalue is zero" << std::endl;
    tm_destroy(op);
    exit(-1);
  }
  const int ncv = info.nconv;
  std::vector<std::complex<double>> vals(ncv);
  for (int i = 0; i < ncv; ++i) vals[i] = {vr[i], vi[i]};
  latttmat::write_val(in.outprefix + "_val.dat", vals, sym);
  if (in.savevec[0]) {
    if (sym)
      latttmat::write_vec_sym(in.outprefix + "_vec.dat", std::vector<double>(vecs.begin(), vecs.begin() + (size_t)ncv * n));
    else
      latttmat::write_vec_gen(in.outprefix + "_vec.dat", vecs, n, ncv);
  }
  int64_t count = info.matvecs;
  if (in.savevec[1]) {
    std::vector<double> qr(n), ql;
    for (int64_t i = 0; i < n; ++i) qr[i] = sym ? vecs[i] : vecs[2 * i];
    if (!sym) {
      // left eigenvector from the transpose operator, nev=1 (TMat/pfunc.hpp:47-68)
      tm_op* top = nullptr;
      tm_transpose(op, &top);
      double lr = 0, li = 0;
      std::vector<double> lvec(2 * n);
      tm_eigs_info linfo{};
      tm_status lst = tm_eigs(top, 1, 7, 1e-10, 1, mode, &lr, &li, lvec.data(), nullptr, &linfo);
      count += linfo.matvecs;
      if (lst != TM_OK || linfo.nconv == 0) {
        std::cout << "Warning: left eigenvalue calculation failed." << std::endl;
      } else {
        ql.resize(n);
        for (int64_t i = 0; i < n; ++i) ql[i] = lvec[2 * i];
        if (in.savevec[0]) latttmat::write_vecl(in.outprefix + "_vecl.dat", ql);
        std::streamsize ss = std::cout.precision();
        std::cout.precision(10);
        std::cout << "Eigensolver check: " << std::abs(std::complex<double>(vr[0], vi[0]) / std::complex<double>(lr, li))
                  << std::endl;
        std::cout.precision(ss);
      }
      tm_destroy(top);
    }
    const double* qlp = ql.empty() ? qr.data() : ql.data();
    double mom[4] = {0, 0, 0, 0};
    int mst = 0;
    tm_moments(op, qlp, qr.data(), mom, &mst);
    double ext[16];
    int next = 0, pst = 0;
    tm_phys_extend(op, qlp, qr.data(), ext, 16, &next, &pst);
    latttmat::write_phys(in.outprefix + "_phys.dat", mom, std::vector<double>(ext, ext + next));
  }
  *opcount = count;
  (void)nf;
  tm_destroy(op);
  return 0;
}

int main(int argc, char** argv) {
  const char* infile = "input.dat";
  int mode = TM_EIGS_F64;
  bool parse_only = false;
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--mixed"))
      mode = TM_EIGS_MIXED;
    else if (!std::strcmp(argv[i], "--f64"))
      mode = TM_EIGS_F64;
    else if (!std::strcmp(argv[i], "--parse-only"))
      parse_only = true;
    else
      infile = argv[i];
  }
  ReadInput input;
  int err = input.read(infile);
  if (err) return err;
  if (parse_only) return 0;
  auto t1 = std::chrono::steady_clock::now();
  int64_t opcount = 0;
  int rc = pfunc(input, mode, &opcount);
  auto t2 = std::chrono::steady_clock::now();
  float tc = std::chrono::duration<double>(t2 - t1).count();
  if (tc >= 1.0f) std::cout << "Time consumed: " << tc << " s" << std::endl;
  if (opcount > 0) std::cout << "Number of iteration: " << opcount << std::endl;
  return rc < 0 ? 1 : 0;
}
