// Host-side algebra of the Krylov-Schur restart for general operators
// (tm_arnoldi.cu), shared with the batched parameter sweep (tm_sweep.cu).
#pragma once
#include <complex>
#include <vector>

namespace ltm {

struct Ritz {
  std::vector<std::complex<double>> theta;           // sorted by |theta| desc
  std::vector<double> resid;                         // |beta| |y[m-1]| per computed vector
  std::vector<std::vector<std::complex<double>>> y;  // eigenvectors of H (m)
  double beta = 0;
};

Ritz krylov_project(const double* Hh, int m, int kvec);
int krylov_kvec(int m, int nev);
int krylov_keep(int m, int nev, int nconv, int kvec);
int krylov_basis(const Ritz& R, int m, int kk, std::vector<double>& Wm);
void krylov_restart_h(const double* Hh, int m, const std::vector<double>& Wm, int k, double beta,
                      std::vector<double>& Hn);

}  // namespace ltm
