// Small dense nonsymmetric eigenproblem (m <= 48), host/device code.
//
//  geneig_values: Householder reduction to upper Hessenberg form, then the
//    Francis double-shift QR iteration with deflation (Golub & Van Loan,
//    Matrix Computations, Alg. 7.4.2, 7.5.1, 7.5.2) for all eigenvalues.
//  geneig_vector: right eigenvector for one (complex) eigenvalue by inverse
//    iteration on (A - lambda I) with complex LU and partial pivoting.
// The Arnoldi solver (tm_arnoldi.cu) calls these on the host, where the
// projected matrices are brought back anyway; a CPU test compiles the same
// header with the host compiler.
#pragma once
#include <math.h>

#include "tm_bits.cuh"

namespace ltm {

constexpr int HQR_MMAX = 48;

// H: m x m column-major (overwritten).  Returns 0 on success, 1 when the
// iteration limit was hit (remaining diagonal copied out).
TM_HD int geneig_values(double* H, int m, double* wr, double* wi) {
#define Hm(i, j) H[(i) + (j) * m]
  for (int k = 0; k + 2 < m; ++k) {
    double nrm = 0.0;
    for (int i = k + 1; i < m; ++i) nrm += Hm(i, k) * Hm(i, k);
    nrm = sqrt(nrm);
    if (nrm == 0.0) continue;
    double x0 = Hm(k + 1, k);
    double alpha = (x0 > 0) ? -nrm : nrm;
    double v[HQR_MMAX];
    for (int i = k + 1; i < m; ++i) v[i] = Hm(i, k);
    v[k + 1] -= alpha;
    double vn = 0.0;
    for (int i = k + 1; i < m; ++i) vn += v[i] * v[i];
    if (vn == 0.0) continue;
    double sc = 2.0 / vn;
    for (int j = k; j < m; ++j) {
      double d = 0.0;
      for (int i = k + 1; i < m; ++i) d += v[i] * Hm(i, j);
      d *= sc;
      for (int i = k + 1; i < m; ++i) Hm(i, j) -= d * v[i];
    }
    for (int i = 0; i < m; ++i) {
      double d = 0.0;
      for (int j = k + 1; j < m; ++j) d += Hm(i, j) * v[j];
      d *= sc;
      for (int j = k + 1; j < m; ++j) Hm(i, j) -= d * v[j];
    }
    for (int i = k + 2; i < m; ++i) Hm(i, k) = 0.0;
  }
  const double eps = 2.220446049250313e-16;
  double anorm = 0.0;
  for (int j = 0; j < m; ++j)
    for (int i = 0; i <= (j + 1 < m ? j + 1 : m - 1); ++i) anorm += fabs(Hm(i, j));
  int hi = m - 1, its = 0, total = 0;
  while (hi >= 0) {
    int lo = hi;
    while (lo > 0) {
      double s = fabs(Hm(lo - 1, lo - 1)) + fabs(Hm(lo, lo));
      if (s == 0.0) s = anorm;
      if (fabs(Hm(lo, lo - 1)) <= eps * s) {
        Hm(lo, lo - 1) = 0.0;
        break;
      }
      --lo;
    }
    if (lo == hi) {
      wr[hi] = Hm(hi, hi);
      wi[hi] = 0.0;
      --hi;
      its = 0;
      continue;
    }
    if (lo == hi - 1) {
      double a = Hm(hi - 1, hi - 1), b = Hm(hi - 1, hi), c = Hm(hi, hi - 1), d = Hm(hi, hi);
      double p = 0.5 * (a - d), q = p * p + b * c, mid = 0.5 * (a + d);
      if (q >= 0.0) {
        double z = sqrt(q);
        double e1 = mid + (p >= 0 ? z : -z);
        double e2 = (e1 != 0.0) ? (a * d - b * c) / e1 : mid - (p >= 0 ? z : -z);
        wr[hi - 1] = e1;
        wr[hi] = e2;
        wi[hi - 1] = wi[hi] = 0.0;
      } else {
        double z = sqrt(-q);
        wr[hi - 1] = wr[hi] = mid;
        wi[hi - 1] = z;
        wi[hi] = -z;
      }
      hi -= 2;
      its = 0;
      continue;
    }
    if (++total > 60 * m) {
      for (int i = 0; i <= hi; ++i) {
        wr[i] = Hm(i, i);
        wi[i] = 0.0;
      }
      return 1;
    }
    ++its;
    double s, t;
    if (its % 10 == 0) {
      double e = fabs(Hm(hi, hi - 1)) + fabs(Hm(hi - 1, hi - 2));
      s = 1.5 * e + Hm(hi, hi);
      t = e * e;
    } else {
      s = Hm(hi - 1, hi - 1) + Hm(hi, hi);
      t = Hm(hi - 1, hi - 1) * Hm(hi, hi) - Hm(hi - 1, hi) * Hm(hi, hi - 1);
    }
    double x = Hm(lo, lo) * Hm(lo, lo) + Hm(lo, lo + 1) * Hm(lo + 1, lo) - s * Hm(lo, lo) + t;
    double y = Hm(lo + 1, lo) * (Hm(lo, lo) + Hm(lo + 1, lo + 1) - s);
    double z = Hm(lo + 1, lo) * Hm(lo + 2, lo + 1);
    for (int k = lo; k <= hi - 2; ++k) {
      double nr = sqrt(x * x + y * y + z * z);
      if (nr != 0.0) {
        double alpha = (x > 0) ? -nr : nr;
        double v0 = x - alpha, v1 = y, v2 = z;
        double vn = v0 * v0 + v1 * v1 + v2 * v2;
        if (vn != 0.0) {
          double sc = 2.0 / vn;
          int q0 = (lo > k - 1) ? lo : k - 1;
          for (int j = q0; j <= hi; ++j) {
            double d = sc * (v0 * Hm(k, j) + v1 * Hm(k + 1, j) + v2 * Hm(k + 2, j));
            Hm(k, j) -= d * v0;
            Hm(k + 1, j) -= d * v1;
            Hm(k + 2, j) -= d * v2;
          }
          int r = (k + 3 < hi) ? k + 3 : hi;
          for (int i = lo; i <= r; ++i) {
            double d = sc * (Hm(i, k) * v0 + Hm(i, k + 1) * v1 + Hm(i, k + 2) * v2);
            Hm(i, k) -= d * v0;
            Hm(i, k + 1) -= d * v1;
            Hm(i, k + 2) -= d * v2;
          }
        }
      }
      x = Hm(k + 1, k);
      y = Hm(k + 2, k);
      if (k < hi - 2) z = Hm(k + 3, k);
    }
    {
      double nr = sqrt(x * x + y * y);
      if (nr != 0.0) {
        double alpha = (x > 0) ? -nr : nr;
        double v0 = x - alpha, v1 = y;
        double sc = 2.0 / (v0 * v0 + v1 * v1);
        int k = hi - 1;
        int q0 = (lo > k - 1) ? lo : k - 1;
        for (int j = q0; j <= hi; ++j) {
          double d = sc * (v0 * Hm(k, j) + v1 * Hm(k + 1, j));
          Hm(k, j) -= d * v0;
          Hm(k + 1, j) -= d * v1;
        }
        for (int i = lo; i <= hi; ++i) {
          double d = sc * (Hm(i, k) * v0 + Hm(i, k + 1) * v1);
          Hm(i, k) -= d * v0;
          Hm(i, k + 1) -= d * v1;
        }
      }
    }
  }
  return 0;
#undef Hm
}

// Eigenvector of A (m x m, column-major, lda) for eigenvalue lr + i*li.
// Br, Bi: m*m scratch.  y = (yr, yi) unit 2-norm, largest component real
// positive.
TM_HD void geneig_vector(const double* A, int m, int lda, double lr, double li, double* Br, double* Bi, double* yr,
                         double* yi) {
  double anorm = 0.0;
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) anorm = fmax(anorm, fabs(A[i + j * lda]));
  const double tiny = 1e-14 * fmax(anorm, 1e-300);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) {
      Br[i + j * m] = A[i + j * lda] - (i == j ? lr : 0.0);
      Bi[i + j * m] = (i == j ? -li : 0.0);
    }
  int piv[HQR_MMAX];
  for (int k = 0; k < m; ++k) {
    int p = k;
    double best = -1.0;
    for (int i = k; i < m; ++i) {
      double a = fabs(Br[i + k * m]) + fabs(Bi[i + k * m]);
      if (a > best) {
        best = a;
        p = i;
      }
    }
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < m; ++j) {
        double tr = Br[k + j * m], ti = Bi[k + j * m];
        Br[k + j * m] = Br[p + j * m];
        Bi[k + j * m] = Bi[p + j * m];
        Br[p + j * m] = tr;
        Bi[p + j * m] = ti;
      }
    double dr = Br[k + k * m], di = Bi[k + k * m];
    if (fabs(dr) + fabs(di) < tiny) {
      dr = tiny;
      di = 0.0;
      Br[k + k * m] = dr;
      Bi[k + k * m] = di;
    }
    double den = dr * dr + di * di;
    for (int i = k + 1; i < m; ++i) {
      double ar = Br[i + k * m], ai = Bi[i + k * m];
      double fr = (ar * dr + ai * di) / den, fi = (ai * dr - ar * di) / den;
      Br[i + k * m] = fr;
      Bi[i + k * m] = fi;
      for (int j = k + 1; j < m; ++j) {
        double br = Br[k + j * m], bi = Bi[k + j * m];
        Br[i + j * m] -= fr * br - fi * bi;
        Bi[i + j * m] -= fr * bi + fi * br;
      }
    }
  }
  for (int i = 0; i < m; ++i) {
    yr[i] = (1.0 + 0.01 * i) / sqrt((double)m);
    yi[i] = 0.0;
  }
  for (int it = 0; it < 3; ++it) {
    for (int k = 0; k < m; ++k) {
      int p = piv[k];
      if (p != k) {
        double tr = yr[k], ti = yi[k];
        yr[k] = yr[p];
        yi[k] = yi[p];
        yr[p] = tr;
        yi[p] = ti;
      }
    }
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < i; ++j) {
        double a = Br[i + j * m], b = Bi[i + j * m];
        yr[i] -= a * yr[j] - b * yi[j];
        yi[i] -= a * yi[j] + b * yr[j];
      }
    for (int i = m - 1; i >= 0; --i) {
      double sr = yr[i], si = yi[i];
      for (int j = i + 1; j < m; ++j) {
        double ur = Br[i + j * m], ui = Bi[i + j * m];
        sr -= ur * yr[j] - ui * yi[j];
        si -= ur * yi[j] + ui * yr[j];
      }
      double dr = Br[i + i * m], di = Bi[i + i * m], den = dr * dr + di * di;
      yr[i] = (sr * dr + si * di) / den;
      yi[i] = (si * dr - sr * di) / den;
    }
    double nr = 0.0;
    for (int i = 0; i < m; ++i) nr += yr[i] * yr[i] + yi[i] * yi[i];
    nr = 1.0 / sqrt(nr);
    for (int i = 0; i < m; ++i) {
      yr[i] *= nr;
      yi[i] *= nr;
    }
  }
  int ib = 0;
  double bm = -1;
  for (int i = 0; i < m; ++i) {
    double a = yr[i] * yr[i] + yi[i] * yi[i];
    if (a > bm) {
      bm = a;
      ib = i;
    }
  }
  double pr = yr[ib], pi_ = yi[ib], pn = sqrt(pr * pr + pi_ * pi_);
  pr /= pn;
  pi_ /= pn;
  for (int i = 0; i < m; ++i) {
    double a = yr[i] * pr + yi[i] * pi_, b = yi[i] * pr - yr[i] * pi_;
    yr[i] = a;
    yi[i] = b;
  }
}

}  // namespace ltm
