// Forward/backward of latttmat::EigenFunction on the GPU against central
// finite differences of its own forward pass (step 1e-5): the gradients of
// ln(lambda0) and of xi with respect to betaJ, kappa and h.  Prints one line
// per parameter and exits 0 when every gradient is within tolerance.
//   usage: eigen_function_check model dim axialdir extend_cond betaJ kappa h size
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "latttmat.hpp"

int main(int argc, char** argv) {
  if (argc != 9) {
    std::fprintf(stderr, "usage: %s model dim axialdir extend_cond betaJ kappa h size\n", argv[0]);
    return 2;
  }
  const char model = argv[1][0];
  const int dim = std::atoi(argv[2]), ax = std::atoi(argv[3]), ec = std::atoi(argv[4]);
  const double p0[4] = {std::atof(argv[5]), std::atof(argv[6]), 0.0, std::atof(argv[7])};
  const int size = std::atoi(argv[8]);
  const double step = 1e-5;
  auto make = [&](const double* p) { return latttmat::GpuMatVecProd(p[0], p[1], p[2], p[3], size, model, dim, ax, ec); };
  try {
    latttmat::GpuMatVecProd op = make(p0);
    const latttmat::EigenForward f = latttmat::EigenFunction::forward(op);
    const auto g_log = latttmat::EigenFunction::backward(op, f, 1.0, 0.0);
    const auto g_xi = latttmat::EigenFunction::backward(op, f, 0.0, 1.0);
    int bad = 0;
    for (int t : {0, 1, 3}) {
      if (t == 3 && p0[3] == 0.0) continue;
      double pp[4], pm[4];
      for (int i = 0; i < 4; ++i) pp[i] = pm[i] = p0[i];
      pp[t] += step;
      pm[t] -= step;
      latttmat::GpuMatVecProd opp = make(pp), opm = make(pm);
      const latttmat::EigenForward fp = latttmat::EigenFunction::forward(opp);
      const latttmat::EigenForward fm = latttmat::EigenFunction::forward(opm);
      const double fd_log = (fp.log_lambda0 - fm.log_lambda0) / (2 * step);
      const double fd_xi = (fp.xi - fm.xi) / (2 * step);
      const bool ok = std::fabs(g_log[t] - fd_log) < 2e-6 * std::fmax(1.0, std::fabs(fd_log)) &&
                      std::fabs(g_xi[t] - fd_xi) < 1e-5 * std::fmax(1.0, std::fabs(fd_xi));
      std::printf("param %d: dlnlam0 %.12e fd %.12e | dxi %.12e fd %.12e %s\n", t, g_log[t], fd_log, g_xi[t], fd_xi,
                  ok ? "ok" : "MISMATCH");
      bad += !ok;
    }
    std::printf("lambda0 %.15e xi %.15e\n", f.lambda0, f.xi);
    return bad ? 1 : 0;
  } catch (const latttmat::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", (int)e.code, e.what());
    return 3;
  }
}
