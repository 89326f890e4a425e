// Drives the reference-shaped Davidson() of include/pisces_gb300_ref.hpp the
// way DVR::davdriver does (src/davdriver.cpp:58-86): host arrays, host H*x
// one vector at a time.  Test program: prints the number of converged roots,
// the H*x count and the eigenvalues.
//
//   check_ref_shim            anisotropic harmonic well on a 10 x 11 x 12 sine-DVR grid
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pisces_gb300_ref.hpp"

int main() {
  const int n[3] = {10, 11, 12};
  const double L[3] = {12.0, 13.0, 14.0};
  const double kf[3] = {0.10, 0.15, 0.20};
  const int ng = n[0] * n[1] * n[2];
  std::vector<double> x[3], t[3];
  for (int a = 0; a < 3; ++a) {
    x[a].resize(n[a]);
    t[a].resize((size_t)n[a] * n[a]);
    sine_dvr(n[a], 1.0, -0.5 * L[a], 0.5 * L[a], x[a].data(), t[a].data(), n[a], 0);
  }
  std::vector<double> v(ng), diag(ng);
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int g = i + n[0] * (j + n[1] * k);
        v[g] = 0.5 * (kf[0] * x[0][i] * x[0][i] + kf[1] * x[1][j] * x[1][j] + kf[2] * x[2][k] * x[2][k]);
        diag[g] = v[g] + t[0][(size_t)i * n[0] + i] + t[1][(size_t)j * n[1] + j] + t[2][(size_t)k * n[2] + k];
      }
  long n_mtx = 0;
  auto hx = [&](const double* in, double* out) {  // y = V x + sum_a T_a x along axis a
    ++n_mtx;
    for (int k = 0; k < n[2]; ++k)
      for (int j = 0; j < n[1]; ++j)
        for (int i = 0; i < n[0]; ++i) {
          const int g = i + n[0] * (j + n[1] * k);
          double s = v[g] * in[g];
          for (int b = 0; b < n[0]; ++b) s += t[0][(size_t)i * n[0] + b] * in[b + n[0] * (j + n[1] * k)];
          for (int b = 0; b < n[1]; ++b) s += t[1][(size_t)j * n[1] + b] * in[i + n[0] * (b + n[1] * k)];
          for (int b = 0; b < n[2]; ++b) s += t[2][(size_t)k * n[2] + b] * in[i + n[0] * (j + n[1] * b)];
          out[g] = s;
        }
  };
  const int nstates = 3, maxsub = 24, maxiter = 100, ptol = 8, corrflag = 1;
  std::vector<double> B((size_t)ng * maxsub), Z((size_t)ng * maxsub), ev(nstates);
  std::vector<double> work(DavidsonWorkSize(ng, maxsub, nstates, corrflag));
  // start vectors as the reference's Randm11 (src/DVR.cpp:52-59) draws them
  // from the C library's rand() in an unseeded process: sign, then magnitude
  for (size_t e = 0; e < (size_t)ng * nstates; ++e) {
    if (std::rand() > RAND_MAX / 2) B[e] = (double)std::rand() / RAND_MAX;
    else B[e] = -(double)std::rand() / RAND_MAX;
  }
  int inout[3] = {0, 0, 0}, nconv = 0;
  while (Davidson(ng, maxsub, nstates, maxiter, ptol, corrflag, 0, ev.data(), nconv, B.data(), Z.data(),
                  diag.data(), work.data(), inout) != 0)
    for (int c = 0; c < inout[2]; ++c) hx(&B[(size_t)(inout[0] + c) * ng], &Z[(size_t)(inout[1] + c) * ng]);
  std::printf("%d %ld", nconv, n_mtx);
  for (int r = 0; r < nstates; ++r) std::printf(" %.17g", ev[r]);
  std::printf("\n");
  return nconv == nstates ? 0 : 1;
}
