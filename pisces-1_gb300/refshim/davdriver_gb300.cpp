// DVR::davdriver on the GB300 library: a drop-in for the reference's
// src/davdriver.cpp (same signature, DVR.h:125), built into the reference
// in place of that file.  The reference multiplies one vector at a time on
// the host inside its reverse-communication loop (src/davdriver.cpp:28-96);
// here the whole Davidson runs on the device through pg_solve, with the
// start vectors Diagonalize has set in wavefn (src/DVR.cpp:405-453) and the
// potential ComputePotential has set in v_diag.
//
// Kinetic term: DVRType 2 (sine DVR) and 3 (periodic FFT kinetic term, as
// three per-axis circulant contractions).  gridpara holds the box lengths,
// walls at -L/2 and +L/2 (src/DVR.cpp:603).  Errors print and exit, as the
// reference does.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "DVR.h"
#include "pisces_gb300.h"

namespace {

// The grid handle of the last call, kept while n, L and the type stay the
// same (a single-point stream solves many configurations on one grid).
struct GridCache {
  pg_grid* g = nullptr;
  int n[3] = {0, 0, 0}, type = 0;
  double L[3] = {0, 0, 0};
  ~GridCache() {
    if (g) pg_grid_destroy(g);
  }
};

void fail(const char* what) {
  std::cout << "davdriver (GB300): " << what << ": " << pg_last_error() << "\n";
  exit(1);
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::cout << "davdriver (GB300): " << what << ": " << cudaGetErrorString(e) << "\n";
    exit(1);
  }
}

}  // namespace

int DVR::davdriver(int ng, int nstates, int maxsub, int maxiter, int ptol, int corrflag, double* ev) {
  if (dvrtype != 2 && dvrtype != 3) {
    std::cout << "davdriver (GB300): DVRType " << dvrtype << " is not supported (2: sine DVR, 3: FFT)\n";
    exit(1);
  }
  static GridCache cache;
  const int type = dvrtype == 3 ? 3 : 2;
  bool same = cache.g && cache.type == type;
  for (int a = 0; a < 3 && same; ++a) same = cache.n[a] == n_1dbas[a] && cache.L[a] == gridpara[a];
  if (!same) {
    if (cache.g) pg_grid_destroy(cache.g);
    cache.g = nullptr;
    for (int a = 0; a < 3; ++a) cache.n[a] = n_1dbas[a], cache.L[a] = gridpara[a];
    cache.type = type;
    if (pg_grid_create_dvr(cache.n, cache.L, type, &cache.g) != PG_OK) fail("grid");
  }
  if (pg_grid_npoints(cache.g) != ng) fail("grid size");
  double *v = nullptr, *vec = nullptr;
  cuda_check(cudaMalloc(&v, sizeof(double) * ng), "cudaMalloc");
  cuda_check(cudaMalloc(&vec, sizeof(double) * ng * nstates), "cudaMalloc");
  cuda_check(cudaMemcpy(v, v_diag, sizeof(double) * ng, cudaMemcpyHostToDevice), "copy of V");
  cuda_check(cudaMemcpy(vec, &wavefn[0], sizeof(double) * ng * nstates, cudaMemcpyHostToDevice), "copy of start vectors");
  // the reference's arithmetic (FP64) and correction; start vectors as given
  pg_solve_params p = {nstates, maxsub, maxiter, ptol, corrflag, PG_FP64, 0, 0};
  pg_solve_stats st;
  const pg_status s = pg_solve(cache.g, v, &p, ev, vec, &st, nullptr);
  if (s != PG_OK && s != PG_NOT_CONVERGED) fail("pg_solve");
  cuda_check(cudaMemcpy(&wavefn[0], vec, sizeof(double) * ng * nstates, cudaMemcpyDeviceToHost), "copy of vectors");
  cudaFree(v);
  cudaFree(vec);
  if (verbose > 0) {
    printf("-----------------------------------------------\n");
    printf("Davidson finishes after %i matrix-times-vector operations\n", st.n_matvec);
    printf("%i states have been converged.\n", st.nconv);
  }
  // as the reference: not converging only reports fewer converged roots
  return st.nconv;
}
