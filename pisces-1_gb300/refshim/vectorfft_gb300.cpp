// VectorFFT on the GB300 library: a drop-in for the reference's
// src/VectorFFTW.cpp (struct in src/VectorFFT.hpp:10-33), built into the
// reference in place of that file.  VectorFFT::apply computes
// y = V x + ifft(KE fft(x)) / N for the periodic FFT kinetic term
// (src/VectorFFTW.cpp:56-112); the operator is separable, so here it is the
// library's DVRType-3 grid (three per-axis circulant contractions) applied
// by pg_hx in FP64.  The box length is recovered from KE_diag: KE_diag at
// (k, 0, 0) is the plane-wave energy (dK k)^2 / 2 of axis 0, dK = 2 pi /
// (n dx), L = (n + 1) dx (src/KE_diag.cpp:33-80, src/DVR.cpp:617-630); the
// reference's FFT path assumes a cubic grid (src/VectorFFTW.cpp:83), so one
// axis gives L for all three.  The FFTW plans and work arrays of the
// original are not needed; their members stay unused.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "VectorFFT.hpp"
#include "pisces_gb300.h"

namespace {

struct FftGrid {
  pg_grid* g = nullptr;
  double* dev = nullptr;  // V, X and Y on the device
  size_t ngp = 0;
  double L = 0;
};

FftGrid& state(const VectorFFT* self) {
  // one set per process: the reference builds one VectorFFT per solve
  static FftGrid s;
  (void)self;
  return s;
}

void stop(const char* what) {
  std::cout << "VectorFFT (GB300): " << what << "\n";
  exit(1);
}

}  // namespace

VectorFFT::VectorFFT(int* ndim) {
  n_1dbas[0] = ndim[0];
  n_1dbas[1] = ndim[1];
  n_1dbas[2] = ndim[2];
  ngp = (size_t)ndim[0] * ndim[1] * ndim[2];
  ngp2 = (size_t)ndim[0] * ndim[1] * (ndim[2] / 2 + 1);
  phi_xk = nullptr;
  phi_x = nullptr;
  KE_phi_xk = nullptr;
}

VectorFFT::~VectorFFT() {
  FftGrid& s = state(this);
  if (s.g) pg_grid_destroy(s.g);
  if (s.dev) cudaFree(s.dev);
  s = FftGrid();
}

void VectorFFT::apply(const double* x, double* y, const double* v_diag, const double* KE_diag) {
  FftGrid& s = state(this);
  const int n = n_1dbas[0];
  if (n_1dbas[1] != n || n_1dbas[2] != n) stop("the FFT kinetic path needs a cubic grid, as the reference's");
  if (n < 2) stop("the grid needs two points per axis");
  const double pi = 3.14159265358979;  // the reference's (src/KE_diag.cpp:28-30)
  const double dk = sqrt(2.0 * KE_diag[(size_t)n * n]);
  const double L = (double)(n + 1) * (2.0 * pi / (double)n) / dk;
  if (!s.g || s.L != L || s.ngp != ngp) {
    if (s.g) pg_grid_destroy(s.g);
    if (s.dev) cudaFree(s.dev);
    s = FftGrid();
    const int nn[3] = {n, n, n};
    const double LL[3] = {L, L, L};
    if (pg_grid_create_dvr(nn, LL, 3, &s.g) != PG_OK) stop(pg_last_error());
    if (cudaMalloc(&s.dev, 3 * sizeof(double) * ngp) != cudaSuccess) stop("cudaMalloc failed");
    s.ngp = ngp;
    s.L = L;
  }
  double *dv = s.dev, *dx = s.dev + ngp, *dy = s.dev + 2 * ngp;
  if (cudaMemcpy(dv, v_diag, sizeof(double) * ngp, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dx, x, sizeof(double) * ngp, cudaMemcpyHostToDevice) != cudaSuccess)
    stop("copy to the device failed");
  if (pg_hx(s.g, dv, dx, dy, 1, PG_FP64, nullptr) != PG_OK) stop(pg_last_error());
  if (cudaMemcpy(y, dy, sizeof(double) * ngp, cudaMemcpyDeviceToHost) != cudaSuccess) stop("copy to the host failed");
}
