// Reference-shaped C++ entry points over the C ABI of libpisces_gb300.
//
// Header-only.  Each function keeps the signature and argument meaning of
// the reference function it replaces, so a reference-shaped caller
// (DVR::davdriver's loop, the kinetic builders) recompiles against this
// header without changes:
//
//   sine_dvr          src/sine_dvr.h:1, src/sine_dvr.cpp:45-131
//   Tdiag             src/KE_diag.cpp:33-80   (FFT kinetic energies; ldt ignored)
//   DavidsonWorkSize  src/Davidson.h:1, src/Davidson.cpp:46-52
//   Davidson          src/Davidson.h:2-15, src/Davidson.cpp:61-376
//
// Davidson() here takes the reference's HOST arrays B, Z, diag, davwork and
// keeps their device mirrors itself: at the first call of a solve it uploads
// the start vectors and diag(H); when it returns 1 it has copied the block
// B[inout[0] .. inout[0]+inout[2]) to the host for the caller's H*x; at the
// next call it uploads the Z columns the caller filled; when it returns 0 it
// has copied the converged vectors B[0 .. nroots) to the host.  davwork is not
// used (the work array lives on the device).  Like the reference it keeps one
// solve's state in a static and is not re-entrant; pg_davidson_rci is the
// re-entrant form.  Errors print pg_last_error() and end the solve (return 0),
// where the reference exits.
#ifndef PISCES_GB300_REF_HPP
#define PISCES_GB300_REF_HPP

#include <cuda_runtime.h>

#include <cstdio>

#include "pisces_gb300.h"

inline void sine_dvr(int ngp, double mu, double x0, double xNp1, double* x, double* ekin, int ldt, int /*verbose*/) {
  if (pg_sine_dvr(ngp, mu, x0, xNp1, x, ekin, ldt) != PG_OK) std::fprintf(stderr, "sine_dvr: %s\n", pg_last_error());
}

inline void Tdiag(int ngp, double mu, double x0, double xNp1, double* x, double* ekin, int /*ldt*/, int /*verbose*/) {
  if (pg_fft_kinetic(ngp, mu, x0, xNp1, x, ekin, nullptr) != PG_OK)
    std::fprintf(stderr, "Tdiag: %s\n", pg_last_error());
}

inline int DavidsonWorkSize(int ndim, int maxsub, int nroots, int jdflag) {
  return (int)pg_davidson_work_size(ndim, maxsub, nroots, jdflag);
}

namespace pisces_gb300_ref {

struct DavidsonMirror {
  pg_davidson* handle = nullptr;
  double *B = nullptr, *Z = nullptr, *diag = nullptr, *work = nullptr;
  int ndim = 0, maxsub = 0, nroots = 0, corrflag = -1;
  bool in_solve = false;

  void release() {
    cudaFree(B);
    cudaFree(Z);
    cudaFree(diag);
    cudaFree(work);
    B = Z = diag = work = nullptr;
  }
  bool ensure(int nd, int ms, int nr, int cf) {
    if (handle == nullptr && pg_davidson_create(&handle) != PG_OK) return false;
    if (B && nd == ndim && ms == maxsub && nr == nroots && cf == corrflag) return true;
    release();
    ndim = nd, maxsub = ms, nroots = nr, corrflag = cf;
    const size_t nb = sizeof(double) * (size_t)nd * ms;
    const size_t nw = sizeof(double) * (size_t)pg_davidson_work_size(nd, ms, nr, cf);
    return cudaMalloc(&B, nb) == cudaSuccess && cudaMalloc(&Z, nb) == cudaSuccess &&
           cudaMalloc(&diag, sizeof(double) * (size_t)nd) == cudaSuccess && cudaMalloc(&work, nw) == cudaSuccess;
  }
};

inline DavidsonMirror& mirror() {
  static DavidsonMirror m;
  return m;
}

}  // namespace pisces_gb300_ref

inline int Davidson(int ndim, int maxsub, int nroots, int maxmacro, int tol, int corrflag, int /*verbose*/,
                    double* eval, int& nConv, double* B, double* Z, double* diag, double* /*davwork*/,
                    int* inout) {
  pisces_gb300_ref::DavidsonMirror& m = pisces_gb300_ref::mirror();
  const size_t col = sizeof(double) * (size_t)ndim;
  if (!m.in_solve) {
    if (!m.ensure(ndim, maxsub, nroots, corrflag) ||
        cudaMemcpy(m.B, B, col * nroots, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m.diag, diag, col, cudaMemcpyHostToDevice) != cudaSuccess) {
      std::fprintf(stderr, "Davidson: device set-up failed\n");
      return 0;
    }
    m.in_solve = true;
  } else if (cudaMemcpy(m.Z + (size_t)inout[1] * ndim, Z + (size_t)inout[1] * ndim, col * inout[2],
                        cudaMemcpyHostToDevice) != cudaSuccess) {
    std::fprintf(stderr, "Davidson: upload of H*B failed\n");
    m.in_solve = false;
    return 0;
  }
  int ret = 0, nc = nConv;
  const pg_status s = pg_davidson_rci(m.handle, ndim, maxsub, nroots, maxmacro, tol, corrflag, eval, &nc, m.B, m.Z,
                                      m.diag, m.work, inout, &ret, nullptr);
  nConv = nc;
  if (s != PG_OK && s != PG_NOT_CONVERGED) {
    std::fprintf(stderr, "Davidson: %s\n", pg_last_error());
    m.in_solve = false;
    return 0;
  }
  if (ret == 1) {  // the caller computes Z = H B for this block
    cudaMemcpy(B + (size_t)inout[0] * ndim, m.B + (size_t)inout[0] * ndim, col * inout[2], cudaMemcpyDeviceToHost);
    return 1;
  }
  cudaMemcpy(B, m.B, col * nroots, cudaMemcpyDeviceToHost);
  m.in_solve = false;
  return 0;
}

#endif  // PISCES_GB300_REF_HPP
