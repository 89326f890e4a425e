/* Link-time stand-ins for the libraries the reference CPU code expects, used
 * only to build that code as the test oracle:
 *  - BLAS/LAPACK entry points forwarded to the OpenBLAS that ships inside the
 *    installed scipy wheel (its symbols carry a "scipy_" prefix);
 *  - FFTW 3 (a third-party library the reference links, absent from its
 *    tree; its CMake file takes any installed FFTW 3): the plan constructors
 *    and fftw_execute the reference calls, computing the transforms FFTW
 *    defines -- the multi-dimensional DFT y[k] = sum_j x[j] e^{s 2 pi i j.k / n}
 *    (s = -1 forward, +1 backward, unnormalised), row-major arrays, the real
 *    input (r2c) giving the n_last/2 + 1 non-redundant outputs of the last
 *    dimension and c2r the real inverse of such a half spectrum -- directly
 *    from that definition, one axis at a time, in FP64 (O(N sum n) work);
 *  - ARPACK and L-BFGS symbols that abort (neither is on the Davidson path). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <stddef.h>
#include <string.h>

typedef double fftw_complex[2];
typedef struct oracle_fftw_plan_s {
  int kind;  /* 0 c2c, 1 r2c, 2 c2r */
  int n[3];  /* leading dimensions padded with 1 */
  int sign;
  void* in;
  void* out;
}* fftw_plan;
static void die(const char* what) { fprintf(stderr, "oracle shim: %s is not available in the oracle build\n", what); abort(); }
void* fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void* p) { free(p); }

static fftw_plan make_plan(int kind, int rank, const int* n, void* in, void* out, int sign) {
  if (rank < 1 || rank > 3) die("a transform of rank other than 1-3");
  fftw_plan p = (fftw_plan)malloc(sizeof(*p));
  if (!p) die("plan allocation");
  p->kind = kind;
  p->n[0] = p->n[1] = p->n[2] = 1;
  for (int a = 0; a < rank; ++a) p->n[3 - rank + a] = n[a];
  p->sign = sign;
  p->in = in;
  p->out = out;
  return p;
}
fftw_plan fftw_plan_dft_r2c(int r, const int* n, double* i, fftw_complex* o, unsigned f) { (void)f; return make_plan(1, r, n, i, o, -1); }
fftw_plan fftw_plan_dft_c2r(int r, const int* n, fftw_complex* i, double* o, unsigned f) { (void)f; return make_plan(2, r, n, i, o, +1); }
fftw_plan fftw_plan_dft(int r, const int* n, fftw_complex* i, fftw_complex* o, int s, unsigned f) { (void)f; return make_plan(0, r, n, i, o, s); }
fftw_plan fftw_plan_dft_r2c_3d(int a, int b, int c, double* i, fftw_complex* o, unsigned f) { const int n[3] = {a, b, c}; return fftw_plan_dft_r2c(3, n, i, o, f); }
fftw_plan fftw_plan_dft_c2r_3d(int a, int b, int c, fftw_complex* i, double* o, unsigned f) { const int n[3] = {a, b, c}; return fftw_plan_dft_c2r(3, n, i, o, f); }
fftw_plan fftw_plan_dft_3d(int a, int b, int c, fftw_complex* i, fftw_complex* o, int s, unsigned f) { const int n[3] = {a, b, c}; return fftw_plan_dft(3, n, i, o, s, f); }

/* In-place DFT of the complex array z[n0][n1][n2] along axis ax, sign s:
 * the twiddles e^{s 2 pi i m / n} for m = j k mod n (exact arguments). */
static void dft_axis(double* z, const int* n, int ax, int s) {
  const int len = n[ax];
  const long stride = ax == 2 ? 1 : (ax == 1 ? n[2] : (long)n[1] * n[2]);
  const long count = (long)n[0] * n[1] * n[2] / len;
  double* cw = (double*)malloc(sizeof(double) * 2 * len);
  double* buf = (double*)malloc(sizeof(double) * 2 * len);
  if (!cw || !buf) die("DFT scratch");
  const double pi = 3.14159265358979323846;
  for (int m = 0; m < len; ++m) {
    cw[2 * m] = cos(2.0 * pi * m / len);
    cw[2 * m + 1] = s * sin(2.0 * pi * m / len);
  }
  for (long line = 0; line < count; ++line) {
    /* the line's first element: all index combinations of the other axes */
    long base;
    if (ax == 2) base = line * len;
    else if (ax == 1) base = (line / n[2]) * (long)n[1] * n[2] + line % n[2];
    else base = line;
    for (int k = 0; k < len; ++k) {
      double re = 0, im = 0;
      for (int j = 0; j < len; ++j) {
        const int m = (int)(((long)j * k) % len);
        const double xr = z[2 * (base + j * stride)], xi = z[2 * (base + j * stride) + 1];
        re += xr * cw[2 * m] - xi * cw[2 * m + 1];
        im += xr * cw[2 * m + 1] + xi * cw[2 * m];
      }
      buf[2 * k] = re;
      buf[2 * k + 1] = im;
    }
    for (int k = 0; k < len; ++k) {
      z[2 * (base + k * stride)] = buf[2 * k];
      z[2 * (base + k * stride) + 1] = buf[2 * k + 1];
    }
  }
  free(cw);
  free(buf);
}

void fftw_execute(const fftw_plan p) {
  const int n0 = p->n[0], n1 = p->n[1], n2 = p->n[2], nh = n2 / 2 + 1;
  const long N = (long)n0 * n1 * n2;
  double* z = (double*)calloc((size_t)(2 * N), sizeof(double));
  if (!z) die("DFT array");
  if (p->kind == 0) {
    memcpy(z, p->in, sizeof(double) * 2 * N);
  } else if (p->kind == 1) {
    const double* x = (const double*)p->in;
    for (long g = 0; g < N; ++g) z[2 * g] = x[g];
  } else {
    /* the full spectrum from its half: X[k] = conj(X[-k]) for k2 > n2/2 */
    const double* h = (const double*)p->in;
    for (int a = 0; a < n0; ++a)
      for (int b = 0; b < n1; ++b)
        for (int c = 0; c < n2; ++c) {
          const long g = ((long)a * n1 + b) * n2 + c;
          if (c < nh) {
            const long q = ((long)a * n1 + b) * nh + c;
            z[2 * g] = h[2 * q];
            z[2 * g + 1] = h[2 * q + 1];
          } else {
            const long q = ((long)((n0 - a) % n0) * n1 + (n1 - b) % n1) * nh + (n2 - c);
            z[2 * g] = h[2 * q];
            z[2 * g + 1] = -h[2 * q + 1];
          }
        }
  }
  for (int ax = 0; ax < 3; ++ax)
    if (p->n[ax] > 1) dft_axis(z, p->n, ax, p->sign);
  if (p->kind == 0) {
    memcpy(p->out, z, sizeof(double) * 2 * N);
  } else if (p->kind == 1) {
    double* h = (double*)p->out;
    for (int a = 0; a < n0; ++a)
      for (int b = 0; b < n1; ++b)
        for (int c = 0; c < nh; ++c) {
          const long g = ((long)a * n1 + b) * n2 + c, q = ((long)a * n1 + b) * nh + c;
          h[2 * q] = z[2 * g];
          h[2 * q + 1] = z[2 * g + 1];
        }
  } else {
    double* y = (double*)p->out;
    for (long g = 0; g < N; ++g) y[g] = z[2 * g];
  }
  free(z);
}
void fftw_destroy_plan(fftw_plan p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void)n; }
void fftw_cleanup_threads(void) {}

/* BLAS level 1-3 and LAPACK, Fortran calling convention (all by reference). */
#define FWD(ret, name, params, args) \
  extern ret scipy_##name##_ params; \
  ret name##_ params { return scipy_##name##_ args; }
FWD(void, dscal, (int* n, double* a, double* x, int* ix), (n, a, x, ix))
FWD(void, dcopy, (int* n, double* x, int* ix, double* y, int* iy), (n, x, ix, y, iy))
FWD(void, daxpy, (int* n, double* a, double* x, int* ix, double* y, int* iy), (n, a, x, ix, y, iy))
FWD(double, dnrm2, (int* n, double* x, int* ix), (n, x, ix))
FWD(double, ddot, (int* n, const double* x, int* ix, const double* y, int* iy), (n, x, ix, y, iy))
FWD(void, dsyev, (const char* jz, const char* ul, int* n, double* a, int* lda, double* w, double* wk, int* lw, int* info), (jz, ul, n, a, lda, w, wk, lw, info))
FWD(void, dgeev, (const char* jl, const char* jr, int* n, double* a, int* lda, double* wr, double* wi, double* vl, int* ldvl, double* vr, int* ldvr, double* wk, int* lw, int* info), (jl, jr, n, a, lda, wr, wi, vl, ldvl, vr, ldvr, wk, lw, info))
FWD(void, dsteqr, (const char* c, int* n, double* d, double* e, double* z, int* ldz, double* wk, int* info), (c, n, d, e, z, ldz, wk, info))
FWD(void, dgemv, (const char* t, const int* m, const int* n, const double* al, const double* a, const int* lda, const double* x, const int* ix, const double* be, double* y, const int* iy), (t, m, n, al, a, lda, x, ix, be, y, iy))
FWD(void, dsymv, (const char* u, const int* n, const double* al, const double* a, const int* lda, const double* x, const int* ix, const double* be, double* y, const int* iy), (u, n, al, a, lda, x, ix, be, y, iy))
FWD(void, dgemm, (const char* ta, const char* tb, const int* m, const int* n, const int* k, const double* al, const double* a, const int* lda, const double* b, const int* ldb, const double* be, double* c, const int* ldc), (ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc))
FWD(void, dsytrf, (const char* u, int* n, double* a, int* lda, int* ipiv, double* w, int* lw, int* info), (u, n, a, lda, ipiv, w, lw, info))
FWD(void, dsytri, (const char* u, int* n, double* a, int* lda, int* ipiv, double* w, int* info), (u, n, a, lda, ipiv, w, info))
FWD(void, dspmv, (const char* u, const int* n, const double* al, const double* ap, const double* x, const int* ix, const double* be, double* y, const int* iy), (u, n, al, ap, x, ix, be, y, iy))
FWD(void, dgetrf, (int* m, int* n, double* a, int* lda, int* ipiv, int* info), (m, n, a, lda, ipiv, info))
FWD(void, dgetri, (int* n, double* a, int* lda, int* ipiv, double* w, int* lw, int* info), (n, a, lda, ipiv, w, lw, info))

/* ARPACK (Lanczos alternative) and L-BFGS (geometry optimiser): not on the path. */
void dsaupd_(void) { die("ARPACK dsaupd"); }
void dseupd_(void) { die("ARPACK dseupd"); }
void lbfgs_(void) { die("L-BFGS"); }
