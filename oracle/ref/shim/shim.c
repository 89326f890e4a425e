/* Link-time stand-ins for the libraries the reference CPU code expects, used
 * only to build that code as the test oracle:
 *  - BLAS/LAPACK entry points forwarded to the OpenBLAS that ships inside the
 *    installed scipy wheel (its symbols carry a "scipy_" prefix);
 *  - FFTW plan constructors that hand back a dummy plan (the sine-DVR Davidson
 *    driver builds an FFT engine it never executes) and an fftw_execute that
 *    aborts, so the FFT kinetic path can never return a silent wrong answer;
 *  - ARPACK and L-BFGS symbols that abort (neither is on the Davidson path). */
#include <stdio.h>
#include <stdlib.h>
#include <stddef.h>

typedef double fftw_complex[2];
typedef struct oracle_fftw_plan_s* fftw_plan;
static int dummy_plan;
static void die(const char* what) { fprintf(stderr, "oracle shim: %s is not available in the oracle build\n", what); abort(); }
void* fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void* p) { free(p); }
fftw_plan fftw_plan_dft_r2c(int r, const int* n, double* i, fftw_complex* o, unsigned f) { (void)r; (void)n; (void)i; (void)o; (void)f; return (fftw_plan)&dummy_plan; }
fftw_plan fftw_plan_dft_c2r(int r, const int* n, fftw_complex* i, double* o, unsigned f) { (void)r; (void)n; (void)i; (void)o; (void)f; return (fftw_plan)&dummy_plan; }
fftw_plan fftw_plan_dft(int r, const int* n, fftw_complex* i, fftw_complex* o, int s, unsigned f) { (void)r; (void)n; (void)i; (void)o; (void)s; (void)f; return (fftw_plan)&dummy_plan; }
fftw_plan fftw_plan_dft_r2c_3d(int a, int b, int c, double* i, fftw_complex* o, unsigned f) { (void)a; (void)b; (void)c; (void)i; (void)o; (void)f; return (fftw_plan)&dummy_plan; }
fftw_plan fftw_plan_dft_c2r_3d(int a, int b, int c, fftw_complex* i, double* o, unsigned f) { (void)a; (void)b; (void)c; (void)i; (void)o; (void)f; return (fftw_plan)&dummy_plan; }
fftw_plan fftw_plan_dft_3d(int a, int b, int c, fftw_complex* i, fftw_complex* o, int s, unsigned f) { (void)a; (void)b; (void)c; (void)i; (void)o; (void)s; (void)f; return (fftw_plan)&dummy_plan; }
void fftw_execute(const fftw_plan p) { (void)p; die("fftw_execute"); }
void fftw_destroy_plan(fftw_plan p) { (void)p; }
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
