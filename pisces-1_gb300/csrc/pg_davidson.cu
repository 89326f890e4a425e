// Reverse-communication Davidson on the device, the driver loop, and the
// whole single point from host data.
//
// pg_davidson_rci restates the reference algorithm of Davidson()
// (src/Davidson.cpp:61-376) step for step -- same subspace growth, restart
// rule, locking weight, correction vectors and return protocol -- with every
// O(N) operation a device kernel (pg_linalg.cu) and only O(maxsub^2) data on
// the host: the subspace matrix S, its eigenvectors and the convergence
// bookkeeping.  Differences that do not change the subspace:
//   - S = Z^T B is extended by its new columns only (the reference recomputes
//     all of it each iteration, src/Davidson.cpp:220, 385-393; the values it
//     reads -- the upper triangle -- are the same dot products);
//   - the correction vectors are orthogonalised against the basis and among
//     themselves as one block, by two passes of block Gram-Schmidt with the
//     Pythagorean Gram (block_orthonormalise), where the reference projects
//     and renormalises against one basis vector at a time, twice each
//     (src/Davidson.cpp:447-514); both produce an orthonormal basis of the
//     same span;
//   - the subspace eigenproblem (LAPACK dsyev of all m pairs in the
//     reference, src/Davidson.cpp:224) computes only the nroots lowest pairs,
//     the only ones the iteration reads (pg_subspace.cpp), from the same
//     upper triangle.
// Two differences do change the subspace, both where the reference's
// iteration breaks down: locking stops at nroots, and a restart
// re-orthonormalises the kept block of B and Z (see the restart below).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <tuple>
#include <mutex>
#include <memory>
#include <map>
#include <deque>
#include <vector>

#include "pg_linalg.cuh"
#include "pg_solve.cuh"

struct pg_davidson {
  int status = 0;
  int jmacro = 0, nsub = 0, nnewB = 0, nnewZ = 0;
  int s_valid = 0;  // columns of S that hold Z^T B of the current basis
  int ndim = 0, maxsub = 0, nroots = 0;
  double thresh = 0;
  std::vector<double> S, V, sse, residuals, conv_w;
  std::vector<int> ccode, bindex;
  pg::RedScratch rs;
  pg::DevBuf<double> dcoef;  // maxsub * maxsub coefficients / Gram blocks
  pg::DevBuf<double> dsq;    // device scalars (norms, Ritz values, constants)
  pg::DevBuf<double> dgram;  // small Gram matrices of the Cholesky-QR step
  // double-float twins of B and Z (a float2 (hi, lo) per point, the form the
  // double-float kernels compute with), kept next to the FP64 arrays in the
  // mixed form so that B and Z are not converted again by every kernel that
  // reads them; Z rows [0, zt_valid) have current twins, B rows always do
  // where the double-float kernels read them
  pg::DevBuf<double> bt, zt;
  int zt_valid = 0;
  // page-locked staging of the per-iteration host<->device copies (offsets
  // kPin* below); a region is rewritten only after a later stream sync, so
  // no copy from it is still pending
  pg::HostPinned<double> hpin;
  // kinetic preconditioner (corrflag 3): grid, arithmetic, work blocks
  const pg_grid* pc_grid = nullptr;
  int pc_precision = PG_FP64;
  // subspace products (S, Ritz/residual combinations, orthogonalisation) in
  // double-float arithmetic on the FP32 pipe instead of FP64 (mixed form)
  bool dfloat = false;
  pg::DevBuf<double> pc_w1, pc_w2, pc_ru;
  // corrflag 3 on a grid where V is identically zero: the plain correction
  // M r is the Ritz vector itself there, so the Olsen form is used instead
  bool pc_olsen = false;
  pg::DevBuf<int> pc_flag;
  // set by the first block Gram-Schmidt pass when its Cholesky pivots show
  // that no correction lost enough of its norm for the second pass to matter
  pg::DevBuf<int> pip_skip;
  // counters for the solve statistics
  long n_iter = 0, n_restart = 0;
  double t_eig = 0, t_wait = 0;  // host seconds in the subspace eigensolver / waiting for the device
};

namespace pg {

// pg_subspace.cpp
bool lowest_eigenpairs(int m, const double* S, int ld, int k, double* w, double* V, int ldv);

namespace {

constexpr int kT = 256;

int blocks_for(long N) {
  long b = (N + kT - 1) / kT;
  return (int)(b < 152L * 8 ? (b > 0 ? b : 1) : 152L * 8);
}

// ritz_r = U_r / |U_r|;  res_r = W_r - lambda_r ritz_r   (src/Davidson.cpp:240-260),
// with per-block partial sums of |res_r|^2, reduced by the last block into
// rsq (|res_r|^2, then 1/|res_r|).  uinv[r] = 1/|U_r| (written by the
// combine that formed U).
template <int NR>
__global__ void __launch_bounds__(kT) k_ritz_residual(long N, long chunk, int nr, double* __restrict__ U,
                                                      double* __restrict__ W, const double* __restrict__ uinv,
                                                      const double* __restrict__ lam, double* __restrict__ partial,
                                                      double* rsq, unsigned* counter) {
  pdl_wait();
  pdl_release();
  __shared__ double red[kT / 32][NR];
  double inv[NR], nl[NR], acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    inv[r] = r < nr ? uinv[r] : 0.0;
    nl[r] = r < nr ? -lam[r] : 0.0;
    acc[r] = 0.0;
  }
  const long g_begin = blockIdx.x * chunk;
  const long g_end = g_begin + chunk < N ? g_begin + chunk : N;
  for (long g = g_begin + threadIdx.x; g < g_end; g += kT) {
    double u[NR], w[NR];  // all loads of the point first, then the arithmetic and stores
#pragma unroll
    for (int r = 0; r < NR; ++r)
      if (r < nr) {
        u[r] = U[(long)r * N + g];
        w[r] = W[(long)r * N + g];
      }
#pragma unroll
    for (int r = 0; r < NR; ++r)
      if (r < nr) {
        u[r] = u[r] * inv[r];
        w[r] = w[r] + nl[r] * u[r];
        acc[r] += w[r] * w[r];
        U[(long)r * N + g] = u[r];
        W[(long)r * N + g] = w[r];
      }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    double v = acc[r];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < nr) {
    double t = 0;
    for (int w = 0; w < kT / 32; ++w) t += red[w][threadIdx.x];
    partial[(long)blockIdx.x * nr + threadIdx.x] = t;
  }
  reduce_in_last_block(partial, nr, rsq, 1, counter);
}

// Davidson correction (lambda - diag H)^-1 r with the 1e-12 floor
// (DavidsonCorrectionVector, src/Davidson.cpp:557-566).
__global__ void k_precond(long N, double* __restrict__ r, const double* __restrict__ diag, double lambda) {
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    double d = lambda - diag[g];
    if (fabs(d) < 1e-12) d = 1e-12;
    r[g] /= d;
  }
}

// First half of the zeroth-order Jacobi-Davidson correction
// (src/Davidson.cpp:537-545): r <- -M r, jd <- M u, M = (diag H - lambda)^-1.
__global__ void k_jd_prep(long N, double* __restrict__ r, double* __restrict__ jd, const double* __restrict__ u,
                          const double* __restrict__ diag, double lambda) {
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    double m = diag[g] - lambda;
    if (fabs(m) < 1e-12) m = 1e-12;
    m = 1.0 / m;
    r[g] *= -m;
    jd[g] = m * u[g];
  }
}

// Diagonal of the kinetic preconditioner in the DST-I eigenbasis:
// y_v(i,j,k) /= (dx_i + dy_j + dz_k - sigma_v), the denominator kept at
// least `floor` in magnitude.  fast: the scale factor in FP32 (it only sets
// the convergence rate; the mixed form uses it to stay off the FP64 pipe).
template <int NR>
__global__ void __launch_bounds__(kT) k_kin_scale(int nx, int ny, int nz, const double* __restrict__ dx,
                                                  const double* __restrict__ dy, const double* __restrict__ dz,
                                                  const double* __restrict__ sigma, double floor,
                                                  double* __restrict__ Y, int nvec, int fast) {
  // 32-bit index arithmetic (the grid has fewer than 2^31 points)
  const unsigned N = (unsigned)nx * ny * nz;
  for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < N; g += gridDim.x * blockDim.x) {
    const unsigned i = g % (unsigned)nx;
    const unsigned r = g / (unsigned)nx;
    double y[NR];  // all loads of the point first
#pragma unroll
    for (int v = 0; v < NR; ++v)
      if (v < nvec) y[v] = Y[(size_t)v * N + g];
    if (fast) {
      const float dk = (float)dx[i] + (float)dy[r % (unsigned)ny] + (float)dz[r / (unsigned)ny];
#pragma unroll
      for (int v = 0; v < NR; ++v)
        if (v < nvec) {
          float den = dk - (float)sigma[v];
          if (fabsf(den) < (float)floor) den = den < 0 ? -(float)floor : (float)floor;
          Y[(size_t)v * N + g] = y[v] * (double)(1.0f / den);
        }
    } else {
      const double dk = dx[i] + dy[r % (unsigned)ny] + dz[r / (unsigned)ny];
#pragma unroll
      for (int v = 0; v < NR; ++v)
        if (v < nvec) {
          double den = dk - sigma[v];
          if (fabs(den) < floor) den = den < 0 ? -floor : floor;
          Y[(size_t)v * N + g] = y[v] / den;
        }
    }
  }
}

// r += f jd with f = dots[0] / dots[1]  (src/Davidson.cpp:547-548)
__global__ void k_jd_finish(long N, double* __restrict__ r, const double* __restrict__ jd,
                            const double* __restrict__ dots) {
  const double f = dots[0] / dots[1];
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x)
    r[g] += f * jd[g];
}

}  // namespace
}  // namespace pg

extern "C" pg_status pg_davidson_create(pg_davidson** out) {
  PG_ARG(out, "pg_davidson_create: null argument");
  *out = new pg_davidson();
  return PG_OK;
}

extern "C" pg_status pg_davidson_destroy(pg_davidson* d) {
  delete d;
  return PG_OK;
}

extern "C" pg_status pg_davidson_set_arithmetic(pg_davidson* d, int precision) {
  PG_ARG(d && (precision == PG_FP64 || precision == PG_MIXED), "pg_davidson_set_arithmetic: bad arguments");
  // the mixed form's double-float twins of B and Z are set up at a solve's
  // first call, so the arithmetic is fixed while a solve is in progress
  PG_ARG(d->status == 0 || (precision == PG_MIXED) == d->dfloat,
         "pg_davidson_set_arithmetic: the arithmetic cannot change while a solve is in progress");
  d->dfloat = precision == PG_MIXED;
  return PG_OK;
}

extern "C" pg_status pg_davidson_set_preconditioner(pg_davidson* d, const pg_grid* g, int precision) {
  PG_ARG(d && (precision == PG_FP64 || precision == PG_MIXED), "pg_davidson_set_preconditioner: bad arguments");
  d->pc_grid = g;
  d->pc_precision = precision;
  return PG_OK;
}

extern "C" pg_status pg_kinetic_precondition(const pg_grid* g, double* R, int k, const double* sigma, int precision,
                                             void* stream) {
  PG_ARG(g && k >= 0 && (precision == PG_FP64 || precision == PG_MIXED), "pg_kinetic_precondition: bad arguments");
  if (k == 0) return PG_OK;
  PG_ARG(R && sigma, "pg_kinetic_precondition: null R or sigma");
  cudaStream_t st = pg::as_stream(stream);
  pg::DevBuf<double> w, sg;
  PG_TRY(w.alloc((size_t)2 * k * g->N));
  PG_TRY(sg.alloc((size_t)k));
  PG_CUDA_TRY(cudaMemcpyAsync(sg.p, sigma, sizeof(double) * k, cudaMemcpyHostToDevice, st));
  PG_TRY(pg::kinetic_precondition(g, R, k, sg.p, w.p, w.p + (long)k * g->N, precision, st));
  // the scratch is freed on return: finish with it first
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  return precision == PG_MIXED ? pg::check_tc_error(g, st) : PG_OK;
}

extern "C" pg_status pg_grid_set_precond_kernel(pg_grid* g, int kind) {
  PG_ARG(g && (kind == 0 || kind == 1), "pg_grid_set_precond_kernel: kind must be 0 or 1");
  g->pc_kernel = kind;
  return PG_OK;
}

extern "C" pg_status pg_grid_precond_plan(const pg_grid* g, char* text, int len) {
  PG_ARG(g && text && len > 0, "pg_grid_precond_plan: bad arguments");
  if (g->pc_kernel != 1 && pg::kin_f16_ok(g)) {
    pg::kin_f16_plan_text(g, text, len);
  } else {
    char why[200] = "forced";
    if (g->pc_kernel != 1) pg::kin_f16_plan_text(g, why, sizeof(why));
    snprintf(text, (size_t)len, "axis passes (k_hx_tc x 6, k_kin_scale); %s", why);
  }
  return PG_OK;
}

extern "C" long pg_davidson_work_size(int ndim, int maxsub, int nroots, int corrflag) {
  // DavidsonWorkSize (src/Davidson.cpp:46-52); same layout of the work array.
  if (corrflag == 2) return 2L * maxsub * maxsub + 11L * maxsub + (2L * nroots + 1) * ndim;
  return 2L * maxsub * maxsub + 11L * maxsub + 2L * nroots * ndim;
}

namespace pg {
namespace {

// Device scalars of one Davidson handle (offsets into pg_davidson::dsq).
constexpr int kUsq = 0;     // |U_r|^2 and 1/|U_r| (2 x 16); mixed form: |U_r|^2 and |W_r|^2 (k_ritz_df)
constexpr int kLam = 32;    // Ritz values (16)
constexpr int kRsq = 64;    // |r_r|^2 and 1/|r_r| (2 x 16)
constexpr int kOnes = 96;   // 1.0 (16), the "keep X" coefficients of combine
constexpr int kDots = 112;  // Jacobi-Davidson dot products (2)
constexpr int kSigma = 128; // shifts of the kinetic preconditioner (2 x 16)
constexpr int kScalars = 256;

// Regions of pg_davidson::hpin (doubles)
constexpr int kPinCols = 0;                    // new S columns, m x nc <= 128 x 128
constexpr int kPinHsq = kPinCols + 128 * 128;  // |U_r|^2 ... |r_r|^2 (kRsq + 16)
constexpr int kPinV = kPinHsq + 96;            // Ritz coefficients, maxsub x nroots <= 128 x 16
constexpr int kPinLam = kPinV + 128 * 16;      // Ritz values (16)
constexpr int kPinSig = kPinLam + 16;          // preconditioner shifts (2 x 16)
constexpr int kPinTotal = kPinSig + 32;
static_assert(kRsq + 16 <= 96, "hsq region");

pg_status ensure_scratch(pg_davidson* d, int ndim, int maxsub, int nroots) {
  // grow-only scratch: a reused handle allocates only while its problems grow
  PG_TRY(d->dcoef.ensure((size_t)std::max(maxsub * maxsub, 2 * kMaxGramOut)));
  PG_TRY(d->dgram.ensure((size_t)kMaxGramOut));
  PG_TRY(d->rs.ensure());
  PG_TRY(d->pip_skip.ensure(1));
  PG_TRY(d->hpin.ensure(kPinTotal));
  if (d->dfloat) {
    PG_TRY(d->bt.ensure((size_t)maxsub * ndim));
    PG_TRY(d->zt.ensure((size_t)maxsub * ndim));
  }
  d->zt_valid = 0;
  if (!d->dsq.p) {
    PG_TRY(d->dsq.alloc(kScalars));
    std::vector<double> init(kScalars, 0.0);
    for (int i = 0; i < 16; ++i) init[kOnes + i] = 1.0;
    PG_CUDA_TRY(cudaMemcpy(d->dsq.p, init.data(), sizeof(double) * kScalars, cudaMemcpyHostToDevice));
  }
  d->ndim = ndim;
  d->maxsub = maxsub;
  d->nroots = nroots;
  return PG_OK;
}

// Coefficients of one block Gram-Schmidt pass with the Pythagorean Gram (the
// BCGS-PIP form): the corrections R (k vectors) sit right after the nb basis
// vectors of B, and G holds the Gram products of [B R] against R,
// G[a*k + j] = [B R]_a . R_j, so the first nb rows are C = B^T R and the last
// k rows are R^T R.  With B orthonormal, (R - B C)^T (R - B C) = R^T R - C^T C,
// whose Cholesky factor L gives U = L^-T; the pass is then one combine over
// [B R] with coef[a*k + j] = -(C U)[a][j] for a < nb and U[a-nb][j] below.
// A pivot is floored at 1e-24 of that vector's R^T R diagonal: where the
// subtraction cancels (R almost inside span(B)) the pass yields scaled
// rounding noise, mostly orthogonal to B, which the second pass (no
// cancellation left) projects and normalises.  One block; k <= 16, nb <= 128.
//
// skip_out (first pass): 1 when every squared pivot L_jj^2 keeps at least
// kPipKeep of that correction's squared norm R_j^T R_j, else 0.  Pivot j is
// what remains of R_j after removing span(B) and the corrections before it;
// with ratios that large the pass's rounding leaves the block orthonormal to
// about u / kPipKeep (u: the unit roundoff of the products, 2^-53 in FP64,
// about 2^-48 in double-float), and the second pass, which would change the
// vectors only by that much, is skipped.  skip_in (second pass): return at
// once when set.
constexpr double kPipKeep = 1e-3;
__global__ void __launch_bounds__(256) k_pip_coef(const double* __restrict__ G, int nb, int k,
                                                  double* __restrict__ coef, int* __restrict__ skip_out,
                                                  const int* __restrict__ skip_in) {
  pdl_wait();
  pdl_release();
  if (skip_in && *skip_in) return;
  __shared__ double Cs[128][kMaxCombine];
  __shared__ double L[kMaxCombine][kMaxCombine + 1];
  __shared__ double U[kMaxCombine][kMaxCombine + 1];
  __shared__ int Keep[kMaxCombine];
  const int tid = threadIdx.x;
  for (int e = tid; e < nb * k; e += blockDim.x) Cs[e / k][e % k] = G[e];
  __syncthreads();
  if (tid < k * k) {  // R^T R - C^T C, each entry summed in basis order
    const int i = tid / k, j = tid % k;
    double s = G[(long)(nb + i) * k + j];
    for (int a = 0; a < nb; ++a) s -= Cs[a][i] * Cs[a][j];
    L[i][j] = s;
  }
  __syncthreads();
  if (tid < 32) {
    const int lane = tid;
    for (int j = 0; j < k; ++j) {
      if (lane == 0) {
        double s = L[j][j];
        for (int p = 0; p < j; ++p) s -= L[j][p] * L[j][p];
        const double floor = 1e-24 * G[(long)(nb + j) * k + j];
        const double piv = s > floor ? s : (floor > 1e-300 ? floor : 1e-300);
        L[j][j] = sqrt(piv);
        Keep[j] = piv >= kPipKeep * G[(long)(nb + j) * k + j];
      }
      __syncwarp();
      if (lane > j && lane < k) {
        double t = L[lane][j];
        for (int p = 0; p < j; ++p) t -= L[lane][p] * L[j][p];
        L[lane][j] = t / L[j][j];
      }
      __syncwarp();
    }
    if (skip_out && lane == 0) {
      int all = 1;
      for (int j = 0; j < k; ++j) all &= Keep[j];
      *skip_out = all;
    }
    if (lane < k) {  // U = L^-T, column c on lane c (upper triangular)
      const int c = lane;
      for (int i = k - 1; i >= 0; --i) {
        double s = i == c ? 1.0 : 0.0;
        for (int p = i + 1; p < k; ++p) s -= L[p][i] * U[p][c];
        U[i][c] = i > c ? 0.0 : s / L[i][i];
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < (nb + k) * k; e += blockDim.x) {
    const int a = e / k, j = e % k;
    double s;
    if (a < nb) {
      s = 0.0;
      for (int i = 0; i <= j; ++i) s -= Cs[a][i] * U[i][j];
    } else {
      s = U[a - nb][j];
    }
    coef[e] = s;
  }
}

// C = L^-T for the Cholesky factor of the k x k Gram matrix G (row-major,
// G[a*k+b] = R_a . R_b), so that R C has orthonormal columns and, C being
// upper triangular, the same nested spans as Gram-Schmidt.  One warp: lane i
// updates row i of L at each column step, then lane c solves column c of C.
// A pivot is floored at 1e-300 so that a numerically dependent vector yields
// a (normalised) noise direction, as the reference's normalisation does.
__global__ void __launch_bounds__(32) k_cholinv(const double* __restrict__ G, int k, double* __restrict__ C) {
  __shared__ double L[kMaxCombine][kMaxCombine + 1];
  const int lane = threadIdx.x;
  for (int e = lane; e < k * k; e += 32) L[e / k][e % k] = G[e];
  __syncwarp();
  for (int j = 0; j < k; ++j) {
    if (lane == 0) {
      double s = L[j][j];
      for (int p = 0; p < j; ++p) s -= L[j][p] * L[j][p];
      L[j][j] = sqrt(s > 1e-300 ? s : 1e-300);
    }
    __syncwarp();
    if (lane > j && lane < k) {
      double t = L[lane][j];
      for (int p = 0; p < j; ++p) t -= L[lane][p] * L[j][p];
      L[lane][j] = t / L[j][j];
    }
    __syncwarp();
  }
  // C = L^-T: solve L^T C = I, column c on lane c (C upper triangular)
  if (lane < k) {
    const int c = lane;
    for (int i = k - 1; i >= 0; --i) {
      double s = i == c ? 1.0 : 0.0;
      for (int p = i + 1; p < k; ++p) s -= L[p][i] * C[p * k + c];
      C[i * k + c] = i > c ? 0.0 : s / L[i][i];
    }
  }
}

// flag = 1 if diag(H) differs anywhere from the kinetic diagonal, i.e. V is
// not identically zero (any nonzero difference sets the same value).
__global__ void k_potential_nonzero(int nx, int ny, int nz, const double* __restrict__ diag,
                                    const double* __restrict__ tx, const double* __restrict__ ty,
                                    const double* __restrict__ tz, int* __restrict__ flag) {
  const unsigned N = (unsigned)nx * ny * nz;
  for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < N; g += gridDim.x * blockDim.x) {
    const unsigned i = g % (unsigned)nx, r = g / (unsigned)nx;
    const unsigned j = r % (unsigned)ny, k = r / (unsigned)ny;
    double t = 0.0;
    t = __dadd_rn(t, tx[(size_t)i * nx + i]);
    t = __dadd_rn(t, ty[(size_t)j * ny + j]);
    t = __dadd_rn(t, tz[(size_t)k * nz + k]);
    if (diag[g] != t) *flag = 1;
  }
}

// Coefficients of the Olsen correction c_j = -M r_j + (u_j.M r_j / u_j.M u_j) M u_j
// from the Gram block G[j*2k + b] = u_j . [M R, M U]_b, as a 2k x k matrix
// C[a*k + j] for a combine over [M R, M U].
__global__ void k_olsen_coef(const double* __restrict__ G, int k, double* __restrict__ C) {
  for (int e = threadIdx.x; e < 2 * k * k; e += blockDim.x) {
    const int a = e / k, j = e % k;
    double c = 0.0;
    if (a == j) {
      c = -1.0;
    } else if (a == k + j) {
      const double den = G[(long)j * 2 * k + k + j];
      c = den != 0.0 ? G[(long)j * 2 * k + j] / den : 0.0;
    }
    C[e] = c;
  }
}

pg_status kinetic_precondition(pg_davidson* d, double* R, int k, const double* sigma_dev, cudaStream_t st) {
  const long N = d->pc_grid->N;
  PG_TRY(d->pc_w1.ensure((size_t)k * N));
  PG_TRY(d->pc_w2.ensure((size_t)k * N));
  return pg::kinetic_precondition(d->pc_grid, R, k, sigma_dev, d->pc_w1.p, d->pc_w2.p, d->pc_precision, st);
}

}  // namespace

// Kinetic preconditioner on the k contiguous vectors R: R <- (T - sigma_j)^-1 R
// with T = Q diag(d) Q^T per axis (DST-I for the sine DVR, the real Fourier
// basis for the periodic FFT kinetic term): three forward contractions
// (Q^T), a diagonal scale and three backward contractions (Q).  The mixed
// form runs them as one FP16-split tensor-core kernel where the grid allows
// (k_kin_f16), else as six axis passes and a scale kernel.
pg_status kinetic_precondition(const pg_grid* g, double* R, int k, const double* sigma_dev, double* w1, double* w2,
                               int pr, cudaStream_t st) {
  const long N = g->N;
  // the smallest kinetic level, a scale for the denominator floor
  double dmin = 0;
  for (int a = 0; a < 3; ++a) dmin += 0.5 * (M_PI / g->L[a]) * (M_PI / g->L[a]);
  if (pr == PG_MIXED && g->pc_kernel != 1 && kin_f16_ok(g) && (((uintptr_t)R | (uintptr_t)w1 | (uintptr_t)w2) & 15u) == 0)
    return kin_f16(g, R, w1, w2, k, sigma_dev, 0.1 * dmin, st);
  PG_TRY(axis_apply(g, 2, g->q_dev[2].p, g->q_hi[2].p, g->q_lo[2].p, R, w1, k, 0, pr, st));
  PG_TRY(axis_apply(g, 1, g->q_dev[1].p, g->q_hi[1].p, g->q_lo[1].p, w1, w2, k, 0, pr, st));
  PG_TRY(axis_apply(g, 0, g->q_dev[0].p, g->q_hi[0].p, g->q_lo[0].p, w2, w1, k, 0, pr, st));
  for (int v0 = 0; v0 < k; v0 += 16) {  // at most 16 vectors per launch
    const int kk = std::min(16, k - v0);
#define PG_KIN_SCALE(NRV)                                                                                     \
  k_kin_scale<NRV><<<blocks_for(N), kT, 0, st>>>(g->n[0], g->n[1], g->n[2], g->d_dev[0].p, g->d_dev[1].p,      \
                                                 g->d_dev[2].p, sigma_dev + v0, 0.1 * dmin, w1 + (long)v0 * N, \
                                                 kk, pr == PG_MIXED ? 1 : 0)
    if (kk <= 1) PG_KIN_SCALE(1);
    else if (kk <= 2) PG_KIN_SCALE(2);
    else if (kk <= 4) PG_KIN_SCALE(4);
    else if (kk <= 8) PG_KIN_SCALE(8);
    else PG_KIN_SCALE(16);
#undef PG_KIN_SCALE
    PG_TRY(check_launch("k_kin_scale"));
  }
  PG_TRY(axis_apply(g, 2, g->qb_dev[2].p, g->qb_hi[2].p, g->qb_lo[2].p, w1, w2, k, 0, pr, st));
  PG_TRY(axis_apply(g, 1, g->qb_dev[1].p, g->qb_hi[1].p, g->qb_lo[1].p, w2, w1, k, 0, pr, st));
  PG_TRY(axis_apply(g, 0, g->qb_dev[0].p, g->qb_hi[0].p, g->qb_lo[0].p, w1, R, k, 0, pr, st));
  return PG_OK;
}

namespace {

// Orthonormalise the k vectors R (contiguous, R[j*N]) against the first nbas
// columns of B and among themselves, into B[nbas .. nbas+k) (out must be
// B + nbas*N; R is copied there first when it lives elsewhere).  Two passes of
// block Gram-Schmidt with the Pythagorean Gram (k_pip_coef): one Gram over
// [B R] against R, one coefficient kernel, one combine over [B R] in place.
// The second pass repairs what the first leaves (rounding, or the cancellation
// of a correction that lies almost inside span(B)).  Same spans as the
// reference's vector-by-vector orthogonalisation, which projects and
// renormalises one vector at a time (src/Davidson.cpp:447-514).
pg_status block_orthonormalise(pg_davidson* d, long N, double* R, int k, double* B, int nbas, double* out,
                               cudaStream_t st) {
  PG_ARG(out == B + (long)nbas * N && k > 0 && k <= kMaxCombine && nbas + k <= 128,
         "block_orthonormalise: output must follow the basis (nbas=%d k=%d)", nbas, k);
  // mixed form: both passes read the twins of [B R] and the combines write the
  // twin of their output, so [B R] is converted once (R here, B as it was
  // written); R is copied into place and split in one pass
  double* Bt = d->dfloat ? d->bt.p : nullptr;
  double* Rt = Bt ? Bt + (long)nbas * N : nullptr;
  if (Bt) PG_TRY(split_twin(N * k, R, Rt, st, R != out ? out : nullptr));
  else if (R != out) PG_CUDA_TRY(cudaMemcpyAsync(out, R, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, st));
  // the second pass runs only where the first one's pivots ask for it
  // (k_pip_coef); the decision stays on the device
  for (int pass = 0; pass < 2; ++pass) {
    const int* skip = pass == 1 ? d->pip_skip.p : nullptr;
    PG_TRY(gram(N, B, nbas + k, out, k, d->dgram.p, d->rs, st, d->dfloat, Bt, Rt, skip));
    PG_CUDA_TRY(launch_dependent(k_pip_coef, dim3(1), dim3(256), 0, st, d->dgram.p, nbas, k, d->dcoef.p,
                                 pass == 0 ? d->pip_skip.p : nullptr, skip));
    PG_TRY(check_launch("k_pip_coef"));
    PG_TRY(combine(N, B, nbas + k, d->dcoef.p, k, 1, 1.0, nullptr, nullptr, false, out, k, nullptr, d->rs, st,
                   d->dfloat, Bt, Rt, skip));
  }
  return PG_OK;
}

}  // namespace
}  // namespace pg

extern "C" pg_status pg_davidson_rci(pg_davidson* d, int ndim, int maxsub, int nroots, int maxmacro, int tol,
                                     int corrflag, double* evals, int* nconv, double* B, double* Z,
                                     const double* diag, double* work, int* inout, int* ret, void* stream) {
  using namespace pg;
  PG_ARG(d && evals && nconv && B && Z && diag && work && inout && ret, "pg_davidson_rci: null argument");
  PG_ARG(ndim > 0 && nroots > 0 && maxsub > nroots && maxsub <= 128 && nroots <= kMaxCombine,
         "pg_davidson_rci: need 0 < nroots <= %d, nroots < maxsub <= 128 (ndim=%d maxsub=%d nroots=%d)",
         kMaxCombine, ndim, maxsub, nroots);
  cudaStream_t st = as_stream(stream);
  const long N = ndim;
  const int ms = maxsub;
  // device work-array layout (src/Davidson.cpp:181-187); S and V live on the host
  double* ritz = work + 2L * ms * ms + 11L * ms;
  double* res = ritz + N * nroots;
  double* jd = res + N * nroots;
  if (corrflag == 3 && !d->pc_grid) {
    set_error("pg_davidson_rci: corrflag 3 needs pg_davidson_set_preconditioner");
    return PG_BAD_ARG;
  }
  if (corrflag < 0 || corrflag > 3) corrflag = 1;
  if (corrflag == 3) PG_ARG(d->pc_grid->N == ndim, "pg_davidson_rci: preconditioner grid does not match ndim");

  if (d->status == 0) {  // first call (src/Davidson.cpp:145-193)
    PG_TRY(ensure_scratch(d, ndim, maxsub, nroots));
    d->pc_olsen = false;
    if (corrflag == 3) {  // is V identically zero? (diag(H) equals the kinetic diagonal)
      const pg_grid* g = d->pc_grid;
      PG_TRY(d->pc_flag.ensure(1));
      PG_CUDA_TRY(cudaMemsetAsync(d->pc_flag.p, 0, sizeof(int), st));
      k_potential_nonzero<<<blocks_for(N), kT, 0, st>>>(g->n[0], g->n[1], g->n[2], diag, g->t_dev[0].p,
                                                         g->t_dev[1].p, g->t_dev[2].p, d->pc_flag.p);
      PG_TRY(check_launch("k_potential_nonzero"));
      int nonzero = 1;
      PG_CUDA_TRY(cudaMemcpyAsync(&nonzero, d->pc_flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
      PG_CUDA_TRY(cudaStreamSynchronize(st));
      d->pc_olsen = nonzero == 0;
    }
    d->jmacro = 1;
    d->nsub = 0;
    d->nnewB = nroots;
    d->s_valid = 0;
    d->thresh = pow(10.0, -tol);
    d->S.assign((size_t)ms * ms, 0.0);
    d->V.assign((size_t)ms * ms, 0.0);
    d->sse.assign(ms, 0.0);
    d->residuals.assign(nroots, 0.0);
    d->conv_w.assign(nroots, 0.0);
    d->ccode.assign(nroots, 0);
    d->bindex.assign(nroots, 0);
    d->n_iter = d->n_restart = 0;
    d->t_eig = d->t_wait = 0;
    // orthonormalise the start vectors (GramSchmidt, src/Davidson.cpp:482-514)
    PG_TRY(block_orthonormalise(d, N, B, nroots, B, 0, B, st));
    d->status = 1;
  }
  PG_ARG(d->status == 1 && d->ndim == ndim, "pg_davidson_rci: state does not match this problem");

  for (;;) {
    if (d->nnewB > 0) {  // hand the new block to the caller (src/Davidson.cpp:209-217)
      inout[0] = d->nsub;
      inout[1] = d->nsub;
      inout[2] = d->nnewB;
      d->nnewZ = d->nnewB;
      d->nnewB = 0;
      *ret = 1;
      return PG_OK;
    }
    d->n_iter++;
    const int m = d->nsub + d->nnewZ;
    // new columns of S = Z^T B (upper triangle is what the eigensolver reads)
    {
      const int c0 = d->s_valid;
      const int nc = m - c0;
      const int per = std::max(1, std::min(kMaxGramOut / m, std::min(16, 144 - m)));
      if (d->dfloat && d->zt_valid < m) {  // twins of the Z rows the caller has just written
        PG_TRY(split_twin((long)(m - d->zt_valid) * N, Z + (long)d->zt_valid * N, d->zt.p + (long)d->zt_valid * N, st));
        d->zt_valid = m;
      }
      for (int cb = 0; cb < nc; cb += per) {
        const int k = std::min(per, nc - cb);
        PG_TRY(gram(N, Z, m, B + (long)(c0 + cb) * N, k, d->dcoef.p + (size_t)cb * m, d->rs, st, d->dfloat,
                    d->dfloat ? d->zt.p : nullptr, d->dfloat ? d->bt.p + (long)(c0 + cb) * N : nullptr));
      }
      const double* cols = d->hpin.p + kPinCols;
      const auto w0 = std::chrono::steady_clock::now();
      PG_CUDA_TRY(cudaMemcpyAsync(d->hpin.p + kPinCols, d->dcoef.p, sizeof(double) * m * nc, cudaMemcpyDeviceToHost,
                                  st));
      PG_CUDA_TRY(cudaStreamSynchronize(st));
      d->t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
      // gram output is [a*nb + b] per chunk: a = Z column i, b = new B column
      for (int cb = 0; cb < nc; cb += per) {
        const int k = std::min(per, nc - cb);
        const double* blk = cols + (size_t)cb * m;
        for (int i = 0; i < m; ++i)
          for (int b = 0; b < k; ++b) d->S[i + (size_t)(c0 + cb + b) * ms] = blk[(size_t)i * k + b];
      }
      d->s_valid = m;
    }
    d->nsub = m;
    const auto e0 = std::chrono::steady_clock::now();
    const bool eig_ok = lowest_eigenpairs(m, d->S.data(), ms, nroots, d->sse.data(), d->V.data(), ms);
    d->t_eig += std::chrono::duration<double>(std::chrono::steady_clock::now() - e0).count();
    if (!eig_ok) {
      set_error("pg_davidson_rci: subspace eigensolve produced a non-finite value");
      d->status = 0;
      return PG_NUMERIC;
    }
    // overlap of each root with the converged space (src/Davidson.cpp:229-237)
    for (int r = 0; r < nroots; ++r) {
      double s = 0;
      for (int c = 0; c < *nconv; ++c) s += d->V[c + (size_t)r * ms] * d->V[c + (size_t)r * ms];
      d->conv_w[r] = *nconv > 0 ? sqrt(s) : 0.0;
    }
    // Ritz vectors u = B v (renormalised) and residuals Z v - lambda u
    // (src/Davidson.cpp:240-269), all roots in one pass
    double* dV = d->dcoef.p;
    double* dlam = d->dsq.p + kLam;
    double* usq = d->dsq.p + kUsq;
    double* rsq = d->dsq.p + kRsq;
    memcpy(d->hpin.p + kPinV, d->V.data(), sizeof(double) * ms * nroots);
    memcpy(d->hpin.p + kPinLam, d->sse.data(), sizeof(double) * nroots);
    PG_CUDA_TRY(cudaMemcpyAsync(dV, d->hpin.p + kPinV, sizeof(double) * ms * nroots, cudaMemcpyHostToDevice, st));
    PG_CUDA_TRY(cudaMemcpyAsync(dlam, d->hpin.p + kPinLam, sizeof(double) * nroots, cudaMemcpyHostToDevice, st));
    if (d->dfloat) {
      // mixed form: both products, the residual and the norms in one pass
      // over the twins of B and Z (U is not renormalised: |U| = 1 to ~1e-14)
      PG_TRY(ritz_df(N, d->bt.p, d->zt.p, m, dV, ms, dlam, ritz, res, nroots, usq, d->rs, st));
    } else {
      PG_TRY(combine(N, B, m, dV, 1, ms, 1.0, nullptr, nullptr, false, ritz, nroots, usq, d->rs, st));
      PG_TRY(combine(N, Z, m, dV, 1, ms, 1.0, nullptr, nullptr, false, res, nroots, nullptr, d->rs, st));
      const long chunk = (N + kRedBlocks - 1) / kRedBlocks;
      const int nblk = (int)((N + chunk - 1) / chunk);
#define PG_RITZ(NRV) \
  PG_CUDA_TRY(launch_dependent(k_ritz_residual<NRV>, dim3(nblk), dim3(kT), 0, st, N, chunk, nroots, ritz, res, \
                               usq + nroots, dlam, d->rs.partial.p, rsq, d->rs.counter.p))
      if (nroots <= 1) PG_RITZ(1);
      else if (nroots <= 2) PG_RITZ(2);
      else if (nroots <= 4) PG_RITZ(4);
      else if (nroots <= 8) PG_RITZ(8);
      else PG_RITZ(16);
#undef PG_RITZ
      PG_TRY(check_launch("k_ritz_residual"));
    }
    // |r_r|^2 and |U_r|^2 in one read (rsq and usq both live in dsq; the
    // mixed form's pass leaves |W_r|^2 right after |U_r|^2)
    static_assert(kUsq == 0 && kRsq > kUsq, "dsq layout");
    const auto w1 = std::chrono::steady_clock::now();
    PG_CUDA_TRY(cudaMemcpyAsync(d->hpin.p + kPinHsq, d->dsq.p, sizeof(double) * (kRsq + nroots),
                                cudaMemcpyDeviceToHost, st));
    const double* hr = d->hpin.p + kPinHsq + (d->dfloat ? kUsq + nroots : kRsq);
    const double* hu = d->hpin.p + kPinHsq + kUsq;
    PG_CUDA_TRY(cudaStreamSynchronize(st));
    d->t_wait += std::chrono::duration<double>(std::chrono::steady_clock::now() - w1).count();
    for (int r = 0; r < nroots; ++r) {
      d->residuals[r] = d->dfloat ? sqrt(hr[r] / hu[r]) : sqrt(hr[r]);  // |Z v - lambda B v| / |B v|
      if (!std::isfinite(d->residuals[r])) {
        set_error("pg_davidson_rci: non-finite residual norm for root %d", r);
        d->status = 0;
        return PG_NUMERIC;
      }
      // with an orthonormal basis |B v| = 1 for every unit subspace vector v;
      // a deviation means the basis lost orthonormality and the Ritz pairs
      // (which the reference would renormalise and accept) are spurious
      if (!(fabs(hu[r] - 1.0) < 1e-6)) {
        set_error("pg_davidson_rci: subspace basis lost orthonormality (|Bv|^2 = %.3e for root %d)", hu[r], r);
        d->status = 0;
        return PG_NUMERIC;
      }
    }
    // convergence and locking (src/Davidson.cpp:272-289).  The reference
    // skips a root whose overlap with the converged space exceeds 0.95; at
    // most nconv roots can (their squared overlaps sum to at most nconv), and
    // with separated eigenvalues exactly the nconv locked ones do.  Inside a
    // degenerate set the rotation of the Ritz vectors can leave every overlap
    // below 0.95, and the reference would lock the same state again (nConv
    // past nroots).  Here the nconv roots of largest overlap are the ones
    // skipped: the same choice whenever the reference's is well defined.
    std::vector<char> in_conv(nroots, 0);
    {
      std::vector<int> order(nroots);
      for (int r = 0; r < nroots; ++r) order[r] = r;
      std::stable_sort(order.begin(), order.end(),
                       [&](int a, int b) { return d->conv_w[a] > d->conv_w[b]; });
      for (int c = 0; c < *nconv && c < nroots; ++c) in_conv[order[c]] = 1;
    }
    int newly = 0;
    for (int r = 0; r < nroots; ++r) {
      if (in_conv[r] || d->conv_w[r] > 0.95) {
        d->ccode[r] = 0;
      } else if (d->residuals[r] < d->thresh && *nconv < nroots) {
        d->ccode[r] = 1;
        d->bindex[r] = *nconv;
        PG_CUDA_TRY(cudaMemcpyAsync(B + (long)(*nconv) * N, ritz + (long)r * N, sizeof(double) * N,
                                    cudaMemcpyDeviceToDevice, st));
        *nconv += 1;
        newly += 1;
      } else {
        d->ccode[r] = 2;
      }
    }
    if (*nconv == nroots) {  // src/Davidson.cpp:290-297
      memcpy(evals, d->sse.data(), sizeof(double) * nroots);
      PG_CUDA_TRY(cudaMemcpyAsync(B, ritz, sizeof(double) * N * nroots, cudaMemcpyDeviceToDevice, st));
      PG_CUDA_TRY(cudaStreamSynchronize(st));
      d->status = 0;
      *ret = 0;
      return PG_OK;
    }
    // restart (src/Davidson.cpp:303-346)
    const bool restarted = d->nsub == ms || newly > 0;
    if (restarted) {
      d->n_restart++;
      d->nnewB = 0;
      for (int r = 0; r < nroots; ++r)
        if (d->ccode[r] == 2) {
          PG_CUDA_TRY(cudaMemcpyAsync(B + (long)(d->nnewB + *nconv) * N, ritz + (long)r * N, sizeof(double) * N,
                                      cudaMemcpyDeviceToDevice, st));
          d->bindex[r] = *nconv + d->nnewB;
          d->nnewB += 1;
        }
      // Z v of the kept vectors, built in the Ritz block (root order, as the
      // reference does) and copied into Z as one block
      for (int r = 0; r < nroots; ++r)
        if (d->ccode[r] > 0) {
          const int jz = d->bindex[r];
          PG_TRY(combine(N, Z, d->nsub, dV + (size_t)r * ms, 1, ms, 1.0, nullptr, nullptr, false,
                         ritz + (long)jz * N, 1, nullptr, d->rs, st, d->dfloat, d->dfloat ? d->zt.p : nullptr));
        }
      const long first = *nconv - newly;
      const long cnt = (long)(d->nnewB + newly);
      if (cnt > 0)
        PG_CUDA_TRY(cudaMemcpyAsync(Z + first * N, ritz + first * N, sizeof(double) * N * cnt,
                                    cudaMemcpyDeviceToDevice, st));
      // The locked vectors are Ritz vectors of an older subspace, so the new
      // Ritz vectors are orthogonal to them only to O(residual / gap).  The
      // reference carries that drift on (src/Davidson.cpp:303-346); inside
      // near-degenerate sets it lets a state be locked twice, and with many
      // roots it wrecks the basis.  One Cholesky-QR step on the kept block,
      // applied to B and Z alike (Z = H B stays exact), restores
      // orthonormality.  With the locked vectors first it only normalises them
      // and orthogonalises the others against them.  The kept block is
      // nconv + nnewB = nroots <= 16 vectors.
      {
        const int kept = *nconv + d->nnewB;
        PG_TRY(gram(N, B, kept, B, kept, d->dgram.p, d->rs, st, d->dfloat));
        k_cholinv<<<1, 32, 0, st>>>(d->dgram.p, kept, d->dcoef.p);
        PG_TRY(check_launch("k_cholinv"));
        // the copies above left these rows' twins stale: read B and Z, write
        // fresh twins
        PG_TRY(combine(N, B, kept, d->dcoef.p, kept, 1, 1.0, nullptr, nullptr, false, B, kept, nullptr, d->rs, st,
                       d->dfloat, nullptr, d->dfloat ? d->bt.p : nullptr));
        PG_TRY(combine(N, Z, kept, d->dcoef.p, kept, 1, 1.0, nullptr, nullptr, false, Z, kept, nullptr, d->rs, st,
                       d->dfloat, nullptr, d->dfloat ? d->zt.p : nullptr));
        d->zt_valid = kept;
      }
      d->nsub = nroots;
      d->s_valid = 0;
      d->jmacro += 1;
      if (d->jmacro >= maxmacro) {
        // The reference returns 0 here with its state still set and only
        // prints the unconverged list (src/Davidson.cpp:332-340).
        PG_CUDA_TRY(cudaStreamSynchronize(st));
        *ret = 0;
        set_error("pg_davidson_rci: %d of %d roots converged after %d macro iterations", *nconv, nroots,
                  d->jmacro);
        d->status = 0;
        return PG_NOT_CONVERGED;
      }
    }
    // correction vectors (src/Davidson.cpp:353-371): the unconverged roots in
    // order while the subspace has room, preconditioned, compacted to the
    // front of the residual block, orthonormalised as one block and appended
    // to B
    std::vector<int> sel;
    for (int r = 0; r < nroots; ++r) {
      if (d->nsub + (int)sel.size() == ms) break;
      if (d->ccode[r] < 2) continue;
      sel.push_back(r);
    }
    for (size_t j = 0; j < sel.size(); ++j) {
      const int r = sel[j];
      double* rv = res + (long)r * N;
      if (corrflag == 1) {
        k_precond<<<blocks_for(N), kT, 0, st>>>(N, rv, diag, d->sse[r]);
        PG_TRY(check_launch("k_precond"));
      } else if (corrflag == 2) {
        k_jd_prep<<<blocks_for(N), kT, 0, st>>>(N, rv, jd, ritz + (long)r * N, diag, d->sse[r]);
        PG_TRY(check_launch("k_jd_prep"));
        double* dots = d->dsq.p + kDots;  // (u . r, u . jd)
        PG_TRY(gram(N, ritz + (long)r * N, 1, rv, 1, dots, d->rs, st));
        PG_TRY(gram(N, ritz + (long)r * N, 1, jd, 1, dots + 1, d->rs, st));
        k_jd_finish<<<blocks_for(N), kT, 0, st>>>(N, rv, jd, dots);
        PG_TRY(check_launch("k_jd_finish"));
      }
      if (r != (int)j)  // sel is increasing, so slot j is free or already moved
        PG_CUDA_TRY(cudaMemcpyAsync(res + (long)j * N, rv, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    }
    d->nnewB = (int)sel.size();
    if (corrflag == 3 && d->nnewB > 0 && !d->pc_olsen) {
      // exact-kinetic correction M r_j, M = (T - lambda_j)^-1
      double* sig = d->hpin.p + kPinSig;
      for (int j = 0; j < d->nnewB; ++j) sig[j] = d->sse[sel[j]];
      double* dsig = d->dsq.p + kSigma;
      PG_CUDA_TRY(cudaMemcpyAsync(dsig, sig, sizeof(double) * d->nnewB, cudaMemcpyHostToDevice, st));
      PG_TRY(kinetic_precondition(d, res, d->nnewB, dsig, st));
    } else if (corrflag == 3 && d->nnewB > 0) {
      // Olsen correction with M = (T - lambda_j)^-1 applied exactly:
      // c_j = -M r_j + (u_j.M r_j / u_j.M u_j) M u_j, orthogonal to u_j.  With
      // V = 0, M r_j is u_j itself and would add no direction.
      const int k = d->nnewB;
      PG_TRY(d->pc_ru.ensure((size_t)3 * nroots * N));
      double* RU = d->pc_ru.p;             // [R (k), U (k), U again (k)]
      double* Uc = RU + (long)2 * k * N;
      PG_CUDA_TRY(cudaMemcpyAsync(RU, res, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, st));
      for (int j = 0; j < k; ++j) {
        // after a restart the Ritz block holds Z v; the Ritz vector is in B
        const double* u = restarted ? B + (long)d->bindex[sel[j]] * N : ritz + (long)sel[j] * N;
        PG_CUDA_TRY(cudaMemcpyAsync(RU + (long)(k + j) * N, u, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
      }
      PG_CUDA_TRY(cudaMemcpyAsync(Uc, RU + (long)k * N, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, st));
      double* sig = d->hpin.p + kPinSig;
      for (int j = 0; j < k; ++j) sig[j] = sig[k + j] = d->sse[sel[j]];
      double* dsig = d->dsq.p + kSigma;
      PG_CUDA_TRY(cudaMemcpyAsync(dsig, sig, sizeof(double) * 2 * k, cudaMemcpyHostToDevice, st));
      PG_TRY(kinetic_precondition(d, RU, 2 * k, dsig, st));  // RU = [M R, M U]
      PG_TRY(gram(N, Uc, k, RU, 2 * k, d->dgram.p, d->rs, st, d->dfloat));
      k_olsen_coef<<<1, 256, 0, st>>>(d->dgram.p, k, d->dcoef.p);
      PG_TRY(check_launch("k_olsen_coef"));
      PG_TRY(combine(N, RU, 2 * k, d->dcoef.p, k, 1, 1.0, nullptr, nullptr, false, res, k, nullptr, d->rs, st,
                     d->dfloat));
    }
    if (d->nnewB > 0)
      PG_TRY(block_orthonormalise(d, N, res, d->nnewB, B, d->nsub, B + (long)d->nsub * N, st));
  }
}

// ----------------------------------------------------------------- driver

namespace pg {
namespace {

// glibc's rand(): the additive feedback generator r[i] = r[i-3] + r[i-31]
// seeded by a Lehmer sequence, outputs r[i] >> 1 after 310 discarded values.
// The reference draws its random start vectors from rand() in an unseeded
// process (seed 1, src/DVR.cpp:52-59, 440-445); this reproduces that stream.
struct GlibcRand {
  unsigned ring[34];
  long pos = 34;
  explicit GlibcRand(unsigned seed) {
    long long v[34];
    v[0] = seed;
    for (int i = 1; i < 31; ++i) {
      v[i] = (16807LL * v[i - 1]) % 2147483647LL;
      if (v[i] < 0) v[i] += 2147483647LL;
    }
    for (int i = 31; i < 34; ++i) v[i] = v[i - 31];
    for (int i = 0; i < 34; ++i) ring[i] = (unsigned)v[i];
    for (int i = 34; i < 344; ++i) next_raw();
  }
  unsigned next_raw() {
    const unsigned x = ring[(pos - 31) % 34] + ring[(pos - 3) % 34];
    ring[pos % 34] = x;
    ++pos;
    return x;
  }
  int operator()() { return (int)(next_raw() >> 1); }
};

constexpr int kRandMax = 2147483647;

}  // namespace

// Start vectors of DVR::Diagonalize (src/DVR.cpp:405-453): startvec 1 puts
// the particle-in-a-box product in column 0, the other columns (all of them
// for startvec 2) are uniform in [-1, 1] from the C library generator.
pg_status start_vectors(const pg_grid* g, int nroots, int startvec, double* B, cudaStream_t st) {
  const long N = g->N;
  int istart = 0;
  if (startvec == 1) {
    PG_TRY(pg_piab_start(g, B, st));
    istart = 1;
  }
  if (istart < nroots) {
    // Randm11 (src/DVR.cpp:52-59): sign draw, then magnitude draw.  The
    // sequence restarts at seed 1 for every solve, so the grid keeps it.
    const size_t cnt = (size_t)(nroots - istart) * N;
    std::lock_guard<std::mutex> l(g->start_m);
    if (g->start_rand.n < cnt) {
      GlibcRand rnd(1);
      std::vector<double> h(cnt);
      for (auto& x : h) {
        if (rnd() > kRandMax / 2) x = (double)rnd() / kRandMax;
        else x = -(double)rnd() / kRandMax;
      }
      PG_TRY(g->start_rand.alloc(cnt));
      PG_CUDA_TRY(cudaMemcpyAsync(g->start_rand.p, h.data(), sizeof(double) * cnt, cudaMemcpyHostToDevice, st));
    }
    PG_CUDA_TRY(cudaMemcpyAsync(B + (long)istart * N, g->start_rand.p, sizeof(double) * cnt,
                                cudaMemcpyDeviceToDevice, st));
    PG_CUDA_TRY(cudaStreamSynchronize(st));  // before another solve may regrow the cache
  }
  return PG_OK;
}

}  // namespace pg

extern "C" int pg_glibc_rand_check(int count, int* out) {
  pg::GlibcRand r(1);
  for (int i = 0; i < count; ++i) out[i] = r();
  return 0;
}

namespace pg {

// Buffers of one eigensolve, kept by a long-lived caller (a serving worker)
// so that repeated solves allocate only while their sizes grow.
struct SolveWorkspace {
  DevBuf<double> B, Z, diag, work;
  pg_davidson d;
};

SolveWorkspace* workspace_create() { return new SolveWorkspace(); }
void workspace_destroy(SolveWorkspace* w) { delete w; }

// Device bytes a workspace keeps between solves (its grow-only buffers and
// those of its Davidson handle).
double workspace_bytes(const SolveWorkspace* w) {
  if (!w) return 0;
  const pg_davidson& d = w->d;
  const size_t doubles = w->B.n + w->Z.n + w->diag.n + w->work.n + d.rs.partial.n + d.dcoef.n + d.dsq.n +
                         d.dgram.n + d.bt.n + d.zt.n + d.pc_w1.n + d.pc_w2.n + d.pc_ru.n;
  return 8.0 * (double)doubles + 4.0 * (double)(d.rs.counter.n + d.pc_flag.n + d.pip_skip.n);
}

// The device eigensolve of pg_solve with the H*X product supplied by the
// caller (the serving engine routes it through its cross-solve batcher).
pg_status solve_with(const pg_grid* g, const double* v, const pg_solve_params* p, double* evals, double* evecs,
                     pg_solve_stats* stats, cudaStream_t st,
                     const std::function<pg_status(const double*, double*, int)>& matvec, SolveWorkspace* wsp) {
  PG_ARG(g && v && p && evals && evecs, "pg_solve: null argument");
  PG_ARG(p->nroots > 0 && p->maxsub > p->nroots && p->maxiter > 0 && p->ptol > 0, "pg_solve: bad parameters");
  PG_ARG(p->precision == PG_FP64 || p->precision == PG_MIXED, "pg_solve: unknown precision");
  PG_ARG(p->startvec >= 0 && p->startvec <= 3, "pg_solve: startvec %d is not 0, 1, 2 or 3", p->startvec);
  PG_ARG(g->N < (1L << 31), "pg_solve: grid too large for the reverse-communication interface");
  auto t0 = std::chrono::steady_clock::now();
  const long N = g->N;
  const int ms = p->maxsub, nr = p->nroots;
  SolveWorkspace local;
  SolveWorkspace& ws = wsp ? *wsp : local;
  DevBuf<double>&B = ws.B, &Z = ws.Z, &diag = ws.diag, &work = ws.work;
  PG_TRY(B.ensure((size_t)ms * N));
  PG_TRY(Z.ensure((size_t)ms * N));
  PG_TRY(diag.ensure(N));
  PG_TRY(work.ensure((size_t)pg_davidson_work_size((int)N, ms, nr, p->corrflag)));
  if (p->startvec == 0) {
    PG_CUDA_TRY(cudaMemcpyAsync(B.p, evecs, sizeof(double) * N * nr, cudaMemcpyDeviceToDevice, st));
  } else if (p->startvec == 3) {
    // SVFlag 3 (src/DVR.cpp:422-434): column 0 given (the coarse state
    // interpolated onto this grid), the others random
    PG_CUDA_TRY(cudaMemcpyAsync(B.p, evecs, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    if (nr > 1) PG_TRY(start_vectors(g, nr - 1, 2, B.p + N, st));
  } else {
    PG_TRY(start_vectors(g, nr, p->startvec, B.p, st));
  }
  PG_TRY(pg_diagonal(g, v, diag.p, st));
  pg_davidson& d = ws.d;
  d.status = 0;  // a fresh solve, whatever the last one left behind
  d.pc_grid = nullptr;
  if (p->corrflag == 3) PG_TRY(pg_davidson_set_preconditioner(&d, g, p->precision));
  d.dfloat = p->precision == PG_MIXED;
  int inout[3] = {0, 0, 0}, nconv = 0, ret = 1;
  long nmv = 0;
  pg_status s = PG_OK;
  while (ret != 0) {  // DVR::davdriver loop (src/davdriver.cpp:58-86)
    s = pg_davidson_rci(&d, (int)N, ms, nr, p->maxiter, p->ptol, p->corrflag, evals, &nconv, B.p, Z.p, diag.p,
                        work.p, inout, &ret, st);
    if (s != PG_OK && s != PG_NOT_CONVERGED) return s;
    if (ret == 1) {
      // the whole block in one launch (the reference multiplies vector by vector)
      PG_TRY(matvec(B.p + (long)inout[0] * N, Z.p + (long)inout[1] * N, inout[2]));
      nmv += inout[2];
    }
  }
  const pg_status conv_status = s;
  if (nconv < nr)  // not converged: report the current Ritz values
    for (int r = 0; r < nr && r < (int)d.sse.size(); ++r) evals[r] = d.sse[r];
  if (p->precision == PG_MIXED) PG_TRY(check_tc_error(g, st));
  if (p->precision == PG_MIXED && p->refine == 1) {
    // FP64 Rayleigh-Ritz on the converged vectors: Z = H B with the FP64
    // operator, S = B^T Z, eigenpairs of S rotate the vectors.
    PG_TRY(hx(g, v, B.p, Z.p, nr, PG_FP64, st));
    nmv += nr;
    PG_TRY(gram(N, Z.p, nr, B.p, nr, d.dcoef.p, d.rs, st));
    std::vector<double> S((size_t)nr * nr), w(nr), V((size_t)nr * nr);
    PG_CUDA_TRY(cudaMemcpyAsync(S.data(), d.dcoef.p, sizeof(double) * nr * nr, cudaMemcpyDeviceToHost, st));
    PG_CUDA_TRY(cudaStreamSynchronize(st));
    std::vector<double> Sc((size_t)nr * nr);  // gram gives [i*nr + j] = Z_i . B_j = S(i,j)
    for (int i = 0; i < nr; ++i)
      for (int j = 0; j < nr; ++j) Sc[i + (size_t)j * nr] = S[(size_t)i * nr + j];
    if (!lowest_eigenpairs(nr, Sc.data(), nr, nr, w.data(), V.data(), nr)) return PG_NUMERIC;
    PG_CUDA_TRY(cudaMemcpyAsync(d.dcoef.p, V.data(), sizeof(double) * nr * nr, cudaMemcpyHostToDevice, st));
    PG_TRY(combine(N, B.p, nr, d.dcoef.p, 1, nr, 1.0, nullptr, nullptr, false, evecs, nr, nullptr, d.rs, st));
    for (int r = 0; r < nr; ++r) evals[r] = w[r];
  } else {
    PG_CUDA_TRY(cudaMemcpyAsync(evecs, B.p, sizeof(double) * N * nr, cudaMemcpyDeviceToDevice, st));
  }
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->nconv = nconv;
    stats->n_matvec = (int)nmv;
    stats->n_iter = (int)d.n_iter;
    stats->n_restart = (int)d.n_restart;
    for (int r = 0; r < nr && r < 64; ++r) stats->residual[r] = r < (int)d.residuals.size() ? d.residuals[r] : 0;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    stats->host_eig_seconds = d.t_eig;
    stats->device_wait_seconds = d.t_wait;
  }
  if (p->precision == PG_MIXED && p->refine == 2 && conv_status == PG_OK) {
    // FP64 polish: the plain FP64 Davidson continued from the mixed form's
    // converged vectors to residual 10^-max(ptol+2, 8), so that eigenvectors
    // (not only eigenvalues) reach FP64 accuracy even for close states
    pg_solve_params q = *p;
    q.precision = PG_FP64;
    q.startvec = 0;
    q.refine = 0;
    q.ptol = std::max(p->ptol + 2, 8);
    pg_solve_stats s2;
    const pg_status s = solve_with(
        g, v, &q, evals, evecs, &s2, st,
        [&](const double* x, double* y, int nvec) { return hx(g, v, x, y, nvec, PG_FP64, st, true); }, &ws);
    if (stats) {
      stats->nconv = s2.nconv;
      stats->n_matvec += s2.n_matvec;
      stats->n_iter += s2.n_iter;
      stats->n_restart += s2.n_restart;
      for (int r = 0; r < 64; ++r) stats->residual[r] = s2.residual[r];
      stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      stats->host_eig_seconds += s2.host_eig_seconds;
      stats->device_wait_seconds += s2.device_wait_seconds;
    }
    return s;
  }
  return conv_status;
}

// V(r) of a water cluster (default model) plus Bloomfield ions, on the device.
pg_status cluster_potential(const pg_grid* g, int nw, const double* waters, int nions, const double* ions, double* v,
                            cudaStream_t st) {
  const long N = g->N;
  if (nw > 0) {
    std::vector<double> sites(12 * (size_t)nw), q(3 * (size_t)nw), dip(9 * (size_t)nw), sto(8 * (size_t)nw),
        pa(nw);
    std::vector<int> qs(3 * (size_t)nw), ds(3 * (size_t)nw), ss(4 * (size_t)nw), ps(nw);
    int it = 0;
    PG_TRY(pg_water_sites(nw, waters, sites.data(), q.data(), qs.data(), dip.data(), ds.data(), &it));
    pg_sites t;
    PG_TRY(pg_water_default_tables(nw, sites.data(), q.data(), qs.data(), dip.data(), ds.data(), sto.data(),
                                   ss.data(), pa.data(), ps.data(), &t));
    PG_TRY(pg_potential_eval(g, &t, v, nullptr, st));
  } else {
    PG_CUDA_TRY(cudaMemsetAsync(v, 0, sizeof(double) * N, st));
  }
  if (nions > 0) {
    std::vector<double> pos(3 * (size_t)nions), qi(nions);
    const double a2b = 1.0 / 0.52917720859;
    for (int i = 0; i < nions; ++i) {
      for (int c = 0; c < 3; ++c) pos[3 * i + c] = ions[4 * i + c] * a2b;
      qi[i] = ions[4 * i + 3];
    }
    PG_TRY(pg_potential_ions_add(g, nions, pos.data(), qi.data(), 2.9, 1.0, v, st));
  }
  return PG_OK;
}

}  // namespace pg

extern "C" pg_status pg_solve(const pg_grid* g, const double* v, const pg_solve_params* p, double* evals,
                              double* evecs, pg_solve_stats* stats, void* stream) {
  using namespace pg;
  cudaStream_t st = as_stream(stream);
  const int prec = p ? p->precision : PG_FP64;
  return solve_with(
      g, v, p, evals, evecs, stats, st,
      [&](const double* x, double* y, int nvec) { return hx(g, v, x, y, nvec, prec, st, true); }, nullptr);
}

namespace pg {
namespace {

// Grids of pg_cluster_solve, kept per (device, n, L) so that a stream of
// single points on one grid builds its kinetic matrices once (at most
// kGridCacheMax grids; the oldest is dropped when a new one does not fit).
constexpr size_t kGridCacheMax = 16;
struct GridCache {
  std::mutex m;
  std::map<std::tuple<int, int, int, int, double, double, double>, std::shared_ptr<pg_grid>> grids;
  std::deque<std::tuple<int, int, int, int, double, double, double>> order;
};
GridCache& grid_cache() {
  static GridCache c;
  return c;
}

pg_status cached_grid(const int n[3], const double L[3], std::shared_ptr<pg_grid>* out) {
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev));
  const auto key = std::make_tuple(dev, n[0], n[1], n[2], L[0], L[1], L[2]);
  GridCache& c = grid_cache();
  std::lock_guard<std::mutex> l(c.m);
  auto it = c.grids.find(key);
  if (it != c.grids.end()) {
    *out = it->second;
    return PG_OK;
  }
  pg_grid* g = nullptr;
  PG_TRY(pg_grid_create(n, L, &g));
  std::shared_ptr<pg_grid> sp(g, [](pg_grid* q) { pg_grid_destroy(q); });
  if (c.order.size() >= kGridCacheMax) {  // in-flight users keep their shared_ptr
    c.grids.erase(c.order.front());
    c.order.pop_front();
  }
  c.grids[key] = sp;
  c.order.push_back(key);
  *out = sp;
  return PG_OK;
}

}  // namespace
}  // namespace pg

extern "C" pg_status pg_cluster_solve(const int n[3], const double L[3], int nw, const double* waters, int nions,
                                      const double* ions, const pg_solve_params* p, double* evals, double* evecs_host,
                                      pg_solve_stats* stats, void* stream) {
  using namespace pg;
  PG_ARG(n && L && p && evals && nw >= 0 && nions >= 0, "pg_cluster_solve: bad arguments");
  PG_ARG(nw == 0 || waters, "pg_cluster_solve: null water coordinates");
  PG_ARG(nions == 0 || ions, "pg_cluster_solve: null ion list");
  PG_ARG(p->startvec == 1 || p->startvec == 2, "pg_cluster_solve: start vectors 0 and 3 need pg_solve");
  PG_ARG(p->nroots > 0, "pg_cluster_solve: bad parameters");
  cudaStream_t st = as_stream(stream);
  std::shared_ptr<pg_grid> gs;
  PG_TRY(cached_grid(n, L, &gs));
  const pg_grid* g = gs.get();
  const long N = g->N;
  // per-thread, grow-only buffers: repeated single points allocate nothing
  static thread_local SolveWorkspace ws;
  static thread_local DevBuf<double> v, vec;
  PG_TRY(v.ensure(N));
  PG_TRY(vec.ensure((size_t)N * p->nroots));
  PG_TRY(cluster_potential(g, nw, waters, nions, ions, v.p, st));
  const int prec = p->precision;
  const double* vp = v.p;
  pg_status s = solve_with(
      g, vp, p, evals, vec.p, stats, st,
      [&](const double* x, double* y, int nvec) { return hx(g, vp, x, y, nvec, prec, st, true); }, &ws);
  if (s != PG_OK && s != PG_NOT_CONVERGED) return s;
  if (evecs_host)
    PG_CUDA_TRY(cudaMemcpyAsync(evecs_host, vec.p, sizeof(double) * N * p->nroots, cudaMemcpyDeviceToHost, st));
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  return s;
}
