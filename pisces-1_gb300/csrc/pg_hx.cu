// Y = H X on the 3-D sine-DVR grid, FP64 form.
//
// H = diag(V) + Tx (+) Ty (+) Tz: for every grid point and vector,
//   y = v x + sum_b Tx[i,b] x[b,j,k] + sum_b Ty[j,b] x[i,b,k] + sum_b Tz[k,b] x[i,j,b]
// (src/mtx.cpp:35-104 applies the same operator line by line with dspmv).
//
// On GB300 the FP64 pipe retires about 1 TFLOP/s (a warp-wide DFMA every ~70
// cycles per SM sub-partition), two orders of magnitude below the load and
// FP32 throughput, so this form is bound by DFMA issue and the kernel is
// organised around it: one thread owns one grid point for up to four vectors
// (four independent accumulators), every operand load is either coalesced
// (consecutive i across the warp: x along y and z, and Tx read as T[b][i],
// T being symmetric) or a warp-wide broadcast (x along x, Ty, Tz), and X
// stays in L2 between the three sweeps.  No tiling is needed to reach the
// DFMA roofline; the mixed form (pg_hx_tc.cu) is the fast path.
#include "pg_common.cuh"

namespace {

template <int NV>
__global__ void __launch_bounds__(256) k_hx_fp64(int nx, int ny, int nz, const double* __restrict__ tx,
                                                 const double* __restrict__ ty, const double* __restrict__ tz,
                                                 const double* __restrict__ v, const double* __restrict__ X,
                                                 double* __restrict__ Y, int nvec) {
  const long N = (long)nx * ny * nz;
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int v0 = blockIdx.y * NV;
  if (g >= N) return;
  const int i = (int)(g % nx);
  const long r = g / nx;
  const int j = (int)(r % ny);
  const int k = (int)(r / ny);
  const int nv = nvec - v0 < NV ? nvec - v0 : NV;
  const double* Xv = X + (long)v0 * N;
  double acc[NV];
  const double vg = v[g];
#pragma unroll
  for (int q = 0; q < NV; ++q) acc[q] = q < nv ? vg * Xv[(long)q * N + g] : 0.0;
  // x sweep: T[b][i] (coalesced over i), x[b,j,k] broadcast
  {
    const long base = (long)nx * (j + (long)ny * k);
    for (int b = 0; b < nx; ++b) {
      const double t = tx[(long)b * nx + i];
#pragma unroll
      for (int q = 0; q < NV; ++q)
        if (q < nv) acc[q] += t * Xv[(long)q * N + base + b];
    }
  }
  // y sweep: Ty[j][b] broadcast, x[i,b,k] coalesced
  {
    const long base = i + (long)nx * ny * k;
    const double* trow = ty + (long)j * ny;
    for (int b = 0; b < ny; ++b) {
      const double t = trow[b];
#pragma unroll
      for (int q = 0; q < NV; ++q)
        if (q < nv) acc[q] += t * Xv[(long)q * N + base + (long)nx * b];
    }
  }
  // z sweep: Tz[k][b] broadcast, x[i,j,b] coalesced
  {
    const long base = i + (long)nx * j;
    const long sz = (long)nx * ny;
    const double* trow = tz + (long)k * nz;
    for (int b = 0; b < nz; ++b) {
      const double t = trow[b];
#pragma unroll
      for (int q = 0; q < NV; ++q)
        if (q < nv) acc[q] += t * Xv[(long)q * N + base + sz * b];
    }
  }
#pragma unroll
  for (int q = 0; q < NV; ++q)
    if (q < nv) Y[(long)(v0 + q) * N + g] = acc[q];
}

// Y (mode) A x_axis X: one axis contraction in FP64, mode 0 write, 1 add.
template <int NV>
__global__ void __launch_bounds__(256) k_axis_fp64(int nx, int ny, int nz, int axis, const double* __restrict__ A,
                                                   const double* __restrict__ X, double* __restrict__ Y, int nvec,
                                                   int mode) {
  const long N = (long)nx * ny * nz;
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int v0 = blockIdx.y * NV;
  if (g >= N) return;
  const int i = (int)(g % nx);
  const long r = g / nx;
  const int j = (int)(r % ny);
  const int k = (int)(r / ny);
  const int na = axis == 0 ? nx : (axis == 1 ? ny : nz);
  const int idx = axis == 0 ? i : (axis == 1 ? j : k);
  const long stride = axis == 0 ? 1 : (axis == 1 ? nx : (long)nx * ny);
  const long base = g - (long)idx * stride;
  const int nv = nvec - v0 < NV ? nvec - v0 : NV;
  double acc[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) acc[q] = (q < nv && mode == 1) ? Y[(long)(v0 + q) * N + g] : 0.0;
  const double* arow = A + (long)idx * na;
  for (int b = 0; b < na; ++b) {
    const double t = arow[b];
#pragma unroll
    for (int q = 0; q < NV; ++q)
      if (q < nv) acc[q] += t * X[(long)(v0 + q) * N + base + (long)b * stride];
  }
#pragma unroll
  for (int q = 0; q < NV; ++q)
    if (q < nv) Y[(long)(v0 + q) * N + g] = acc[q];
}

}  // namespace

namespace pg {

pg_status tc_axis(const pg_grid* g, int a, const float* Ahi, const float* Alo, const double* v, const double* x,
                  double* y, int nvec, int mode, cudaStream_t st);

pg_status axis_apply(const pg_grid* g, int axis, const double* A64, const float* Ahi, const float* Alo,
                     const double* x, double* y, int nvec, int mode, int precision, cudaStream_t st) {
  PG_ARG(g && x && y && x != y && axis >= 0 && axis < 3 && (mode == 0 || mode == 1), "axis_apply: bad arguments");
  if (precision == PG_MIXED) return tc_axis(g, axis, Ahi, Alo, nullptr, x, y, nvec, mode, st);
  constexpr int NV = 4;
  dim3 grid((unsigned)((g->N + 255) / 256), (unsigned)((nvec + NV - 1) / NV));
  k_axis_fp64<NV><<<grid, 256, 0, st>>>(g->n[0], g->n[1], g->n[2], axis, A64, x, y, nvec, mode);
  return check_launch("k_axis_fp64");
}

pg_status hx_mixed(const pg_grid* g, const double* v, const double* x, double* y, int nvec, cudaStream_t st,
                   bool check, bool unit);

pg_status hx(const pg_grid* g, const double* v, const double* x, double* y, int nvec, int precision,
             cudaStream_t st, bool unit) {
  PG_ARG(g && v && nvec >= 0, "pg_hx: bad arguments");
  if (nvec == 0) return PG_OK;  // an empty block may come with null X and Y
  PG_ARG(x && y, "pg_hx: null X or Y");
  PG_ARG(x != y, "pg_hx: X and Y must not alias");
  if (precision == PG_MIXED) return hx_mixed(g, v, x, y, nvec, st, false, unit);
  PG_ARG(precision == PG_FP64, "pg_hx: unknown precision %d", precision);
  constexpr int NV = 4;
  dim3 grid((unsigned)((g->N + 255) / 256), (unsigned)((nvec + NV - 1) / NV));
  k_hx_fp64<NV><<<grid, 256, 0, st>>>(g->n[0], g->n[1], g->n[2], g->t_dev[0].p, g->t_dev[1].p, g->t_dev[2].p, v, x,
                                     y, nvec);
  return check_launch("k_hx_fp64");
}

}  // namespace pg

extern "C" pg_status pg_hx(const pg_grid* g, const double* v, const double* x, double* y, int nvec, int precision,
                           void* stream) {
  cudaStream_t st = pg::as_stream(stream);
  PG_TRY(pg::hx(g, v, x, y, nvec, precision, st));
  return precision == PG_MIXED ? pg::check_tc_error(g, st) : PG_OK;
}

extern "C" pg_status pg_hx_async(const pg_grid* g, const double* v, const double* x, double* y, int nvec,
                                 int precision, void* stream) {
  return pg::hx(g, v, x, y, nvec, precision, pg::as_stream(stream));
}

extern "C" pg_status pg_grid_check(const pg_grid* g, void* stream) {
  PG_ARG(g, "pg_grid_check: null grid");
  cudaStream_t st = pg::as_stream(stream);
  const pg_status s = pg::check_tc_error(g, st);
  if (s == PG_DEVICE_TIMEOUT) PG_CUDA_TRY(cudaMemsetAsync(g->tc_err.p, 0, sizeof(int), st));
  return s;
}
