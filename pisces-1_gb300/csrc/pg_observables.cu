// Observables of converged states on the grid, and the coarse-grid start
// vector: psi^2-weighted grid reductions (DVR::ExpectationValues,
// DVR::EnergyPartitioning) and trilinear interpolation from a smaller
// equidistant grid (Small2Large).
//
// The reductions sum per-block partials in a fixed order (a second launch),
// so the results are the same bits run to run.  Arithmetic is FP64, as the
// reference's; this file is built without fused multiply-adds so that the
// interpolation weights round as the reference's do.
#include <cmath>
#include <vector>

#include "pg_common.cuh"

namespace {

constexpr int kT = 256;
constexpr int kBlocks = 296;  // partial-sum blocks per state (two per SM)
constexpr int kMom = 8;       // norm, <x>, <y>, <z>, <r^2>, <n|x|0>, <n|y|0>, <n|z|0>

// Block-wide sum of kMom values per thread into partial[(s * gridDim.x + b) * kMom + m].
__device__ __forceinline__ void block_sums(double (&a)[kMom], double* partial, int nvals) {
  __shared__ double red[kT / 32][kMom];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < kMom; ++m) {
    double v = a[m];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][m] = v;
  }
  __syncthreads();
  if (threadIdx.x < nvals) {
    double s = 0.0;
    for (int k = 0; k < kT / 32; ++k) s += red[k][threadIdx.x];
    partial[((long)blockIdx.y * gridDim.x + blockIdx.x) * kMom + threadIdx.x] = s;
  }
}

// State s = blockIdx.y: psi_s^2 times 1, x, y, z, r^2, and psi_s psi_0 times
// x, y, z (DVR::ExpectationValues, src/DVR.cpp:2383-2412).
__global__ void __launch_bounds__(kT) k_moments(long N, int nx, int ny, const double* __restrict__ X,
                                                const double* __restrict__ xg, const double* __restrict__ yg,
                                                const double* __restrict__ zg, long chunk, double* partial) {
  const int s = blockIdx.y;
  const double* __restrict__ w = X + (long)s * N;
  double a[kMom] = {0, 0, 0, 0, 0, 0, 0, 0};
  const long g0 = (long)blockIdx.x * chunk, g1 = g0 + chunk < N ? g0 + chunk : N;
  for (long g = g0 + threadIdx.x; g < g1; g += kT) {
    const int i = (int)(g % nx);
    const long r = g / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    const double x = xg[i], y = yg[j], z = zg[k];
    const double p = w[g], rho = p * p;
    a[0] += rho;
    a[1] += rho * x;
    a[2] += rho * y;
    a[3] += rho * z;
    a[4] += rho * (x * x + y * y + z * z);
    if (s > 0) {
      const double p0 = X[g];
      a[5] += p * x * p0;
      a[6] += p * y * p0;
      a[7] += p * z * p0;
    }
  }
  block_sums(a, partial, kMom);
}

// State s = blockIdx.y: psi_s^2 times the four potential parts
// (DVR::EnergyPartitioning, src/DVR.cpp:2286-2312).
__global__ void __launch_bounds__(kT) k_energy_parts(long N, const double* __restrict__ X,
                                                     const double* __restrict__ parts, long chunk, double* partial) {
  const int s = blockIdx.y;
  const double* __restrict__ w = X + (long)s * N;
  double a[kMom] = {0, 0, 0, 0, 0, 0, 0, 0};
  const long g0 = (long)blockIdx.x * chunk, g1 = g0 + chunk < N ? g0 + chunk : N;
  for (long g = g0 + threadIdx.x; g < g1; g += kT) {
    const double rho = w[g] * w[g];
#pragma unroll
    for (int c = 0; c < 4; ++c) a[c] += rho * parts[(long)c * N + g];
  }
  block_sums(a, partial, 4);
}

// out[s * nv + m] = sum over the blocks of partial[(s * nb + b) * kMom + m], in block order.
__global__ void k_sum_partials(const double* __restrict__ partial, int nb, int nstates, int nv, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nstates * nv) return;
  const int s = t / nv, m = t - s * nv;
  double acc = 0.0;
  for (int b = 0; b < nb; ++b) acc += partial[((long)s * nb + b) * kMom + m];
  out[t] = acc;
}

struct SmallGrid {
  int n[3];
  double xmin[3], dx[3];
};

// Trilinear interpolation of a small-grid function (cube order: z fastest,
// stride n1 n2 along x) at the large-grid point (X, Y, Z) = XMIN + I * DX
// (Small2Large, src/Small2Large.cpp:135-205: lower corner by truncation,
// clamped to the second-to-last point, eight weights normalised by their sum).
__global__ void k_small2large(SmallGrid s, const double* __restrict__ wf, int NX, int NY, int NZ, double X0, double Y0,
                              double Z0, double DX, double DY, double DZ, double* __restrict__ WF) {
  const long Ntot = (long)NX * NY * NZ;
  const long G = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (G >= Ntot) return;
  const int IX = (int)(G % NX);
  const long R = G / NX;
  const int IY = (int)(R % NY);
  const int IZ = (int)(R / NY);
  const long xs = (long)s.n[1] * s.n[2], ys = s.n[2];
  int lo[3], hi[3];
  double wgt[3];
  const double P[3] = {X0 + IX * DX, Y0 + IY * DY, Z0 + IZ * DZ};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int l = (int)((P[a] - s.xmin[a]) / s.dx[a]);
    int u;
    if (l < 0) {
      l = 0;
      u = 1;
    } else if (l > s.n[a] - 2) {
      l = s.n[a] - 2;
      u = s.n[a] - 1;
    } else {
      u = l + 1;
    }
    lo[a] = l;
    hi[a] = u;
    wgt[a] = (P[a] - (s.xmin[a] + l * s.dx[a])) / s.dx[a];
  }
  const double wx = wgt[0], wy = wgt[1], wz = wgt[2];
  auto at = [&](int ix, int iy, int iz) { return wf[ix * xs + iy * ys + iz]; };
  double sum = 0.0, w, v;
  w = (1 - wx) * (1 - wy) * (1 - wz);
  sum += w;
  v = at(lo[0], lo[1], lo[2]) * w;
  w = wx * (1 - wy) * (1 - wz);
  sum += w;
  v += at(hi[0], lo[1], lo[2]) * w;
  w = (1 - wx) * wy * (1 - wz);
  sum += w;
  v += at(lo[0], hi[1], lo[2]) * w;
  w = (1 - wx) * (1 - wy) * wz;
  sum += w;
  v += at(lo[0], lo[1], hi[2]) * w;
  w = wx * wy * (1 - wz);
  sum += w;
  v += at(hi[0], hi[1], lo[2]) * w;
  w = wx * (1 - wy) * wz;
  sum += w;
  v += at(hi[0], lo[1], hi[2]) * w;
  w = (1 - wx) * wy * wz;
  sum += w;
  v += at(lo[0], hi[1], hi[2]) * w;
  w = wx * wy * wz;
  sum += w;
  v += at(hi[0], hi[1], hi[2]) * w;
  WF[G] = v / sum;
}

// sum of squares, per block, then in block order
__global__ void __launch_bounds__(kT) k_sumsq(long N, const double* __restrict__ x, long chunk, double* partial) {
  double a[kMom] = {0, 0, 0, 0, 0, 0, 0, 0};
  const long g0 = (long)blockIdx.x * chunk, g1 = g0 + chunk < N ? g0 + chunk : N;
  for (long g = g0 + threadIdx.x; g < g1; g += kT) a[0] += x[g] * x[g];
  block_sums(a, partial, 1);
}

__global__ void k_scale_rsqrt_norm(long N, const double* __restrict__ sumsq, double* __restrict__ x) {
  const double f = 1.0 / sqrt(*sumsq);
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) x[g] *= f;
}

long chunk_of(long N) { return ((N + kBlocks - 1) / kBlocks + kT - 1) / kT * kT; }

}  // namespace

extern "C" pg_status pg_expectation_values(const pg_grid* g, const double* vecs, int nstates, pg_moments* out,
                                           void* stream) {
  PG_ARG(g && vecs && out && nstates > 0 && nstates <= 1024, "pg_expectation_values: bad arguments");
  cudaStream_t st = pg::as_stream(stream);
  const long N = g->N;
  const long chunk = chunk_of(N);
  const int nb = (int)((N + chunk - 1) / chunk);
  pg::DevBuf<double> partial, sums;
  PG_TRY(partial.alloc((size_t)nb * nstates * kMom));
  PG_TRY(sums.alloc((size_t)nstates * kMom));
  k_moments<<<dim3(nb, nstates), kT, 0, st>>>(N, g->n[0], g->n[1], vecs, g->x_dev[0].p, g->x_dev[1].p,
                                              g->x_dev[2].p, chunk, partial.p);
  PG_TRY(pg::check_launch("k_moments"));
  k_sum_partials<<<(nstates * kMom + 127) / 128, 128, 0, st>>>(partial.p, nb, nstates, kMom, sums.p);
  PG_TRY(pg::check_launch("k_sum_partials"));
  std::vector<double> h((size_t)nstates * kMom);
  PG_CUDA_TRY(cudaMemcpyAsync(h.data(), sums.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  for (int s = 0; s < nstates; ++s) {
    const double* a = &h[(size_t)s * kMom];
    out[s].norm = a[0];
    for (int k = 0; k < 3; ++k) out[s].r[k] = a[1 + k];
    out[s].r2 = a[4];
    for (int k = 0; k < 3; ++k) out[s].trans_dipole[k] = s > 0 ? a[5 + k] : 0.0;
  }
  return PG_OK;
}

extern "C" pg_status pg_energy_partition(const pg_grid* g, const double* vecs, int nstates, const double* parts,
                                         double* out, void* stream) {
  PG_ARG(g && vecs && parts && out && nstates > 0 && nstates <= 1024, "pg_energy_partition: bad arguments");
  cudaStream_t st = pg::as_stream(stream);
  const long N = g->N;
  const long chunk = chunk_of(N);
  const int nb = (int)((N + chunk - 1) / chunk);
  pg::DevBuf<double> partial, sums;
  PG_TRY(partial.alloc((size_t)nb * nstates * kMom));
  PG_TRY(sums.alloc((size_t)nstates * 4));
  k_energy_parts<<<dim3(nb, nstates), kT, 0, st>>>(N, vecs, parts, chunk, partial.p);
  PG_TRY(pg::check_launch("k_energy_parts"));
  k_sum_partials<<<(nstates * 4 + 127) / 128, 128, 0, st>>>(partial.p, nb, nstates, 4, sums.p);
  PG_TRY(pg::check_launch("k_sum_partials"));
  PG_CUDA_TRY(cudaMemcpyAsync(out, sums.p, sizeof(double) * nstates * 4, cudaMemcpyDeviceToHost, st));
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  return PG_OK;
}

extern "C" pg_status pg_small_to_large(const int n[3], const double xmin[3], const double dx[3], const double* wf_small,
                                       const pg_grid* g, double* wf, void* stream) {
  PG_ARG(n && xmin && dx && wf_small && g && wf, "pg_small_to_large: null argument");
  SmallGrid s;
  long ns = 1;
  for (int a = 0; a < 3; ++a) {
    PG_ARG(n[a] >= 2 && dx[a] > 0, "pg_small_to_large: the small grid needs two points and a positive step per axis");
    s.n[a] = n[a];
    s.xmin[a] = xmin[a];
    s.dx[a] = dx[a];
    ns *= n[a];
  }
  cudaStream_t st = pg::as_stream(stream);
  pg::DevBuf<double> small, partial;
  PG_TRY(small.alloc((size_t)ns));
  PG_CUDA_TRY(cudaMemcpyAsync(small.p, wf_small, sizeof(double) * ns, cudaMemcpyHostToDevice, st));
  // the large grid: its first point and the sine-DVR spacing L / (n + 1)
  double X0[3], D[3];
  for (int a = 0; a < 3; ++a) {
    X0[a] = g->x[a][0];
    D[a] = g->L[a] / (double)(g->n[a] + 1);
  }
  const long N = g->N;
  k_small2large<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(s, small.p, g->n[0], g->n[1], g->n[2], X0[0], X0[1],
                                                             X0[2], D[0], D[1], D[2], wf);
  PG_TRY(pg::check_launch("k_small2large"));
  // normalised as a DVR vector: sum of squares 1 (src/Small2Large.cpp:207-219)
  const long chunk = chunk_of(N);
  const int nb = (int)((N + chunk - 1) / chunk);
  PG_TRY(partial.alloc((size_t)nb * kMom + 1));
  k_sumsq<<<nb, kT, 0, st>>>(N, wf, chunk, partial.p);
  PG_TRY(pg::check_launch("k_sumsq"));
  double* total = partial.p + (size_t)nb * kMom;
  k_sum_partials<<<1, 128, 0, st>>>(partial.p, nb, 1, 1, total);
  PG_TRY(pg::check_launch("k_sum_partials"));
  k_scale_rsqrt_norm<<<296, 256, 0, st>>>(N, total, wf);
  PG_TRY(pg::check_launch("k_scale_rsqrt_norm"));
  PG_CUDA_TRY(cudaStreamSynchronize(st));  // the temporary buffers are released on return
  return PG_OK;
}
