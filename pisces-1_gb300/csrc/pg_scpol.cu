// Self-consistent polarisation of the electron-water model (PolType 3, 5, 6)
// and the electron part of the Hellmann-Feynman gradient that stands on it.
//
// The model: every polarisable atom i of the cluster sees the field of the
// electron, e_i(r) = g(|r - R_i|) (r - R_i), plus the fixed field Epc_i of the
// water charges.  The induced dipoles are mu(r) = A E(r) with the (3 npp)^2
// matrix A = (alpha^-1 - T)^-1 of Thole-damped dipole tensors, and the
// electron feels V_pol(r) = -1/2 E(r)^T A E(r) - V_ww
// (Potential::SelfConsistentPolarizability, src/Potential.cpp:1495-1628).
//
// Over the grid the dipoles are one dense product MU = E A (N x 3npp times
// 3npp x 3npp).  The work is FP64 (the reference's precision), on this
// part's FP64 pipe: tiled in shared memory, 64 points x 64 dipole components
// per CTA, 4 x 4 outputs per thread.  V_pol is that product's epilogue: each
// CTA forms the row dots E . MU of its tile, and a second pass sums the
// column tiles of a point in a fixed order (no atomics; bit-stable).
//
// The gradient (DVR::ComputeGradient, src/DVR.cpp:1099-1176, with
// Potential::EvaluateDPPGTOPGradient / DerivElecField / MuCrossMu /
// FinalGradient / SubtractWWGradient, src/Gradients.cpp:80-289) needs MU
// itself: the dipoles enter the field-derivative term of each polarisable
// site, and the density-weighted sums  tmu = sum_g psi_g^2 mu_g  and
// mCm = sum_g psi_g^2 mu_g mu_g^T  feed the dipole-tensor derivative terms.
// mCm is a second product, MU^T diag(psi^2) MU, split over point slices whose
// partial tiles are summed in slice order.
//
// Points are processed in chunks that keep E and MU within a fixed budget of
// device memory, so the largest grids need no more than that.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pg_solve.cuh"

namespace {

constexpr int kBM = 64;   // points per product tile
constexpr int kBN = 64;   // dipole components per product tile
constexpr int kBK = 16;   // reduction depth per shared-memory stage
constexpr int kGT = 256;  // threads per product CTA (16 x 16, 4 x 4 outputs each)
constexpr size_t kChunkBytes = size_t(1) << 30;  // E (and MU) per chunk of points

// ------------------------------------------------------------------ host side

// Thole-damped dipole-dipole tensor of sites i, j (CalcDDTensor,
// src/MolPolAux.cpp:311-336): T = f5 3 r r^T / r^5 - f3 / r^3 with
// f3 = 1 - exp(-x), f5 = 1 - (1 + x) exp(-x), x = a r^3 / sqrt(alpha_i alpha_j).
void dd_tensor(double T[9], const double r[3], double ai, double aj, double a) {
  const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  const double rr = sqrt(r2);
  const double r3 = rr * r2, r5 = r2 * r3;
  const double x = a * r3 / sqrt(ai * aj);
  const double ex = exp(-x);
  const double f3 = 1 - ex, f5 = 1 - (1 + x) * ex;
  const double c1 = f5 * 3.0 / r5, c2 = f3 / r3;
  for (int p = 0; p < 3; ++p)
    for (int q = 0; q < 3; ++q) T[3 * p + q] = c1 * r[p] * r[q] - (p == q ? c2 : 0.0);
}

// In-place inverse of a row-major n x n matrix by Gauss-Jordan elimination
// with partial (row) pivoting; false if a pivot is zero.
bool invert_in_place(int n, double* a) {
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = fabs(a[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (fabs(a[(size_t)i * n + k]) > best) best = fabs(a[(size_t)i * n + k]), p = i;
    if (!(best > 0)) return false;
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(a[(size_t)k * n + j], a[(size_t)p * n + j]);
    double* rk = a + (size_t)k * n;
    const double d = 1.0 / rk[k];
    rk[k] = 1.0;
    for (int j = 0; j < n; ++j) rk[j] *= d;
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      double* ri = a + (size_t)i * n;
      const double f = ri[k];
      if (f == 0) continue;
      ri[k] = 0.0;
      for (int j = 0; j < n; ++j) ri[j] -= f * rk[j];
    }
  }
  for (int k = n - 1; k >= 0; --k)
    if (piv[k] != k)
      for (int i = 0; i < n; ++i) std::swap(a[(size_t)i * n + k], a[(size_t)i * n + piv[k]]);
  return true;
}

pg_status check_model(const char* who, const pg_sites* t, const pg_scpol_model* m) {
  PG_ARG(t && m, "%s: null argument", who);
  PG_ARG(t->nsites > 0 && t->sites, "%s: the site list is empty", who);
  PG_ARG(m->npp > 0 && m->pol_site && m->inva && m->epc, "%s: bad polarisation model", who);
  PG_ARG(m->damp_type == 1 || m->damp_type == 2, "%s: damp_type %d (1: cubic exponential, 2: effective radius)", who,
         m->damp_type);
  PG_ARG(m->damp > 0, "%s: the damping parameter must be positive", who);
  PG_ARG(3L * m->npp <= 6144, "%s: %d polarisable sites exceed the limit of 2048", who, m->npp);
  for (int i = 0; i < m->npp; ++i)
    PG_ARG(m->pol_site[i] >= 0 && m->pol_site[i] < t->nsites, "%s: polarisable site %d refers to site %d of %d", who,
           i, m->pol_site[i], t->nsites);
  return PG_OK;
}

// Device copies of a model: positions of the polarisable sites, Epc and A.
struct ModelDev {
  pg::DevBuf<double> pos, epc, inva;
  pg_status upload(const pg_sites* t, const pg_scpol_model* m, cudaStream_t st) {
    const int n = 3 * m->npp;
    std::vector<double> p(n);
    for (int i = 0; i < m->npp; ++i)
      for (int c = 0; c < 3; ++c) p[3 * i + c] = t->sites[3 * m->pol_site[i] + c];
    PG_TRY(pos.alloc(n));
    PG_TRY(epc.alloc(n));
    PG_TRY(inva.alloc((size_t)n * n));
    PG_CUDA_TRY(cudaMemcpyAsync(pos.p, p.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    PG_CUDA_TRY(cudaMemcpyAsync(epc.p, m->epc, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    PG_CUDA_TRY(cudaMemcpyAsync(inva.p, m->inva, sizeof(double) * n * n, cudaMemcpyHostToDevice, st));
    // the host arrays may be released as soon as the call returns
    PG_CUDA_TRY(cudaStreamSynchronize(st));
    return PG_OK;
  }
};

long chunk_points(long N, int n) {
  long c = (long)(kChunkBytes / (sizeof(double) * (size_t)n));
  c = c / kBM * kBM;
  if (c < kBM) c = kBM;
  return c < N ? c : N;
}

// ---------------------------------------------------------------- device side

// Field of the electron at every polarisable site plus Epc, for points
// [p0, p0 + np) of the grid (x fastest), or of a point list (list[p0 + p]):
// E[p*n + 3i + c] (src/Potential.cpp:1518-1552; distances as
// Potential::Evaluate, src/Potential.cpp:136-146).
__global__ void k_scpol_field(long p0, long np, const int* __restrict__ list, int nx, int ny,
                              const double* __restrict__ gx, const double* __restrict__ gy,
                              const double* __restrict__ gz, int npp, const double* __restrict__ pos,
                              const double* __restrict__ epc, int damp_type, double damp, double* __restrict__ E) {
  const long total = np * npp;
  const int n = 3 * npp;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long p = t / npp;
    const int i = (int)(t - p * npp);
    const long gi = list ? (long)list[p0 + p] : p0 + p;
    const int ix = (int)(gi % nx);
    const long r = gi / nx;
    const int iy = (int)(r % ny), iz = (int)(r / ny);
    const double rx = gx[ix] - pos[3 * i], ry = gy[iy] - pos[3 * i + 1], rz = gz[iz] - pos[3 * i + 2];
    const double r2 = rx * rx + ry * ry + rz * rz;
    const double rr = sqrt(r2);
    double g = 1.0 / (r2 * rr);
    if (damp_type == 1) {
      g *= 1.0 - exp(-damp * rr * r2);
    } else if (rr < damp) {
      const double q = rr / damp;
      const double reff = damp * (0.5 + q * q * q * (1.0 - 0.5 * q));
      g = 1.0 / (reff * reff * reff);
    }
    double* e = E + p * n + 3 * i;
    e[0] = g * rx + epc[3 * i];
    e[1] = g * ry + epc[3 * i + 1];
    e[2] = g * rz + epc[3 * i + 2];
  }
}

// Y = E A for np points (E: np x n, A: n x n, both row-major).  kStore:
// Y -> out[p*n + c]; otherwise out[ct*np + p] = sum over the 64 columns c of
// column tile ct of E[p][c] Y[p][c] (fixed shuffle order).
template <bool kStore>
__global__ void __launch_bounds__(kGT) k_scpol_gemm(long np, int n, const double* __restrict__ E,
                                                    const double* __restrict__ A, double* __restrict__ out) {
  __shared__ double Es[kBK][kBM + 1];
  __shared__ double As[kBK][kBN];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const long pb = (long)blockIdx.x * kBM;
  const int cb = blockIdx.y * kBN;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < n; k0 += kBK) {
#pragma unroll
    for (int e = t; e < kBM * kBK; e += kGT) {
      const int pp = e / kBK, kk = e - pp * kBK;
      const long p = pb + pp;
      const int k = k0 + kk;
      Es[kk][pp] = (p < np && k < n) ? E[p * n + k] : 0.0;
    }
#pragma unroll
    for (int e = t; e < kBK * kBN; e += kGT) {
      const int kk = e / kBN, cc = e - kk * kBN;
      const int k = k0 + kk, c = cb + cc;
      As[kk][cc] = (k < n && c < n) ? A[(long)k * n + c] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = Es[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = As[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  if (kStore) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long p = pb + ty + 16 * i;
      if (p >= np) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = cb + tx + 16 * j;
        if (c < n) out[p * n + c] = acc[i][j];
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long p = pb + ty + 16 * i;
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = cb + tx + 16 * j;
        if (p < np && c < n) s += E[p * n + c] * acc[i][j];
      }
#pragma unroll
      for (int off = 8; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (tx == 0 && p < np) out[(long)blockIdx.y * np + p] = s;
    }
  }
}

// v[g] += -1/2 sum_ct part[ct*np + p] - vww (and the polarisation part),
// g = p0 + p or list[p0 + p]
__global__ void k_scpol_finish(long p0, long np, const int* __restrict__ list, int nct, const double* __restrict__ part,
                               double vww, double* __restrict__ v, double* __restrict__ vpol) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np; p += (long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int ct = 0; ct < nct; ++ct) s += part[(long)ct * np + p];
    const double val = -0.5 * s - vww;
    const long g = list ? (long)list[p0 + p] : p0 + p;
    v[g] += val;
    if (vpol) vpol[g] += val;
  }
}

// Per-site record for the gradient: position, charge, up to two Slater
// terms, index among the polarisable sites (-1: none).
struct SiteRec {
  double x, y, z, q, z0, c0, z1, c1;
  int has_q, nsto, pol, pad;
};

// One point's gradient of V with respect to site j, in the reference's order:
// charge, Slater terms in list order, field derivative of a polarisable site
// (src/Gradients.cpp:88-137, 164-228).
__device__ __forceinline__ void site_gradient(const SiteRec& s, double ex, double ey, double ez, double cdamp,
                                              double pdamp, const double* __restrict__ mu, double g[3]) {
  const double rx = ex - s.x, ry = ey - s.y, rz = ez - s.z;
  const double r2 = rx * rx + ry * ry + rz * rz;
  const double R = sqrt(r2);
  g[0] = g[1] = g[2] = 0.0;
  if (s.has_q) {
    double vg;
    if (R < cdamp) {
      const double q = R / cdamp;
      const double reff = cdamp * (0.5 + q * q * q * (1.0 - 0.5 * q));
      vg = s.q * (3.0 * q * q - 2.0 * q * q * q) / (reff * reff);
    } else {
      vg = s.q / (R * R);
    }
    g[0] += -vg * rx / R;
    g[1] += -vg * ry / R;
    g[2] += -vg * rz / R;
  }
  if (s.nsto > 0) {
    const double d = s.c0 * (-s.z0) * exp(-s.z0 * R);
    g[0] += -d * rx / R;
    g[1] += -d * ry / R;
    g[2] += -d * rz / R;
  }
  if (s.nsto > 1) {
    const double d = s.c1 * (-s.z1) * exp(-s.z1 * R);
    g[0] += -d * rx / R;
    g[1] += -d * ry / R;
    g[2] += -d * rz / R;
  }
  if (s.pol >= 0) {
    double gij = 1.0 / (r2 * R);
    double reff = R;
    double dg = -3.0 / (reff * reff * reff * reff);
    if (reff < pdamp) {
      const double q = reff / pdamp;
      reff = pdamp * (0.5 + q * q * q * (1.0 - 0.5 * q));
      dg = -3.0 / (reff * reff * reff * reff);
      const double dr = 3.0 * q * q - 0.5 * 4.0 * q * q * q;
      gij = 1.0 / (reff * reff * reff);
      dg = dr * dg;
    }
    const double m0 = mu[0], m1 = mu[1], m2 = mu[2];
    const double rv[3] = {rx, ry, rz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double f = -dg * rv[a] / R;
      const double d0 = f * rx - (a == 0 ? gij : 0.0);
      const double d1 = f * ry - (a == 1 ? gij : 0.0);
      const double d2 = f * rz - (a == 2 ? gij : 0.0);
      g[a] += -0.5 * 2.0 * (d0 * m0 + d1 * m1 + d2 * m2);
    }
  }
}

// Density-weighted gradient sums of one slice of points per CTA:
// part[blk][3j + a] = sum_g psi_g^2 dV_g/dR_j,a and part[blk][3 ns + k] =
// sum_g psi_g^2 MU[g][k].
__global__ void __launch_bounds__(256) k_grad_sites(long p0, long np, long per, int nx, int ny,
                                                    const double* __restrict__ gx, const double* __restrict__ gy,
                                                    const double* __restrict__ gz, const double* __restrict__ psi,
                                                    const double* __restrict__ MU, int n, int ns,
                                                    const SiteRec* __restrict__ sites, double cdamp, double pdamp,
                                                    double* __restrict__ part) {
  const long g0 = blockIdx.x * per;
  const long g1 = g0 + per < np ? g0 + per : np;
  double* out = part + (long)blockIdx.x * (3L * ns + n);
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    const SiteRec s = sites[j];
    double a0 = 0, a1 = 0, a2 = 0;
    for (long p = g0; p < g1; ++p) {
      const long gi = p0 + p;
      const int ix = (int)(gi % nx);
      const long r = gi / nx;
      const int iy = (int)(r % ny), iz = (int)(r / ny);
      double g[3];
      site_gradient(s, gx[ix], gy[iy], gz[iz], cdamp, pdamp, s.pol >= 0 ? MU + p * n + 3 * s.pol : nullptr, g);
      const double w = psi[gi] * psi[gi];
      a0 += w * g[0];
      a1 += w * g[1];
      a2 += w * g[2];
    }
    out[3 * j] = a0;
    out[3 * j + 1] = a1;
    out[3 * j + 2] = a2;
  }
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double a = 0;
    for (long p = g0; p < g1; ++p) {
      const double w = psi[p0 + p] * psi[p0 + p];
      a += w * MU[p * n + k];
    }
    out[3 * ns + k] = a;
  }
}

// tot[e] += sum_b part[b*m + e], blocks in order
__global__ void k_sum_blocks(int nb, long m, const double* __restrict__ part, double* __restrict__ tot) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < m; e += (long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[(long)b * m + e];
    tot[e] += s;
  }
}

// Lower-triangle tiles (bi >= bj) of  C = MU^T diag(psi^2) MU  over one slice
// of points per blockIdx.y: part[(slice*ntiles + tile)*64*64 + ii*64 + jj].
// The left factor is psi^2 mu_i, rounded, then times mu_j, as MuCrossMu
// (src/Gradients.cpp:231-241).
__global__ void __launch_bounds__(kGT) k_grad_mcm(long p0, long np, long per, int n, const double* __restrict__ psi,
                                                  const double* __restrict__ MU, const int2* __restrict__ tiles,
                                                  int ntiles, double* __restrict__ part) {
  __shared__ double Ls[kBK][kBN];
  __shared__ double Rs[kBK][kBN];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int2 tile = tiles[blockIdx.x];
  const int ib = tile.x * kBN, jb = tile.y * kBN;
  const long g0 = blockIdx.y * per;
  const long g1 = g0 + per < np ? g0 + per : np;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (long k0 = g0; k0 < g1; k0 += kBK) {
#pragma unroll
    for (int e = t; e < kBK * kBN; e += kGT) {
      const int kk = e / kBN, cc = e - kk * kBN;
      const long p = k0 + kk;
      const bool in = p < g1;
      const int ci = ib + cc, cj = jb + cc;
      const double w = in ? psi[p0 + p] * psi[p0 + p] : 0.0;
      Ls[kk][cc] = (in && ci < n) ? w * MU[p * n + ci] : 0.0;
      Rs[kk][cc] = (in && cj < n) ? MU[p * n + cj] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = Ls[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Rs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  double* out = part + ((long)blockIdx.y * ntiles + blockIdx.x) * (kBM * kBN);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) out[(ty + 16 * i) * kBN + tx + 16 * j] = acc[i][j];
}

// C[i][j] (and C[j][i]) += sum over slices of the tile partials
__global__ void k_mcm_reduce(int n, int ntiles, int nslices, const int2* __restrict__ tiles,
                             const double* __restrict__ part, double* __restrict__ C) {
  const long total = (long)ntiles * kBM * kBN;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int tile = (int)(e / (kBM * kBN));
    const int w = (int)(e - (long)tile * kBM * kBN);
    const int i = tiles[tile].x * kBN + w / kBN, j = tiles[tile].y * kBN + w % kBN;
    if (i >= n || j >= n || j > i) continue;
    double s = 0.0;
    for (int sl = 0; sl < nslices; ++sl) s += part[((long)sl * ntiles + tile) * (kBM * kBN) + w];
    C[(long)i * n + j] += s;
    if (i != j) C[(long)j * n + i] += s;
  }
}

int stride_blocks(long work) {
  long b = (work + 255) / 256;
  return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace

extern "C" pg_status pg_scpol_inva(int npp, const double* pos, const double* alpha, double a_thole, double* inva) {
  PG_ARG(npp > 0 && pos && alpha && inva, "pg_scpol_inva: bad arguments");
  PG_ARG(a_thole >= 0, "pg_scpol_inva: negative Thole parameter");
  for (int i = 0; i < npp; ++i) PG_ARG(alpha[i] > 0, "pg_scpol_inva: polarisability %d is not positive", i);
  const int n = 3 * npp;
  // A = alpha^-1 on the diagonal 3 x 3 blocks, -T_ij off them
  // (BuildPolarizationMatrix, src/MolPolAux.cpp:100-136)
  std::fill(inva, inva + (size_t)n * n, 0.0);
  for (int i = 0; i < npp; ++i)
    for (int c = 0; c < 3; ++c) inva[(size_t)(3 * i + c) * n + 3 * i + c] = 1.0 / alpha[i];
  for (int i = 0; i < npp; ++i)
    for (int j = i + 1; j < npp; ++j) {
      const double r[3] = {pos[3 * i] - pos[3 * j], pos[3 * i + 1] - pos[3 * j + 1], pos[3 * i + 2] - pos[3 * j + 2]};
      double T[9];
      dd_tensor(T, r, alpha[i], alpha[j], a_thole);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          inva[(size_t)(3 * j + a) * n + 3 * i + b] = inva[(size_t)(3 * i + a) * n + 3 * j + b] = -T[3 * a + b];
    }
  if (!invert_in_place(n, inva)) {
    pg::set_error("pg_scpol_inva: the polarisation matrix is singular");
    return PG_NUMERIC;
  }
  // the inverse of a symmetric matrix, symmetric to round-off: keep the
  // average of the two triangles
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const double s = 0.5 * (inva[(size_t)i * n + j] + inva[(size_t)j * n + i]);
      inva[(size_t)i * n + j] = inva[(size_t)j * n + i] = s;
    }
  return PG_OK;
}

namespace pg {

pg_status scpol_add_points(const pg_grid* g, const pg_sites* t, const pg_scpol_model* m, const int* list, long count,
                           double* v, double* vpol, cudaStream_t st) {
  PG_TRY(check_model("pg_potential_scpol_add", t, m));
  if (count == 0) return PG_OK;
  ModelDev md;
  PG_TRY(md.upload(t, m, st));
  const int n = 3 * m->npp;
  const long chunk = chunk_points(count, n);
  const int nct = (n + kBN - 1) / kBN;
  pg::DevBuf<double> E, part;
  PG_TRY(E.alloc((size_t)chunk * n));
  PG_TRY(part.alloc((size_t)chunk * nct));
  for (long p0 = 0; p0 < count; p0 += chunk) {
    const long np = chunk < count - p0 ? chunk : count - p0;
    k_scpol_field<<<stride_blocks(np * m->npp), 256, 0, st>>>(p0, np, list, g->n[0], g->n[1], g->x_dev[0].p,
                                                             g->x_dev[1].p, g->x_dev[2].p, m->npp, md.pos.p, md.epc.p,
                                                             m->damp_type, m->damp, E.p);
    PG_TRY(pg::check_launch("k_scpol_field"));
    k_scpol_gemm<false><<<dim3((unsigned)((np + kBM - 1) / kBM), nct), kGT, 0, st>>>(np, n, E.p, md.inva.p, part.p);
    PG_TRY(pg::check_launch("k_scpol_gemm"));
    k_scpol_finish<<<stride_blocks(np), 256, 0, st>>>(p0, np, list, nct, part.p, m->vpol_ww, v, vpol);
    PG_TRY(pg::check_launch("k_scpol_finish"));
  }
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  return PG_OK;
}

}  // namespace pg

extern "C" pg_status pg_potential_scpol_add(const pg_grid* g, const pg_sites* t, const pg_scpol_model* m, double* v,
                                            double* parts, void* stream) {
  PG_ARG(g && v, "pg_potential_scpol_add: null argument");
  return pg::scpol_add_points(g, t, m, nullptr, g->N, v, parts ? parts + 3 * g->N : nullptr, pg::as_stream(stream));
}

extern "C" pg_status pg_hf_gradient_grid(const pg_grid* g, const pg_sites* t, const pg_scpol_model* m,
                                         const double* psi, double* grad, double* tmu, double* mcm, void* stream) {
  PG_ARG(g && psi && grad && tmu && mcm, "pg_hf_gradient_grid: null argument");
  PG_TRY(check_model("pg_hf_gradient_grid", t, m));
  PG_ARG(m->damp_type == 2,
         "pg_hf_gradient_grid: the reference gradient damps the polarisable sites by the effective radius only");
  cudaStream_t st = pg::as_stream(stream);
  ModelDev md;
  PG_TRY(md.upload(t, m, st));
  const int ns = t->nsites, n = 3 * m->npp;
  // site records: charges, Slater terms, polarisable index
  std::vector<SiteRec> rec(ns);
  for (int j = 0; j < ns; ++j) {
    SiteRec& s = rec[j];
    std::memset(&s, 0, sizeof(s));
    s.x = t->sites[3 * j], s.y = t->sites[3 * j + 1], s.z = t->sites[3 * j + 2];
    s.pol = -1;
  }
  for (int e = 0; e < t->ncharges; ++e) {
    const int j = t->charge_site[e];
    PG_ARG(j >= 0 && j < ns && !rec[j].has_q, "pg_hf_gradient_grid: charge %d on site %d", e, j);
    rec[j].has_q = 1, rec[j].q = t->charges[e];
  }
  for (int e = 0; e < t->nsto; ++e) {
    const int j = t->sto_site[e];
    PG_ARG(j >= 0 && j < ns && rec[j].nsto < 2, "pg_hf_gradient_grid: Slater term %d on site %d", e, j);
    if (rec[j].nsto == 0) rec[j].z0 = t->sto[2 * e], rec[j].c0 = t->sto[2 * e + 1];
    else rec[j].z1 = t->sto[2 * e], rec[j].c1 = t->sto[2 * e + 1];
    rec[j].nsto++;
  }
  for (int i = 0; i < m->npp; ++i) {
    const int j = m->pol_site[i];
    PG_ARG(rec[j].pol < 0, "pg_hf_gradient_grid: two polarisable sites on site %d", j);
    rec[j].pol = i;
  }
  // The reference walks the polarisable sites in site order
  // (DerivElecField, src/Gradients.cpp:164-228): only an increasing list
  // reaches every site.
  for (int i = 1; i < m->npp; ++i)
    PG_ARG(m->pol_site[i] > m->pol_site[i - 1], "pg_hf_gradient_grid: polarisable sites must be in site order");
  const long N = g->N;
  const long chunk = chunk_points(N, n);
  // tiles of the lower triangle of mCm, and point slices per chunk
  const int nt = (n + kBN - 1) / kBN;
  std::vector<int2> tl;
  for (int bi = 0; bi < nt; ++bi)
    for (int bj = 0; bj <= bi; ++bj) tl.push_back(make_int2(bi, bj));
  const int ntiles = (int)tl.size();
  const long want = (4L * 152 + ntiles - 1) / ntiles;
  const long mcm_per = std::max<long>(kBK, ((chunk + want - 1) / want + kBK - 1) / kBK * kBK);
  const int mcm_slices = (int)((chunk + mcm_per - 1) / mcm_per);
  const long site_per = std::max<long>(1, (chunk + 607) / 608);
  const int site_blocks = (int)((chunk + site_per - 1) / site_per);
  const long m1 = 3L * ns + n;
  pg::DevBuf<double> E, MU, spart, mpart, tot, C;
  pg::DevBuf<SiteRec> srec;
  pg::DevBuf<int2> dtiles;
  PG_TRY(E.alloc((size_t)chunk * n));
  PG_TRY(MU.alloc((size_t)chunk * n));
  PG_TRY(spart.alloc((size_t)site_blocks * m1));
  PG_TRY(mpart.alloc((size_t)mcm_slices * ntiles * kBM * kBN));
  PG_TRY(tot.alloc(m1));
  PG_TRY(C.alloc((size_t)n * n));
  PG_TRY(srec.alloc(ns));
  PG_TRY(dtiles.alloc(ntiles));
  PG_CUDA_TRY(cudaMemcpyAsync(srec.p, rec.data(), sizeof(SiteRec) * ns, cudaMemcpyHostToDevice, st));
  PG_CUDA_TRY(cudaMemcpyAsync(dtiles.p, tl.data(), sizeof(int2) * ntiles, cudaMemcpyHostToDevice, st));
  PG_CUDA_TRY(cudaMemsetAsync(tot.p, 0, sizeof(double) * m1, st));
  PG_CUDA_TRY(cudaMemsetAsync(C.p, 0, sizeof(double) * n * n, st));
  const int nct = (n + kBN - 1) / kBN;
  for (long p0 = 0; p0 < N; p0 += chunk) {
    const long np = chunk < N - p0 ? chunk : N - p0;
    k_scpol_field<<<stride_blocks(np * m->npp), 256, 0, st>>>(p0, np, nullptr, g->n[0], g->n[1], g->x_dev[0].p,
                                                             g->x_dev[1].p, g->x_dev[2].p, m->npp, md.pos.p, md.epc.p,
                                                             2, m->damp, E.p);
    PG_TRY(pg::check_launch("k_scpol_field"));
    k_scpol_gemm<true><<<dim3((unsigned)((np + kBM - 1) / kBM), nct), kGT, 0, st>>>(np, n, E.p, md.inva.p, MU.p);
    PG_TRY(pg::check_launch("k_scpol_gemm"));
    const int sb = (int)((np + site_per - 1) / site_per);
    k_grad_sites<<<sb, 256, 0, st>>>(p0, np, site_per, g->n[0], g->n[1], g->x_dev[0].p, g->x_dev[1].p,
                                     g->x_dev[2].p, psi, MU.p, n, ns, srec.p, t->charge_damp, m->damp, spart.p);
    PG_TRY(pg::check_launch("k_grad_sites"));
    k_sum_blocks<<<stride_blocks(m1), 256, 0, st>>>(sb, m1, spart.p, tot.p);
    PG_TRY(pg::check_launch("k_sum_blocks"));
    const int ms = (int)((np + mcm_per - 1) / mcm_per);
    k_grad_mcm<<<dim3(ntiles, ms), kGT, 0, st>>>(p0, np, mcm_per, n, psi, MU.p, dtiles.p, ntiles, mpart.p);
    PG_TRY(pg::check_launch("k_grad_mcm"));
    k_mcm_reduce<<<stride_blocks((long)ntiles * kBM * kBN), 256, 0, st>>>(n, ntiles, ms, dtiles.p, mpart.p, C.p);
    PG_TRY(pg::check_launch("k_mcm_reduce"));
  }
  std::vector<double> h(m1);
  PG_CUDA_TRY(cudaMemcpyAsync(h.data(), tot.p, sizeof(double) * m1, cudaMemcpyDeviceToHost, st));
  PG_CUDA_TRY(cudaMemcpyAsync(mcm, C.p, sizeof(double) * n * n, cudaMemcpyDeviceToHost, st));
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  std::memcpy(grad, h.data(), sizeof(double) * 3 * ns);
  std::memcpy(tmu, h.data() + 3 * ns, sizeof(double) * n);
  return PG_OK;
}

extern "C" pg_status pg_hf_gradient_final(int nsites, int npp, const double* tmu, const double* mcm,
                                          const double* dT_x, const double* dT_y, const double* dT_z,
                                          const double* dEfield, const double* pol_grad, double* gradient) {
  PG_ARG(tmu && mcm && dT_x && dT_y && dT_z && dEfield && gradient, "pg_hf_gradient_final: null argument");
  PG_ARG(npp > 0 && npp % 3 == 0 && nsites == npp / 3 * 4,
         "pg_hf_gradient_final: %d sites and %d polarisable atoms are not the rigid-water layout (O,H,H,M; O,H,H)",
         nsites, npp);
  // FinalGradient (src/Gradients.cpp:252-275)
  const int n3 = 3 * npp, n9 = 9 * npp;
  const double* dT[3] = {dT_x, dT_y, dT_z};
  for (int j = 0; j < nsites; ++j) {
    for (int d = 0; d < 3; ++d) {
      const double* row = dEfield + (size_t)n3 * (3 * j + d);
      double s = 0.0;
      for (int k = 0; k < n3; ++k) s += row[k] * tmu[k];
      gradient[3 * j + d] += -0.5 * 2.0 * s;
    }
    if ((j + 1) % 4 != 0) {
      const int aj = 3 * (j / 4) + j % 4;
      for (int d = 0; d < 3; ++d) {
        const double* a = dT[d] + (size_t)aj * n9;
        const double* b = mcm + (size_t)aj * n9;
        double s = 0.0;
        for (int k = 0; k < n9; ++k) s += a[k] * b[k];
        gradient[3 * j + d] += -0.5 * 2.0 * s;
      }
    }
  }
  // SubtractWWGradient (src/Gradients.cpp:278-289)
  if (pol_grad)
    for (int k = 0; k < 3 * nsites; ++k) gradient[k] -= pol_grad[k];
  return PG_OK;
}
