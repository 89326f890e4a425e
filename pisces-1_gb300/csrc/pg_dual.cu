// The dual-grid single point of the self-consistent polarisation model
// (PolType 6): a coarse grid of double spacing (odd point count per axis)
// or triple spacing (even count) over a slightly larger box is solved
// first; on the fine grid V is then taken from the coarse V by
// inverse-distance interpolation wherever every site is farther than Rtol
// (and wherever a fine point coincides with a coarse one), and evaluated
// exactly elsewhere; the coarse ground state, interpolated the same way,
// starts the fine solve (ClusterAnion::EnergyFromConfiguration,
// src/ClusterAnion.cpp:211-290; DVR::ComputePotential, src/DVR.cpp:751-832;
// DVR::InterpolVtriple / InterpolVdouble, src/DVR.cpp:1240-1444;
// DVR::ExtendWfThree / ExtendWfDouble, src/DVR.cpp:1446-1723).
//
// Index arithmetic: fine point f of an axis maps to coarse position
// p = f - h (h = 0 for double spacing; h = c/2 for triple spacing with
// c = n - 3 nc + 2, the reference's checkM), coarse cell p / s, remainder
// p % s.  Triple spacing zeroes the fine points with p < 0 or p >= n - c.
// A point with remainders r_a on the axes where r_a != 0 takes the 2^m
// coarse corners of its cell; with double spacing each weighs 1/2^m; with
// triple spacing the weight is the inverse distance in fine steps,
// normalised, as tabulated by the reference (its decimal constants).
// One kernel serves V and the start vector; the exactly evaluated points
// are gathered into a list, in grid order, and get the charge and Slater
// terms from the full-grid V kernel and the polarisation term from the
// tiled dipole product on the list only.
#include <cmath>
#include <vector>

#include "pg_solve.cuh"

namespace {

struct DualGeom {
  int n, nc, s, h, cut;  // fine and coarse points per axis, spacing, offset, first zeroed coarse position
};

pg_status dual_geom(const char* who, const pg_grid* g, const int nc[3], DualGeom& d) {
  PG_ARG(g && nc, "%s: null argument", who);
  PG_ARG(g->n[0] == g->n[1] && g->n[0] == g->n[2] && nc[0] == nc[1] && nc[0] == nc[2],
         "%s: the dual grid needs the same point count on every axis (as the reference)", who);
  d.n = g->n[0];
  d.nc = nc[0];
  if (d.n % 2 == 1) {
    PG_ARG(d.nc == (d.n + 1) / 2, "%s: %d coarse points for %d fine (double spacing needs %d)", who, d.nc, d.n,
           (d.n + 1) / 2);
    d.s = 2, d.h = 0, d.cut = d.n;
  } else {
    const int want = (d.n / 2 + 1) / 3 * 2;
    PG_ARG(d.nc == want && want >= 2, "%s: %d coarse points for %d fine (triple spacing needs %d)", who, d.nc, d.n,
           want);
    const int c = d.n - 3 * d.nc + 2;  // 0, 2 or 4
    d.s = 3, d.h = c / 2, d.cut = d.n - c;
  }
  return PG_OK;
}

// Inverse-distance weights of the reference's triple-spacing interpolation:
// 1-D 2/3, 1/3; 2-D 1/sqrt(2,5,8) and 3-D 1/sqrt(3,6,9,12), normalised
// (src/DVR.cpp:1245-1248, 1341-1344).
__device__ __forceinline__ double triple_weight(int m, int d2) {
  if (m == 1) return d2 == 1 ? 2.0 / 3.0 : 1.0 / 3.0;
  if (m == 2) return (d2 == 2 ? 0.707107 : d2 == 5 ? 0.447214 : 0.353553) / 1.955087;
  return (d2 == 3 ? 0.57735 : d2 == 6 ? 0.408248 : d2 == 9 ? 0.33333 : 0.288675) / 3.09077;
}

// Value at fine point (i, j, k) interpolated from the coarse array F
// (x fastest); 0 on the zeroed boundary layers.  The corners are summed in
// the reference's order, (0,0,0), x, y, z, xy, yz, xz, xyz, each product
// rounded before it is added (this file is built without contraction), so
// the value is the reference's bit for bit.  extend: the start-vector
// form, whose table differs from the potential's in two cases
// (DVR::ExtendWfThree against InterpolVtriple): remainders (2, 0, 1) weigh
// the corner (x, z + 1) by 1/sqrt(2) instead of 1/sqrt(8)
// (src/DVR.cpp:1563-1566 against :1329-1332), and remainders (2, 1, 2)
// weigh the corner x + 1 by 1/sqrt(9) and (x + 1, y + 1) by 1/sqrt(6),
// the other way round (src/DVR.cpp:1610-1615 against :1374-1379).
__device__ double dual_value(const DualGeom& d, const double* __restrict__ F, int i, int j, int k, bool extend,
                             bool& coincident) {
  const int p[3] = {i - d.h, j - d.h, k - d.h};
  coincident = false;
  for (int a = 0; a < 3; ++a)
    if (p[a] < 0 || p[a] >= d.cut) return 0.0;
  int c[3], r[3], m = 0;
  for (int a = 0; a < 3; ++a) {
    c[a] = p[a] / d.s;
    r[a] = p[a] - c[a] * d.s;
    m += r[a] != 0;
  }
  const long sy = d.nc, sz = (long)d.nc * d.nc;
  if (m == 0) {
    coincident = true;
    return F[c[0] + c[1] * sy + c[2] * sz];
  }
  constexpr int kOrder[8] = {0, 1, 2, 4, 3, 6, 5, 7};  // corner bits: x 1, y 2, z 4
  double v = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int corner = kOrder[q];
    const int o[3] = {corner & 1, (corner >> 1) & 1, (corner >> 2) & 1};
    bool skip = false;
    int d2 = 0;
    for (int a = 0; a < 3; ++a) {
      if (r[a] == 0 && o[a]) skip = true;
      const int dist = r[a] == 0 ? 0 : (o[a] ? d.s - r[a] : r[a]);
      d2 += dist * dist;
    }
    if (skip) continue;
    if (extend && d.s == 3) {
      if (r[0] == 2 && r[1] == 0 && r[2] == 1 && corner == 4) d2 = 2;
      if (r[0] == 2 && r[1] == 1 && r[2] == 2 && corner == 1) d2 = 9;
      if (r[0] == 2 && r[1] == 1 && r[2] == 2 && corner == 3) d2 = 6;
    }
    const double f = F[(c[0] + o[0]) + (c[1] + o[1]) * sy + (c[2] + o[2]) * sz];
    v += d.s == 2 ? f : f * triple_weight(m, d2);
  }
  return d.s == 2 ? v / (double)(1 << m) : v;
}

// V on the fine grid: interpolated where every site is farther than rtol
// (the distance is capped at 50 bohr, as Potential::MinDistCheck,
// src/Potential.cpp:95-113) or the point is on the coarse lattice; zero on
// the zeroed layers; flag 1 (exact) elsewhere.
__global__ void k_dual_classify(DualGeom d, const double* __restrict__ gx, const double* __restrict__ gy,
                                const double* __restrict__ gz, int ns, const double* __restrict__ sites, double rtol,
                                const double* __restrict__ vc, double* __restrict__ v, int* __restrict__ exact) {
  const long N = (long)d.n * d.n * d.n;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int i = (int)(g % d.n), j = (int)((g / d.n) % d.n), k = (int)(g / ((long)d.n * d.n));
    bool on_lattice;
    const double vi = dual_value(d, vc, i, j, k, false, on_lattice);
    bool zero = false;
    for (int a = 0; a < 3; ++a) {
      const int p = (a == 0 ? i : a == 1 ? j : k) - d.h;
      zero |= p < 0 || p >= d.cut;
    }
    double md = 50.0;
    const double x = gx[i], y = gy[j], z = gz[k];
    for (int s = 0; s < ns; ++s) {
      const double rx = x - sites[3 * s], ry = y - sites[3 * s + 1], rz = z - sites[3 * s + 2];
      const double r = sqrt(rx * rx + ry * ry + rz * rz);
      if (md > r) md = r;
    }
    int e = 0;
    if (zero) v[g] = 0.0;
    else if (md > rtol || on_lattice) v[g] = vi;
    else e = 1;
    exact[g] = e;
  }
}

// Per-block counts of the exact points (blocks of kSeg points).
constexpr int kSeg = 1024;
__global__ void k_dual_count(long N, const int* __restrict__ exact, int* __restrict__ counts) {
  __shared__ int c;
  if (threadIdx.x == 0) c = 0;
  __syncthreads();
  const long g0 = (long)blockIdx.x * kSeg;
  int mine = 0;
  for (long g = g0 + threadIdx.x; g < g0 + kSeg && g < N; g += blockDim.x) mine += exact[g];
  atomicAdd(&c, mine);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

// Exact points of each segment, in grid order, from its offset on (one
// warp per segment: ballots keep the order).
__global__ void k_dual_gather(long N, const int* __restrict__ exact, const int* __restrict__ offsets,
                              int* __restrict__ list) {
  const long g0 = (long)blockIdx.x * kSeg;
  int out = offsets[blockIdx.x];
  const int lane = threadIdx.x;
  for (long b = g0; b < g0 + kSeg && b < N; b += 32) {
    const long g = b + lane;
    const bool e = g < N && g < g0 + kSeg && exact[g];
    const unsigned mask = __ballot_sync(0xffffffffu, e);
    if (e) list[out + __popc(mask & ((1u << lane) - 1))] = (int)g;
    out += __popc(mask);
  }
}

// Start vector on the fine grid from the coarse state.
__global__ void k_dual_extend(DualGeom d, const double* __restrict__ wc, double* __restrict__ wf) {
  const long N = (long)d.n * d.n * d.n;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int i = (int)(g % d.n), j = (int)((g / d.n) % d.n), k = (int)(g / ((long)d.n * d.n));
    bool on;
    wf[g] = dual_value(d, wc, i, j, k, true, on);
  }
}

int blocks_for(long work) {
  const long b = (work + 255) / 256;
  return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace

extern "C" pg_status pg_dual_grid_coarse(const int n[3], const double L[3], int nc[3], double Lc[3], int* spacing) {
  PG_ARG(n && L && nc && Lc, "pg_dual_grid_coarse: null argument");
  PG_ARG(n[0] == n[1] && n[0] == n[2] && n[0] >= 3, "pg_dual_grid_coarse: the dual grid needs n x n x n points");
  PG_ARG(L[0] > 0 && L[0] == L[1] && L[0] == L[2], "pg_dual_grid_coarse: the dual grid needs a cubic box");
  // src/ClusterAnion.cpp:216-233
  const double h = L[0] / (n[0] + 1);
  const bool odd = n[0] % 2 == 1;
  for (int a = 0; a < 3; ++a) {
    nc[a] = odd ? (n[a] + 1) / 2 : (n[a] / 2 + 1) / 3 * 2;
    Lc[a] = odd ? nc[a] * 2 * h + 2 * h : nc[a] * 3 * h + 3 * h;
  }
  PG_ARG(nc[0] >= 2, "pg_dual_grid_coarse: %d points are too few for a coarse grid", n[0]);
  if (spacing) *spacing = odd ? 2 : 3;
  return PG_OK;
}

extern "C" pg_status pg_dual_grid_potential(const pg_grid* g, const int nc[3], const double* v_coarse,
                                            const pg_sites* t, const pg_scpol_model* m, double rtol, double* v,
                                            long* n_exact, void* stream) {
  DualGeom d;
  PG_TRY(dual_geom("pg_dual_grid_potential", g, nc, d));
  PG_ARG(v_coarse && v && t && m, "pg_dual_grid_potential: null argument");
  PG_ARG(t->ndipoles == 0 && t->npol == 0,
         "pg_dual_grid_potential: PolType 6 has no induced dipoles and no one-site polarisation term");
  cudaStream_t st = pg::as_stream(stream);
  const long N = g->N;
  // charges and Slater cores everywhere (cheap), then the split
  PG_TRY(pg_potential_eval(g, t, v, nullptr, stream));
  pg::DevBuf<double> sites;
  pg::DevBuf<int> exact, counts, offs, list;
  PG_TRY(sites.alloc(3 * (size_t)t->nsites));
  PG_TRY(exact.alloc(N));
  const int nseg = (int)((N + kSeg - 1) / kSeg);
  PG_TRY(counts.alloc(nseg));
  PG_TRY(offs.alloc(nseg));
  PG_CUDA_TRY(cudaMemcpyAsync(sites.p, t->sites, sizeof(double) * 3 * t->nsites, cudaMemcpyHostToDevice, st));
  k_dual_classify<<<blocks_for(N), 256, 0, st>>>(d, g->x_dev[0].p, g->x_dev[1].p, g->x_dev[2].p, t->nsites, sites.p,
                                                 rtol, v_coarse, v, exact.p);
  PG_TRY(pg::check_launch("k_dual_classify"));
  k_dual_count<<<nseg, 256, 0, st>>>(N, exact.p, counts.p);
  PG_TRY(pg::check_launch("k_dual_count"));
  std::vector<int> hc(nseg), ho(nseg);
  PG_CUDA_TRY(cudaMemcpyAsync(hc.data(), counts.p, sizeof(int) * nseg, cudaMemcpyDeviceToHost, st));
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  long total = 0;
  for (int b = 0; b < nseg; ++b) ho[b] = (int)total, total += hc[b];
  if (n_exact) *n_exact = total;
  if (total == 0) return PG_OK;
  PG_TRY(list.alloc(total));
  PG_CUDA_TRY(cudaMemcpyAsync(offs.p, ho.data(), sizeof(int) * nseg, cudaMemcpyHostToDevice, st));
  k_dual_gather<<<nseg, 32, 0, st>>>(N, exact.p, offs.p, list.p);
  PG_TRY(pg::check_launch("k_dual_gather"));
  return pg::scpol_add_points(g, t, m, list.p, total, v, nullptr, st);
}

extern "C" pg_status pg_dual_grid_extend(const pg_grid* g, const int nc[3], const double* wf_coarse, double* wf,
                                         void* stream) {
  DualGeom d;
  PG_TRY(dual_geom("pg_dual_grid_extend", g, nc, d));
  PG_ARG(wf_coarse && wf, "pg_dual_grid_extend: null argument");
  k_dual_extend<<<blocks_for(g->N), 256, 0, pg::as_stream(stream)>>>(d, wf_coarse, wf);
  return pg::check_launch("k_dual_extend");
}
