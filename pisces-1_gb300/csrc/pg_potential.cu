// V(r) on the grid: electron-water DPP model, Bloomfield ions, harmonic well.
//
// Compiled with -fmad=false: every product and sum is rounded separately, in
// the reference's evaluation order.  The differences from the CPU code are
// last-place ones: exp/erf, and the undamped inverse powers of R taken from
// one reciprocal square root per site instead of a square root and divisions;
// and a Slater core term c exp(-z R) with z R > 50 (below 2e-22 c) is not
// added.
//
// Layout: the reference's per-term lists (charges, dipoles, Slater cores,
// polarisable sites, each with a site index) are packed on the host into one
// 128-byte record per site.  One thread owns one grid point and walks the
// records; records are staged into shared memory in tiles by the bulk-copy
// (TMA) engine, double buffered, so every thread of a CTA reads the same
// record from shared memory (a broadcast).  Walking sites in site order keeps
// each term's sum in the reference's list order for the default model (its
// lists are all in site order), and the four sums are combined as
// Vpc + Vind + Vrep + Vpol (src/Potential.cpp:928).
#include <cmath>
#include <cstring>
#include <vector>

#include "pg_common.cuh"

namespace {

constexpr int kRec = 16;        // doubles per site record
constexpr int kTile = 64;       // records per shared-memory tile (8 KiB)
constexpr int kThreads = 256;

// record fields
enum { R_X, R_Y, R_Z, R_Q, R_MX, R_MY, R_MZ, R_ALPHA, R_Z0, R_C0, R_Z1, R_C1, R_FLAGS };
enum { F_CHARGE = 1, F_DIPOLE = 2, F_POL = 4 };  // bits 3..4: number of Slater terms

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait on an mbarrier phase; false if the bound ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned phase) {
  for (long it = 0; it < (1L << 24); ++it) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    if (ok) return true;
  }
  return false;
}

constexpr double kStoCut = 50.0;  // z R beyond which a Slater core term is dropped

__device__ __forceinline__ double reff(double r, double r0) {
  // Effective-distance damping (DampType 2), src/Potential.cpp:1192-1196.
  if (r < r0) {
    const double q = r / r0;
    return r0 * (0.5 + q * q * q * (1.0 - 0.5 * q));
  }
  return r;
}

__global__ void __launch_bounds__(kThreads) k_potential_dpp(
    int nx, int ny, int nz, const double* __restrict__ xs, const double* __restrict__ ys,
    const double* __restrict__ zs, const double* __restrict__ rec, int nrec, double dq, double dd, double dp,
    double* __restrict__ v, double* __restrict__ parts, int* __restrict__ err) {
  __shared__ __align__(128) double tile[2][kTile * kRec];
  __shared__ __align__(8) unsigned long long bar[2];
  const long N = (long)nx * ny * nz;
  const long g = blockIdx.x * (long)kThreads + threadIdx.x;
  const int ntiles = (nrec + kTile - 1) / kTile;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int cnt = nrec < kTile ? nrec : kTile;
    bulk_load(tile[0], rec, cnt * kRec * 8, &bar[0]);
  }
  double px = 0, py = 0, pz = 0;
  if (g < N) {
    const int i = (int)(g % nx);
    const long r = g / nx;
    px = xs[i];
    py = ys[(int)(r % ny)];
    pz = zs[(int)(r / ny)];
  }
  double vpc = 0, vind = 0, vrep = 0, spol = 0;
  bool ok = true;
  for (int t = 0; t < ntiles; ++t) {
    const int buf = t & 1;
    // Issue the next tile into the other buffer (freed by the barrier at the
    // end of the previous iteration).
    if (threadIdx.x == 0 && t + 1 < ntiles) {
      const int first = (t + 1) * kTile;
      const int cnt = nrec - first < kTile ? nrec - first : kTile;
      bulk_load(tile[buf ^ 1], rec + (long)first * kRec, cnt * kRec * 8, &bar[buf ^ 1]);
    }
    // Every thread polls the barrier (bounded); the CTA then agrees on the
    // outcome so that all threads leave the loop together on a timeout.
    if (!__syncthreads_and(mbar_wait(&bar[buf], (t >> 1) & 1) ? 1 : 0)) {
      ok = false;
      // drain the copy already issued into the other buffer before leaving
      if (threadIdx.x == 0 && t + 1 < ntiles) mbar_wait(&bar[buf ^ 1], ((t + 1) >> 1) & 1);
      break;
    }
    const int cnt = nrec - t * kTile < kTile ? nrec - t * kTile : kTile;
    if (g < N) {
      for (int s = 0; s < cnt; ++s) {
        const double* R = tile[buf] + s * kRec;
        const int flags = (int)R[R_FLAGS];
        // distance table entry, src/Potential.cpp:136-146
        const double rx = px - R[R_X], ry = py - R[R_Y], rz = pz - R[R_Z];
        const double r2 = rx * rx + ry * ry + rz * rz;
        // one reciprocal square root per site serves every undamped term
        // (1/R, 1/R^3, 1/R^4); R = R^2 / R.  The damped branches (R < r0,
        // including R = 0 on a site) keep the reference's divisions.
        const double ir = rsqrt(r2);
        const double r = r2 > 0.0 ? r2 * ir : 0.0;
        if (flags & F_CHARGE) vpc += r < dq ? -R[R_Q] / reff(r, dq) : -R[R_Q] * ir;  // :1188-1204
        if (flags & F_DIPOLE) {                                                       // :1246-1262
          double m3;
          if (r < dd) {
            const double re = reff(r, dd);
            m3 = 1.0 / (re * re * re);
          } else {
            m3 = ir * ir * ir;
          }
          vind += -(rx * R[R_MX] + ry * R[R_MY] + rz * R[R_MZ]) * m3;
        }
        // repulsive Slater cores c exp(-z R) (:1301-1308); a term with
        // z R > kStoCut is below c e^-50 (< 1e-20 Eh for the water model's
        // c <= 43) and is not evaluated
        const int nsto = (flags >> 3) & 3;
        if (nsto > 0) {
          const double zr = R[R_Z0] * r;
          if (zr < kStoCut) vrep += R[R_C0] * exp(-zr);
        }
        if (nsto > 1) {
          const double zr = R[R_Z1] * r;
          if (zr < kStoCut) vrep += R[R_C1] * exp(-zr);
        }
        if (flags & F_POL) {                                  // :1350-1366
          if (r < dp) {
            const double re = reff(r, dp);
            const double re2 = re * re;
            spol += R[R_ALPHA] * r2 / (re2 * re2 * re2);
          } else {
            const double ir2 = ir * ir;
            spol += R[R_ALPHA] * (ir2 * ir2);
          }
        }
      }
    }
    __syncthreads();  // everyone is done with tile[buf] before it is refilled
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    return;
  }
  if (g < N) {
    const double vpol = spol * -0.5;  // first-order polarisation, :884
    v[g] = vpc + vind + vrep + vpol;
    if (parts) {
      parts[g] = vpc;
      parts[N + g] = vind;
      parts[2 * N + g] = vrep;
      parts[3 * N + g] = vpol;
    }
  }
}

__global__ void k_potential_ions(int nx, int ny, int nz, const double* __restrict__ xs, const double* __restrict__ ys,
                                 const double* __restrict__ zs, const double* __restrict__ ion, int nions,
                                 double dcat, double dan, double* __restrict__ v) {
  const long N = (long)nx * ny * nz;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int i = (int)(g % nx);
    const long r0 = g / nx;
    const double px = xs[i], py = ys[(int)(r0 % ny)], pz = zs[(int)(r0 / ny)];
    double acc = 0;
    for (int s = 0; s < nions; ++s) {  // src/NaCl.cpp:300-307
      const double rx = px - ion[4 * s], ry = py - ion[4 * s + 1], rz = pz - ion[4 * s + 2];
      const double r = sqrt(rx * rx + ry * ry + rz * rz);
      const double q = ion[4 * s + 3];
      const double damp = q > 0 ? dcat : dan;
      acc += -q * erf(damp * r) / r;
    }
    v[g] = v[g] + acc;
  }
}

__global__ void k_potential_spherical(int nx, int ny, int nz, const double* __restrict__ xs,
                                      const double* __restrict__ ys, const double* __restrict__ zs, double k,
                                      double* __restrict__ v) {
  const long N = (long)nx * ny * nz;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int i = (int)(g % nx);
    const long r0 = g / nx;
    const double px = xs[i], py = ys[(int)(r0 % ny)], pz = zs[(int)(r0 / ny)];
    const double d = sqrt(px * px + py * py + pz * pz);  // src/Model_pot.cpp:147-149
    v[g] = 0.5 * k * d * d;
  }
}

int grid_stride_blocks(long N) {
  long b = (N + 255) / 256;
  return (int)(b < 152L * 16 ? (b > 0 ? b : 1) : 152L * 16);
}

}  // namespace

extern "C" pg_status pg_potential_eval(const pg_grid* g, const pg_sites* t, double* v, double* parts, void* stream) {
  PG_ARG(g && t && v, "pg_potential_eval: null argument");
  PG_ARG(t->nsites >= 0 && (t->nsites == 0 || t->sites), "pg_potential_eval: bad site list");
  const int ns = t->nsites;
  std::vector<double> rec((size_t)(ns > 0 ? ns : 1) * kRec, 0.0);
  std::vector<int> nsto(ns, 0);
  for (int s = 0; s < ns; ++s)
    for (int c = 0; c < 3; ++c) rec[(size_t)s * kRec + c] = t->sites[3 * s + c];
  auto site_of = [&](const int* idx, int e, const char* what) -> long {
    const int s = idx[e];
    if (s < 0 || s >= ns) {
      pg::set_error("pg_potential_eval: %s %d refers to site %d of %d", what, e, s, ns);
      return -1;
    }
    return (long)s * kRec;
  };
  int flags_err = 0;
  std::vector<int> flags(ns, 0);
  for (int e = 0; e < t->ncharges; ++e) {
    const long o = site_of(t->charge_site, e, "charge");
    if (o < 0) return PG_BAD_ARG;
    if (flags[o / kRec] & F_CHARGE) flags_err = 1;
    flags[o / kRec] |= F_CHARGE;
    rec[o + R_Q] = t->charges[e];
  }
  for (int e = 0; e < t->ndipoles; ++e) {
    const long o = site_of(t->dipole_site, e, "dipole");
    if (o < 0) return PG_BAD_ARG;
    if (flags[o / kRec] & F_DIPOLE) flags_err = 1;
    flags[o / kRec] |= F_DIPOLE;
    for (int c = 0; c < 3; ++c) rec[o + R_MX + c] = t->dipoles[3 * e + c];
  }
  for (int e = 0; e < t->nsto; ++e) {
    const long o = site_of(t->sto_site, e, "Slater term");
    if (o < 0) return PG_BAD_ARG;
    const int k = nsto[o / kRec]++;
    if (k > 1) { flags_err = 1; continue; }
    rec[o + R_Z0 + 2 * k] = t->sto[2 * e];
    rec[o + R_C0 + 2 * k] = t->sto[2 * e + 1];
  }
  for (int e = 0; e < t->npol; ++e) {
    const long o = site_of(t->pol_site, e, "polarisable site");
    if (o < 0) return PG_BAD_ARG;
    if (flags[o / kRec] & F_POL) flags_err = 1;
    flags[o / kRec] |= F_POL;
    rec[o + R_ALPHA] = t->pol_alpha[e];
  }
  if (flags_err) {
    pg::set_error("pg_potential_eval: more than one charge, dipole or polarisable site, or more than two "
                  "Slater terms, on one site");
    return PG_UNSUPPORTED;
  }
  // The reference sums each term over its own list; walking records in site
  // order reproduces that order only if every list is sorted by site.
  for (int s = 0; s < ns; ++s) rec[(size_t)s * kRec + R_FLAGS] = (double)(flags[s] | ((nsto[s] > 2 ? 2 : nsto[s]) << 3));

  // per-thread, grow-only device copies of the site records (the call waits
  // for its stream before returning, so the next call may overwrite them)
  static thread_local pg::DevBuf<double> drec;
  static thread_local pg::DevBuf<int> derr;
  PG_TRY(drec.ensure(rec.size()));
  PG_TRY(derr.ensure(1));
  cudaStream_t st = pg::as_stream(stream);
  PG_CUDA_TRY(cudaMemcpyAsync(drec.p, rec.data(), rec.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  PG_CUDA_TRY(cudaMemsetAsync(derr.p, 0, sizeof(int), st));
  const long blocks = (g->N + kThreads - 1) / kThreads;
  if (ns > 0) {
    k_potential_dpp<<<(unsigned)blocks, kThreads, 0, st>>>(g->n[0], g->n[1], g->n[2], g->x_dev[0].p, g->x_dev[1].p,
                                                           g->x_dev[2].p, drec.p, ns, t->charge_damp, t->dipole_damp,
                                                           t->pol_damp, v, parts, derr.p);
    PG_TRY(pg::check_launch("k_potential_dpp"));
  } else {
    PG_CUDA_TRY(cudaMemsetAsync(v, 0, g->N * sizeof(double), st));
    if (parts) PG_CUDA_TRY(cudaMemsetAsync(parts, 0, 4 * g->N * sizeof(double), st));
  }
  int herr = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&herr, derr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    pg::set_error("pg_potential_eval: site-tile copy did not complete in time");
    return PG_DEVICE_TIMEOUT;
  }
  return PG_OK;
}

extern "C" pg_status pg_potential_ions_add(const pg_grid* g, int nions, const double* pos, const double* q,
                                           double r_cation, double r_anion, double* v, void* stream) {
  PG_ARG(g && v && nions >= 0 && (nions == 0 || (pos && q)), "pg_potential_ions_add: bad arguments");
  PG_ARG(r_cation > 0 && r_anion > 0, "pg_potential_ions_add: damping radii must be positive");
  if (nions == 0) return PG_OK;
  std::vector<double> ion(4 * (size_t)nions);
  for (int s = 0; s < nions; ++s) {
    for (int c = 0; c < 3; ++c) ion[4 * s + c] = pos[3 * s + c];
    ion[4 * s + 3] = q[s];
  }
  static thread_local pg::DevBuf<double> d;  // per-thread, grow-only; idle again on return
  PG_TRY(d.ensure(ion.size()));
  cudaStream_t st = pg::as_stream(stream);
  PG_CUDA_TRY(cudaMemcpyAsync(d.p, ion.data(), ion.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  k_potential_ions<<<grid_stride_blocks(g->N), 256, 0, st>>>(g->n[0], g->n[1], g->n[2], g->x_dev[0].p,
                                                             g->x_dev[1].p, g->x_dev[2].p, d.p, nions,
                                                             1.0 / r_cation, 1.0 / r_anion, v);
  PG_TRY(pg::check_launch("k_potential_ions"));
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  return PG_OK;
}

extern "C" pg_status pg_potential_spherical(const pg_grid* g, double k, double* v, void* stream) {
  PG_ARG(g && v, "pg_potential_spherical: null argument");
  k_potential_spherical<<<grid_stride_blocks(g->N), 256, 0, pg::as_stream(stream)>>>(
      g->n[0], g->n[1], g->n[2], g->x_dev[0].p, g->x_dev[1].p, g->x_dev[2].p, k, v);
  return pg::check_launch("k_potential_spherical");
}
