// Grid handle, kinetic builders (sine DVR; periodic FFT kinetic), diag(H)
// and the particle-in-a-box start vector.
#include <cuda_fp16.h>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <vector>

#include "pg_common.cuh"

namespace pg {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

const char* last_error() { return g_err; }

static std::atomic<long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
static std::atomic<long> g_device_allocs{0};
void count_device_alloc() { g_device_allocs.fetch_add(1, std::memory_order_relaxed); }

// The reference defines the sine DVR with a 15-digit value of pi
// (src/sine_dvr.cpp:24, src/constants.h:4); the kinetic matrix and the
// particle-in-a-box start vector use it, so it is kept here.
constexpr double kRefPi = 3.14159265358979;

}  // namespace pg

extern "C" const char* pg_last_error(void) { return pg::last_error(); }
extern "C" int pg_version(void) { return 100; }
extern "C" long pg_kernel_launches(void) { return pg::g_launches.load(); }
extern "C" long pg_device_allocations(void) { return pg::g_device_allocs.load(); }

extern "C" pg_status pg_sine_dvr(int n, double mu, double x0, double xNp1, double* x, double* ekin, int ldt) {
  PG_ARG(n > 0 && x && ekin && mu > 0 && xNp1 > x0, "pg_sine_dvr: bad arguments");
  PG_ARG(ldt == 0 || ldt >= n, "pg_sine_dvr: ldt must be 0 (packed) or >= n");
  // Equidistant interior points and the analytic DVR kinetic matrix of the
  // particle-in-a-box basis (Colbert-Miller / Light-Carrington, Phys. Rep.
  // 324, 1 (2000) eq. B.62, B.65), term order as src/sine_dvr.cpp:47-111.
  const double dx = (xNp1 - x0) / (double)(n + 1);
  for (int j = 0; j < n; ++j) x[j] = x0 + dx * (double)(j + 1);
  const double f1 = 0.5 * pg::kRefPi * pg::kRefPi / (mu * (dx * dx));
  const double f2 = pg::kRefPi / (double)(n + 1);
  const double f3 = (double)((n + 1) * (n + 1));
  auto at = [&](int a, int b) -> double& {
    return ldt > 0 ? ekin[a + (long)ldt * b] : ekin[(long)a * (a + 1) / 2 + b];
  };
  for (int a = 0; a < n; ++a) {
    const double s = sin((a + 1) * f2);
    at(a, a) = f1 * (1.0 / 3.0 + 1.0 / (6.0 * f3) - 0.5 / (f3 * (s * s)));
  }
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < a; ++b) {
      const double d = cos(f2 * (a + 1)) - cos(f2 * (b + 1));
      double v = f1 * 2.0 / f3 * sin(f2 * (a + 1)) * sin(f2 * (b + 1)) / (d * d);
      if ((a - b) % 2 == 1) v *= -1.0;
      at(a, b) = v;
    }
  if (ldt > 0)
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < a; ++b) ekin[b + (long)a * ldt] = ekin[a + (long)b * ldt];
  return PG_OK;
}

extern "C" pg_status pg_fft_kinetic(int n, double mu, double x0, double xNp1, double* x, double* ekin, double* t) {
  PG_ARG(n > 1 && x && ekin && mu > 0 && xNp1 > x0, "pg_fft_kinetic: bad arguments");
  // Tdiag (src/KE_diag.cpp:33-80): the same interior points as the sine DVR
  // and, for the periodic FFT kinetic term, the plane-wave energies
  // (dK kpoint)^2 / (2 mu) with dK = 2 pi / (n dx) and kpoint = a for
  // a < n/2, a - n otherwise (the reference's 15-digit pi).
  const double dx = (xNp1 - x0) / (double)(n + 1);
  for (int j = 0; j < n; ++j) x[j] = x0 + dx * (double)(j + 1);
  const double f2 = pg::kRefPi / (double)n;
  const double dk = 2.0 * f2 / dx;
  for (int a = 0; a < n; ++a) {
    const int kp = a >= n / 2 ? a - n : a;
    const double q = dk * kp;
    ekin[a] = q * q / (2.0 * mu);
  }
  // The operator VectorFFT::apply uses per axis, ifft(ekin * fft(.)) / n
  // (src/VectorFFTW.cpp:56-112), as a real symmetric circulant matrix:
  // T[p][q] = (1/n) sum_m ekin[m] cos(2 pi m (p - q) / n).
  if (t) {
    std::vector<double> c(n);
    for (int d = 0; d < n; ++d) {
      double s = 0;
      for (int m = 0; m < n; ++m) s += ekin[m] * cos(2.0 * M_PI * (double)(((long)m * d) % n) / (double)n);
      c[d] = s / (double)n;
    }
    for (int p = 0; p < n; ++p)
      for (int q = 0; q < n; ++q) t[(long)p * n + q] = c[(p - q + n) % n];
  }
  return PG_OK;
}

namespace {

// Round to the TF32 grid (10 explicit mantissa bits), nearest-even, as fp32.
// Row-major n x n matrix -> tensor-core operand images: rows padded to 16,
// K split into chunks of tc_kchunk(n) (zero fill past n), one K-major image
// per chunk, stored one after the other.
std::vector<float> tc_image(const std::vector<float>& M, int n) {
  const int npad = pg::tc_npad(n), kpad = pg::tc_kpad(n), kc = pg::tc_kchunk(n);
  const int nch = (kpad + kc - 1) / kc;
  std::vector<float> img((size_t)nch * npad * kc, 0.f);
  for (int r = 0; r < n; ++r)
    for (int k = 0; k < n; ++k)
      img[(size_t)(k / kc) * npad * kc + pg::tc_kmajor_off(r, k % kc, kc) / 4] = M[(size_t)r * n + k];
  return img;
}

// FP16 hi/lo images of the kinetic matrices of a grid (all axes <= 128
// points), T scaled by one power of two 2^tau so that max |T| * 2^tau lies in
// [2^14, 2^15): hi = fp16(T 2^tau), lo = fp16(T 2^tau - hi), each rounded to
// nearest, about 22 significant bits together.
pg_status build_t16(pg_grid* g) {
  for (int a = 0; a < 3; ++a)
    if (g->n[a] > 128) return PG_OK;
  double tmax = 0.0;
  for (int a = 0; a < 3; ++a)
    for (double v : g->t[a]) tmax = std::max(tmax, std::fabs(v));
  int e = 0;
  if (tmax > 0.0) std::frexp(tmax, &e);  // tmax = m 2^e, m in [0.5, 1)
  const int tau = tmax > 0.0 ? 15 - e : 0;
  g->t16_scale = tau;
  for (int a = 0; a < 3; ++a) {
    const int m = g->n[a], npad = pg::tc_npad(m), kpad = pg::tc16_kpad(m);
    std::vector<unsigned short> hi((size_t)npad * kpad, 0), lo((size_t)npad * kpad, 0);
    for (int r = 0; r < m; ++r)
      for (int k = 0; k < m; ++k) {
        const double v = std::ldexp(g->t[a][(size_t)r * m + k], tau);
        const __half h = __float2half_rn((float)v);
        const __half l = __float2half_rn((float)(v - (double)__half2float(h)));
        const size_t o = pg::tc16_kmajor_off(r, k, kpad) / 2;
        hi[o] = __half_as_ushort(h);
        lo[o] = __half_as_ushort(l);
      }
    PG_TRY(g->t16_hi[a].alloc(hi.size()));
    PG_TRY(g->t16_lo[a].alloc(lo.size()));
    PG_CUDA_TRY(cudaMemcpy(g->t16_hi[a].p, hi.data(), sizeof(unsigned short) * hi.size(), cudaMemcpyHostToDevice));
    PG_CUDA_TRY(cudaMemcpy(g->t16_lo[a].p, lo.data(), sizeof(unsigned short) * lo.size(), cudaMemcpyHostToDevice));
  }
  return PG_OK;
}

// FP16 images of the eigenbasis (forward Q^T and backward Q, n x n row-major,
// [output][input]) scaled by 2^tau, the largest entry in [2^14, 2^15).
pg_status build_q16(pg_grid* g, const std::vector<double>& q, const std::vector<double>& qt, int m) {
  double qmax = 0.0;
  for (double v : q) qmax = std::max(qmax, std::fabs(v));
  int e = 0;
  if (qmax > 0.0) std::frexp(qmax, &e);
  const int tau = qmax > 0.0 ? 15 - e : 0;
  g->q16_scale = tau;
  g->q16_sym = q == qt;
  const int npad = pg::tc_npad(m), kpad = pg::tc16_kpad(m);
  auto image = [&](const std::vector<double>& M, pg::DevBuf<unsigned short>& dhi,
                   pg::DevBuf<unsigned short>& dlo) -> pg_status {
    std::vector<unsigned short> hi((size_t)npad * kpad, 0), lo((size_t)npad * kpad, 0);
    for (int r = 0; r < m; ++r)
      for (int k = 0; k < m; ++k) {
        const double v = std::ldexp(M[(size_t)r * m + k], tau);
        const __half h = __float2half_rn((float)v);
        const __half l = __float2half_rn((float)(v - (double)__half2float(h)));
        const size_t o = pg::tc16_kmajor_off(r, k, kpad) / 2;
        hi[o] = __half_as_ushort(h);
        lo[o] = __half_as_ushort(l);
      }
    PG_TRY(dhi.alloc(hi.size()));
    PG_TRY(dlo.alloc(lo.size()));
    PG_CUDA_TRY(cudaMemcpy(dhi.p, hi.data(), sizeof(unsigned short) * hi.size(), cudaMemcpyHostToDevice));
    PG_CUDA_TRY(cudaMemcpy(dlo.p, lo.data(), sizeof(unsigned short) * lo.size(), cudaMemcpyHostToDevice));
    return PG_OK;
  };
  PG_TRY(image(qt, g->q16f_hi, g->q16f_lo));
  if (!g->q16_sym) PG_TRY(image(q, g->q16b_hi, g->q16b_lo));
  return PG_OK;
}

float to_tf32(float f) {
  unsigned u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return f;
  const unsigned lsb = (u >> 13) & 1u;
  u += 0xfffu + lsb;
  u &= 0xffffe000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
}

__global__ void k_diagonal(int nx, int ny, int nz, const double* __restrict__ v, const double* __restrict__ tx,
                           const double* __restrict__ ty, const double* __restrict__ tz, double* __restrict__ diag) {
  const long N = (long)nx * ny * nz;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int i = (int)(g % nx);
    const long r = g / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    // V first, then the axis diagonals in x, y, z order (src/DVR.cpp:1811-1831).
    double d = v[g];
    d = __dadd_rn(d, tx[(long)i * nx + i]);
    d = __dadd_rn(d, ty[(long)j * ny + j]);
    d = __dadd_rn(d, tz[(long)k * nz + k]);
    diag[g] = d;
  }
}

__global__ void k_piab(int nx, int ny, int nz, const double* __restrict__ xs, const double* __restrict__ ys,
                       const double* __restrict__ zs, double* __restrict__ wf) {
  const long N = (long)nx * ny * nz;
  const int n[3] = {nx, ny, nz};
  const double* xa[3] = {xs, ys, zs};
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int i = (int)(g % nx);
    const long r = g / nx;
    const int idx[3] = {i, (int)(r % ny), (int)(r / ny)};
    // Product of half-box sines, zero outside [x0/2, -x0/2] with x0 the first
    // grid point and L the first-to-last span (src/DVR.cpp:1737-1789).
    double w = 1;
    for (int a = 0; a < 3; ++a) {
      const double x0 = xa[a][0];
      const double L = xa[a][n[a] - 1] - x0;
      const double q = xa[a][idx[a]];
      if (q < x0 / 2 || q > -x0 / 2) w = 0.0;
      else w *= sin(pg::kRefPi / L * 2.0 * (q - x0 / 2.0));
    }
    wf[g] = w;
  }
}

int grid_blocks(long N, int threads) {
  long b = (N + threads - 1) / threads;
  const long cap = 152L * 16;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

}  // namespace

extern "C" pg_status pg_grid_create(const int n[3], const double L[3], pg_grid** out) {
  return pg_grid_create_dvr(n, L, 2, out);
}

extern "C" pg_status pg_grid_create_dvr(const int n[3], const double L[3], int dvrtype, pg_grid** out) {
  PG_ARG(n && L && out, "pg_grid_create: null argument");
  PG_ARG(dvrtype == 2 || dvrtype == 3, "pg_grid_create: dvrtype %d (2: sine DVR, 3: periodic FFT kinetic)", dvrtype);
  for (int a = 0; a < 3; ++a) {
    PG_ARG(n[a] >= 2 && n[a] <= 1024, "pg_grid_create: n[%d] = %d out of range [2, 1024]", a, n[a]);
    PG_ARG(L[a] > 0 && std::isfinite(L[a]), "pg_grid_create: L[%d] must be positive", a);
  }
  PG_ARG((double)n[0] * n[1] * n[2] < 2.0e9, "pg_grid_create: too many grid points");
  pg_grid* g = new pg_grid();
  g->dvrtype = dvrtype;
  cudaGetDevice(&g->device);
  g->N = 1;
  for (int a = 0; a < 3; ++a) {
    g->n[a] = n[a];
    g->L[a] = L[a];
    g->N *= n[a];
    const int m = n[a];
    g->x[a].resize(m);
    g->t[a].resize((size_t)m * m);
    std::vector<double> ek(m);
    pg_status s = dvrtype == 3 ? pg_fft_kinetic(m, 1.0, -0.5 * L[a], 0.5 * L[a], g->x[a].data(), ek.data(),
                                                g->t[a].data())
                               : pg_sine_dvr(m, 1.0, -0.5 * L[a], 0.5 * L[a], g->x[a].data(), g->t[a].data(), m);
    if (s != PG_OK) { delete g; return s; }
    g->ekin[a] = ek;
    std::vector<float> hi((size_t)m * m), lo((size_t)m * m);
    for (size_t e = 0; e < hi.size(); ++e) {
      hi[e] = to_tf32((float)g->t[a][e]);
      lo[e] = to_tf32((float)(g->t[a][e] - (double)hi[e]));
    }
    const std::vector<float> hi_img = tc_image(hi, m), lo_img = tc_image(lo, m);
    if ((s = g->t_dev[a].alloc((size_t)m * m)) != PG_OK || (s = g->t_hi[a].alloc(hi_img.size())) != PG_OK ||
        (s = g->t_lo[a].alloc(lo_img.size())) != PG_OK || (s = g->x_dev[a].alloc(m)) != PG_OK) {
      delete g;
      return s;
    }
    if (cudaMemcpy(g->t_dev[a].p, g->t[a].data(), sizeof(double) * m * m, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(g->t_hi[a].p, hi_img.data(), sizeof(float) * hi_img.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(g->t_lo[a].p, lo_img.data(), sizeof(float) * lo_img.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(g->x_dev[a].p, g->x[a].data(), sizeof(double) * m, cudaMemcpyHostToDevice) != cudaSuccess) {
      pg::set_error("pg_grid_create: upload failed: %s", cudaGetErrorString(cudaGetLastError()));
      delete g;
      return PG_CUDA;
    }
  }
  {
    const pg_status s16 = build_t16(g);
    if (s16 != PG_OK) {
      delete g;
      return s16;
    }
  }
  // Eigenbasis of the kinetic matrix of each axis, T = Q diag(d) Q^T, for the
  // kinetic preconditioner (forward transform Q^T, backward Q).
  //   sine DVR: the DVR is the particle-in-a-box basis, Q is the orthonormal
  //     DST-I matrix Q[i][k] = sqrt(2/(n+1)) sin(pi (i+1)(k+1)/(n+1)) (symmetric,
  //     Q^T = Q) and d_k = (pi (k+1) / L)^2 / 2 (src/sine_dvr.cpp:1-12);
  //   periodic FFT kinetic: the real Fourier basis, columns 1/sqrt(n),
  //     sqrt(2/n) cos(2 pi m i / n), sqrt(2/n) sin(2 pi m i / n) for
  //     0 < m < n/2, and (-1)^i / sqrt(n) for even n; d = the plane-wave
  //     energy of m.
  for (int a = 0; a < 3; ++a) {
    const int m = n[a];
    std::vector<double> q((size_t)m * m), qt((size_t)m * m), d(m);
    if (dvrtype == 3) {
      const std::vector<double>& ek = g->ekin[a];
      int col = 0;
      auto put = [&](int c, auto f, double e) {
        for (int i = 0; i < m; ++i) q[(size_t)i * m + c] = f(i);
        d[c] = e;
      };
      put(col++, [&](int) { return 1.0 / sqrt((double)m); }, ek[0]);
      for (int f = 1; 2 * f < m; ++f) {
        const double s2 = sqrt(2.0 / m);
        put(col++, [&](int i) { return s2 * cos(2.0 * M_PI * (double)(((long)f * i) % m) / m); }, ek[f]);
        put(col++, [&](int i) { return s2 * sin(2.0 * M_PI * (double)(((long)f * i) % m) / m); }, ek[f]);
      }
      if (m % 2 == 0) put(col++, [&](int i) { return (i % 2 ? -1.0 : 1.0) / sqrt((double)m); }, ek[m / 2]);
    } else {
      const double s = sqrt(2.0 / (m + 1));
      for (int i = 0; i < m; ++i)
        for (int k = 0; k < m; ++k)
          q[(size_t)i * m + k] = s * sin(M_PI * (double)((long)(i + 1) * (k + 1) % (2 * (m + 1))) / (m + 1));
      for (int k = 0; k < m; ++k) d[k] = 0.5 * (M_PI * (k + 1) / L[a]) * (M_PI * (k + 1) / L[a]);
    }
    for (int i = 0; i < m; ++i)
      for (int k = 0; k < m; ++k) qt[(size_t)k * m + i] = q[(size_t)i * m + k];
    // forward (Q^T) and backward (Q) transforms in FP64 and as TF32 operand images
    auto upload = [&](const std::vector<double>& M, pg::DevBuf<double>& dv, pg::DevBuf<float>& hi,
                      pg::DevBuf<float>& lo) -> bool {
      std::vector<float> h((size_t)m * m), l((size_t)m * m);
      for (size_t e = 0; e < M.size(); ++e) {
        h[e] = to_tf32((float)M[e]);
        l[e] = to_tf32((float)(M[e] - (double)h[e]));
      }
      const std::vector<float> hi_img = tc_image(h, m), lo_img = tc_image(l, m);
      return dv.alloc((size_t)m * m) == PG_OK && hi.alloc(hi_img.size()) == PG_OK &&
             lo.alloc(lo_img.size()) == PG_OK &&
             cudaMemcpy(dv.p, M.data(), sizeof(double) * M.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(hi.p, hi_img.data(), sizeof(float) * hi_img.size(), cudaMemcpyHostToDevice) ==
                 cudaSuccess &&
             cudaMemcpy(lo.p, lo_img.data(), sizeof(float) * lo_img.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    };
    if (!upload(qt, g->q_dev[a], g->q_hi[a], g->q_lo[a]) || !upload(q, g->qb_dev[a], g->qb_hi[a], g->qb_lo[a]) ||
        g->d_dev[a].alloc(m) != PG_OK ||
        cudaMemcpy(g->d_dev[a].p, d.data(), sizeof(double) * m, cudaMemcpyHostToDevice) != cudaSuccess) {
      pg::set_error("pg_grid_create: kinetic eigenbasis upload failed");
      delete g;
      return PG_OOM;
    }
    if (a == 0 && n[1] == m && n[2] == m && m <= 128) {
      const pg_status s16 = build_q16(g, q, qt, m);
      if (s16 != PG_OK) {
        delete g;
        return s16;
      }
    }
  }
  if (g->tc_err.alloc(1) != PG_OK || cudaMemset(g->tc_err.p, 0, sizeof(int)) != cudaSuccess) {
    pg::set_error("pg_grid_create: allocation of the status word failed");
    delete g;
    return PG_OOM;
  }
  *out = g;
  return PG_OK;
}

extern "C" pg_status pg_grid_destroy(pg_grid* g) {
  delete g;
  return PG_OK;
}

extern "C" long pg_grid_npoints(const pg_grid* g) { return g ? g->N : 0; }

extern "C" pg_status pg_grid_points(const pg_grid* g, double* x, double* y, double* z) {
  PG_ARG(g, "pg_grid_points: null grid");
  double* o[3] = {x, y, z};
  for (int a = 0; a < 3; ++a)
    if (o[a]) memcpy(o[a], g->x[a].data(), sizeof(double) * g->n[a]);
  return PG_OK;
}

extern "C" pg_status pg_grid_kinetic(const pg_grid* g, int axis, double* t) {
  PG_ARG(g && t && axis >= 0 && axis < 3, "pg_grid_kinetic: bad arguments");
  memcpy(t, g->t[axis].data(), sizeof(double) * g->t[axis].size());
  return PG_OK;
}

extern "C" pg_status pg_diagonal(const pg_grid* g, const double* v, double* diag, void* stream) {
  PG_ARG(g && v && diag, "pg_diagonal: null argument");
  k_diagonal<<<grid_blocks(g->N, 256), 256, 0, pg::as_stream(stream)>>>(g->n[0], g->n[1], g->n[2], v, g->t_dev[0].p,
                                                                        g->t_dev[1].p, g->t_dev[2].p, diag);
  return pg::check_launch("k_diagonal");
}

extern "C" pg_status pg_piab_start(const pg_grid* g, double* wf, void* stream) {
  PG_ARG(g && wf, "pg_piab_start: null argument");
  k_piab<<<grid_blocks(g->N, 256), 256, 0, pg::as_stream(stream)>>>(g->n[0], g->n[1], g->n[2], g->x_dev[0].p,
                                                                     g->x_dev[1].p, g->x_dev[2].p, wf);
  return pg::check_launch("k_piab");
}
