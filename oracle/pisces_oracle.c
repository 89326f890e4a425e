/*
 * CPU oracle for the PISCES excess-electron eigensolve path -- TEST
 * INFRASTRUCTURE ONLY (see pisces_oracle.h).  Plain C + OpenMP restatement of
 * the reference algorithms; each function cites the reference file:line it
 * follows.  Built with -ffp-contract=off so that no multiply-add is fused and
 * results do not depend on the host's FMA policy.
 */
#include "pisces_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Thread count of the OpenMP loops below (results do not depend on it). */
void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* The reference's own value of pi, truncated to 15 digits
 * (src/sine_dvr.cpp:24, src/constants.h:4); the kinetic matrix and the
 * start vector are defined with it. */
#define OR_PI 3.14159265358979

/* ------------------------------------------------------------------ grid */

void or_sine_dvr(int n, double mu, double x0, double xNp1, double* x, double* t) {
  /* src/sine_dvr.cpp:47,61-62: equidistant interior points of the box. */
  const double dx = (xNp1 - x0) / (double)(n + 1);
  for (int j = 0; j < n; ++j) x[j] = x0 + dx * (double)(j + 1);
  /* src/sine_dvr.cpp:72-74 (eq. B.65 of Phys. Rep. 324, 1). */
  const double f1 = 0.5 * OR_PI * OR_PI / (mu * (dx * dx));
  const double f2 = OR_PI / (double)(n + 1);
  const double f3 = (double)((n + 1) * (n + 1));
  for (int a = 0; a < n; ++a) { /* diagonal, :80-86 */
    const double s = sin((a + 1) * f2);
    t[(long)a * (a + 1) / 2 + a] = f1 * (1.0 / 3.0 + 1.0 / (6.0 * f3) - 0.5 / (f3 * (s * s)));
  }
  for (int a = 0; a < n; ++a) { /* off-diagonal, :101-111 */
    for (int b = 0; b < a; ++b) {
      const double d = cos(f2 * (a + 1)) - cos(f2 * (b + 1));
      double v = f1 * 2.0 / f3 * sin(f2 * (a + 1)) * sin(f2 * (b + 1)) / (d * d);
      if ((a - b) % 2 == 1) v *= -1.0;
      t[(long)a * (a + 1) / 2 + b] = v;
    }
  }
}

static inline double tp_at(const double* tp, int a, int b) {
  return a >= b ? tp[(long)a * (a + 1) / 2 + b] : tp[(long)b * (b + 1) / 2 + a];
}

/* ---------------------------------------------------------------- matvec */

void or_matvec(const int n[3], const double* const tp[3], const double* v, const double* x, double* y) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const long N = (long)nx * ny * nz;
  const long stride[3] = {1, nx, (long)nx * ny};
  /* Unpack the symmetric matrices once (the reference applies them packed with
   * dspmv; the arithmetic per line is the same dense symmetric product). */
  double* full[3];
  for (int a = 0; a < 3; ++a) {
    full[a] = (double*)malloc(sizeof(double) * n[a] * n[a]);
    for (int r = 0; r < n[a]; ++r)
      for (int c = 0; c < n[a]; ++c) full[a][(long)r * n[a] + c] = tp_at(tp[a], r, c);
  }
  /* y = V x (src/mtx.cpp:35-38). */
#pragma omp parallel for schedule(static)
  for (long g = 0; g < N; ++g) y[g] = v[g] * x[g];
  /* Three axis sweeps, each line y_line += T_axis x_line (src/mtx.cpp:61-104). */
  for (int ax = 0; ax < 3; ++ax) {
    const int len = n[ax];
    const long st = stride[ax];
    const int o1 = ax == 0 ? ny : nx;                  /* the two other axes */
    const int o2 = ax == 2 ? ny : nz;
    const long s1 = ax == 0 ? stride[1] : stride[0];
    const long s2 = ax == 2 ? stride[1] : stride[2];
    const double* T = full[ax];
#pragma omp parallel for collapse(2) schedule(static)
    for (int q2 = 0; q2 < o2; ++q2) {
      for (int q1 = 0; q1 < o1; ++q1) {
        const long off = (long)q1 * s1 + (long)q2 * s2;
        for (int a = 0; a < len; ++a) {
          const double* Ta = T + (long)a * len;
          double s = 0.0;
          for (int b = 0; b < len; ++b) s += Ta[b] * x[off + (long)b * st];
          y[off + (long)a * st] += s;
        }
      }
    }
  }
  for (int a = 0; a < 3; ++a) free(full[a]);
}

void or_diagonal(const int n[3], const double* const tp[3], const double* v, double* diag) {
  /* src/DVR.cpp:1808-1881: V first, then the T diagonals axis by axis. */
  const int nx = n[0], ny = n[1], nz = n[2];
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long g = i + (long)nx * (j + (long)ny * k);
        double d = v[g];
        d += tp_at(tp[0], i, i);
        d += tp_at(tp[1], j, j);
        d += tp_at(tp[2], k, k);
        diag[g] = d;
      }
}

void or_piab_start(const int n[3], const double* const x[3], double* wf) {
  /* src/DVR.cpp:1737-1799: x0 = first grid point, L = last - first; nonzero
   * only on the half box [x0/2, -x0/2] along every axis. */
  double x0[3], L[3];
  for (int a = 0; a < 3; ++a) { x0[a] = x[a][0]; L[a] = x[a][n[a] - 1] - x0[a]; }
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const long g = i + (long)n[0] * (j + (long)n[1] * k);
        const double q[3] = {x[0][i], x[1][j], x[2][k]};
        double w = 1;
        for (int a = 0; a < 3; ++a) {
          if (q[a] < x0[a] / 2 || q[a] > -x0[a] / 2) w = 0.0;
          else w *= sin(OR_PI / L[a] * 2.0 * (q[a] - x0[a] / 2.0));
        }
        wf[g] = w;
      }
}

void or_random_start(int count, double* out) {
  /* src/DVR.cpp:52-59 (Randm11): the sign draw and the magnitude draw are two
   * separate rand() calls. */
  for (int i = 0; i < count; ++i) {
    if (rand() > RAND_MAX / 2) out[i] = (double)rand() / RAND_MAX;
    else out[i] = -(double)rand() / RAND_MAX;
  }
}

/* ------------------------------------------------------------ water model */

#define OR_BOHR2ANGS 0.52917720859                  /* src/constants.h:18 */
#define OR_ANGS2BOHR (1 / OR_BOHR2ANGS)             /* src/constants.h:19 */
/* Rigid DPP monomer in its centre-of-mass frame, Angstrom (src/ttm_data.h:28-48). */
#define OR_TTM_OZ 0.0650980307
#define OR_TTM_HZ (-0.5207842453)
#define OR_TTM_HY 0.756950327
#define OR_TTM_MZ (OR_TTM_OZ - 0.25)
#define OR_TTM_QH 0.5742185854046506                /* src/ttm_data.h:15-16 */
#define OR_TTM_QM (-2 * OR_TTM_QH)

typedef struct { double x[4], y[4], z[4]; double ox, oy, oz, phi, theta, psi; } or_water;

static void or_water_update(or_water* w) {
  /* Water::UpdatePositions = ResetPositions + ApplyEuler (src/Water.cpp:850-943). */
  const double rx[4] = {0, 0, 0, 0};
  const double ry[4] = {0, OR_TTM_HY * OR_ANGS2BOHR, -(OR_TTM_HY * OR_ANGS2BOHR), 0};
  const double rz[4] = {OR_TTM_OZ * OR_ANGS2BOHR, OR_TTM_HZ * OR_ANGS2BOHR, OR_TTM_HZ * OR_ANGS2BOHR,
                        OR_TTM_MZ * OR_ANGS2BOHR};
  for (int s = 0; s < 4; ++s) {
    w->x[s] = w->ox + rx[s];
    w->y[s] = s == 2 ? w->oy - (OR_TTM_HY * OR_ANGS2BOHR) : w->oy + ry[s];
    w->z[s] = w->oz + rz[s];
  }
  const double c1 = cos(w->phi), c2 = cos(w->theta), c3 = cos(w->psi);
  const double s1 = sin(w->phi), s2 = sin(w->theta), s3 = sin(w->psi);
  const double m[9] = {c1 * c2 * c3 - s1 * s3, -c1 * c2 * s3 - s1 * c3, c1 * s2,
                       s1 * c2 * c3 + c1 * s3, -s1 * c2 * s3 + c1 * c3, s1 * s2,
                       -s2 * c3,               s2 * s3,                 c2};
  for (int s = 0; s < 4; ++s) {
    const double px = w->x[s] - w->ox, py = w->y[s] - w->oy, pz = w->z[s] - w->oz;
    const double nx = m[0] * px + m[1] * py + m[2] * pz;
    const double ny = m[3] * px + m[4] * py + m[5] * pz;
    const double nz = m[6] * px + m[7] * py + m[8] * pz;
    w->x[s] = nx + w->ox; w->y[s] = ny + w->oy; w->z[s] = nz + w->oz;
  }
}

static void or_water_reposition(or_water* w, const double* a) {
  /* Water::Reposition (src/Water.cpp:695-824): project O,H,H (bohr) onto the
   * rigid model: CoM origin plus z-y-z Euler angles of the molecular frame. */
  const double ox = a[0], oy = a[1], oz = a[2];
  const double r1x = a[3] - ox, r1y = a[4] - oy, r1z = a[5] - oz;
  const double r3x = a[6] - ox, r3y = a[7] - oy, r3z = a[8] - oz;
  double zx = r1x + r3x, zy = r1y + r3y, zz = r1z + r3z;
  const double zm = sqrt(zx * zx + zy * zy + zz * zz);
  zx /= zm; zy /= zm; zz /= zm;
  zx = -zx; zy = -zy; zz = -zz;
  const double p = r1x * zx + r1y * zy + r1z * zz;
  double yx = r1x - p * zx, yy = r1y - p * zy, yz = r1z - p * zz;
  const double ym = sqrt(yx * yx + yy * yy + yz * yz);
  yx /= ym; yy /= ym; yz /= ym;
  const double xy = yz * zx - yx * zz;
  const double xz = yx * zy - yy * zx;
  double phi, psi;
  const double theta = acos(zz);
  const double st = sin(theta);
  if (fabs(st) > 1e-5) {
    double tc = -xz / st;
    double ac = acos(tc);
    if (tc <= -1) ac = OR_PI;
    psi = yz >= 0 ? ac : 2 * OR_PI - ac;
    tc = zx / st;
    if (tc > 1) tc = 1;
    if (tc < -1) tc = -1;
    phi = zy >= 0 ? acos(tc) : 2 * OR_PI - acos(tc);
  } else {
    phi = 0.0;
    psi = xy >= 0 ? acos(yy) : 2 * OR_PI - acos(yy);
  }
  w->ox = (a[3] + a[6] + 16.0 * ox) / 18.0;
  w->oy = (a[4] + a[7] + 16.0 * oy) / 18.0;
  w->oz = (a[5] + a[8] + 16.0 * oz) / 18.0;
  w->phi = phi; w->theta = theta; w->psi = psi;
  or_water_update(w);
}

static double or_damp_dc(double r, double ai, double aj, double a) {
  /* ElectrostaticDCDamp (src/DPP.cpp:1798-1804). */
  const double A = pow(ai * aj, 1.0 / 6.0);
  const double x = a * pow(r / A, 3);
  return 1.0 - exp(-x);
}

static double or_damp_dd(double r, double ai, double aj, double a) {
  /* ElectrostaticDDDamp (src/DPP.cpp:1806-1814). */
  const double A = pow(ai * aj, 1.0 / 6.0);
  const double x = a * pow(r / A, 3);
  return 1.0 - (1 + x) * exp(-x);
}

int or_dpp_sites(int nw, const double* wa, double* sites, double* charges, int* charge_site, double* dipoles,
                 int* dipole_site) {
  const double pol_o = 1.22 * pow(OR_ANGS2BOHR, 3), pol_h = 0.28 * pow(OR_ANGS2BOHR, 3); /* src/ttm_data.h:55-56 */
  const double damp_cd = 0.21, damp_dd = 0.3;   /* DPP Damping[1], Damping[2]: src/Water.cpp:240 */
  or_water* w = (or_water*)calloc(nw, sizeof(or_water));
  for (int i = 0; i < nw; ++i) {
    double b[9];
    for (int c = 0; c < 9; ++c) b[c] = wa[9 * i + c] * OR_ANGS2BOHR;   /* Reposition_A, src/Water.cpp:679-693 */
    or_water_reposition(&w[i], b);
  }
  /* Polarisable sites: O, H1, H2 of every water (alpha != 0; M has none). */
  const int ns = 3 * nw;
  double *px = malloc(sizeof(double) * ns), *py = malloc(sizeof(double) * ns), *pz = malloc(sizeof(double) * ns);
  double *al = malloc(sizeof(double) * ns);
  double *f1 = calloc(3 * ns, sizeof(double)), *f2 = malloc(sizeof(double) * 3 * ns);
  double *mu = malloc(sizeof(double) * 3 * ns), *old = malloc(sizeof(double) * 3 * ns);
  for (int j = 0; j < nw; ++j)
    for (int k = 0; k < 3; ++k) {
      const int i = 3 * j + k;
      px[i] = w[j].x[k]; py[i] = w[j].y[k]; pz[i] = w[j].z[k];
      al[i] = k == 0 ? pol_o : pol_h;
    }
  /* Field of the permanent charges at the polarisable sites of other waters
   * (src/DPP.cpp:815-855); the charge carries its own damping polarisability
   * ("sigma": H -> alpha_H, M -> alpha_O, src/Water.cpp:229-232). */
  for (int j = 0; j < nw; ++j)
    for (int k = 1; k < 4; ++k) {
      const double q = k == 3 ? OR_TTM_QM : OR_TTM_QH;
      const double ak = k == 3 ? pol_o : pol_h;
      for (int i = 0; i < ns; ++i) {
        if (i / 3 == j) continue;
        const double rx = px[i] - w[j].x[k], ry = py[i] - w[j].y[k], rz = pz[i] - w[j].z[k];
        const double tensor = q * pow(rx * rx + ry * ry + rz * rz, -1.5);
        const double dist = sqrt(rx * rx + ry * ry + rz * rz);
        const double damp = or_damp_dc(dist, al[i], ak, damp_cd);
        f1[3 * i + 0] += tensor * rx * damp;
        f1[3 * i + 1] += tensor * ry * damp;
        f1[3 * i + 2] += tensor * rz * damp;
      }
    }
  /* Damped SCF with mixing 1/2, threshold 1e-12 on the mean change
   * (src/DPP.cpp:858-868, 948-1033). */
  for (int i = 0; i < ns; ++i)
    for (int c = 0; c < 3; ++c) mu[3 * i + c] = 0.5 * al[i] * f1[3 * i + c];
  const int maxit = 5 * (ns + 10);
  int iters = -1;
  for (int it = 0; it < maxit; ++it) {
    for (int i = 0; i < 3 * ns; ++i) f2[i] = 0;
    for (int i = 0; i < ns; ++i)
      for (int j = 0; j < ns; ++j) {
        if (j == i) continue;
        /* FieldOfDipole (src/DPP.cpp:2377-2410): field at site i of dipole j. */
        const double rx = px[i] - px[j], ry = py[i] - py[j], rz = pz[i] - pz[j];
        const double r2 = rx * rx + ry * ry + rz * rz;
        const double r5 = pow(r2, -2.5);
        const double d1 = or_damp_dd(sqrt(r2), al[i], al[j], damp_dd);
        const double d2 = or_damp_dc(sqrt(r2), al[i], al[j], damp_dd);
        const double txx = (d1 * 3. * rx * rx - d2 * r2) * r5;
        const double tyy = (d1 * 3. * ry * ry - d2 * r2) * r5;
        const double tzz = (d1 * 3. * rz * rz - d2 * r2) * r5;
        const double txy = d1 * 3. * rx * ry * r5;
        const double txz = d1 * 3. * rx * rz * r5;
        const double tyz = d1 * 3. * ry * rz * r5;
        const double mx = mu[3 * j], my = mu[3 * j + 1], mz = mu[3 * j + 2];
        f2[3 * i + 0] += txx * mx + txy * my + txz * mz;
        f2[3 * i + 1] += txy * mx + tyy * my + tyz * mz;
        f2[3 * i + 2] += txz * mx + tyz * my + tzz * mz;
      }
    double tester = 0;
    for (int i = 0; i < ns; ++i)
      for (int c = 0; c < 3; ++c) {
        old[3 * i + c] = mu[3 * i + c];
        mu[3 * i + c] = 0.5 * old[3 * i + c] + 0.5 * al[i] * (f1[3 * i + c] + f2[3 * i + c]);
      }
    for (int i = 0; i < ns; ++i) {
      const double tx = old[3 * i] - mu[3 * i], ty = old[3 * i + 1] - mu[3 * i + 1], tz = old[3 * i + 2] - mu[3 * i + 2];
      tester += tx * tx + ty * ty + tz * tz;
    }
    tester = sqrt(tester) / 3 / ns;
    if (tester < 1e-12) { iters = it + 1; break; }
  }
  /* Lists for the electron (src/DPP.cpp:402-529). */
  for (int j = 0; j < nw; ++j) {
    for (int s = 0; s < 4; ++s) {
      sites[12 * j + 3 * s + 0] = w[j].x[s];
      sites[12 * j + 3 * s + 1] = w[j].y[s];
      sites[12 * j + 3 * s + 2] = w[j].z[s];
    }
    for (int c = 0; c < 3; ++c) {
      charges[3 * j + c] = c == 2 ? OR_TTM_QM : OR_TTM_QH;
      charge_site[3 * j + c] = 4 * j + 1 + c;
      dipole_site[3 * j + c] = 4 * j + c;
      for (int d = 0; d < 3; ++d) dipoles[9 * j + 3 * c + d] = mu[3 * (3 * j + c) + d];
    }
  }
  free(px); free(py); free(pz); free(al); free(f1); free(f2); free(mu); free(old); free(w);
  return iters;
}

void or_dpp_default_tables(int nw, const double* sites, const double* charges, const int* charge_site,
                           const double* dipoles, const int* dipole_site, double* sto, int* sto_site,
                           double* pol_alpha, int* pol_site, or_dpp_tables* t) {
  /* Set4STORepCore (src/Potential.cpp:699-728) with RepCoreScale 4.4837 and
   * one polarisable site per water on M with Alpha 9.745 (:326-338); damping
   * radii CoulombDamping = DipoleDamping = 1.7724, PolDamping = 2.536
   * (src/GetInput.cpp:43-63, src/Potential.cpp:283-287). */
  const double sig = 1.0 / 4.4837;
  for (int i = 0; i < nw; ++i) {
    double* g = sto + 8 * i;
    g[0] = 9.98526; g[1] = 192.608 * sig; g[2] = 1.67075; g[3] = 13.8937 * sig;
    g[4] = 1.64121; g[5] = 1.7643 * sig;  g[6] = 1.64121; g[7] = 1.7643 * sig;
    sto_site[4 * i + 0] = 4 * i; sto_site[4 * i + 1] = 4 * i; sto_site[4 * i + 2] = 4 * i + 1; sto_site[4 * i + 3] = 4 * i + 2;
    pol_alpha[i] = 9.745; pol_site[i] = 4 * i + 3;
  }
  t->nsites = 4 * nw; t->sites = sites;
  t->ncharges = 3 * nw; t->charges = charges; t->charge_site = charge_site;
  t->ndipoles = 3 * nw; t->dipoles = dipoles; t->dipole_site = dipole_site;
  t->nsto = 4 * nw; t->sto = sto; t->sto_site = sto_site;
  t->npol = nw; t->pol_alpha = pol_alpha; t->pol_site = pol_site;
  t->charge_damp = 1.7724; t->dipole_damp = 1.7724; t->pol_damp = 2.536;
}

static inline double or_reff(double r, double r0) {
  /* Effective-distance damping, DampType 2 (src/Potential.cpp:1192-1196). */
  if (r < r0) {
    const double q = r / r0;
    return r0 * (0.5 + q * q * q * (1.0 - 0.5 * q));
  }
  return r;
}

void or_potential_dpp(const int n[3], const double* const x[3], const or_dpp_tables* t, double* v, double* v_pc,
                      double* v_ind, double* v_rep, double* v_pol) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const int ns = t->nsites;
#pragma omp parallel
  {
    double* rx = malloc(sizeof(double) * ns);
    double* ry = malloc(sizeof(double) * ns);
    double* rz = malloc(sizeof(double) * ns);
    double* r2 = malloc(sizeof(double) * ns);
    double* r = malloc(sizeof(double) * ns);
    double* rm3 = malloc(sizeof(double) * ns);
#pragma omp for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double p[3] = {x[0][i], x[1][j], x[2][k]};
          /* Distance table (src/Potential.cpp:136-146). */
          for (int s = 0; s < ns; ++s) {
            rx[s] = p[0] - t->sites[3 * s + 0];
            ry[s] = p[1] - t->sites[3 * s + 1];
            rz[s] = p[2] - t->sites[3 * s + 2];
            r2[s] = rx[s] * rx[s] + ry[s] * ry[s] + rz[s] * rz[s];
            r[s] = sqrt(r2[s]);
            rm3[s] = 1.0 / (r2[s] * r[s]);
          }
          double vpc = 0; /* charges, src/Potential.cpp:1188-1204 */
          for (int c = 0; c < t->ncharges; ++c) {
            const double reff = or_reff(r[t->charge_site[c]], t->charge_damp);
            vpc += -t->charges[c] / reff;
          }
          double vind = 0; /* dipoles, :1246-1262 */
          for (int d = 0; d < t->ndipoles; ++d) {
            const int s = t->dipole_site[d];
            double m3 = rm3[s];
            if (r[s] < t->dipole_damp) {
              const double reff = or_reff(r[s], t->dipole_damp);
              m3 = 1.0 / (reff * reff * reff);
            }
            const double* mu = t->dipoles + 3 * d;
            vind += -(rx[s] * mu[0] + ry[s] * mu[1] + rz[s] * mu[2]) * m3;
          }
          double vrep = 0; /* Slater repulsive core, :1301-1308 */
          for (int g = 0; g < t->nsto; ++g) vrep += t->sto[2 * g + 1] * exp(-t->sto[2 * g] * r[t->sto_site[g]]);
          double spol = 0; /* polarisable sites, :1350-1366 */
          for (int q = 0; q < t->npol; ++q) {
            const int s = t->pol_site[q];
            const double a = t->pol_alpha[q];
            if (r[s] < t->pol_damp) {
              const double reff = or_reff(r[s], t->pol_damp);
              const double re2 = reff * reff;
              spol += a * r2[s] / (re2 * re2 * re2);
            } else {
              spol += a / (r2[s] * r2[s]);
            }
          }
          const double vpol = spol * -0.5; /* first-order adiabatic form, :884 */
          const long gidx = i + (long)nx * (j + (long)ny * k);
          v[gidx] = vpc + vind + vrep + vpol;
          if (v_pc) v_pc[gidx] = vpc;
          if (v_ind) v_ind[gidx] = vind;
          if (v_rep) v_rep[gidx] = vrep;
          if (v_pol) v_pol[gidx] = vpol;
        }
    free(rx); free(ry); free(rz); free(r2); free(r); free(rm3);
  }
}

void or_potential_ions_add(const int n[3], const double* const x[3], int nions, const double* pos, const double* q,
                           double r_cation, double r_anion, double* v) {
  /* EvaluateBloomfield (src/NaCl.cpp:285-318): -q erf(R/r_ion)/R, the damping
   * radius chosen by the sign of the charge (:262-266). */
  const double dc = 1.0 / r_cation, da = 1.0 / r_anion;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        double acc = 0;
        for (int s = 0; s < nions; ++s) {
          const double rx = x[0][i] - pos[3 * s], ry = x[1][j] - pos[3 * s + 1], rz = x[2][k] - pos[3 * s + 2];
          const double r = sqrt(rx * rx + ry * ry + rz * rz);
          const double damp = q[s] > 0 ? dc : da;
          acc += -q[s] * erf(damp * r) / r;
        }
        v[i + (long)n[0] * (j + (long)n[1] * k)] += acc;
      }
}

void or_potential_spherical(const int n[3], const double* const x[3], double k, double* v) {
  for (int c = 0; c < n[2]; ++c)
    for (int b = 0; b < n[1]; ++b)
      for (int a = 0; a < n[0]; ++a) {
        const double d = sqrt(x[0][a] * x[0][a] + x[1][b] * x[1][b] + x[2][c] * x[2][c]);
        v[a + (long)n[0] * (b + (long)n[1] * c)] = 0.5 * k * d * d;
      }
}

/* ---------------------------------------------------------- small linalg */

/* Dot product over 64 fixed blocks summed in order: the same bits for any
 * thread count (an OpenMP reduction combines its partial sums in an
 * unspecified order). */
#define OR_DOT_BLOCKS 64
static double or_dot(long n, const double* a, const double* b) {
  double part[OR_DOT_BLOCKS];
  const long chunk = (n + OR_DOT_BLOCKS - 1) / OR_DOT_BLOCKS;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < OR_DOT_BLOCKS; ++k) {
    const long b0 = (long)k * chunk, b1 = b0 + chunk < n ? b0 + chunk : n;
    double s = 0;
    for (long i = b0; i < b1; ++i) s += a[i] * b[i];
    part[k] = s;
  }
  double s = 0;
  for (int k = 0; k < OR_DOT_BLOCKS; ++k) s += part[k];
  return s;
}
static double or_nrm2(long n, const double* a) { return sqrt(or_dot(n, a, a)); }
static void or_scal(long n, double f, double* a) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) a[i] *= f;
}
static void or_axpy(long n, double f, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) y[i] += f * x[i];
}
/* y = A c, A = ncol columns of length n (ld n). */
static void or_gemv(long n, int ncol, const double* A, const double* c, double* y) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    double s = 0;
    for (int j = 0; j < ncol; ++j) s += A[(long)j * n + i] * c[j];
    y[i] = s;
  }
}

int or_syev(int n, double* a, int lda, double* w, double* v, int ldv) {
  /* Cyclic Jacobi on the upper triangle (the part dsyev("V","U") reads). */
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) a[i + (long)j * lda] = a[j + (long)i * lda];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) v[i + (long)j * ldv] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double e = a[i + (long)j * lda] * a[i + (long)j * lda];
        tot += e;
        if (i != j) off += e;
      }
    if (off <= 1e-30 * tot || off == 0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p + (long)q * lda];
        if (apq == 0) continue;
        const double app = a[p + (long)p * lda], aqq = a[q + (long)q * lda];
        const double th = (aqq - app) / (2 * apq);
        const double tt = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
        const double c = 1 / sqrt(tt * tt + 1), s = tt * c;
        for (int k = 0; k < n; ++k) { /* columns p, q */
          const double akp = a[k + (long)p * lda], akq = a[k + (long)q * lda];
          a[k + (long)p * lda] = c * akp - s * akq;
          a[k + (long)q * lda] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) { /* rows p, q */
          const double apk = a[p + (long)k * lda], aqk = a[q + (long)k * lda];
          a[p + (long)k * lda] = c * apk - s * aqk;
          a[q + (long)k * lda] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[k + (long)p * ldv], vkq = v[k + (long)q * ldv];
          v[k + (long)p * ldv] = c * vkp - s * vkq;
          v[k + (long)q * ldv] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = a[i + (long)i * lda];
  /* ascending order, like dsyev */
  for (int i = 0; i < n - 1; ++i) {
    int m = i;
    for (int j = i + 1; j < n; ++j)
      if (w[j] < w[m]) m = j;
    if (m != i) {
      const double tw = w[i]; w[i] = w[m]; w[m] = tw;
      for (int k = 0; k < n; ++k) {
        const double tv = v[k + (long)i * ldv]; v[k + (long)i * ldv] = v[k + (long)m * ldv]; v[k + (long)m * ldv] = tv;
      }
    }
  }
  return 0;
}

/* -------------------------------------------------------------- Davidson */

struct or_davidson_state {
  int status, jmacro, nsub, nnewB, nnewZ;
  double thresh;
  double *residuals, *conv_w;
  int *ccode, *bindex;
  int cap;
};

or_davidson_state* or_davidson_create(void) { return (or_davidson_state*)calloc(1, sizeof(or_davidson_state)); }
void or_davidson_destroy(or_davidson_state* s) {
  if (!s) return;
  free(s->residuals); free(s->conv_w); free(s->ccode); free(s->bindex); free(s);
}

long or_davidson_work_size(int ndim, int maxsub, int nroots, int corrflag) {
  /* src/Davidson.cpp:46-52 */
  if (corrflag == 2) return 2L * maxsub * maxsub + 11L * maxsub + (2L * nroots + 1) * ndim;
  return 2L * maxsub * maxsub + 11L * maxsub + 2L * nroots * ndim;
}

/* Orthonormalise vec against nbas vectors of B, each twice, renormalising
 * after every step (OrthoVecOnB, src/Davidson.cpp:447-474). */
static void or_ortho_on_b(long n, int nbas, double* vec, const double* B) {
  if (nbas == 0) return;
  or_scal(n, 1.0 / or_nrm2(n, vec), vec);
  for (int i = 0; i < nbas; ++i)
    for (int rep = 0; rep < 2; ++rep) {
      const double ovl = -or_dot(n, vec, B + (long)i * n);
      or_axpy(n, ovl, B + (long)i * n, vec);
      or_scal(n, 1.0 / or_nrm2(n, vec), vec);
    }
}

/* GramSchmidt of the start vectors (src/Davidson.cpp:482-514). */
static void or_gram_schmidt(long n, int nvec, double* vec) {
  for (int i = 0; i < nvec; ++i) {
    double* vi = vec + (long)i * n;
    or_scal(n, 1.0 / or_nrm2(n, vi), vi);
    for (int j = 0; j < i; ++j)
      for (int rep = 0; rep < 2; ++rep) {
        const double ovl = -or_dot(n, vi, vec + (long)j * n);
        or_axpy(n, ovl, vec + (long)j * n, vi);
        or_scal(n, 1.0 / or_nrm2(n, vi), vi);
      }
  }
}

int or_davidson(or_davidson_state* st, int ndim, int maxsub, int nroots, int maxmacro, int tol, int corrflag,
                double* evals, int* nconv, double* B, double* Z, const double* diag, double* work, int* inout) {
  const long N = ndim;
  /* davwork layout (src/Davidson.cpp:181-187). */
  double* S = work;
  double* V = S + (long)maxsub * maxsub;
  double* Wk = V + (long)maxsub * maxsub;
  double* sse = Wk + 10L * maxsub;
  double* ritz = sse + maxsub;
  double* res = ritz + N * nroots;
  double* jd = res + N * nroots;

  if (st->status == 0) { /* first call: src/Davidson.cpp:145-193 */
    st->jmacro = 1; st->nsub = 0; st->nnewB = nroots;
    st->thresh = pow(10.0, -tol);
    if (st->cap < nroots) {
      free(st->residuals); free(st->conv_w); free(st->ccode); free(st->bindex);
      st->residuals = malloc(sizeof(double) * nroots); st->conv_w = malloc(sizeof(double) * nroots);
      st->ccode = malloc(sizeof(int) * nroots); st->bindex = malloc(sizeof(int) * nroots);
      st->cap = nroots;
    }
    if (corrflag < 0 || corrflag > 2) corrflag = 1;
    or_gram_schmidt(N, nroots, B);
    st->status = 1;
  }

  for (;;) {
    if (st->nnewB > 0) { /* hand the new block to the caller (:209-217) */
      inout[0] = st->nsub; inout[1] = st->nsub; inout[2] = st->nnewB;
      st->nnewZ = st->nnewB; st->nnewB = 0;
      return 1;
    }
    /* S = Z^T B over the whole subspace (ComputeS, :385-393) and its eigenpairs (:220-226). */
    const int m = st->nsub + st->nnewZ;
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) S[i + (long)j * maxsub] = or_dot(N, Z + (long)i * N, B + (long)j * N);
    st->nsub = m;
    {
      double* a = malloc(sizeof(double) * (long)maxsub * maxsub);
      memcpy(a, S, sizeof(double) * (long)maxsub * maxsub);
      or_syev(m, a, maxsub, sse, V, maxsub);
      free(a);
    }
    /* overlap of each root with the converged space (:229-237) */
    for (int r = 0; r < nroots; ++r) {
      if (*nconv > 0) {
        double s = 0;
        for (int c = 0; c < *nconv; ++c) s += V[c + (long)r * maxsub] * V[c + (long)r * maxsub];
        st->conv_w[r] = sqrt(s);
      } else {
        st->conv_w[r] = 0;
      }
    }
    /* Ritz vectors u = B v, renormalised (:240-246) */
    for (int r = 0; r < nroots; ++r) {
      double* u = ritz + (long)r * N;
      or_gemv(N, m, B, V + (long)r * maxsub, u);
      or_scal(N, 1.0 / or_nrm2(N, u), u);
    }
    /* residuals r = Z v - lambda u (:251-269) */
    for (int r = 0; r < nroots; ++r) {
      double* rv = res + (long)r * N;
      or_gemv(N, m, Z, V + (long)r * maxsub, rv);
      or_axpy(N, -sse[r], ritz + (long)r * N, rv);
      st->residuals[r] = or_nrm2(N, rv);
    }
    if (getenv("ORACLE_TRACE")) { /* iteration trace, as the reference prints at verbose > 1 (:262-267) */
      fprintf(stderr, "%3d", m);
      for (int r = 0; r < nroots; ++r) fprintf(stderr, "  %16.12f %10.3e", sse[r], st->residuals[r]);
      fprintf(stderr, "  nconv=%d\n", *nconv);
    }
    /* convergence and locking (:272-297) */
    int newly = 0;
    for (int r = 0; r < nroots; ++r) {
      if (st->conv_w[r] > 0.95) {
        st->ccode[r] = 0;
      } else if (st->residuals[r] < st->thresh) {
        if (*nconv >= maxsub) { /* the reference's copy would land past B's maxsub columns */
          st->status = 0;
          return -2;
        }
        st->ccode[r] = 1;
        st->bindex[r] = *nconv;
        memcpy(B + (long)(*nconv) * N, ritz + (long)r * N, sizeof(double) * N);
        *nconv += 1;
        newly += 1;
      } else {
        st->ccode[r] = 2;
      }
    }
    /* Inside a near-degenerate set every root's overlap with the locked space
     * can stay below 0.95, and the same state is locked again, so nconv can
     * pass nroots.  The reference then keeps nconv + (unconverged roots) >
     * nroots vectors: its restart writes the extra Z combinations past the
     * nroots Ritz slots, into the residual (and JD) slots that follow them in
     * the work array (src/Davidson.cpp:181-187, 303-346), and later locks copy
     * Ritz vectors to B[nconv] whatever nconv is (:279-284).  The oracle does
     * the same while those writes stay inside the work array and B; where the
     * reference's would leave them it stops with -2. */
    {
      int kept = *nconv;
      for (int r = 0; r < nroots; ++r) kept += st->ccode[r] == 2;
      const int slots = 2 * nroots + (corrflag == 2 ? 1 : 0); /* N-vectors from ritz to the end of work */
      if (kept > slots || kept > maxsub) {
        st->status = 0;
        return -2;
      }
    }
    if (*nconv == nroots) {
      memcpy(evals, sse, sizeof(double) * nroots);
      memcpy(B, ritz, sizeof(double) * N * nroots);
      st->status = 0;
      return 0;
    }
    /* restart on a full subspace or on new convergence (:303-346) */
    if (st->nsub == maxsub || newly > 0) {
      st->nnewB = 0;
      for (int r = 0; r < nroots; ++r)
        if (st->ccode[r] == 2) {
          memcpy(B + (long)(st->nnewB + *nconv) * N, ritz + (long)r * N, sizeof(double) * N);
          st->bindex[r] = *nconv + st->nnewB;
          st->nnewB += 1;
        }
      /* Z for the kept vectors, built in the Ritz block and copied as one block */
      for (int r = 0; r < nroots; ++r)
        if (st->ccode[r] > 0) {
          const int jz = st->bindex[r];
          or_gemv(N, st->nsub, Z, V + (long)r * maxsub, ritz + (long)jz * N);
        }
      const long cnt = (long)(st->nnewB + newly) * N;
      memcpy(Z + (long)(*nconv - newly) * N, ritz + (long)(*nconv - newly) * N, sizeof(double) * cnt);
      st->nsub = nroots;
      st->jmacro += 1;
      if (st->jmacro >= maxmacro) return 0; /* the reference leaves its status set here */
    }
    /* correction vectors (:353-371) */
    st->nnewB = 0;
    for (int r = 0; r < nroots; ++r) {
      if (st->nsub + st->nnewB == maxsub) break;
      if (st->ccode[r] < 2) continue;
      double* rv = res + (long)r * N;
      if (corrflag == 1) {
        /* DavidsonCorrectionVector (:557-566) */
#pragma omp parallel for schedule(static)
        for (long k = 0; k < N; ++k) {
          double dv = sse[r] - diag[k];
          if (fabs(dv) < 1e-12) dv = 1e-12;
          rv[k] /= dv;
        }
      } else if (corrflag == 2) {
        /* DavidsonJacobiCorrectionVector (:530-549) */
        const double* u = ritz + (long)r * N;
#pragma omp parallel for schedule(static)
        for (long k = 0; k < N; ++k) {
          double mk = diag[k] - sse[r];
          if (fabs(mk) < 1e-12) mk = 1e-12;
          mk = 1.0 / mk;
          rv[k] *= -mk;
          jd[k] = mk * u[k];
        }
        const double f = or_dot(N, u, rv) / or_dot(N, u, jd);
        or_axpy(N, f, jd, rv);
      }
      or_ortho_on_b(N, st->nsub + st->nnewB, rv, B);
      memcpy(B + (long)(st->nsub + st->nnewB) * N, rv, sizeof(double) * N);
      st->nnewB += 1;
    }
  }
}

int or_solve(const int n[3], const double* const tp[3], const double* const x[3], const double* v, int nstates,
             int maxsub, int maxiter, int ptol, int corrflag, int startvec, double* evals, double* B,
             long* n_matvec, long max_matvec) {
  const long N = (long)n[0] * n[1] * n[2];
  /* start vectors (src/DVR.cpp:405-453) */
  srand(1);
  int istart = 0;
  if (startvec == 1) { or_piab_start(n, x, B); istart = 1; }
  for (int s = istart; s < nstates; ++s) or_random_start((int)N, B + (long)s * N);
  double* Z = malloc(sizeof(double) * N * maxsub);
  double* diag = malloc(sizeof(double) * N);
  double* work = malloc(sizeof(double) * or_davidson_work_size((int)N, maxsub, nstates, corrflag));
  or_diagonal(n, tp, v, diag);
  or_davidson_state* st = or_davidson_create();
  int inout[3] = {0, 0, 0}, nconv = 0, ido = 1;
  long nmv = 0;
  int stopped = 0;
  while (ido != 0) { /* src/davdriver.cpp:58-86 */
    ido = or_davidson(st, (int)N, maxsub, nstates, maxiter, ptol, corrflag, evals, &nconv, B, Z, diag, work, inout);
    if (ido < 0) { stopped = ido; break; }
    if (ido == 1) {
      for (int k = 0; k < inout[2]; ++k) {
        or_matvec(n, tp, v, B + (long)(inout[0] + k) * N, Z + (long)(inout[1] + k) * N);
        ++nmv;
      }
      if (max_matvec > 0 && nmv >= max_matvec) { stopped = 1; break; }
    }
  }
  or_davidson_destroy(st);
  free(Z); free(diag); free(work);
  if (n_matvec) *n_matvec = nmv;
  return stopped == 1 ? -1 : stopped < 0 ? stopped : nconv;
}

/* ---------------------------------------------------------------- observables */

/* DVR::ExpectationValues (src/DVR.cpp:2329-2449): for each state the sums
 * over the grid of psi^2, psi^2 x, psi^2 y, psi^2 z, psi^2 r^2, and for
 * states n >= 1 psi_n x psi_0 (and y, z), in the reference's loop order
 * (x slowest, z fastest).  out[8*s + m]. */
void or_expectation_values(const int n[3], const double* const xg[3], const double* wf, int nstates, double* out) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const long ngp = (long)nx * ny * nz;
  for (int m = 0; m < 8 * nstates; ++m) out[m] = 0.0;
  for (int ix = 0; ix < nx; ++ix)
    for (int iy = 0; iy < ny; ++iy)
      for (int iz = 0; iz < nz; ++iz) {
        const long idx = ix + (long)nx * (iy + (long)ny * iz);
        const double x = xg[0][ix], y = xg[1][iy], z = xg[2][iz];
        for (int s = 0; s < nstates; ++s) {
          const double w = wf[s * ngp + idx], rho = w * w;
          double* o = out + 8 * s;
          o[0] += rho;
          o[1] += rho * x;
          o[2] += rho * y;
          o[3] += rho * z;
          o[4] += rho * (x * x + y * y + z * z);
          if (s > 0) {
            const double w0 = wf[idx];
            o[5] += w * x * w0;
            o[6] += w * y * w0;
            o[7] += w * z * w0;
          }
        }
      }
}

/* DVR::EnergyPartitioning (src/DVR.cpp:2240-2325): sums of psi^2 times the
 * four potential parts (charges, induced dipoles, repulsion, polarisation),
 * in the reference's loop order.  parts[c*ngp + g]; out[4*s + c]. */
void or_energy_partition(const int n[3], const double* wf, int nstates, const double* parts, double* out) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const long ngp = (long)nx * ny * nz;
  for (int m = 0; m < 4 * nstates; ++m) out[m] = 0.0;
  for (int ix = 0; ix < nx; ++ix)
    for (int iy = 0; iy < ny; ++iy)
      for (int iz = 0; iz < nz; ++iz) {
        const long idx = ix + (long)nx * (iy + (long)ny * iz);
        for (int s = 0; s < nstates; ++s) {
          const double w = wf[s * ngp + idx], rho = w * w;
          for (int c = 0; c < 4; ++c) out[4 * s + c] += rho * parts[c * ngp + idx];
        }
      }
}

/* Small2Large, eight-point branch (src/Small2Large.cpp:135-219): the small
 * grid in cube order (z fastest), the large grid XMIN + I DX with x fastest,
 * normalised so that the sum of squares is 1 (summed in the large grid's
 * order). */
void or_small_to_large(const int n[3], const double xmin[3], const double dx[3], const double* wf, const int N[3],
                       const double XMIN[3], const double DX[3], double* WF) {
  const long xs = (long)n[1] * n[2], ys = n[2];
  double nrm = 0.0;
  long c = 0;
  for (int IZ = 0; IZ < N[2]; ++IZ) {
    const double Z = XMIN[2] + IZ * DX[2];
    int iz = (int)((Z - xmin[2]) / dx[2]), izu;
    if (iz < 0) { iz = 0; izu = 1; }
    else if (iz > n[2] - 2) { iz = n[2] - 2; izu = n[2] - 1; }
    else izu = iz + 1;
    const double wz = (Z - (xmin[2] + iz * dx[2])) / dx[2];
    for (int IY = 0; IY < N[1]; ++IY) {
      const double Y = XMIN[1] + IY * DX[1];
      int iy = (int)((Y - xmin[1]) / dx[1]), iyu;
      if (iy < 0) { iy = 0; iyu = 1; }
      else if (iy > n[1] - 2) { iy = n[1] - 2; iyu = n[1] - 1; }
      else iyu = iy + 1;
      const double wy = (Y - (xmin[1] + iy * dx[1])) / dx[1];
      for (int IX = 0; IX < N[0]; ++IX) {
        const double X = XMIN[0] + IX * DX[0];
        int ix = (int)((X - xmin[0]) / dx[0]), ixu;
        if (ix < 0) { ix = 0; ixu = 1; }
        else if (ix > n[0] - 2) { ix = n[0] - 2; ixu = n[0] - 1; }
        else ixu = ix + 1;
        const double wx = (X - (xmin[0] + ix * dx[0])) / dx[0];
        double sum = 0, w, v;
        w = (1 - wx) * (1 - wy) * (1 - wz); sum += w; v = wf[ix * xs + iy * ys + iz] * w;
        w = wx * (1 - wy) * (1 - wz); sum += w; v += wf[ixu * xs + iy * ys + iz] * w;
        w = (1 - wx) * wy * (1 - wz); sum += w; v += wf[ix * xs + iyu * ys + iz] * w;
        w = (1 - wx) * (1 - wy) * wz; sum += w; v += wf[ix * xs + iy * ys + izu] * w;
        w = wx * wy * (1 - wz); sum += w; v += wf[ixu * xs + iyu * ys + iz] * w;
        w = wx * (1 - wy) * wz; sum += w; v += wf[ixu * xs + iy * ys + izu] * w;
        w = (1 - wx) * wy * wz; sum += w; v += wf[ix * xs + iyu * ys + izu] * w;
        w = wx * wy * wz; sum += w; v += wf[ixu * xs + iyu * ys + izu] * w;
        v /= sum;
        WF[c++] = v;
        nrm += v * v;
      }
    }
  }
  nrm = 1.0 / sqrt(nrm);
  for (long k = 0; k < c; ++k) WF[k] *= nrm;
}

/* ------------------------------------------------------------------------ */
/* Self-consistent polarisation and the Hellmann-Feynman gradient.          */

/* BuildPolarizationMatrix + CalcDDTensor (src/MolPolAux.cpp:100-136,
 * 311-336), then the inverse column by column from an LU factorisation with
 * partial pivoting (the reference inverts with LAPACK dsytrf/dsytri,
 * src/MolPolAux.cpp:264-293; any exact inverse agrees to round-off). */
int or_scpol_inva(int npp, const double* pos, const double* alpha, double a_thole, double* inva) {
  const int n = 3 * npp;
  double* a = calloc((size_t)n * n, sizeof(double));
  int* piv = malloc(sizeof(int) * n);
  for (int i = 0; i < npp; ++i)
    for (int c = 0; c < 3; ++c) a[(size_t)(3 * i + c) * n + 3 * i + c] = 1.0 / alpha[i];
  for (int i = 0; i < npp; ++i)
    for (int j = i + 1; j < npp; ++j) {
      const double r[3] = {pos[3 * i] - pos[3 * j], pos[3 * i + 1] - pos[3 * j + 1], pos[3 * i + 2] - pos[3 * j + 2]};
      const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2], rr = sqrt(r2);
      const double r3 = rr * r2, r5 = r2 * r3;
      const double te = a_thole * r3 / sqrt(alpha[i] * alpha[j]);
      const double tf = exp(-te);
      const double f3 = 1 - tf, f5 = 1 - (1 + te) * tf;
      const double c1 = f5 * 3.0 / r5, c2 = f3 / r3;
      for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q) {
          const double t = c1 * r[p] * r[q] - (p == q ? c2 : 0.0);
          a[(size_t)(3 * j + p) * n + 3 * i + q] = a[(size_t)(3 * i + p) * n + 3 * j + q] = -t;
        }
    }
  /* LU = P A (Doolittle, row pivoting) */
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (fabs(a[(size_t)i * n + k]) > fabs(a[(size_t)p * n + k])) p = i;
    piv[k] = p;
    if (a[(size_t)p * n + k] == 0) { free(a); free(piv); return -1; }
    if (p != k)
      for (int j = 0; j < n; ++j) { double t = a[(size_t)k * n + j]; a[(size_t)k * n + j] = a[(size_t)p * n + j]; a[(size_t)p * n + j] = t; }
    for (int i = k + 1; i < n; ++i) {
      const double l = a[(size_t)i * n + k] / a[(size_t)k * n + k];
      a[(size_t)i * n + k] = l;
      for (int j = k + 1; j < n; ++j) a[(size_t)i * n + j] -= l * a[(size_t)k * n + j];
    }
  }
#pragma omp parallel for schedule(static)
  for (int col = 0; col < n; ++col) {
    double* y = malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) y[i] = 0.0;
    /* e_col permuted */
    int src = col;
    double* e = calloc(n, sizeof(double));
    e[src] = 1.0;
    for (int k = 0; k < n; ++k) { const double t = e[k]; e[k] = e[piv[k]]; e[piv[k]] = t; }
    for (int i = 0; i < n; ++i) {
      double s = e[i];
      for (int j = 0; j < i; ++j) s -= a[(size_t)i * n + j] * y[j];
      y[i] = s;
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = y[i];
      for (int j = i + 1; j < n; ++j) s -= a[(size_t)i * n + j] * y[j];
      y[i] = s / a[(size_t)i * n + i];
    }
    for (int i = 0; i < n; ++i) inva[(size_t)i * n + col] = y[i];
    free(y); free(e);
  }
  free(a); free(piv);
  return 0;
}

/* Damped field of the electron at r on every polarisable atom plus Epc
 * (src/Potential.cpp:1518-1552). */
static void scpol_field(const double r[3], int npp, const double* pos, const double* epc, int damp_type, double damp,
                        double* E) {
  for (int i = 0; i < npp; ++i) {
    const double rx = r[0] - pos[3 * i], ry = r[1] - pos[3 * i + 1], rz = r[2] - pos[3 * i + 2];
    const double r2 = rx * rx + ry * ry + rz * rz, R = sqrt(r2);
    double g = 1.0 / (r2 * R);
    if (damp_type == 1) {
      g *= 1.0 - exp(-damp * R * r2);
    } else if (R < damp) {
      const double q = R / damp;
      const double reff = damp * (0.5 + q * q * q * (1.0 - 0.5 * q));
      g = 1.0 / (reff * reff * reff);
    }
    E[3 * i] = g * rx + epc[3 * i];
    E[3 * i + 1] = g * ry + epc[3 * i + 1];
    E[3 * i + 2] = g * rz + epc[3 * i + 2];
  }
}

void or_potential_scpol_add(const int n[3], const double* const x[3], int npp, const double* pos, const double* inva,
                            const double* epc, int damp_type, double damp, double vww, double* v) {
  const int m = 3 * npp;
  const long N = (long)n[0] * n[1] * n[2];
#pragma omp parallel
  {
    double* E = malloc(sizeof(double) * m);
#pragma omp for schedule(static)
    for (long g = 0; g < N; ++g) {
      const int ix = (int)(g % n[0]), iy = (int)((g / n[0]) % n[1]), iz = (int)(g / ((long)n[0] * n[1]));
      const double r[3] = {x[0][ix], x[1][iy], x[2][iz]};
      scpol_field(r, npp, pos, epc, damp_type, damp, E);
      double e = 0.0;
      for (int i = 0; i < m; ++i) {
        double mu = 0.0;
        for (int j = 0; j < m; ++j) mu += inva[(size_t)i * m + j] * E[j];
        e += E[i] * mu;
      }
      v[g] += -0.5 * e - vww;
    }
    free(E);
  }
}

void or_hf_gradient_grid(const int n[3], const double* const x[3], int nsites, const double* sites, int ncharges,
                         const double* charges, const int* charge_site, double charge_damp, int nsto,
                         const double* sto, const int* sto_site, int npp, const int* pol_site, const double* inva,
                         const double* epc, double pol_damp, const double* psi, double* grad, double* tmu,
                         double* mcm) {
  const int m = 3 * npp;
  const long N = (long)n[0] * n[1] * n[2];
  double* pos = malloc(sizeof(double) * m);
  for (int i = 0; i < npp; ++i)
    for (int c = 0; c < 3; ++c) pos[3 * i + c] = sites[3 * pol_site[i] + c];
  for (int k = 0; k < 3 * nsites; ++k) grad[k] = 0.0;
  for (int k = 0; k < m; ++k) tmu[k] = 0.0;
  for (long k = 0; k < (long)m * m; ++k) mcm[k] = 0.0;
  /* serial over points: the sums are the checker's, in grid order */
  double *E = malloc(sizeof(double) * m), *mu = malloc(sizeof(double) * m);
  double *Rx = malloc(sizeof(double) * nsites), *Ry = malloc(sizeof(double) * nsites),
         *Rz = malloc(sizeof(double) * nsites), *R = malloc(sizeof(double) * nsites),
         *tg = malloc(sizeof(double) * 3 * nsites);
  for (long g = 0; g < N; ++g) {
    const double w = psi[g] * psi[g];
    if (w == 0.0) continue; /* contributes nothing; lets tests use sparse densities on large grids */
    const int ix = (int)(g % n[0]), iy = (int)((g / n[0]) % n[1]), iz = (int)(g / ((long)n[0] * n[1]));
    const double r[3] = {x[0][ix], x[1][iy], x[2][iz]};
    for (int s = 0; s < nsites; ++s) {
      Rx[s] = r[0] - sites[3 * s];
      Ry[s] = r[1] - sites[3 * s + 1];
      Rz[s] = r[2] - sites[3 * s + 2];
      R[s] = sqrt(Rx[s] * Rx[s] + Ry[s] * Ry[s] + Rz[s] * Rz[s]);
    }
    for (int k = 0; k < 3 * nsites; ++k) tg[k] = 0.0;
    /* charges (src/Gradients.cpp:88-107) */
    for (int e = 0; e < ncharges; ++e) {
      const int s = charge_site[e];
      double vg;
      if (R[s] < charge_damp) {
        const double q = R[s] / charge_damp;
        const double reff = charge_damp * (0.5 + q * q * q * (1.0 - 0.5 * q));
        vg = charges[e] * (3.0 * q * q - 2.0 * q * q * q) / (reff * reff);
      } else {
        vg = charges[e] / (R[s] * R[s]);
      }
      tg[3 * s] += -vg * Rx[s] / R[s];
      tg[3 * s + 1] += -vg * Ry[s] / R[s];
      tg[3 * s + 2] += -vg * Rz[s] / R[s];
    }
    /* Slater repulsive cores (src/Gradients.cpp:110-116) */
    for (int e = 0; e < nsto; ++e) {
      const int s = sto_site[e];
      const double d = sto[2 * e + 1] * (-sto[2 * e]) * exp(-sto[2 * e] * R[s]);
      tg[3 * s] += -d * Rx[s] / R[s];
      tg[3 * s + 1] += -d * Ry[s] / R[s];
      tg[3 * s + 2] += -d * Rz[s] / R[s];
    }
    /* dipoles mu = A E (src/Gradients.cpp:125-152) */
    scpol_field(r, npp, pos, epc, 2, pol_damp, E);
    for (int i = 0; i < m; ++i) {
      double t = 0.0;
      for (int j = 0; j < m; ++j) t += inva[(size_t)i * m + j] * E[j];
      mu[i] = t;
    }
    /* DerivElecField (src/Gradients.cpp:164-228) */
    for (int i = 0; i < npp; ++i) {
      const int s = pol_site[i];
      const double Rs = R[s];
      double gij = 1.0 / (Rs * Rs * Rs);
      double reff = Rs, dg = -3.0 / (reff * reff * reff * reff);
      if (reff < pol_damp) {
        const double q = reff / pol_damp;
        reff = pol_damp * (0.5 + q * q * q * (1.0 - 0.5 * q));
        dg = (3.0 * q * q - 2.0 * q * q * q) * (-3.0 / (reff * reff * reff * reff));
        gij = 1.0 / (reff * reff * reff);
      }
      const double rv[3] = {Rx[s], Ry[s], Rz[s]};
      for (int a = 0; a < 3; ++a) {
        double d = 0.0;
        for (int b = 0; b < 3; ++b) d += (-dg * rv[a] / Rs * rv[b] - (a == b ? gij : 0.0)) * mu[3 * i + b];
        tg[3 * s + a] += -d;
      }
    }
    for (int k = 0; k < 3 * nsites; ++k) grad[k] += w * tg[k];
    /* MuCrossMu (src/Gradients.cpp:231-241) */
    for (int i = 0; i < m; ++i) {
      const double t0 = w * mu[i];
      tmu[i] += t0;
      for (int j = 0; j < m; ++j) mcm[(size_t)i * m + j] += t0 * mu[j];
    }
  }
  free(E); free(mu); free(Rx); free(Ry); free(Rz); free(R); free(tg); free(pos);
}

void or_hf_gradient_final(int nsites, int npp, const double* tmu, const double* mcm, const double* dT_x,
                          const double* dT_y, const double* dT_z, const double* dEfield, const double* pol_grad,
                          double* gradient) {
  const int n3 = 3 * npp, n9 = 9 * npp;
  const double* dT[3] = {dT_x, dT_y, dT_z};
  for (int j = 0; j < nsites; ++j) {
    for (int d = 0; d < 3; ++d) {
      double s = 0.0;
      for (int k = 0; k < n3; ++k) s += dEfield[(size_t)n3 * (3 * j + d) + k] * tmu[k];
      gradient[3 * j + d] -= s;
    }
    if ((j + 1) % 4 != 0) {
      const int aj = 3 * (j / 4) + j % 4;
      for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int k = 0; k < n9; ++k) s += dT[d][(size_t)aj * n9 + k] * mcm[(size_t)aj * n9 + k];
        gradient[3 * j + d] -= s;
      }
    }
  }
  if (pol_grad)
    for (int k = 0; k < 3 * nsites; ++k) gradient[k] -= pol_grad[k];
}

/* ------------------------------------------------------------------------ */
/* Dual grid.                                                               */

/* Interpolated value at coarse position (px, py, pz) (fine steps from the
 * first coarse point), spacing sp, nc coarse points per axis, following
 * DVR::InterpolVtriple / InterpolVdouble (src/DVR.cpp:1240-1444): corners
 * in the reference's order (0,0,0), x, y, z, xy, yz, xz, xyz, products
 * rounded before they are added.  extend: the start-vector form
 * (DVR::ExtendWfThree, src/DVR.cpp:1446-1642), whose table differs in two
 * cases: remainders (2, 0, 1) weigh the corner (x, z + 1) by 1/sqrt(2)
 * instead of 1/sqrt(8) (:1563-1566 against :1329-1332), and remainders
 * (2, 1, 2) weigh the corner x + 1 by 1/sqrt(9) and (x + 1, y + 1) by
 * 1/sqrt(6) (:1610-1615 against :1374-1379). */
static double dual_interp_w(const double* F, int nc, int sp, int px, int py, int pz, int extend) {
  static const int order[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                  {1, 1, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 1}};
  const int P[3] = {px, py, pz};
  int c[3], r[3], nz = 0;
  for (int a = 0; a < 3; ++a) {
    c[a] = P[a] / sp;
    r[a] = P[a] % sp;
    if (r[a]) ++nz;
  }
  const long s1 = nc, s2 = (long)nc * nc;
  if (nz == 0) return F[c[0] + c[1] * s1 + c[2] * s2];
  double sum = 0.0;
  for (int q = 0; q < 8; ++q) {
    const int* o = order[q];
    int used = 1, d2 = 0;
    for (int a = 0; a < 3; ++a) {
      if (o[a] && !r[a]) used = 0;
      if (r[a]) {
        const int dd = o[a] ? sp - r[a] : r[a];
        d2 += dd * dd;
      }
    }
    if (!used) continue;
    const double f = F[(c[0] + o[0]) + (c[1] + o[1]) * s1 + (c[2] + o[2]) * s2];
    if (sp == 2) {
      sum += f;
      continue;
    }
    if (extend && r[0] == 2 && r[1] == 0 && r[2] == 1 && !o[0] && o[2]) d2 = 2;
    if (extend && r[0] == 2 && r[1] == 1 && r[2] == 2 && o[0] && !o[1] && !o[2]) d2 = 9;
    if (extend && r[0] == 2 && r[1] == 1 && r[2] == 2 && o[0] && o[1] && !o[2]) d2 = 6;
    double w;
    if (nz == 1) w = d2 == 1 ? 2.0 / 3.0 : 1.0 / 3.0;
    else if (nz == 2) w = (d2 == 2 ? 0.707107 : d2 == 5 ? 0.447214 : 0.353553) / 1.955087;
    else w = (d2 == 3 ? 0.57735 : d2 == 6 ? 0.408248 : d2 == 9 ? 0.33333 : 0.288675) / 3.09077;
    sum += f * w;
  }
  return sp == 2 ? sum / (double)(1 << nz) : sum;
}

static double dual_interp(const double* F, int nc, int sp, int px, int py, int pz) {
  return dual_interp_w(F, nc, sp, px, py, pz, 0);
}

void or_dual_potential(int n, int nc, const double* const x[3], int nsites, const double* sites, double rtol,
                       const double* v_coarse, const double* v_exact, double* v) {
  const int sp = n % 2 == 1 ? 2 : 3;
  const int checkM = sp == 3 ? n - (nc * 3 / 2 - 1) * 2 : 0;
  long g = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i, ++g) {
        const int px = i - checkM / 2, py = j - checkM / 2, pz = k - checkM / 2;
        double md = 50.0;
        for (int s = 0; s < nsites; ++s) {
          const double rx = x[0][i] - sites[3 * s], ry = x[1][j] - sites[3 * s + 1], rz = x[2][k] - sites[3 * s + 2];
          const double r = sqrt(rx * rx + ry * ry + rz * rz);
          if (md > r) md = r;
        }
        if (sp == 3 && (px < 0 || py < 0 || pz < 0 || px >= n - checkM || py >= n - checkM || pz >= n - checkM)) {
          v[g] = 0.0;
        } else if (md > rtol || (px % sp == 0 && py % sp == 0 && pz % sp == 0)) {
          v[g] = dual_interp(v_coarse, nc, sp, px, py, pz);
        } else {
          v[g] = v_exact[g];
        }
      }
}

void or_dual_extend(int n, int nc, const double* wf_coarse, double* wf) {
  const int sp = n % 2 == 1 ? 2 : 3;
  const int checkM = sp == 3 ? n - (nc * 3 / 2 - 1) * 2 : 0;
  long g = 0, coarse = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i, ++g) {
        const int px = i - checkM / 2, py = j - checkM / 2, pz = k - checkM / 2;
        if (sp == 3 && (px < 0 || py < 0 || pz < 0 || px >= n - checkM || py >= n - checkM || pz >= n - checkM)) {
          wf[g] = 0.0;
        } else if (px % sp == 0 && py % sp == 0 && pz % sp == 0) {
          wf[g] = wf_coarse[coarse++]; /* the coarse points in their own order, as the reference counts them */
        } else {
          wf[g] = dual_interp_w(wf_coarse, nc, sp, px, py, pz, 1);
        }
      }
}
