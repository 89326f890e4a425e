// Rigid-water DPP site producer (host) and the default electron-water model
// tables.  This is the input stage of the eigensolve: it turns water
// coordinates into the charges, self-consistent induced dipoles, repulsive
// cores and polarisable sites that the V(r) kernel sums over.  It is O(n_w^2)
// per SCF sweep for a few hundred sites and stays on the CPU, as it does in
// the reference.
//
// Model constants of the DPP monomer (src/ttm_data.h:8-58, src/Water.cpp:197-243,
// src/constants.h:18-19) and the default electron-model parameters
// (src/GetInput.cpp:43-63, src/Potential.cpp:699-728) are kept identical.
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "pisces_gb300.h"

namespace pg {
void set_error(const char* fmt, ...);
}

namespace {

constexpr double kBohr2Angs = 0.52917720859;
constexpr double kAngs2Bohr = 1 / kBohr2Angs;
constexpr double kPi = 3.14159265358979;  // the reference's constant (src/constants.h:4)
// monomer frame (centre of mass), Angstrom
constexpr double kOz = 0.0650980307, kHz = -0.5207842453, kHy = 0.756950327, kMz = kOz - 0.25;
constexpr double kQH = 0.5742185854046506, kQM = -2 * kQH;
constexpr double kDampCharge = 0.21, kDampDipole = 0.3;  // Thole-like damping of the SCF
const double kPolO = 1.22 * std::pow(kAngs2Bohr, 3), kPolH = 0.28 * std::pow(kAngs2Bohr, 3);

// One rigid monomer: centre of mass, z-y-z Euler angles and its four sites.
struct Monomer {
  double com[3];
  double euler[3];  // phi, theta, psi
  std::array<std::array<double, 3>, 4> site;  // O, H1, H2, M (bohr)

  // Water::ResetPositions + ApplyEuler (src/Water.cpp:850-943): sites of the
  // reference frame placed at the centre, then rotated about it.
  void place() {
    const double ref[4][3] = {{0, 0, kOz * kAngs2Bohr},
                              {0, kHy * kAngs2Bohr, kHz * kAngs2Bohr},
                              {0, kHy * kAngs2Bohr, kHz * kAngs2Bohr},
                              {0, 0, kMz * kAngs2Bohr}};
    for (int s = 0; s < 4; ++s) {
      site[s][0] = com[0] + ref[s][0];
      site[s][1] = s == 2 ? com[1] - ref[s][1] : com[1] + ref[s][1];
      site[s][2] = com[2] + ref[s][2];
    }
    const double c1 = cos(euler[0]), c2 = cos(euler[1]), c3 = cos(euler[2]);
    const double s1 = sin(euler[0]), s2 = sin(euler[1]), s3 = sin(euler[2]);
    const double R[3][3] = {{c1 * c2 * c3 - s1 * s3, -c1 * c2 * s3 - s1 * c3, c1 * s2},
                            {s1 * c2 * c3 + c1 * s3, -s1 * c2 * s3 + c1 * c3, s1 * s2},
                            {-s2 * c3, s2 * s3, c2}};
    for (auto& p : site) {
      const double d[3] = {p[0] - com[0], p[1] - com[1], p[2] - com[2]};
      for (int r = 0; r < 3; ++r) {
        const double rot = R[r][0] * d[0] + R[r][1] * d[1] + R[r][2] * d[2];
        p[r] = rot + com[r];
      }
    }
  }

  // Water::Reposition (src/Water.cpp:695-824): the molecular frame of an
  // O,H,H triple (bohr) -- z along minus the H-H bisector, y in the plane --
  // as Euler angles, and the centre of mass with masses 16,1,1.
  void from_atoms(const double* a) {
    const double* o = a;
    const double h1[3] = {a[3] - o[0], a[4] - o[1], a[5] - o[2]};
    const double h2[3] = {a[6] - o[0], a[7] - o[1], a[8] - o[2]};
    double z[3] = {h1[0] + h2[0], h1[1] + h2[1], h1[2] + h2[2]};
    const double zn = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
    for (double& c : z) c = -(c / zn);
    const double proj = h1[0] * z[0] + h1[1] * z[1] + h1[2] * z[2];
    double y[3] = {h1[0] - proj * z[0], h1[1] - proj * z[1], h1[2] - proj * z[2]};
    const double yn = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    for (double& c : y) c /= yn;
    const double xy = y[2] * z[0] - y[0] * z[2];
    const double xz = y[0] * z[1] - y[1] * z[0];
    const double theta = acos(z[2]);
    const double st = sin(theta);
    double phi, psi;
    if (fabs(st) > 1e-5) {
      double c = -xz / st;
      const double ac = c <= -1 ? kPi : acos(c);
      psi = y[2] >= 0 ? ac : 2 * kPi - ac;
      c = z[0] / st;
      c = c > 1 ? 1 : (c < -1 ? -1 : c);
      phi = z[1] >= 0 ? acos(c) : 2 * kPi - acos(c);
    } else {  // frame axis at a pole
      phi = 0.0;
      psi = xy >= 0 ? acos(y[1]) : 2 * kPi - acos(y[1]);
    }
    for (int c = 0; c < 3; ++c) com[c] = (a[3 + c] + a[6 + c] + 16.0 * a[c]) / 18.0;
    euler[0] = phi;
    euler[1] = theta;
    euler[2] = psi;
    place();
  }
};

// Thole-type damping of charge-dipole and dipole-dipole fields between
// polarisable sites (src/DPP.cpp:1798-1814): x = a (R / (alpha_i alpha_j)^(1/6))^3.
inline double thole_x(double r, double ai, double aj, double a) { return a * pow(r / pow(ai * aj, 1.0 / 6.0), 3); }
inline double damp_cd(double r, double ai, double aj, double a) { return 1.0 - exp(-thole_x(r, ai, aj, a)); }
inline double damp_dd(double r, double ai, double aj, double a) {
  const double x = thole_x(r, ai, aj, a);
  return 1.0 - (1 + x) * exp(-x);
}

// The rigid monomers of a cluster and their damped self-consistent induced
// dipoles (WaterCluster::CalcInducedDipoles, src/DPP.cpp:760-1060): the
// polarisable atoms O, H1, H2 of every water, their polarisabilities, the
// field f1 of the other waters' charges at them and the dipoles mu.
struct Scf {
  std::vector<Monomer> w;
  std::vector<double> alpha, f1, mu;
  int iters = -1;
};

pg_status water_scf(const char* who, int nw, const double* waters, Scf& out) {
  std::vector<Monomer>& w = out.w;
  w.resize(nw);
  for (int i = 0; i < nw; ++i) {
    double b[9];
    for (int c = 0; c < 9; ++c) b[c] = waters[9 * i + c] * kAngs2Bohr;
    if (!std::isfinite(b[0] + b[1] + b[2] + b[3] + b[4] + b[5] + b[6] + b[7] + b[8])) {
      pg::set_error("%s: water %d has a non-finite coordinate", who, i);
      return PG_BAD_ARG;
    }
    w[i].from_atoms(b);
  }
  // Polarisable sites O, H1, H2 of every water; the charged sites H1, H2
  // and M carry a damping polarisability of their own (H: alpha_H, M:
  // alpha_O; src/Water.cpp:229-232).
  const int ns = 3 * nw;
  std::vector<double> pos(3 * (size_t)ns), f2(3 * (size_t)ns), old(3 * (size_t)ns);
  std::vector<double>& alpha = out.alpha;
  std::vector<double>& f1 = out.f1;
  std::vector<double>& mu = out.mu;
  alpha.assign(ns, 0.0);
  f1.assign(3 * (size_t)ns, 0.0);
  mu.assign(3 * (size_t)ns, 0.0);
  for (int j = 0; j < nw; ++j)
    for (int k = 0; k < 3; ++k) {
      for (int c = 0; c < 3; ++c) pos[3 * (3 * j + k) + c] = w[j].site[k][c];
      alpha[3 * j + k] = k == 0 ? kPolO : kPolH;
    }
  // Field of the point charges of other waters (src/DPP.cpp:815-855).
  for (int j = 0; j < nw; ++j)
    for (int k = 1; k < 4; ++k) {
      const double q = k == 3 ? kQM : kQH;
      const double aq = k == 3 ? kPolO : kPolH;
      for (int i = 0; i < ns; ++i) {
        if (i / 3 == j) continue;
        const double rx = pos[3 * i] - w[j].site[k][0], ry = pos[3 * i + 1] - w[j].site[k][1],
                     rz = pos[3 * i + 2] - w[j].site[k][2];
        const double q3 = q * pow(rx * rx + ry * ry + rz * rz, -1.5);
        const double damp = damp_cd(sqrt(rx * rx + ry * ry + rz * rz), alpha[i], aq, kDampCharge);
        f1[3 * i] += q3 * rx * damp;
        f1[3 * i + 1] += q3 * ry * damp;
        f1[3 * i + 2] += q3 * rz * damp;
      }
    }
  // Self-consistent dipoles, mixing 1/2, converged when the mean change is
  // below 1e-12 (src/DPP.cpp:858-868, 948-1033).
  for (int i = 0; i < ns; ++i)
    for (int c = 0; c < 3; ++c) mu[3 * i + c] = 0.5 * alpha[i] * f1[3 * i + c];
  const int maxit = 5 * (ns + 10);
  // The damped dipole field tensors (FieldOfDipole, src/DPP.cpp:2377-2410)
  // depend on the geometry only: computed once, then every SCF sweep is a
  // block matrix-vector product with the same operations in the same order.
  std::vector<double> tens(6 * (size_t)ns * ns, 0.0);
  for (int i = 0; i < ns; ++i)
    for (int j = 0; j < ns; ++j) {
      if (j == i) continue;
      const double rx = pos[3 * i] - pos[3 * j], ry = pos[3 * i + 1] - pos[3 * j + 1],
                   rz = pos[3 * i + 2] - pos[3 * j + 2];
      const double r2 = rx * rx + ry * ry + rz * rz;
      const double r5 = pow(r2, -2.5);
      const double d1 = damp_dd(sqrt(r2), alpha[i], alpha[j], kDampDipole);
      const double d2 = damp_cd(sqrt(r2), alpha[i], alpha[j], kDampDipole);
      double* t = &tens[6 * ((size_t)i * ns + j)];
      t[0] = (d1 * 3. * rx * rx - d2 * r2) * r5;  // xx
      t[1] = (d1 * 3. * ry * ry - d2 * r2) * r5;  // yy
      t[2] = (d1 * 3. * rz * rz - d2 * r2) * r5;  // zz
      t[3] = d1 * 3. * rx * ry * r5;              // xy
      t[4] = d1 * 3. * rx * rz * r5;              // xz
      t[5] = d1 * 3. * ry * rz * r5;              // yz
    }
  for (int it = 0; it < maxit; ++it) {
    std::fill(f2.begin(), f2.end(), 0.0);
    for (int i = 0; i < ns; ++i)
      for (int j = 0; j < ns; ++j) {
        if (j == i) continue;
        const double* t = &tens[6 * ((size_t)i * ns + j)];
        const double* m = &mu[3 * j];
        f2[3 * i] += t[0] * m[0] + t[3] * m[1] + t[4] * m[2];
        f2[3 * i + 1] += t[3] * m[0] + t[1] * m[1] + t[5] * m[2];
        f2[3 * i + 2] += t[4] * m[0] + t[5] * m[1] + t[2] * m[2];
      }
    for (int i = 0; i < ns; ++i)
      for (int c = 0; c < 3; ++c) {
        old[3 * i + c] = mu[3 * i + c];
        mu[3 * i + c] = 0.5 * old[3 * i + c] + 0.5 * alpha[i] * (f1[3 * i + c] + f2[3 * i + c]);
      }
    double change = 0;
    for (int i = 0; i < ns; ++i) {
      const double tx = old[3 * i] - mu[3 * i], ty = old[3 * i + 1] - mu[3 * i + 1], tz = old[3 * i + 2] - mu[3 * i + 2];
      change += tx * tx + ty * ty + tz * tz;
    }
    change = sqrt(change) / 3 / ns;
    if (change < 1e-12) {
      out.iters = it + 1;
      break;
    }
  }
  return PG_OK;
}

}  // namespace

extern "C" pg_status pg_water_sites(int nw, const double* waters, double* sites, double* charges, int* charge_site,
                                    double* dipoles, int* dipole_site, int* scf_iters) {
  if (nw <= 0 || !waters || !sites || !charges || !charge_site || !dipoles || !dipole_site) {
    pg::set_error("pg_water_sites: bad arguments");
    return PG_BAD_ARG;
  }
  Scf scf;
  const pg_status st = water_scf("pg_water_sites", nw, waters, scf);
  if (st != PG_OK) return st;
  // Lists for the electron (GetLists / ReportInducedDipoles, src/DPP.cpp:402-529).
  for (int j = 0; j < nw; ++j) {
    for (int s = 0; s < 4; ++s)
      for (int c = 0; c < 3; ++c) sites[12 * j + 3 * s + c] = scf.w[j].site[s][c];
    for (int k = 0; k < 3; ++k) {
      charges[3 * j + k] = k == 2 ? kQM : kQH;
      charge_site[3 * j + k] = 4 * j + 1 + k;
      dipole_site[3 * j + k] = 4 * j + k;
      for (int c = 0; c < 3; ++c) dipoles[9 * j + 3 * k + c] = scf.mu[3 * (3 * j + k) + c];
    }
  }
  if (scf_iters) *scf_iters = scf.iters;
  return PG_OK;
}

extern "C" pg_status pg_water_scpol(int nw, const double* waters, int* pol_site, double* alpha, double* epc,
                                    double* vpol_ww) {
  if (nw <= 0 || !waters || !pol_site || !alpha || !epc || !vpol_ww) {
    pg::set_error("pg_water_scpol: bad arguments");
    return PG_BAD_ARG;
  }
  Scf scf;
  const pg_status st = water_scf("pg_water_scpol", nw, waters, scf);
  if (st != PG_OK) return st;
  // WaterCluster::ReportPolSitesAndField (src/DPP.cpp:540-640): the field
  // there is the same sum as the SCF's f1.
  for (int j = 0; j < nw; ++j)
    for (int k = 0; k < 3; ++k) {
      pol_site[3 * j + k] = 4 * j + k;
      alpha[3 * j + k] = scf.alpha[3 * j + k];
      for (int c = 0; c < 3; ++c) epc[3 * (3 * j + k) + c] = scf.f1[3 * (3 * j + k) + c];
    }
  // Water-water polarisation energy, summed pair by pair as
  // CalcIntermolecularPotential / WaterWaterPolarizationEnergy
  // (src/DPP.cpp:1648-1691, 1935-2010): each polarisable atom of one water
  // in the damped field of the other water's charges, halved.
  double pol = 0.0;
  for (int a = 0; a < nw - 1; ++a)
    for (int b = a + 1; b < nw; ++b) {
      double e = 0.0;
      for (int k = 0; k < 3; ++k) {
        for (int side = 0; side < 2; ++side) {
          const int w1 = side == 0 ? a : b, w2 = side == 0 ? b : a;
          const double* x1 = scf.w[w1].site[k].data();
          const double* m1 = &scf.mu[3 * (3 * w1 + k)];
          const double al = scf.alpha[3 * w1 + k];
          for (int q = 1; q < 4; ++q) {
            const double qq = q == 3 ? kQM : kQH;
            const double aq = q == 3 ? kPolO : kPolH;
            const double rx = x1[0] - scf.w[w2].site[q][0], ry = x1[1] - scf.w[w2].site[q][1],
                         rz = x1[2] - scf.w[w2].site[q][2];
            const double d = sqrt(rx * rx + ry * ry + rz * rz);
            const double damp = damp_cd(d, al, aq, kDampCharge);
            e -= qq * (m1[0] * rx + m1[1] * ry + m1[2] * rz) * damp * pow(rx * rx + ry * ry + rz * rz, -1.5) / 2.0;
          }
        }
      }
      pol += e;
    }
  *vpol_ww = pol;
  return PG_OK;
}

extern "C" pg_status pg_water_default_tables(int nw, const double* sites, const double* charges,
                                             const int* charge_site, const double* dipoles, const int* dipole_site,
                                             double* sto, int* sto_site, double* pol_alpha, int* pol_site,
                                             pg_sites* out) {
  if (nw <= 0 || !sites || !charges || !charge_site || !dipoles || !dipole_site || !sto || !sto_site || !pol_alpha ||
      !pol_site || !out) {
    pg::set_error("pg_water_default_tables: bad arguments");
    return PG_BAD_ARG;
  }
  // Four Slater repulsive cores per water, coefficients scaled by 1/4.4837
  // (Set4STORepCore, src/Potential.cpp:699-728); one polarisable site of
  // alpha 9.745 on each M site (src/Potential.cpp:326-338).
  const double sig = 1.0 / 4.4837;
  const double zeta[4] = {9.98526, 1.67075, 1.64121, 1.64121};
  const double coef[4] = {192.608, 13.8937, 1.7643, 1.7643};
  const int on[4] = {0, 0, 1, 2};
  for (int i = 0; i < nw; ++i) {
    for (int k = 0; k < 4; ++k) {
      sto[8 * i + 2 * k] = zeta[k];
      sto[8 * i + 2 * k + 1] = coef[k] * sig;
      sto_site[4 * i + k] = 4 * i + on[k];
    }
    pol_alpha[i] = 9.745;
    pol_site[i] = 4 * i + 3;
  }
  std::memset(out, 0, sizeof(*out));
  out->nsites = 4 * nw;
  out->sites = sites;
  out->ncharges = 3 * nw;
  out->charges = charges;
  out->charge_site = charge_site;
  out->ndipoles = 3 * nw;
  out->dipoles = dipoles;
  out->dipole_site = dipole_site;
  out->nsto = 4 * nw;
  out->sto = sto;
  out->sto_site = sto_site;
  out->npol = nw;
  out->pol_alpha = pol_alpha;
  out->pol_site = pol_site;
  out->charge_damp = 1.7724;
  out->dipole_damp = 1.7724;
  out->pol_damp = 2.536;
  return PG_OK;
}
