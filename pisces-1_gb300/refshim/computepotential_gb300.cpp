// DVR::ComputePotential on the GB300 library: a drop-in for the member of
// the same name (DVR.h:63, src/DVR.cpp:661-1059), built into the reference
// in place of that function.  The reference asks Potential::Evaluate for
// every grid point (src/DVR.cpp:751-859); here the site tables the
// Potential was set up with go to pg_potential_eval, which evaluates the
// whole grid on the device, and v_diag and its four parts come back.
//
// Potential keeps its tables private and has no accessors, so this file
// reads them by compiling Potential.h with its members public; the class
// layout is unchanged.  Supported: the electron-water model with STO
// repulsive cores and effective-radius damping (src/GetInput.cpp:43-63),
// with first-order polarisation (PolType 1, the default) or self-consistent
// polarisation (PolType 3: the MolPol[0] tables go to
// pg_potential_scpol_add), or the dual grid's PolType 6 (the coarse V that
// v_diag still holds from the previous call, on the Pre1db grid, goes to
// pg_dual_grid_potential with Rtol; src/DVR.cpp:735-832), and single
// sampling; other models print and exit, as the reference does for what it
// cannot evaluate.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

#define private public
#include "Potential.h"
#undef private
#include "DVR.h"
#include "pisces_gb300.h"

namespace {

void stop(const char* what) {
  std::cout << "ComputePotential (GB300): " << what << "\n";
  exit(1);
}

}  // namespace

void DVR::ComputePotential(class Potential& V) {
  const bool dual = V.PolType == 6;
  const bool sc = V.PolType == 3 || dual;
  if (V.PotFlags.empty() || V.PotFlags[0] != 3 || V.DampType != 2 || (V.PolType != 1 && !sc) ||
      V.AdiabaticPolPot != 0 || V.RepCoreType != 2 || V.nMolPol != (sc ? 1 : 0))
    stop("only the electron-water model with STO cores, DampType 2 and PolType 1, 3 or 6 is supported");
  if (sampling != 1) stop("only single sampling is supported");
  std::vector<int> stosite(V.nGauss), polsite(V.nPPS);
  std::vector<double> alpha(V.nPPS);
  for (int i = 0; i < V.nGauss; ++i) stosite[i] = V.GaussSite[i];
  for (int i = 0; i < V.nPPS; ++i) alpha[i] = V.PPS[2 * i], polsite[i] = V.PPSSite[i];
  pg_sites t;
  t.nsites = V.nSites;
  t.sites = V.Site.data();
  t.ncharges = V.nCharges;
  t.charges = V.Charge.data();
  t.charge_site = V.ChargeSite.data();
  t.ndipoles = V.nDipoles;
  t.dipoles = V.Dipole.data();
  t.dipole_site = V.DipoleSite.data();
  t.nsto = V.nGauss;
  t.sto = V.Gauss.data();
  t.sto_site = stosite.data();
  t.npol = V.nPPS;
  t.pol_alpha = alpha.data();
  t.pol_site = polsite.data();
  t.charge_damp = V.ChargeDamping;
  t.dipole_damp = V.DipoleDamping;
  t.pol_damp = V.PolDamping;
  double L[3] = {gridpara[0], gridpara[1], gridpara[2]};
  pg_grid* g = nullptr;
  if (pg_grid_create_dvr(n_1dbas, L, dvrtype == 3 ? 3 : 2, &g) != PG_OK) stop(pg_last_error());
  double *v = nullptr, *parts = nullptr;
  if (cudaMalloc(&v, sizeof(double) * ngp) != cudaSuccess || cudaMalloc(&parts, 4 * sizeof(double) * ngp) != cudaSuccess)
    stop("cudaMalloc failed");
  if (dual) {
    // PolType 6 has no induced-dipole part (src/Potential.cpp:904-907) and
    // no one-site term; the four parts are not written, as the reference
    // does not write them for this model
    t.ndipoles = 0, t.npol = 0;
    const DistributedPolarizabilities& mp = V.MolPol[0];
    pg_scpol_model m;
    m.npp = mp.nAtoms;
    m.pol_site = mp.SiteList.data();
    m.inva = mp.InvA.data();
    m.epc = mp.Epc.data();
    m.damp_type = V.DampType;
    m.damp = V.PolDamping;
    m.vpol_ww = V.VpolWaterWater;
    const size_t ncg = (size_t)Pre1db[0] * Pre1db[1] * Pre1db[2];
    double* vc = nullptr;
    if (cudaMalloc(&vc, sizeof(double) * ncg) != cudaSuccess) stop("cudaMalloc failed");
    if (cudaMemcpy(vc, v_diag, sizeof(double) * ncg, cudaMemcpyHostToDevice) != cudaSuccess)
      stop("copy of the coarse V failed");
    if (pg_dual_grid_potential(g, Pre1db, vc, &t, &m, V.Rtol, v, nullptr, nullptr) != PG_OK) stop(pg_last_error());
    if (cudaMemcpy(v_diag, v, sizeof(double) * ngp, cudaMemcpyDeviceToHost) != cudaSuccess) stop("copy of V failed");
    cudaFree(vc);
    cudaFree(v);
    cudaFree(parts);
    pg_grid_destroy(g);
    return;
  }
  if (pg_potential_eval(g, &t, v, parts, nullptr) != PG_OK) stop(pg_last_error());
  if (sc) {
    // SelfConsistentPolarizability (src/Potential.cpp:1495-1591); PolType 3
    // sets no dipoles (src/Potential.cpp:325-335), so the second part is zero
    const DistributedPolarizabilities& mp = V.MolPol[0];
    pg_scpol_model m;
    m.npp = mp.nAtoms;
    m.pol_site = mp.SiteList.data();
    m.inva = mp.InvA.data();
    m.epc = mp.Epc.data();
    m.damp_type = V.DampType;
    m.damp = V.PolDamping;
    m.vpol_ww = V.VpolWaterWater;
    if (pg_potential_scpol_add(g, &t, &m, v, parts, nullptr) != PG_OK) stop(pg_last_error());
  }
  double* out[5] = {v_diag, v_diag_pc, v_diag_ind, v_diag_rep, v_diag_pol};
  if (cudaMemcpy(out[0], v, sizeof(double) * ngp, cudaMemcpyDeviceToHost) != cudaSuccess) stop("copy of V failed");
  for (int c = 0; c < 4; ++c)
    if (cudaMemcpy(out[c + 1], parts + (size_t)c * ngp, sizeof(double) * ngp, cudaMemcpyDeviceToHost) != cudaSuccess)
      stop("copy of the parts failed");
  cudaFree(v);
  cudaFree(parts);
  pg_grid_destroy(g);
}
