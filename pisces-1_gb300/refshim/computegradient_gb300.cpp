// DVR::ComputeGradient on the GB300 library: a drop-in for the member of the
// same name (DVR.h:67, src/DVR.cpp:1099-1176), built into the reference in
// place of that function (the reference object keeps it as a weak symbol).
// The reference walks every grid point on the host for the density-weighted
// gradient of the electron's potential with respect to the site positions
// (Potential::EvaluateGradient, src/Gradients.cpp:40-241), then adds the
// dipole-tensor and field-derivative terms and subtracts the water-water
// polarisation gradient (FinalGradient, SubtractWWGradient,
// src/Gradients.cpp:252-289).  Here the grid sums run on the device
// (pg_hf_gradient_grid) for the ground state this DVR holds, and
// pg_hf_gradient_final adds the rest.
//
// Potential keeps its tables private, so this file reads them by compiling
// Potential.h with its members public.  Supported: the self-consistent
// polarisation model (PolType 3, MolPol[0]) with STO cores and
// effective-radius damping, the model the reference's gradient is written
// for.
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
  std::cout << "ComputeGradient (GB300): " << what << "\n";
  exit(1);
}

}  // namespace

void DVR::ComputeGradient(class Potential& V, int nSites, double* Gradient, double* dT_x, double* dT_y, double* dT_z,
                          double* PolGrad, class WaterCluster& WaterN, double* dEfield) {
  (void)WaterN;  // the reference passes it through to Potential::EvaluateGradient unused
  if (V.PotFlags.empty() || V.PotFlags[0] != 3 || V.DampType != 2 || V.PolType != 3 || V.RepCoreType != 2 ||
      V.nMolPol != 1)
    stop("only the self-consistent polarisation model (PolType 3, STO cores, DampType 2) is supported");
  if (nSites != V.nSites) stop("the site count does not match the potential's");
  std::vector<int> stosite(V.nGauss);
  for (int i = 0; i < V.nGauss; ++i) stosite[i] = V.GaussSite[i];
  pg_sites t = {};
  t.nsites = V.nSites;
  t.sites = V.Site.data();
  t.ncharges = V.nCharges;
  t.charges = V.Charge.data();
  t.charge_site = V.ChargeSite.data();
  t.nsto = V.nGauss;
  t.sto = V.Gauss.data();
  t.sto_site = stosite.data();
  t.charge_damp = V.ChargeDamping;
  t.dipole_damp = V.DipoleDamping;
  t.pol_damp = V.PolDamping;
  const DistributedPolarizabilities& mp = V.MolPol[0];
  pg_scpol_model m;
  m.npp = mp.nAtoms;
  m.pol_site = mp.SiteList.data();
  m.inva = mp.InvA.data();
  m.epc = mp.Epc.data();
  m.damp_type = V.DampType;
  m.damp = V.PolDamping;
  m.vpol_ww = V.VpolWaterWater;
  double L[3] = {gridpara[0], gridpara[1], gridpara[2]};
  pg_grid* g = nullptr;
  if (pg_grid_create_dvr(n_1dbas, L, dvrtype == 3 ? 3 : 2, &g) != PG_OK) stop(pg_last_error());
  double* psi = nullptr;
  if (cudaMalloc(&psi, sizeof(double) * ngp) != cudaSuccess) stop("cudaMalloc failed");
  // the ground state (wavefn[igp], src/DVR.cpp:1140-1146)
  if (cudaMemcpy(psi, wavefn.data(), sizeof(double) * ngp, cudaMemcpyHostToDevice) != cudaSuccess)
    stop("copy of the state failed");
  const int n = 3 * m.npp;
  std::vector<double> grid(3 * (size_t)nSites), tmu(n), mcm((size_t)n * n);
  if (pg_hf_gradient_grid(g, &t, &m, psi, grid.data(), tmu.data(), mcm.data(), nullptr) != PG_OK)
    stop(pg_last_error());
  for (int k = 0; k < 3 * nSites; ++k) Gradient[k] += grid[k];
  if (pg_hf_gradient_final(nSites, m.npp, tmu.data(), mcm.data(), dT_x, dT_y, dT_z, dEfield, PolGrad, Gradient) !=
      PG_OK)
    stop(pg_last_error());
  cudaFree(psi);
  pg_grid_destroy(g);
}
