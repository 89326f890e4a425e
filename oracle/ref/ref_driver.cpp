// Oracle driver for the reference PISCES CPU code (test infrastructure only).
//
// Links the reference's own objects (compiled unmodified from their source
// tree) and replays the single-point sequence of
// ClusterAnion::SetUpClusterAnion / SinglePoint / EnergyFromConfiguration
// (src/ClusterAnion.cpp:92-112, 114-125, 192-290) through public APIs:
//   WaterCluster::SetStructure -> GetConfiguration -> SetConfiguration ->
//   CalcEnergy -> GetLists / ReportInducedDipoles / ReportPolSitesAndField,
//   Potential::Setup, DVR::SetupDVR / ComputePotential / DiagonalizeSetup /
//   Diagonalize.
// It writes every intermediate the GPU path must reproduce (grid points,
// kinetic matrices, site tables, V on the grid with its four parts, diag(H),
// one H*x product, eigenvalues and eigenvectors) to a binary record file at
// full double precision, which the fixture generator turns into golden files.
//
// The water + ion configuration has no single reference model: the ions use
// the reference Bloomfield potential (src/NaCl.cpp:260-318) in a second
// Potential object, evaluated on the same grid and added to V before the
// reference Davidson runs.
//
// DVR keeps its grid, V and kinetic matrices private; this driver is test
// code, so it opens the class up to read them.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <fstream>
#include <iostream>
#include <sstream>
#include <chrono>
#include <mpi.h>
#include <fcntl.h>
#include <unistd.h>
#include "vecdefs.h"
#include "constants.h"
#include "GTO.h"
#include "MO.h"
#include "AtomCenter.h"
#include "Water.h"
#include "DPP.h"
#define private public
#include "Potential.h"
#include "DVR.h"
#undef private
#include "lapackblas.h"
#include "WriteCubeFile.h"
#include "ReadCubeFile.h"
#include "Small2Large.h"
#include "VectorFFT.hpp"

namespace {

struct Record {
  std::string name;
  char kind;  // 'd' double, 'i' int32
  std::vector<double> d;
  std::vector<int> i;
};

std::vector<Record> g_records;

void put(const std::string& name, const double* p, size_t n) {
  Record r; r.name = name; r.kind = 'd'; r.d.assign(p, p + n); g_records.push_back(r);
}
void put(const std::string& name, const int* p, size_t n) {
  Record r; r.name = name; r.kind = 'i'; r.i.assign(p, p + n); g_records.push_back(r);
}
void put1(const std::string& name, double v) { put(name, &v, 1); }
void put1i(const std::string& name, int v) { put(name, &v, 1); }

// File layout: magic "PGREC1\0\0", then per record: 64-byte zero-padded name,
// 8-byte kind ('d' or 'i' then zeros), uint64 count, raw little-endian data.
void write_records(const std::string& path) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { perror(path.c_str()); exit(2); }
  fwrite("PGREC1\0\0", 1, 8, f);
  for (const Record& r : g_records) {
    char name[64] = {0}; strncpy(name, r.name.c_str(), 63);
    char kind[8] = {0}; kind[0] = r.kind;
    unsigned long long n = r.kind == 'd' ? r.d.size() : r.i.size();
    fwrite(name, 1, 64, f); fwrite(kind, 1, 8, f); fwrite(&n, 8, 1, f);
    if (r.kind == 'd') fwrite(r.d.data(), 8, n, f); else fwrite(r.i.data(), 4, n, f);
  }
  fclose(f);
}

// splitmix64 -> uniform [-1, 1); the vector is also written out, so nothing
// else has to reproduce this generator.
double next_uniform(unsigned long long& s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

struct Input {
  int n[3] = {16, 16, 16};
  double L[3] = {20, 20, 20};
  int nstates = 1, method = 2, maxsub = 20, maxiter = 100, ptol = 5, startvec = 1;
  std::vector<double> waters;  // 9 per water, Angstrom
  std::vector<double> ions;    // x y z q per ion, Angstrom
  double spherical_k = -1;     // >=0: harmonic model potential instead of waters
  long long matvec_seed = -1;
  int fulldiag = 0;
  int diagonalize = 1;
  int dump_wavefn = 1;
  int s2l[3] = {0, 0, 0};  // > 0: the observables and cube-file records, Small2Large onto this grid
  int poltype = 1;         // 3: self-consistent polarisation (PotFlag[3])
  int gradient = 0;        // 1: the Hellmann-Feynman gradient records (needs poltype 3)
  int dual = 0;            // 1: the dual-grid single point of PotFlag[3] = 6 (coarse solve, then this grid)
  double rtol = 20.0;      // PotPara[10]: distance from every site beyond which V is interpolated
  int fft = 0;             // 1: the FFT kinetic path (DVRType 3): its grid, KE_diag and VectorFFT::apply products
  std::string out = "out.rec";
};

Input read_input(const char* path) {
  Input in;
  std::ifstream f(path);
  if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  std::string key;
  while (f >> key) {
    if (key == "grid") { f >> in.n[0] >> in.n[1] >> in.n[2] >> in.L[0] >> in.L[1] >> in.L[2]; }
    else if (key == "diag") { f >> in.nstates >> in.method >> in.maxsub >> in.maxiter >> in.ptol >> in.startvec; }
    else if (key == "waters") { int nw; f >> nw; in.waters.resize(9 * nw); for (double& v : in.waters) f >> v; }
    else if (key == "ions") { int ni; f >> ni; in.ions.resize(4 * ni); for (double& v : in.ions) f >> v; }
    else if (key == "spherical") { f >> in.spherical_k; }
    else if (key == "matvec_seed") { f >> in.matvec_seed; }
    else if (key == "fulldiag") { f >> in.fulldiag; }
    else if (key == "diagonalize") { f >> in.diagonalize; }
    else if (key == "dump_wavefn") { f >> in.dump_wavefn; }
    else if (key == "observables") { f >> in.s2l[0] >> in.s2l[1] >> in.s2l[2]; }
    else if (key == "poltype") { f >> in.poltype; }
    else if (key == "gradient") { f >> in.gradient; }
    else if (key == "dual") { f >> in.dual; }
    else if (key == "rtol") { f >> in.rtol; }
    else if (key == "fft") { f >> in.fft; }
    else if (key == "out") { f >> in.out; }
    else { fprintf(stderr, "unknown key %s\n", key.c_str()); exit(2); }
  }
  return in;
}

// Everything the process writes to standard output (printf and cout) while
// fn runs, as text.
template <class F>
std::string capture_stdout(const std::string& tmp, F&& fn) {
  fflush(stdout);
  std::cout.flush();
  const int saved = dup(1);
  const int fd = open(tmp.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
  dup2(fd, 1);
  close(fd);
  fn();
  fflush(stdout);
  std::cout.flush();
  dup2(saved, 1);
  close(saved);
  std::ifstream f(tmp);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

void put_text(const std::string& name, const std::string& text) {
  std::vector<int> b(text.begin(), text.end());
  put(name, b.data(), b.size());
}

std::string read_file(const std::string& path) {
  std::ifstream f(path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

}  // namespace

// The FFT kinetic path (DVRType 3): DVR::SetupDVR with type 3 (Tdiag per axis
// and the KE_diag composition, src/DVR.cpp:64-651, src/KE_diag.cpp:33-80), then
// VectorFFT::apply (src/VectorFFTW.cpp:14-112, the product davdriver calls for
// this type, src/davdriver.cpp:48, 72-74) on two seeded vectors with a seeded
// V.  DVR::ComputeDiagonal is not called: with DVRType 3 the per-axis kinetic
// arrays hold n values, and it reads them as packed triangles
// (src/DVR.cpp:1808-1881), past their ends, so the reference's Davidson on this
// path starts from an undefined diagonal.
int fft_records(const Input& in) {
  DVR Hel;
  int n[3] = {in.n[0], in.n[1], in.n[2]};
  Hel.SetupDVR(n, 3, 1, in.L, 0);
  Hel.SetVerbose(0);
  const int ngp = Hel.ngp;
  put("n", in.n, 3);
  put("L", in.L, 3);
  for (int a = 0; a < 3; ++a) {
    int off = a == 0 ? 0 : (a == 1 ? Hel.max1db[0] : Hel.max1db[0] + Hel.max1db[1]);
    put(std::string("x") + char('0' + a), Hel.x_dvr + off, n[a]);
    put(std::string("ekin") + char('0' + a), Hel.e_kin[a], n[a]);
  }
  put("ke_diag", Hel.KE_diag, ngp);
  unsigned long long s = (unsigned long long)(in.matvec_seed >= 0 ? in.matvec_seed : 1);
  dVec v(ngp);
  for (double& t : v) t = next_uniform(s);
  put("fft_v", v.data(), ngp);
  VectorFFT engine(n);
  for (int rep = 0; rep < 2; ++rep) {
    dVec x(ngp), y(ngp);
    for (double& t : x) t = next_uniform(s);
    engine.apply(x.data(), y.data(), v.data(), Hel.KE_diag);
    put(std::string("fft_x") + char('0' + rep), x.data(), ngp);
    put(std::string("fft_y") + char('0' + rep), y.data(), ngp);
  }
  write_records(in.out);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) { fprintf(stderr, "usage: %s input.txt\n", argv[0]); return 2; }
  Input in = read_input(argv[1]);
  int provided; MPI_Init_thread(&argc, &argv, MPI_THREAD_FUNNELED, &provided);
  if (in.fft) return fft_records(in);

  // Default electron-water model parameters (src/GetInput.cpp:43-63).
  iVec potflag(6);
  potflag[0] = 3; potflag[1] = 2; potflag[2] = 0; potflag[3] = in.poltype; potflag[4] = 0; potflag[5] = 0;
  double potpara[100] = {0};
  potpara[0] = 9.745; potpara[1] = 2.536; potpara[2] = 4.4837; potpara[3] = 1.7724;
  potpara[4] = 1.7724; potpara[5] = 4.4837; potpara[6] = 0.5 / sqrt(potpara[0]); potpara[10] = in.rtol;

  DVR Hel;
  Hel.SetupDVR(in.n, 0, 1, in.L, 0);
  Hel.SetVerbose(0);
  Hel.DiagonalizeSetup(in.nstates, in.method, in.maxsub, in.maxiter, in.ptol);
  const int ngp = Hel.ngp;

  put("n", in.n, 3);
  put("L", in.L, 3);
  for (int a = 0; a < 3; ++a) {
    int off = a == 0 ? 0 : (a == 1 ? Hel.max1db[0] : Hel.max1db[0] + Hel.max1db[1]);
    put(std::string("x") + char('0' + a), Hel.x_dvr + off, in.n[a]);
    put(std::string("tpacked") + char('0' + a), Hel.e_kin[a], (size_t)in.n[a] * (in.n[a] + 1) / 2);
  }

  Potential Vel;
  Vel.SetVerbose(0);
  WaterCluster WaterN;
  const int nW = (int)in.waters.size() / 9;
  double t_pot = 0;
  if (in.spherical_k >= 0) {
    // DVR::ComputePotential cannot take this model: it asks every Potential
    // for five energy parts (src/DVR.cpp:767-768), SetupSphericalPotential
    // never sets that count, and ReportEnergies exits
    // (src/Potential.cpp:1897-1900).  Sample Potential::Evaluate directly,
    // in the same point order (x fastest).
    double pp[3] = {0, 0, in.spherical_k};
    Vel.SetupSphericalPotential(pp);
    auto t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < in.n[2]; ++k)
      for (int j = 0; j < in.n[1]; ++j)
        for (int i = 0; i < in.n[0]; ++i) {
          double q[3] = {Hel.x_dvr[i], Hel.x_dvr[Hel.max1db[0] + j], Hel.x_dvr[Hel.max1db[0] + Hel.max1db[1] + k]};
          Hel.v_diag[i + in.n[0] * (j + in.n[1] * k)] = Vel.Evaluate(q);
        }
    t_pot = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  } else if (nW > 0) {
    // src/ClusterAnion.cpp:104-106, 84-88, 204-206: structure in Angstrom,
    // no centre-of-mass shift (CoMOrigin default 0), standard DPP charges.
    WaterN.SetStructure(nW, in.waters.data(), 1, 0, 0, 0);
    dVec conf(6 * nW);
    WaterN.GetConfiguration(nW, conf.data(), 1.0, 0);
    WaterN.SetConfiguration(nW, conf.data(), 1, 0);
    double E0 = WaterN.CalcEnergy(0);
    put1("E0", E0);

    int nSites = 0, nCharges = 0, nDipoles = 0;
    WaterN.ReportNoOfSites(nSites, nCharges, nDipoles);
    int nPntPol = WaterN.ReportNoOfPolSites();
    dVec Sites(3 * nSites), Charges(nCharges), Dipoles(3 * nDipoles), DmuByDR(3 * nSites * 3 * nDipoles);
    iVec iqs(nCharges), ids(nDipoles);
    dVec Alphas(nPntPol), Epc(3 * nPntPol);
    iVec ips(nPntPol);
    WaterN.GetLists(nSites, Sites.data(), nCharges, Charges.data(), iqs.data(), nDipoles, Dipoles.data(),
                    ids.data(), DmuByDR.data(), 0);
    put("mol_dipoles", Dipoles.data(), 3 * nDipoles);
    nDipoles *= 3;
    Dipoles.resize(3 * nDipoles);
    ids.resize(nDipoles);
    WaterN.ReportInducedDipoles(nDipoles, Dipoles.data(), ids.data(), 0);
    WaterN.ReportPolSitesAndField(nPntPol, Alphas.data(), ips.data(), Epc.data(), 0);
    put("sites", Sites.data(), Sites.size());
    put("charges", Charges.data(), Charges.size());
    put("charge_site", iqs.data(), iqs.size());
    put("dipoles", Dipoles.data(), Dipoles.size());
    put("dipole_site", ids.data(), ids.size());
    put("alphas", Alphas.data(), Alphas.size());
    put("alpha_site", ips.data(), ips.size());
    put("epc", Epc.data(), Epc.size());

    // src/ClusterAnion.cpp:173: the water-water polarisation energy is the
    // offset of the self-consistent term
    Vel.VpolWaterWater = WaterN.ReportPolarization();
    put1("vpol_ww", Vel.VpolWaterWater);
    if (in.dual) {
      // ClusterAnion::EnergyFromConfiguration with PotFlag[3] = 6
      // (src/ClusterAnion.cpp:211-236, 274-290): a coarse grid of double
      // (odd point count) or triple (even) spacing over a slightly larger
      // box, the self-consistent model (PolType 3) solved on it, then this
      // grid with PolType 6 and the coarse ground state as start vector.
      int Tn[3];
      double TL[3];
      const double spacing = in.L[0] / (in.n[0] + 1);
      for (int a = 0; a < 3; ++a) {
        if (in.n[0] % 2 == 1) {
          Tn[a] = (in.n[a] + 1) / 2;
          TL[a] = Tn[a] * 2 * spacing + 2 * spacing;
        } else {
          Tn[a] = (in.n[a] / 2 + 1) / 3 * 2;
          TL[a] = Tn[a] * 3 * spacing + 3 * spacing;
        }
      }
      Hel.SetupDVR2(Tn, 0, 1, TL, 0);
      Hel.DiagonalizeSetup(in.nstates, in.method, in.maxsub, in.maxiter, in.ptol);
      potflag[3] = 3;
      Vel.Setup(potflag, nSites, Sites.data(), nCharges, Charges.data(), iqs.data(), nDipoles, Dipoles.data(),
                ids.data(), nPntPol, Alphas.data(), ips.data(), Epc.data(), DmuByDR.data(), potpara);
      Hel.ComputePotential(Vel);
      const int cngp = Hel.ngp;
      put("coarse_n", Tn, 3);
      put("coarse_L", TL, 3);
      for (int a = 0; a < 3; ++a) {
        int off = a == 0 ? 0 : (a == 1 ? Hel.max1db[0] : Hel.max1db[0] + Hel.max1db[1]);
        put(std::string("coarse_x") + char('0' + a), Hel.x_dvr + off, Tn[a]);
      }
      put("coarse_v", Hel.v_diag, cngp);
      dVec cev(in.nstates);
      const int cconv = Hel.Diagonalize(in.startvec, cev.data());
      put1i("coarse_nconv", cconv);
      put("coarse_evals", cev.data(), in.nstates);
      put("coarse_wavefn", Hel.wavefn.data(), (size_t)cngp * in.nstates);
      Hel.SetupDVR2(in.n, 0, 1, in.L, 0);
      Hel.DiagonalizeSetup(in.nstates, in.method, in.maxsub, in.maxiter, in.ptol);
      put1i("idual", Hel.Idual);
      {
        // the start vector DVR::Diagonalize builds from the coarse ground
        // state (src/DVR.cpp:422-434)
        dVec ext(Hel.ngp, 0.0);
        for (int g = 0; g < cngp; ++g) ext[g] = Hel.wavefn[g];
        if (Hel.Idual == 0) Hel.ExtendWfThree(ext.data());
        else Hel.ExtendWfDouble(ext.data());
        put("extended_wf", ext.data(), ext.size());
      }
      potflag[3] = 6;
      in.startvec = 3;
    }
    Vel.Setup(potflag, nSites, Sites.data(), nCharges, Charges.data(), iqs.data(), nDipoles, Dipoles.data(),
              ids.data(), nPntPol, Alphas.data(), ips.data(), Epc.data(), DmuByDR.data(), potpara);
    if (in.poltype == 3) {
      put("inva", Vel.MolPol[0].InvA.data(), Vel.MolPol[0].InvA.size());
      put("pol_site_list", Vel.MolPol[0].SiteList.data(), Vel.MolPol[0].nAtoms);
    }
    auto t0 = std::chrono::steady_clock::now();
    Hel.ComputePotential(Vel);
    t_pot = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    put("v_pc", Hel.v_diag_pc, ngp);
    put("v_ind", Hel.v_diag_ind, ngp);
    put("v_rep", Hel.v_diag_rep, ngp);
    put("v_pol", Hel.v_diag_pol, ngp);
  }
  put1("t_potential", t_pot);

  const int nI = (int)in.ions.size() / 4;
  if (nI > 0) {
    // Ions: Bloomfield erf-damped charges, rNa = 2.9, rCl = 1.0 bohr (src/NaCl.cpp:95-96).
    dVec ipos(3 * nI), iq(nI);
    iVec isite(nI);
    for (int k = 0; k < nI; ++k) {
      for (int c = 0; c < 3; ++c) ipos[3 * k + c] = in.ions[4 * k + c] * Angs2Bohr;
      iq[k] = in.ions[4 * k + 3];
      isite[k] = k;
    }
    double pp[2] = {2.9, 1.0};
    Potential Vion;
    Vion.SetVerbose(0);
    // SetupBloomfield stores its model flag in PotFlags[0] (src/NaCl.cpp:264)
    // without sizing the vector; give it its one element first.
    Vion.PotFlags.resize(1);
    Vion.SetupBloomfield(nI, ipos.data(), nI, iq.data(), isite.data(), pp);
    put("ion_sites", ipos.data(), ipos.size());
    put("ion_charges", iq.data(), iq.size());
    dVec vion(ngp);
    // Same grid-point order as DVR::ComputePotential (x fastest).
    for (int k = 0; k < in.n[2]; ++k)
      for (int j = 0; j < in.n[1]; ++j)
        for (int i = 0; i < in.n[0]; ++i) {
          double q[3] = {Hel.x_dvr[i], Hel.x_dvr[Hel.max1db[0] + j], Hel.x_dvr[Hel.max1db[0] + Hel.max1db[1] + k]};
          vion[i + in.n[0] * (j + in.n[1] * k)] = Vion.Evaluate(q);
        }
    put("v_ion", vion.data(), ngp);
    for (int g = 0; g < ngp; ++g) Hel.v_diag[g] += vion[g];
  }
  put("v", Hel.v_diag, ngp);

  dVec diag(ngp);
  Hel.ComputeDiagonal(diag.data());
  put("diag", diag.data(), ngp);

  if (in.matvec_seed >= 0) {
    unsigned long long s = (unsigned long long)in.matvec_seed;
    dVec x(ngp), y(ngp);
    for (double& v : x) v = next_uniform(s);
    DVR::counter kc; Hel.m_pkc = &kc;
    Hel.MatrixTimesVector(x.data(), y.data());
    put("mv_x", x.data(), ngp);
    put("mv_y", y.data(), ngp);
  }

  if (in.fulldiag) {
    if (ngp > 2000) { fprintf(stderr, "fulldiag needs ngp <= 2000\n"); return 2; }
    dVec h((size_t)ngp * ngp), w(ngp);
    Hel.build_h(h.data());
    int info = 0, lwork = 5 * ngp;
    dVec work(lwork);
    dsyev("N", "U", (int*)&ngp, h.data(), (int*)&ngp, w.data(), work.data(), &lwork, &info);
    if (info != 0) { fprintf(stderr, "dsyev info %d\n", info); return 3; }
    put("full_evals", w.data(), ngp);
  }

  if (in.diagonalize) {
    dVec ev(in.nstates);
    auto t0 = std::chrono::steady_clock::now();
    int nconv = Hel.Diagonalize(in.startvec, ev.data());
    double t_diag = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    put1i("nconv", nconv);
    put("evals", ev.data(), in.nstates);
    put1("t_diagonalize", t_diag);
    if (in.dump_wavefn) put("wavefn", Hel.wavefn.data(), (size_t)ngp * in.nstates);
    fprintf(stderr, "nconv %d t_diag %.3f s\n", nconv, t_diag);

    if (in.gradient && in.poltype == 3 && nW > 0 && nconv > 0) {
      // ClusterAnion::GetAnalGrad (src/ClusterAnion.cpp:322-416) on the
      // converged ground state: water-side inputs, then DVR::ComputeGradient
      // twice, once with every water-side input zero (the grid sums alone)
      // and once as the reference calls it.
      int nSites = 0, nCharges = 0, nDip = 0;
      WaterN.ReportNoOfSites(nSites, nCharges, nDip);
      const int nPntPol = WaterN.ReportNoOfPolSites();
      dVec Sites(3 * nSites), Charges(nCharges), Dipoles(3 * nDip), DmuByDR(3 * nSites * 3 * nDip);
      iVec iqs(nCharges), ids(nDip);
      WaterN.GetLists(nSites, Sites.data(), nCharges, Charges.data(), iqs.data(), nDip, Dipoles.data(), ids.data(),
                      DmuByDR.data(), 0);
      dVec dEfield(3 * nSites * nCharges * 3), dTensor(3 * nSites * 3 * nDip * 3);
      WaterN.Calc_dInducedDipoles(0, DmuByDR.data(), dEfield.data(), dTensor.data());
      dVec Gradient(3 * nSites, 0.0), PolGrad(3 * nSites, 0.0);
      const double E0g = WaterN.CalcGradient(nSites * 3, Gradient.data(), PolGrad.data(), 0);
      put1("grad_E0", E0g);
      put("grad_ww", Gradient.data(), Gradient.size());
      put("pol_grad", PolGrad.data(), PolGrad.size());
      put("dEfield", dEfield.data(), dEfield.size());
      dVec Alphas(nPntPol), Epc(3 * nPntPol);
      iVec ips(nPntPol);
      WaterN.ReportPolSitesAndField(nPntPol, Alphas.data(), ips.data(), Epc.data(), 0);
      dVec Rpps(3 * nPntPol);
      for (int i = 0; i < nPntPol; ++i)
        for (int c = 0; c < 3; ++c) Rpps[3 * i + c] = Sites[3 * ips[i] + c];
      void BuildSuperdT(int, const double*, const double*, double, double*, double*, double*);
      dVec dT_x(9 * nPntPol * nPntPol), dT_y(dT_x.size()), dT_z(dT_x.size());
      BuildSuperdT(nPntPol, Rpps.data(), Alphas.data(), 0.3, dT_x.data(), dT_y.data(), dT_z.data());
      put("dT_x", dT_x.data(), dT_x.size());
      put("dT_y", dT_y.data(), dT_y.size());
      put("dT_z", dT_z.data(), dT_z.size());
      dVec G0(3 * nSites, 0.0), zT(dT_x.size(), 0.0), zP(3 * nSites, 0.0), zE(dEfield.size(), 0.0);
      Hel.ComputeGradient(Vel, nSites, G0.data(), zT.data(), zT.data(), zT.data(), zP.data(), WaterN, zE.data());
      put("grad_grid", G0.data(), G0.size());
      auto tg0 = std::chrono::steady_clock::now();
      Hel.ComputeGradient(Vel, nSites, Gradient.data(), dT_x.data(), dT_y.data(), dT_z.data(), PolGrad.data(), WaterN,
                          dEfield.data());
      put1("t_gradient", std::chrono::duration<double>(std::chrono::steady_clock::now() - tg0).count());
      put("grad_total", Gradient.data(), Gradient.size());
      dVec analgrad(6 * nW);
      WaterN.ConvertF(Gradient.data(), analgrad.data());
      put("grad_rigid", analgrad.data(), analgrad.size());
    }
    for (int k = 0; k < in.nstates; ++k) fprintf(stderr, "E[%d] = %.17g\n", k, ev[k]);

    if (in.s2l[0] > 0 && nconv > 0) {
      // The output side of a single point (src/ClusterAnion.cpp:96-120):
      // expectation values and the energy partition as the reference prints
      // them, the state cube, the cube files it writes, its cube reader on a
      // file of its own writer, and Small2Large onto a second grid.
      const std::string dir = in.out.substr(0, in.out.find_last_of('/') + 1);
      put_text("expect_text", capture_stdout(dir + "expect.txt", [&] { Hel.ExpectationValues(2); }));
      if (nW > 0) put_text("energy_text", capture_stdout(dir + "energy.txt", [&] { Hel.EnergyPartitioning(Vel); }));
      std::vector<int> Z(3 * nW);
      for (int w = 0; w < nW; ++w) Z[3 * w] = 8, Z[3 * w + 1] = 1, Z[3 * w + 2] = 1;
      Hel.SetVerbose(0);
      const int last = nconv < in.nstates ? nconv : in.nstates;
      Hel.WriteCubeFile(1, (dir + "state_gauss.cub").c_str(), 3 * nW, Z.data(), in.waters.data(), 0);
      Hel.WriteCubeFile(last, (dir + "state_gomol.cub").c_str(), 3 * nW, Z.data(), in.waters.data(), 1);
      put_text("cube_gauss", read_file(dir + "state_gauss.cub"));
      put_text("cube_gomol", read_file(dir + "state_gomol.cub"));
      put1i("cube_gomol_state", last);
      dVec cube(ngp);
      Hel.GetWaveFnCube(1, cube.data());
      put("state_cube", cube.data(), ngp);
      int npts[3] = {in.n[0], in.n[1], in.n[2]};
      double x0[3], dx[3];
      for (int a = 0; a < 3; ++a) {
        const double* xa = Hel.x_dvr + (a == 0 ? 0 : (a == 1 ? Hel.max1db[0] : Hel.max1db[0] + Hel.max1db[1]));
        x0[a] = xa[0];
        dx[a] = xa[1] - xa[0];
      }
      put("cube_x0", x0, 3);
      put("cube_dx", dx, 3);
      WriteCubeFile((dir + "StartVector.cub").c_str(), 3 * nW, Z.data(), in.waters.data(), npts, x0, dx, cube.data(),
                    nullptr);
      put_text("cube_free", read_file(dir + "StartVector.cub"));
      // ReadCubeFile reads StartVector.cub from the working directory
      char cwd[4096];
      if (!getcwd(cwd, sizeof(cwd)) || chdir(dir.c_str()) != 0) { fprintf(stderr, "chdir failed\n"); return 2; }
      int rn[3];
      double rx0[3], rdx[3];
      double* rcube = nullptr;
      capture_stdout("read.txt", [&] { ReadCubeFile(rn, rx0, rdx, &rcube); });
      if (chdir(cwd) != 0) { fprintf(stderr, "chdir failed\n"); return 2; }
      put("read_npts", rn, 3);
      put("read_x0", rx0, 3);
      put("read_dx", rdx, 3);
      put("read_cube", rcube, (size_t)rn[0] * rn[1] * rn[2]);
      // Small2Large onto N points over the same box (sine-DVR points)
      int N[3] = {in.s2l[0], in.s2l[1], in.s2l[2]};
      double XMIN[3], DX[3];
      for (int a = 0; a < 3; ++a) {
        DX[a] = in.L[a] / (double)(N[a] + 1);
        XMIN[a] = -0.5 * in.L[a] + DX[a];
      }
      dVec WF((size_t)N[0] * N[1] * N[2]);
      capture_stdout(dir + "s2l.txt", [&] { Small2Large(rn, rx0, rdx, rcube, N, XMIN, DX, WF.data()); });
      put("s2l_N", N, 3);
      put("s2l_xmin", XMIN, 3);
      put("s2l_dx", DX, 3);
      put("s2l", WF.data(), WF.size());
      delete[] rcube;
    }
  }
  write_records(in.out);
  return 0;
}
