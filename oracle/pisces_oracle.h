/*
 * CPU oracle for the PISCES excess-electron eigensolve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (citations per function, paths relative to the reference tree).
 * Only the test suite, the smoke check and the CPU-baseline leg of the bench
 * may load it, and only as the checker or the timed CPU baseline; the product
 * library never links, loads or falls back to it.
 *
 * Parity pinning: every function here is checked against golden vectors
 * produced by the reference's own CPU code, built from the reference sources
 * by oracle/ref/Makefile and driven by oracle/ref/ref_driver.cpp.
 *
 * Conventions (the reference's): grid index g = i + nx*(j + ny*k), x fastest
 * (src/mtx.cpp:15-19); Davidson vectors are contiguous columns B[v*N + g]
 * (src/davdriver.cpp:67-70); kinetic matrices are packed triangles with
 * element (a,b), b<=a, at a*(a+1)/2 + b (src/sine_dvr.cpp:81-84,103-106).
 */
#ifndef PISCES_ORACLE_H
#define PISCES_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Thread count of the OpenMP loops (the results are the same for any count). */
void or_set_threads(int n);

/* 1-D sine DVR: grid points and packed kinetic matrix (src/sine_dvr.cpp:45-131). */
void or_sine_dvr(int n, double mu, double x0, double xNp1, double* x, double* tpacked);

/* y = V.x + (Tx (+) Ty (+) Tz) x, one vector (src/mtx.cpp:22-109). */
void or_matvec(const int n[3], const double* const tp[3], const double* v, const double* x, double* y);

/* diag(H) = V + Tx_ii + Ty_jj + Tz_kk (src/DVR.cpp:1808-1881). */
void or_diagonal(const int n[3], const double* const tp[3], const double* v, double* diag);

/* Half-box particle-in-a-box start vector (src/DVR.cpp:1725-1805). */
void or_piab_start(const int n[3], const double* const x[3], double* wf);

/* Uniform [-1,1] start entries from the C library rand() (src/DVR.cpp:52-59,
 * used at :440-445); the caller seeds rand(). */
void or_random_start(int count, double* out);

/* Rigid-water DPP site producer (src/Water.cpp:197-243, 695-824, 850-943;
 * src/DPP.cpp:114-207, 402-529, 760-1060).  Input: nw waters as O,H,H in
 * Angstrom (9 doubles each).  Outputs (bohr / atomic units):
 *   sites[12*nw]   O,H1,H2,M per water
 *   charges[3*nw], charge_site[3*nw]      (H1, H2, M)
 *   dipoles[9*nw], dipole_site[3*nw]      (self-consistent induced, O,H1,H2)
 * Returns the number of SCF iterations, or -1 if the SCF did not converge. */
int or_dpp_sites(int nw, const double* waters_angstrom, double* sites, double* charges, int* charge_site,
                 double* dipoles, int* dipole_site);

/* Generic electron-site potential tables in the reference's list form
 * (src/Potential.h:38-42, src/Potential.cpp:1817-1861). */
typedef struct {
  int nsites;            const double* sites;        /* 3*nsites */
  int ncharges;          const double* charges;      const int* charge_site;
  int ndipoles;          const double* dipoles;      const int* dipole_site;   /* 3*ndipoles */
  int nsto;              const double* sto;          const int* sto_site;      /* (exponent, coefficient) pairs */
  int npol;              const double* pol_alpha;    const int* pol_site;
  double charge_damp, dipole_damp, pol_damp;          /* effective-radius r0 (DampType 2) */
} or_dpp_tables;

/* Fill the DPPGTOP tables for the default model (PotFlag 3, DampType 2,
 * PolType 1, SigmaOFlag 0; src/Potential.cpp:234-593, 699-728) from the
 * water-site producer output.  Storage for sto/sto_site (8*nw, 4*nw) and
 * pol_alpha/pol_site (nw each) is supplied by the caller. */
void or_dpp_default_tables(int nw, const double* sites, const double* charges, const int* charge_site,
                           const double* dipoles, const int* dipole_site, double* sto, int* sto_site,
                           double* pol_alpha, int* pol_site, or_dpp_tables* t);

/* V(r) on the grid for the DPPGTOP model (src/Potential.cpp:128-182, 844-956,
 * 1169-1374), with the four parts.  Any of parts may be NULL. */
void or_potential_dpp(const int n[3], const double* const x[3], const or_dpp_tables* t, double* v,
                      double* v_pc, double* v_ind, double* v_rep, double* v_pol);

/* Bloomfield erf-damped ions, added into v (src/NaCl.cpp:260-318). */
void or_potential_ions_add(const int n[3], const double* const x[3], int nions, const double* pos,
                           const double* q, double r_cation, double r_anion, double* v);

/* Harmonic model potential 0.5 k r^2 (src/Model_pot.cpp:144-156). */
void or_potential_spherical(const int n[3], const double* const x[3], double k, double* v);

/* Reverse-communication Davidson (src/Davidson.cpp:46-566), state held in a
 * caller-owned struct instead of function statics. */
typedef struct or_davidson_state or_davidson_state;
or_davidson_state* or_davidson_create(void);
void or_davidson_destroy(or_davidson_state* s);
long or_davidson_work_size(int ndim, int maxsub, int nroots, int corrflag);
int or_davidson(or_davidson_state* s, int ndim, int maxsub, int nroots, int maxmacro, int tol, int corrflag,
                double* evals, int* nconv, double* B, double* Z, const double* diag, double* work, int* inout);

/* Full eigensolve through the reverse interface with the sine-DVR matvec:
 * the Davidson driver (src/davdriver.cpp:28-96) with start vectors per
 * src/DVR.cpp:405-453 (startvec 1: PiaB + rand(); 2: all rand(); rand() is
 * seeded with 1, as in a fresh reference process).  B must hold maxsub*N
 * doubles; on return B[0..nstates) are the Ritz vectors.  If n_matvec is
 * given it receives the number of single-vector matvecs; if max_matvec > 0
 * the solve stops after that many (a bounded timing sample) and returns -1.
 * Returns -2 where the reference would lock more than nstates roots and
 * write past its work array (see or_davidson). */
int or_solve(const int n[3], const double* const tp[3], const double* const x[3], const double* v, int nstates,
             int maxsub, int maxiter, int ptol, int corrflag, int startvec, double* evals, double* B,
             long* n_matvec, long max_matvec);

/* Dense symmetric eigensolver (cyclic Jacobi) used for the subspace problem
 * in place of LAPACK dsyev (src/Davidson.cpp:224).  a is n x n column-major
 * with leading dimension lda (overwritten); w ascending, v column-major (ldv). */
int or_syev(int n, double* a, int lda, double* w, double* v, int ldv);

/* Observables and the coarse-grid start vector (src/DVR.cpp:2240-2449,
 * src/Small2Large.cpp:15-220). */
void or_expectation_values(const int n[3], const double* const xg[3], const double* wf, int nstates, double* out);
void or_energy_partition(const int n[3], const double* wf, int nstates, const double* parts, double* out);
void or_small_to_large(const int n[3], const double xmin[3], const double dx[3], const double* wf, const int N[3],
                       const double XMIN[3], const double DX[3], double* WF);

/* Self-consistent polarisation (PolType 3/5/6) and the electron's
 * Hellmann-Feynman gradient on the grid.
 * or_scpol_inva: A = (alpha^-1 - T)^-1, row-major (3 npp)^2
 *   (src/MolPolAux.cpp:39-136, 311-336), inverted by LU with partial pivoting.
 * or_potential_scpol_add: v[g] += -1/2 E(r_g).(A E(r_g)) - vww point by point
 *   (src/Potential.cpp:1495-1591).
 * or_hf_gradient_grid: the density-weighted grid sums of DVR::ComputeGradient
 *   (src/DVR.cpp:1099-1150, src/Gradients.cpp:80-241): grad[3 nsites],
 *   tmu[3 npp], mcm[(3 npp)^2].
 * or_hf_gradient_final: FinalGradient and SubtractWWGradient
 *   (src/Gradients.cpp:252-289). */
int or_scpol_inva(int npp, const double* pos, const double* alpha, double a_thole, double* inva);
void or_potential_scpol_add(const int n[3], const double* const x[3], int npp, const double* pos, const double* inva,
                            const double* epc, int damp_type, double damp, double vww, double* v);
void or_hf_gradient_grid(const int n[3], const double* const x[3], int nsites, const double* sites, int ncharges,
                         const double* charges, const int* charge_site, double charge_damp, int nsto,
                         const double* sto, const int* sto_site, int npp, const int* pol_site, const double* inva,
                         const double* epc, double pol_damp, const double* psi, double* grad, double* tmu,
                         double* mcm);
void or_hf_gradient_final(int nsites, int npp, const double* tmu, const double* mcm, const double* dT_x,
                          const double* dT_y, const double* dT_z, const double* dEfield, const double* pol_grad,
                          double* gradient);

/* Dual grid (PolType 6): or_dual_potential combines the fine grid's exact V
 * (v_exact) with the interpolated coarse V as DVR::ComputePotential's dual
 * branch does (src/DVR.cpp:751-832, InterpolVtriple/InterpolVdouble
 * :1240-1444); or_dual_extend is DVR::ExtendWfThree / ExtendWfDouble
 * (:1446-1723).  n, nc: points per axis (cubic grids). */
void or_dual_potential(int n, int nc, const double* const x[3], int nsites, const double* sites, double rtol,
                       const double* v_coarse, const double* v_exact, double* v);
void or_dual_extend(int n, int nc, const double* wf_coarse, double* wf);

#ifdef __cplusplus
}
#endif
#endif
