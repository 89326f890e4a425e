/*
 * pisces_gb300 -- C ABI of the GB300 (sm_103a) excess-electron eigensolve path.
 *
 * One shared library, libpisces_gb300.so, replaces the reference PISCES hot
 * path: the sine-DVR kinetic builder, the grid evaluation of the
 * electron-water model potential, the H*X product and the reverse-
 * communication Davidson eigensolver.  Reference citations are paths inside
 * the reference source tree.
 *
 * Conventions (identical to the reference):
 *   - grid index g = i + nx*(j + ny*k), x fastest (src/mtx.cpp:15-19);
 *   - box walls at -L/2 and +L/2 per axis, n interior points (src/DVR.cpp:603);
 *   - blocks of vectors are contiguous columns, X[v*N + g]
 *     (src/davdriver.cpp:67-70);
 *   - all reals are IEEE double, lengths in bohr, energies in hartree;
 *     water input coordinates in Angstrom (src/GetInput.cpp:256).
 *
 * Pointers named *_dev are device pointers on the handle's GPU; pointers
 * named *_host are host pointers.  A `stream` argument is a cudaStream_t
 * passed as void* (NULL = the legacy default stream).  No call keeps a
 * caller pointer past its return.  Every call returns a pg_status; the text
 * of the last error on the calling thread is pg_last_error().  Nothing
 * exits the process (the reference calls exit(1)/exit(42) instead).
 */
#ifndef PISCES_GB300_H
#define PISCES_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PG_OK = 0,
  PG_BAD_ARG = 1,        /* invalid size, pointer or flag */
  PG_OOM = 2,            /* device or host allocation failed, or admission refused */
  PG_NOT_CONVERGED = 3,  /* Davidson reached its macro-iteration limit (reference: warning, src/Davidson.cpp:332-340) */
  PG_DEVICE_TIMEOUT = 4, /* a bounded device-side wait ran out */
  PG_NUMERIC = 5,        /* NaN/Inf or a failed small eigensolve (reference: src/Davidson.cpp:225-226) */
  PG_CUDA = 6,           /* a CUDA runtime call failed */
  PG_UNSUPPORTED = 7     /* valid but not implemented on this path */
} pg_status;

typedef enum { PG_FP64 = 0, PG_MIXED = 1 } pg_precision;

const char* pg_last_error(void);
int pg_version(void);
/* Number of CUDA kernels this library has launched since it was loaded. */
long pg_kernel_launches(void);
/* Number of device allocations (cudaMalloc) this library has made since it
 * was loaded, successful or not. */
long pg_device_allocations(void);

/* ------------------------------------------------------------------ kinetic */

/* 1-D sine DVR: grid points x[n] and the kinetic matrix of a particle of
 * mass mu in the box (x0, xNp1).  ldt == 0: packed lower triangle, element
 * (a,b) b<=a at a*(a+1)/2+b; ldt >= n: full symmetric matrix with leading
 * dimension ldt.  Replaces sine_dvr() (src/sine_dvr.h:1, src/sine_dvr.cpp:45-131),
 * same arguments and meaning (the verbose flag is dropped).  Host-only. */
pg_status pg_sine_dvr(int n, double mu, double x0, double xNp1, double* x_host, double* ekin_host, int ldt);

/* Periodic FFT kinetic term of DVRType 3: the grid points and the plane-wave
 * energies ekin[n] = (dK k)^2 / (2 mu), dK = 2 pi / (n dx), k = a or a - n
 * (Tdiag, src/KE_diag.cpp:33-80, same arguments without ldt/verbose); and,
 * if t_host is not NULL, the n x n matrix of the per-axis operator
 * ifft(ekin * fft(.)) / n that VectorFFT::apply applies
 * (src/VectorFFTW.cpp:56-112), a real symmetric circulant.  Host-only. */
pg_status pg_fft_kinetic(int n, double mu, double x0, double xNp1, double* x_host, double* ekin_host,
                         double* t_host);

/* --------------------------------------------------------------------- grid */

typedef struct pg_grid pg_grid;

/* A 3-D sine-DVR grid on the current device: n[3] points per axis, box
 * lengths L[3].  Builds the three kinetic matrices (full, FP64, plus the
 * split-TF32 copies of the mixed form) in device memory.  Replaces
 * DVR::SetupDVR with DVRType 0 (src/DVR.cpp:64-161, 524-651). */
pg_status pg_grid_create(const int n[3], const double L[3], pg_grid** out);
/* The same with the kinetic term chosen as the reference's DVRType: 2 = sine
 * DVR (pg_grid_create), 3 = periodic FFT kinetic (VectorFFT, src/DVR.cpp:
 * 138-142, 596-630), applied here as three per-axis dense circulant
 * contractions, exactly the operator the 3-D FFT applies, by the same H*X
 * kernels.  The reference's FFT path assumes cubic grids
 * (src/VectorFFTW.cpp:83); this one is the separable operator for any box. */
pg_status pg_grid_create_dvr(const int n[3], const double L[3], int dvrtype, pg_grid** out);
pg_status pg_grid_destroy(pg_grid* g);
/* Number of grid points (n0*n1*n2). */
long pg_grid_npoints(const pg_grid* g);
/* Grid points per axis (host copies, n[a] doubles each; any may be NULL). */
pg_status pg_grid_points(const pg_grid* g, double* x_host, double* y_host, double* z_host);
/* Kinetic matrix of one axis as a full n x n host matrix. */
pg_status pg_grid_kinetic(const pg_grid* g, int axis, double* t_host);

/* diag(H) = V + Tx_ii + Ty_jj + Tz_kk (DVR::ComputeDiagonal, src/DVR.cpp:1808-1881). */
pg_status pg_diagonal(const pg_grid* g, const double* v_dev, double* diag_dev, void* stream);

/* Half-box particle-in-a-box start vector (DVR::ParticleInAnDBoxWf, src/DVR.cpp:1725-1805). */
pg_status pg_piab_start(const pg_grid* g, double* wf_dev, void* stream);

/* ----------------------------------------------------------------- potential */

/* Electron-site potential tables in the reference's list form
 * (Potential::Setup arguments, src/Potential.h:38-42; per-term lists set by
 * SetSites/SetCharges/SetDipoles and the repulsive-core and polarisable-site
 * setup, src/Potential.cpp:234-593, 699-728, 1817-1861).  Host pointers.
 * Site indices refer to `sites`.  Damping follows DampType 2 (effective
 * radius r0; src/Potential.cpp:1188-1366); the polarisation term is the
 * first-order -alpha/(2 R^4) form (PolType 1, AdiabaticPolPot 0). */
typedef struct {
  int nsites;   const double* sites;                            /* 3*nsites, bohr */
  int ncharges; const double* charges;   const int* charge_site;
  int ndipoles; const double* dipoles;   const int* dipole_site; /* 3*ndipoles */
  int nsto;     const double* sto;       const int* sto_site;    /* (exponent, coefficient) pairs: c*exp(-z*R) */
  int npol;     const double* pol_alpha; const int* pol_site;
  double charge_damp, dipole_damp, pol_damp;                      /* r0 per term */
} pg_sites;

/* V(r) on every grid point, and optionally its four parts
 * (charges, induced dipoles, repulsive core, polarisation) as parts_dev[4*N]
 * in that order.  Replaces DVR::ComputePotential + Potential::Evaluate /
 * EvaluateDPPGTOP (src/DVR.cpp:661-859, src/Potential.cpp:128-182, 844-956).
 * At most one charge, one dipole, one polarisable site and two repulsive
 * Slater functions may sit on one site (PG_UNSUPPORTED otherwise). */
pg_status pg_potential_eval(const pg_grid* g, const pg_sites* tables, double* v_dev, double* parts_dev, void* stream);

/* Adds Bloomfield erf-damped ion charges, -q erf(R/r_ion)/R, with r_ion =
 * r_cation for q > 0 and r_anion otherwise (Potential::EvaluateBloomfield,
 * src/NaCl.cpp:260-318).  pos_host: 3*nions bohr. */
pg_status pg_potential_ions_add(const pg_grid* g, int nions, const double* pos_host, const double* q_host,
                                double r_cation, double r_anion, double* v_dev, void* stream);

/* Harmonic model potential 0.5*k*r^2 (Potential::EvaluateSphericalPotential,
 * src/Model_pot.cpp:144-156). */
pg_status pg_potential_spherical(const pg_grid* g, double k, double* v_dev, void* stream);

/* --------------------------------------- self-consistent polarisation */

/* The self-consistent polarisation model of the electron-water potential
 * (PolType 3, 5, 6; Potential::SetupDPPGTOP, src/Potential.cpp:383-460,
 * MolPol[0]).  Host pointers.  pol_site: the site (index into the site list
 * of the pg_sites tables it is used with) of each polarisable atom
 * (SiteList); inva: A = (alpha^-1 - T)^-1, (3 npp)^2 doubles (InvA); epc:
 * the water charges' field at those atoms, 3 npp (Epc); damp_type 1:
 * g(R) = (1 - exp(-damp R^3)) / R^3, 2: effective radius r0 = damp
 * (PolDamping); vpol_ww: the water-water polarisation energy subtracted
 * from the term (Potential::VpolWaterWater). */
typedef struct {
  int npp;
  const int* pol_site;
  const double* inva;
  const double* epc;
  int damp_type;
  double damp;
  double vpol_ww;
} pg_scpol_model;

/* A = (alpha^-1 - T)^-1 for npp point-polarisable atoms with Thole-damped
 * dipole tensors (ComputeInvA = BuildPolarizationMatrix + InvertMatrix,
 * src/MolPolAux.cpp:39-136, 264-336).  Host; pos: 3*npp bohr; inva: (3 npp)^2
 * row-major, symmetric.  PG_NUMERIC if the matrix is singular. */
pg_status pg_scpol_inva(int npp, const double* pos_bohr, const double* alpha, double a_thole, double* inva);

/* v_dev[g] += -1/2 E(r_g)^T A E(r_g) - vpol_ww, the self-consistent
 * polarisation term (Potential::SelfConsistentPolarizability,
 * src/Potential.cpp:1495-1628), FP64.  E(r) holds the electron's damped
 * field at every polarisable atom plus epc.  With parts_dev (the four parts
 * of pg_potential_eval, 4*N) the term is also added to its polarisation
 * part.  For the reference's PolType 3 and 6 potentials, evaluate the
 * charges and repulsive core with pg_potential_eval (no dipoles, no
 * non-interacting polarisable sites) and add this term. */
pg_status pg_potential_scpol_add(const pg_grid* g, const pg_sites* tables, const pg_scpol_model* m, double* v_dev,
                                 double* parts_dev, void* stream);

/* ------------------------------------------------------------- dual grid */

/* The coarse grid of the dual-grid single point (PotFlag[3] = 6;
 * ClusterAnion::EnergyFromConfiguration, src/ClusterAnion.cpp:211-236):
 * for n x n x n points over a cubic box of side L, with h = L / (n + 1):
 * odd n: nc = (n + 1) / 2 points over nc*2h + 2h (double spacing);
 * even n: nc = 2 ((n/2 + 1) / 3) points over nc*3h + 3h (triple spacing).
 * *spacing (may be NULL) receives 2 or 3.  PG_BAD_ARG unless the grid is
 * cubic (the reference's dual grid is). */
pg_status pg_dual_grid_coarse(const int n[3], const double L[3], int nc[3], double Lc[3], int* spacing);

/* V of PolType 6 on the fine grid g (DVR::ComputePotential's dual branch,
 * src/DVR.cpp:751-832): the charges and Slater cores of `tables` (no
 * dipoles, no one-site polarisation) everywhere; at points where every
 * site is farther than rtol (PotPara[10]), or that lie on the coarse
 * lattice, V is interpolated from v_coarse_dev (the coarse grid's full V,
 * nc^3 values) by the reference's inverse-distance weights
 * (DVR::InterpolVtriple / InterpolVdouble, src/DVR.cpp:1240-1444); the
 * other points add the self-consistent polarisation term of m.  With
 * triple spacing the reference zeroes V on the outer layers its coarse
 * lattice does not reach; so does this.  *n_exact (may be NULL) receives
 * the number of points evaluated exactly.  Waits for the stream. */
pg_status pg_dual_grid_potential(const pg_grid* g, const int nc[3], const double* v_coarse_dev,
                                 const pg_sites* tables, const pg_scpol_model* m, double rtol, double* v_dev,
                                 long* n_exact, void* stream);

/* Start vector on the fine grid from a coarse state, interpolated the same
 * way (DVR::ExtendWfThree / ExtendWfDouble, src/DVR.cpp:1446-1723). */
pg_status pg_dual_grid_extend(const pg_grid* g, const int nc[3], const double* wf_coarse_dev, double* wf_dev,
                              void* stream);

/* ----------------------------------------------- Hellmann-Feynman gradient */

/* The grid part of the electron's gradient with respect to the site
 * positions (DVR::ComputeGradient's loop, src/DVR.cpp:1099-1150, with
 * Potential::EvaluateDPPGTOPGradient, DerivElecField and MuCrossMu,
 * src/Gradients.cpp:80-241), FP64, for the density psi_dev[g]^2 of a state
 * (N doubles on the device):
 *   grad[3 nsites]  = sum_g psi_g^2 dV(r_g)/dR  over the charges, Slater
 *                     cores and the field derivative at each polarisable atom
 *   tmu[3 npp]      = sum_g psi_g^2 mu(r_g),  mu = A E(r)
 *   mcm[(3 npp)^2]  = sum_g psi_g^2 mu(r_g) mu(r_g)^T
 * Host outputs.  The model's damp_type must be 2 (the reference's gradient
 * damps by the effective radius only) and pol_site increasing. */
pg_status pg_hf_gradient_grid(const pg_grid* g, const pg_sites* tables, const pg_scpol_model* m,
                              const double* psi_dev, double* grad, double* tmu, double* mcm, void* stream);

/* The terms after the grid loop (Potential::FinalGradient and
 * SubtractWWGradient, src/Gradients.cpp:252-289), host:
 *   gradient[3j+d] += -dEfield[3npp (3j+d) + k] tmu[k]
 *                     - dT_d[9 npp a_j + k] mcm[9 npp a_j + k]  (a_j: atom of
 *                       site j, O/H sites only),
 *   gradient -= pol_grad (if not NULL).
 * Rigid-water layout: nsites = 4 nw (O,H,H,M), npp = 3 nw (O,H,H).
 * dT_x/y/z: 9 npp^2 each (BuildSuperdT); dEfield: 3 nsites * 3 npp
 * (WaterCluster::Calc_dInducedDipoles).  Together with
 * pg_hf_gradient_grid this is DVR::ComputeGradient. */
pg_status pg_hf_gradient_final(int nsites, int npp, const double* tmu, const double* mcm, const double* dT_x,
                               const double* dT_y, const double* dT_z, const double* dEfield, const double* pol_grad,
                               double* gradient);

/* Rigid-water DPP site producer (host): projects each O,H,H triple onto the
 * rigid model (Water::Reposition, src/Water.cpp:695-824), solves the damped
 * self-consistent induced dipoles (WaterCluster::CalcInducedDipoles,
 * src/DPP.cpp:760-1060) and returns the electron's lists
 * (WaterCluster::GetLists / ReportInducedDipoles, src/DPP.cpp:402-529):
 *   sites[12*nw] (O,H1,H2,M), charges[3*nw]/charge_site[3*nw] (H1,H2,M),
 *   dipoles[9*nw]/dipole_site[3*nw] (O,H1,H2).
 * *scf_iters receives the SCF iteration count (-1: not converged). */
pg_status pg_water_sites(int nw, const double* waters_angstrom, double* sites, double* charges, int* charge_site,
                         double* dipoles, int* dipole_site, int* scf_iters);

/* The polarisable atoms of the same cluster for the self-consistent model
 * (WaterCluster::ReportPolSitesAndField, src/DPP.cpp:540-640): O, H1, H2 of
 * every water, pol_site[3*nw] = their site indices (4j, 4j+1, 4j+2),
 * alpha[3*nw], epc[9*nw] = the damped field of the other waters' charges at
 * them; *vpol_ww = the water-water polarisation energy with the converged
 * dipoles (WaterCluster::ReportPolarization, src/DPP.cpp:1648-1691,
 * 1935-2010), the offset the reference subtracts from the term. */
pg_status pg_water_scpol(int nw, const double* waters_angstrom, int* pol_site, double* alpha, double* epc,
                         double* vpol_ww);

/* Default electron-water model tables for those lists: 4-STO repulsive core
 * scaled by 1/4.4837, one polarisable site (alpha 9.745) per water on M,
 * damping radii 1.7724/1.7724/2.536 (src/GetInput.cpp:43-63,
 * src/Potential.cpp:699-728, 326-338).  Caller storage: sto[8*nw],
 * sto_site[4*nw], pol_alpha[nw], pol_site[nw]; `out` points into the inputs. */
pg_status pg_water_default_tables(int nw, const double* sites, const double* charges, const int* charge_site,
                                  const double* dipoles, const int* dipole_site, double* sto, int* sto_site,
                                  double* pol_alpha, int* pol_site, pg_sites* out);

/* ------------------------------------------------------------------- H * X */

/* Y = H X for nvec vectors: H = V + Tx (+) Ty (+) Tz.  precision PG_FP64:
 * FP64 arithmetic throughout; PG_MIXED: kinetic contractions as split-TF32
 * tensor-core products accumulated in FP32, V*X in FP64.  nvec = 0 does
 * nothing and accepts null X and Y.  Replaces DVR::MatrixTimesVector applied
 * vector by vector (src/mtx.cpp:22-109, src/davdriver.cpp:67-78). */
pg_status pg_hx(const pg_grid* g, const double* v_dev, const double* x_dev, double* y_dev, int nvec, int precision,
                void* stream);
/* pg_hx without the completion check of the mixed form: returns once the
 * launches are queued (no host wait).  A tensor-core completion wait that
 * timed out is recorded in the grid's status word and reported by the next
 * pg_grid_check. */
pg_status pg_hx_async(const pg_grid* g, const double* v_dev, const double* x_dev, double* y_dev, int nvec,
                      int precision, void* stream);
/* Waits for the stream; PG_DEVICE_TIMEOUT if a tensor-core completion wait on
 * this grid timed out since the last check (the status word is then cleared). */
pg_status pg_grid_check(const pg_grid* g, void* stream);

/* Kernel of the mixed-form H*X on this grid: 0 = automatic (the fused
 * kernel where the grid allows it, else three axis passes), 1 = three axis
 * passes, each a tensor-core contraction over the whole grid, 2 = fused (the
 * x and y contractions of each grid plane in one tensor-memory tile, the z
 * contraction of 128-line tiles, one persistent launch; PG_UNSUPPORTED where
 * the grid does not fit it: more than 128 points along x, an axis above 112
 * points, or operand images beyond shared memory), 3 = the same work items
 * with an FP16 split of the operands scaled by a power of two per item (one
 * plane image read K-major by the x contraction and MN-major by the y
 * contraction, the next item's rows bulk-copied into shared memory; grids of
 * at most 96 points per axis whose axes share one kinetic matrix, nx even;
 * an X block not 16-byte aligned falls back to kind 2).  Automatic selection
 * prefers 3, then 2.  All give the same products to the mixed form's
 * accuracy.  No reference counterpart (the
 * reference multiplies line by line, src/mtx.cpp:61-104). */
pg_status pg_grid_set_hx_kernel(pg_grid* g, int kind);
/* Launch parameters of the mixed-form H*X on this grid, overriding the tuned
 * table: kind as pg_grid_set_hx_kernel; lag = vectors between a vector's xy
 * planes and its z tiles in the fused kernel's work order (0: tuned); ctas =
 * CTAs per launch (0: tuned, at most one per SM); form of the three axis
 * passes: 0 automatic, 1 serial, 2 pipelined (0 = tuned).  The tuned table
 * (pisces-1_gb300/hx_tuned.tsv, written by tune_hx.py on a GB300) holds the
 * fastest measured choice per cubic grid size and block size; other grids
 * use built-in rules.  No reference counterpart. */
pg_status pg_grid_set_hx_params(pg_grid* g, int kind, int lag, int ctas, int form);
/* One line describing the mixed-form H*X kernel and tile shape this grid
 * uses for blocks of nvec vectors (pg_grid_hx_plan: nvec = 1); text of at
 * most len bytes including the terminator. */
pg_status pg_grid_hx_plan(const pg_grid* g, char* text, int len);
pg_status pg_grid_hx_plan_for(const pg_grid* g, int nvec, char* text, int len);

/* ---------------------------------------------------------------- Davidson */

typedef struct pg_davidson pg_davidson;

/* Caller-owned state for the reverse-communication Davidson (the reference
 * keeps it in function statics, src/Davidson.cpp:114-143, so only one solve
 * per process can run; any number of handles can run here). */
pg_status pg_davidson_create(pg_davidson** out);
pg_status pg_davidson_destroy(pg_davidson* d);

/* Arithmetic of the subspace products of this handle (S = Z^T B, the Ritz
 * and residual combinations, the block orthogonalisation): PG_FP64 (default,
 * IEEE FP64 throughout) or PG_MIXED, double-float (two FP32 numbers,
 * ~2^-48 relative) on the FP32 pipe.  The subspace eigensolve, the Cholesky
 * factors and the residual norms stay FP64 either way.  PG_MIXED also keeps
 * double-float copies of B and Z on the device (2 * maxsub * ndim doubles).
 * Set it before a solve's first call: PG_BAD_ARG while a solve is in
 * progress. */
pg_status pg_davidson_set_arithmetic(pg_davidson* d, int precision);

/* Enables corrflag 3 on this handle: the correction vector of a root with
 * Ritz vector u, Ritz value lambda and residual r is M r, M = (T - lambda)^-1,
 * T the grid's kinetic operator applied exactly in its eigenbasis (DST-I for
 * the sine DVR, the real Fourier basis for the periodic FFT kinetic term:
 * three axis contractions, a diagonal scale, three more; precision as
 * pg_hx).  Where V is identically zero M r equals u and adds nothing, so the
 * Olsen form -M r + (u.M r / u.M u) M u is used there (detected from diag(H)
 * at the first call).  Not in the reference, whose corrections use diag(H)
 * only (src/Davidson.cpp:530-566); it changes the convergence rate, not the
 * converged eigenpairs.  T - lambda is definite only for Ritz values below
 * the lowest kinetic level (bound states such as cluster anions); for levels
 * deep inside the kinetic spectrum (a strong confining well) the corrections
 * stall and the solve ends in PG_NOT_CONVERGED: use corrflag 1 there.
 * g must outlive the solve. */
pg_status pg_davidson_set_preconditioner(pg_davidson* d, const pg_grid* g, int precision);

/* The kinetic preconditioner on its own: R <- (T - sigma_j)^-1 R for the k
 * contiguous vectors R (device, N each, 16-byte aligned for the FP16 kernel),
 * sigma[k] on the host; |T - sigma_j| is kept at least a tenth of the lowest
 * kinetic level.  PG_FP64: six FP64 axis passes and a diagonal scale; PG_MIXED:
 * where every axis has the same n <= 96 (n even), one FP16-split tensor-core
 * kernel (k_kin_f16: per vector, xy forward transforms of the planes, z
 * forward transform + diagonal + z backward transform of 128-line tiles, xy
 * backward transforms), else six split-TF32 axis passes.  Allocates 2 k N
 * doubles of scratch and synchronises the stream.  No reference counterpart
 * (corrflag 3 is this library's own). */
pg_status pg_kinetic_precondition(const pg_grid* g, double* R, int k, const double* sigma, int precision,
                                  void* stream);
/* Mixed-form preconditioner kernel of this grid: 0 automatic (the FP16 kernel
 * where it applies), 1 the axis passes. */
pg_status pg_grid_set_precond_kernel(pg_grid* g, int kind);
/* One line describing the mixed-form preconditioner this grid uses. */
pg_status pg_grid_precond_plan(const pg_grid* g, char* text, int len);

/* The subspace eigensolver of the Davidson iteration (host): the k lowest
 * eigenpairs of the symmetric m x m matrix whose upper triangle is stored in
 * S (column-major, leading dimension ld); eigenvalues ascending in w[k],
 * eigenvectors in the columns of V (leading dimension ldv).  Takes the place
 * of the dsyev call of src/Davidson.cpp:224, which computes all m pairs. */
pg_status pg_subspace_lowest(int m, const double* S_host, int ld, int k, double* w_host, double* V_host, int ldv);

/* Block products of the Davidson subspace (device arrays, vectors stored
 * contiguously, vector a at P_dev + a*n), the skinny GEMMs of the reference's
 * S = Z^T B build (src/Davidson.cpp:220, 385-393) and Ritz combinations
 * (src/Davidson.cpp:240-260).  Deterministic (fixed reduction order).
 * precision PG_FP64: FP64; PG_MIXED: double-float on the FP32 pipe.
 *   pg_block_gram:    out[a*nq + b] = P_a . Q_b   (np*nq <= 2048, np+nq <= 144)
 *   pg_block_combine: Y_r = sum_a P_a C[a*ny + r]   (ny <= 16, np*ny <= 2048) */
pg_status pg_block_gram(long n, const double* P_dev, int np, const double* Q_dev, int nq, double* out_dev,
                        int precision, void* stream);
pg_status pg_block_combine(long n, const double* P_dev, int np, const double* C_dev, int ny, double* Y_dev,
                           int precision, void* stream);

/* The same products on double-float twins, the form the mixed Davidson
 * keeps its basis and products in: a twin holds, in the 8 bytes of each
 * value, the float2 (hi, lo) with hi + lo = x to about 2^-48 relative.
 *   pg_split_twin:         twin_dev[i] = twin of x_dev[i]
 *   pg_block_gram_twin:    out[a*nq + b] = P_a . Q_b, P and Q given as twins
 *   pg_block_combine_twin: Y_r = sum_a P_a C[a*ny + r], P given as twins; Yt_dev
 *                          (may be NULL) receives the twins of Y.
 * Limits as pg_block_gram / pg_block_combine.  No reference counterpart
 * (the reference's products are FP64 dgemm, src/Davidson.cpp:220, 240-260). */
pg_status pg_split_twin(long n, const double* x_dev, double* twin_dev, void* stream);
pg_status pg_block_gram_twin(long n, const double* Ptwin_dev, int np, const double* Qtwin_dev, int nq,
                             double* out_dev, void* stream);
pg_status pg_block_combine_twin(long n, const double* Ptwin_dev, int np, const double* C_dev, int ny, double* Y_dev,
                                double* Yt_dev, void* stream);

/* pg_block_gram without any device allocation; no counterpart in the
 * reference.  For callers that must not allocate device memory: a framework
 * may already hold the free memory in its own caching allocator, so a
 * cudaMalloc would fail, or a cudaFree would synchronise the whole device
 * under a latency budget.  The reduction partials go to a fixed file-scope
 * device array of 256 x 296 doubles (592 KiB), so np * nq <= 256
 * (PG_BAD_ARG with a message otherwise).  The first call on a device looks up
 * that array's address and should come before any stream capture; the address
 * is kept for the life of the process, so the entry point must not be called
 * on a device after cudaDeviceReset of that device.  Nothing in the array has
 * to start at zero.  Calls that overlap in time (other streams
 * or threads) share the one array and race: serialise them.  Results are
 * bit-identical to pg_block_gram's. */
pg_status pg_block_gram_noalloc(long n, const double* P_dev, int np, const double* Q_dev, int nq, double* out_dev,
                                int precision, void* stream);

/* Work-array length in doubles (DavidsonWorkSize, src/Davidson.cpp:46-52). */
long pg_davidson_work_size(int ndim, int maxsub, int nroots, int corrflag);

/* One step of the reverse-communication Davidson: same arguments, meaning
 * and return codes as Davidson() (src/Davidson.h:2-15, src/Davidson.cpp:61-376)
 * plus the state handle and a stream.  B_dev, Z_dev (ndim*maxsub), diag_dev
 * (ndim) and work_dev (pg_davidson_work_size) are device arrays; evals_host,
 * nconv and inout are host.  *ret = 1: compute Z[inout[1]+v] = H B[inout[0]+v]
 * for v < inout[2], then call again; *ret = 0: done (converged eigenpairs in
 * evals_host and B_dev[0..nroots), *nconv converged; PG_NOT_CONVERGED if the
 * macro-iteration limit was reached).  Two departures from the reference,
 * both where its iteration breaks down: locking stops at nroots (inside a
 * near-degenerate set the reference can lock a state twice and overrun its
 * arrays), and a restart re-orthonormalises the kept block of B and Z by one
 * Cholesky-QR step (the reference keeps locked and new Ritz vectors that are
 * orthogonal only to O(residual / gap)).  PG_NUMERIC if |B v| of a unit
 * subspace vector still differs from 1 by more than 1e-6. */
pg_status pg_davidson_rci(pg_davidson* d, int ndim, int maxsub, int nroots, int maxmacro, int tol, int corrflag,
                          double* evals_host, int* nconv, double* B_dev, double* Z_dev, const double* diag_dev,
                          double* work_dev, int* inout, int* ret, void* stream);

typedef struct {
  int nroots;     /* states wanted (nStates) */
  int maxsub;     /* max subspace (maxSubspace, default 20) */
  int maxiter;    /* max macro iterations (maxIter, default 100) */
  int ptol;       /* residual threshold 10^-ptol (pTol) */
  int corrflag;   /* 0 residual, 1 Davidson (default), 2 Jacobi-Davidson, 3 exact-kinetic preconditioner */
  int precision;  /* pg_precision of the H*X products */
  int startvec;   /* 0: start vectors given in evecs_dev; 1: PiaB + random; 2: random;
                     3: column 0 given in evecs_dev (pg_dual_grid_extend), the others random */
  int refine;     /* PG_MIXED only: 1 = finish with an FP64 Rayleigh-Ritz step on the converged vectors;
                     2 = continue the plain FP64 Davidson from them to residual 10^-max(ptol+2, 8) */
} pg_solve_params;

typedef struct {
  int nconv;
  int n_matvec;      /* single-vector H*x products */
  int n_iter;        /* Davidson subspace iterations */
  int n_restart;
  double residual[64];   /* final |r| per root (first min(nroots,64)) */
  double seconds;        /* wall time of the solve */
  double host_eig_seconds;     /* of which in the host subspace eigensolver */
  double device_wait_seconds;  /* of which waiting for device results at the two per-iteration reads */
} pg_solve_stats;

/* Full eigensolve on the device: start vectors (DVR::Diagonalize,
 * src/DVR.cpp:405-453), the Davidson driver loop (DVR::davdriver,
 * src/davdriver.cpp:28-96) with block H*X products.  evecs_dev: nroots*N
 * doubles (in: start vectors when startvec == 0; out: eigenvectors).
 * evals_host: nroots. */
pg_status pg_solve(const pg_grid* g, const double* v_dev, const pg_solve_params* p, double* evals_host,
                   double* evecs_dev, pg_solve_stats* stats, void* stream);

/* Whole single point from host data: water coordinates (Angstrom, 9 per
 * water) and optional ions (x,y,z in Angstrom, q) -> site tables (host),
 * V(r) (device), eigensolve (device) -> eigenvalues and, if evecs_host is
 * not NULL, eigenvectors (nroots*N) copied back.  The reference's
 * ClusterAnion::EnergyFromConfiguration (src/ClusterAnion.cpp:192-290)
 * binding-energy part. */
pg_status pg_cluster_solve(const int n[3], const double L[3], int nw, const double* waters_angstrom, int nions,
                           const double* ions_angstrom_q, const pg_solve_params* p, double* evals_host,
                           double* evecs_host, pg_solve_stats* stats, void* stream);

/* ---- Observables and wavefunction files ------------------------------------
 * What the reference reports about converged states and how it stores them
 * (the hot path's output side): grid reductions of psi^2 on the device, and
 * the reference's cube file formats, written byte for byte as it writes
 * them. */

/* Moments of a state psi (a DVR vector: psi^2 at a grid point is the
 * probability there): norm = sum psi^2, r = (<x>, <y>, <z>) in bohr, r2 =
 * <r^2>, and for states n >= 1 the transition dipole (<n|x|0>, <n|y|0>,
 * <n|z|0>) with state 0 (zero for state 0).  |<r>| = |r|, the spread
 * sqrt(r2 - |r|^2). */
typedef struct {
  double norm;
  double r[3];
  double r2;
  double trans_dipole[3];
} pg_moments;

/* Moments of nstates vectors (vecs_dev[s*N + g]) into out_host[nstates].
 * Replaces DVR::ExpectationValues (src/DVR.cpp:2329-2449), which prints the
 * same sums.  Deterministic (fixed summation order). */
pg_status pg_expectation_values(const pg_grid* g, const double* vecs_dev, int nstates, pg_moments* out_host,
                                void* stream);

/* Potential-energy partition: out_host[4*s + c] = sum_g psi_s(g)^2 part_c(g)
 * for the four parts of pg_potential_eval (charges, induced dipoles,
 * repulsive core, polarisation; hartree).  Replaces
 * DVR::EnergyPartitioning (src/DVR.cpp:2240-2325). */
pg_status pg_energy_partition(const pg_grid* g, const double* vecs_dev, int nstates, const double* parts_dev,
                              double* out_host, void* stream);

/* A state's values on the grid in cube order (x slowest, z fastest) scaled
 * by 1/sqrt(dV), i.e. in bohr^-3/2 (DVR::GetWaveFnCube, src/DVR.cpp:2025-2074).
 * wf_host: N doubles; cube_host: N doubles.  dV uses each axis's own extent
 * (the reference takes all three at index nz-1: the same on cubic grids). */
pg_status pg_state_cube(const pg_grid* g, const double* wf_host, double* cube_host);

/* Cube file of a state, as DVR::WriteCubeFile (src/DVR.cpp:1887-2023):
 * cubeflag 1 = gOpenMol text grid, otherwise a Gaussian orbital cube (atom
 * count written negative, then the line "1 iwf").  Atoms: Z[natoms] and
 * pos_angstrom[3*natoms].  integral (may be NULL) receives sum rho^2 dV.
 * Written byte for byte as the reference writes it. */
pg_status pg_write_state_cube(const pg_grid* g, const double* wf_host, int iwf, const char* path, int natoms,
                              const int* Z, const double* pos_angstrom, int cubeflag, double* integral);

/* Gaussian cube of any grid function (WriteCubeFile, src/WriteCubeFile.cpp:
 * 17-78): npts[3] points from x0[3] in steps dx[3] (bohr), values
 * cube_host[npts0*npts1*npts2] with z fastest. */
pg_status pg_write_cube(const char* path, int natoms, const int* Z, const double* pos_angstrom, const int npts[3],
                        const double x0[3], const double dx[3], const double* cube_host);

/* Reads a Gaussian cube (ReadCubeFile, src/ReadCubeFile.cpp:17-104, which
 * reads the fixed name StartVector.cub): the grid into npts/x0/dx, the atom
 * count into natoms (may be NULL; negative for an orbital cube, whose
 * orbital line is skipped), and, if cube_host is not NULL, the values (z
 * fastest; PG_BAD_ARG if capacity is smaller than the grid).  Only
 * cartesian grids (PG_BAD_ARG otherwise; the reference exits). */
pg_status pg_read_cube(const char* path, int npts[3], double x0[3], double dx[3], int* natoms, double* cube_host,
                       long capacity);

/* Start vector from a wavefunction on a smaller equidistant grid (n[3]
 * points from xmin in steps dx, values in cube order as pg_read_cube
 * returns them): trilinear interpolation onto this grid's points, normalised
 * so that sum psi^2 = 1 (Small2Large, src/Small2Large.cpp:15-220, its
 * eight-point branch; the large grid is this grid's points x_0 + I L/(n+1)).
 * wf_dev receives N doubles. */
pg_status pg_small_to_large(const int n[3], const double xmin[3], const double dx[3], const double* wf_small_host,
                            const pg_grid* g, double* wf_dev, void* stream);

/* ---- Serving engine ------------------------------------------------------
 * A request loop for streams of single points (geometry-optimisation and
 * MD-snapshot streams): the role of the reference's repeated
 * ClusterAnion::EnergyFromConfiguration calls (src/ClusterAnion.cpp:192-290,
 * warm start istartvec = 0 after the first solve at :291), which the
 * reference runs one at a time.  Requests of different clusters, grids and
 * state counts are admitted while slots and device memory allow, run
 * concurrently on their own streams, warm-start from the last converged
 * eigenvectors of the same key, and have their mixed-form H*X products on a
 * shared grid merged into one tensor-core launch per axis. */
typedef struct pg_engine pg_engine;

typedef struct {
  int device;             /* CUDA device of the engine (-1: the calling thread's current device) */
  int slots;              /* solves in flight at once, one worker thread + stream each (default 8) */
  double memory_budget;   /* bytes of device memory admitted solves may need together (<= 0: 80% of free) */
  int batch_matvecs;      /* 1: merge concurrent mixed-form H*X products on the same grid */
  int batch_window_us;    /* how long a product waits for partners on its grid (default 200) */
  int warm_start;         /* 1: start from the cached eigenvectors of the request's key */
} pg_engine_config;

typedef struct {
  int n[3];
  double L[3];
  int nw;                       /* waters, 9 doubles each (O, H, H in Angstrom) */
  const double* waters;
  int nions;                    /* ions, 4 doubles each (x, y, z in Angstrom, charge) */
  const double* ions;
  pg_solve_params params;       /* startvec 1 or 2: used when no cached vectors exist */
  long key;                     /* warm-start key (e.g. base cluster id); < 0: none */
  double* evecs_host;           /* optional: receives nroots*N eigenvector values */
} pg_request;

typedef struct {
  long id;
  pg_status status;
  int nroots;
  int warm_started;             /* 1 if the solve started from cached vectors */
  double evals[64];
  pg_solve_stats stats;
  double queue_seconds;         /* submit -> start */
  double latency_seconds;       /* submit -> result */
  char error[256];
} pg_result;

typedef struct {
  long submitted, completed, failed;
  long warm_starts;
  long batches;                 /* merged H*X launches (one per axis counts once) */
  long batched_products;        /* products that went through them */
  int peak_in_flight;
  double peak_bytes;            /* largest admitted footprint sum */
} pg_engine_stats;

/* Footprint of one request in device bytes: the solve buffers (basis and
 * product blocks, their double-float twins in the mixed form, work array,
 * diagonal, potential, eigenvectors). */
double pg_request_footprint(const pg_request* r);
pg_status pg_engine_create(const pg_engine_config* c, pg_engine** out);
/* Copies the request's host data; returns at once.  PG_OOM if the request
 * alone exceeds the memory budget. */
pg_status pg_engine_submit(pg_engine* e, const pg_request* r, long* id);
/* Blocks until request id is done (timeout_s < 0: no limit) and hands over
 * its result; PG_DEVICE_TIMEOUT when the limit passes first. */
pg_status pg_engine_wait(pg_engine* e, long id, pg_result* out, double timeout_s);
/* Hands over up to max finished results in completion order. */
pg_status pg_engine_poll(pg_engine* e, pg_result* out, int max, int* nout);
pg_status pg_engine_get_stats(pg_engine* e, pg_engine_stats* out);
/* Finishes the admitted solves, fails the queued ones, joins the workers. */
pg_status pg_engine_destroy(pg_engine* e);

#ifdef __cplusplus
}
#endif
#endif
