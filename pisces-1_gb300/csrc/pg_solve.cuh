// Internal interfaces between the eigensolver (pg_davidson.cu), the
// tensor-core H*X (pg_hx_tc.cu), the serving engine (pg_serve.cu) and the
// self-consistent polarisation term with the dual grid built on it
// (pg_scpol.cu, pg_dual.cu).
#pragma once

#include <functional>

#include "pg_common.cuh"

namespace pg {

struct SolveWorkspace;
SolveWorkspace* workspace_create();
void workspace_destroy(SolveWorkspace* w);
double workspace_bytes(const SolveWorkspace* w);

// pg_solve with the H*X product supplied by the caller; ws (may be null)
// holds the solve buffers across calls.
pg_status solve_with(const pg_grid* g, const double* v, const pg_solve_params* p, double* evals, double* evecs,
                     pg_solve_stats* stats, cudaStream_t st,
                     const std::function<pg_status(const double*, double*, int)>& matvec, SolveWorkspace* ws);

// Start vectors of the reference (startvec 1: box product + random, 2: random)
// into B (nroots * N doubles); waits for st.
pg_status start_vectors(const pg_grid* g, int nroots, int startvec, double* B, cudaStream_t st);

// V(r) of a water cluster (default model) plus Bloomfield ions on the device.
pg_status cluster_potential(const pg_grid* g, int nw, const double* waters, int nions, const double* ions, double* v,
                            cudaStream_t st);

// v[g] += the self-consistent polarisation term for the grid points
// list[0 .. count) (all points, in order, if list is null; list on the
// device); the same term also added to vpol if not null.  Waits for st.
pg_status scpol_add_points(const pg_grid* g, const pg_sites* t, const pg_scpol_model* m, const int* list, long count,
                           double* v, double* vpol, cudaStream_t st);

constexpr int kMaxBatchJobs = 16;  // job-table entries of one tensor-core launch

// Mixed-form H*X of up to kMaxBatchJobs solves on the same grid: one launch per axis.
// unit: as for hx (every value of the X blocks in [-1, 1]).
pg_status hx_mixed_batch(const pg_grid* g, const double* const* v, const double* const* x, double* const* y,
                         const int* nvec, int njobs, cudaStream_t st, bool unit = false);

// The FP16-split kinetic preconditioner (pg_kin_f16.cu): R <- (T - sigma_v)^-1 R
// for the k contiguous vectors of R, with W1 and W2 k vectors of scratch each;
// sigma on the device; PG_UNSUPPORTED where the grid does not fit it.
bool kin_f16_ok(const pg_grid* g);
void kin_f16_plan_text(const pg_grid* g, char* buf, int len);
pg_status kin_f16(const pg_grid* g, double* R, double* w1, double* w2, int k, const double* sigma, double floor,
                  cudaStream_t st);

// The kinetic preconditioner R <- (T - sigma_v)^-1 R in the given arithmetic
// (pg_davidson.cu), scratch w1 and w2 of k vectors each.
pg_status kinetic_precondition(const pg_grid* g, double* R, int k, const double* sigma_dev, double* w1, double* w2,
                               int precision, cudaStream_t st);

}  // namespace pg
