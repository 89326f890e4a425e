// Skinny FP64 linear algebra of the Davidson subspace on the device.
//
// Every reduction is deterministic: blocks write partial sums, and a second
// launch adds the partials of each output in a fixed order.  Results
// therefore do not depend on scheduling, which keeps a solve bit-identical
// whether it runs alone or next to other solves.
#pragma once

#include "pg_common.cuh"

namespace pg {

constexpr int kRedBlocks = 296;  // partial-sum blocks of a reduction (2 per SM on 148+ SMs)
constexpr int kMaxGramOut = 2048;
constexpr int kMaxCombine = 16;  // columns produced by one combine launch

// Scratch for reductions; one per stream of work.
struct RedScratch {
  DevBuf<double> partial;     // kRedBlocks * kMaxGramOut
  pg_status ensure();
};

// out[o] = sum over b < nb of partial[b*no + o], in a fixed order; with
// sqrt_mode also out[no + o] = 1/sqrt(out[o]).
pg_status reduce_partials(const double* partial, int nb, int no, double* out, bool sqrt_mode, cudaStream_t st);

// out[a*nb + b] = sum_g P[a*N + g] * Q[b*N + g]     (a < na, b < nb; na*nb <= kMaxGramOut)
// dfloat: products and sums in double-float (two-FP32) arithmetic, ~2^-48
// relative, on the FP32 pipe instead of the FP64 pipe.
// Pt / Qt (dfloat only, optional): double-float twins of P / Q, one float2
// (hi, lo) per point as written by split_twin or a combine's Yt, read instead
// of converting P / Q again.
pg_status gram(long N, const double* P, int na, const double* Q, int nb, double* out, RedScratch& rs, cudaStream_t st,
               bool dfloat = false, const double* Pt = nullptr, const double* Qt = nullptr);

// Y[r*N + g] = alpha_r * X[r*N + g] + cscale * sum_a P[a*N + g] * C[a*ca + r*cr]   (r < nr <= kMaxCombine)
// alpha_r: 0 if alpha is null; alpha[r] if inv_sqrt is false; 1/sqrt(alpha[r]) if true.
// X and P may equal Y (each point is read before it is written).  If sq is
// not null, sq[r] = |Y_r|^2 and sq[nr + r] = 1/|Y_r|.
// Pt (dfloat only, optional): twin of P, read instead of P; Yt (dfloat only,
// optional): receives the twin of Y.  Pt and Yt may overlap as P and Y may.
pg_status combine(long N, const double* P, int na, const double* C, int ca, int cr, double cscale, const double* X,
                  const double* alpha, bool inv_sqrt, double* Y, int nr, double* sq, RedScratch& rs,
                  cudaStream_t st, bool dfloat = false, const double* Pt = nullptr, double* Yt = nullptr);

// t[i] = double-float twin of x[i] (float2 (hi, lo) in the 8 bytes of t[i]).
pg_status split_twin(long count, const double* x, double* t, cudaStream_t st);

}  // namespace pg
