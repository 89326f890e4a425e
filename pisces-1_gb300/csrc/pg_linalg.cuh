// Skinny FP64 linear algebra of the Davidson subspace on the device.
//
// Every reduction is deterministic: blocks write partial sums, and the
// partials of each output are added in a fixed order -- by a second launch,
// or, for the few-output norms, by whichever block of the producing kernel
// finishes last (reduce_in_last_block), in the same order.  Results therefore
// do not depend on scheduling, which keeps a solve bit-identical whether it
// runs alone or next to other solves.
#pragma once

#include "pg_common.cuh"

namespace pg {

constexpr int kRedBlocks = 296;  // partial-sum blocks of a reduction (2 per SM on 148+ SMs)
constexpr int kMaxGramOut = 2048;
constexpr int kMaxCombine = 16;  // columns produced by one combine launch

// Scratch for reductions; one per stream of work.
struct RedScratch {
  DevBuf<double> partial;     // kRedBlocks * kMaxGramOut
  DevBuf<unsigned> counter;   // arrival count of reduce_in_last_block (zero between launches)
  pg_status ensure();
};

// Ends a kernel whose block b has written its partial row partial[b*no + o],
// o < no, and that every thread of every block calls last.  The last block to
// arrive adds the rows of each output in the order of k_reduce_partials (one
// warp per output; lanes stride over the rows with eight loads in flight,
// then a shuffle tree), writes out[o] (and 1/sqrt(out[o]) at out[no + o] with
// sqrt_mode), and resets the counter for the next launch.
__device__ __forceinline__ void reduce_in_last_block(const double* partial, int no, double* out, int sqrt_mode,
                                                     unsigned* counter) {
  __shared__ int s_last;
  __threadfence();  // this block's partial row is visible to the last block
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int nb = (int)gridDim.x;
  const int lane = threadIdx.x & 31;
  for (int o = threadIdx.x >> 5; o < no; o += blockDim.x >> 5) {
    double s = 0;
    for (int b0 = 0; b0 < nb; b0 += 8 * 32) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int b = b0 + u * 32 + lane;
        v[u] = b < nb ? __ldcg(partial + (long)b * no + o) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) s += v[u];
    }
    for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
    if (lane == 0) {
      out[o] = s;
      if (sqrt_mode) out[no + o] = 1.0 / sqrt(s);
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// out[a*nb + b] = sum_g P[a*N + g] * Q[b*N + g]     (a < na, b < nb; na*nb <= kMaxGramOut)
// dfloat: products and sums in double-float (two-FP32) arithmetic, ~2^-48
// relative, on the FP32 pipe instead of the FP64 pipe.
// Pt / Qt (dfloat only, optional): double-float twins of P / Q, one float2
// (hi, lo) per point as written by split_twin or a combine's Yt, read instead
// of converting P / Q again.
// skip (optional, device): when *skip is nonzero at the time the launches
// run, they return at once and out is left as it was (a decision taken by an
// earlier kernel on the same stream, without a device-to-host read).
pg_status gram(long N, const double* P, int na, const double* Q, int nb, double* out, RedScratch& rs, cudaStream_t st,
               bool dfloat = false, const double* Pt = nullptr, const double* Qt = nullptr,
               const int* skip = nullptr);

// Y[r*N + g] = alpha_r * X[r*N + g] + cscale * sum_a P[a*N + g] * C[a*ca + r*cr]   (r < nr <= kMaxCombine)
// alpha_r: 0 if alpha is null; alpha[r] if inv_sqrt is false; 1/sqrt(alpha[r]) if true.
// X and P may equal Y (each point is read before it is written).  If sq is
// not null, sq[r] = |Y_r|^2 and sq[nr + r] = 1/|Y_r|.
// Pt (dfloat only, optional): twin of P, read instead of P; Yt (dfloat only,
// optional): receives the twin of Y.  Pt and Yt may overlap as P and Y may.
// skip: as for gram (Y, Yt and sq are left as they were).
pg_status combine(long N, const double* P, int na, const double* C, int ca, int cr, double cscale, const double* X,
                  const double* alpha, bool inv_sqrt, double* Y, int nr, double* sq, RedScratch& rs,
                  cudaStream_t st, bool dfloat = false, const double* Pt = nullptr, double* Yt = nullptr,
                  const int* skip = nullptr);

// t[i] = double-float twin of x[i] (float2 (hi, lo) in the 8 bytes of t[i]);
// with copy (not overlapping x), also copy[i] = x[i] in the same pass.
pg_status split_twin(long count, const double* x, double* t, cudaStream_t st, double* copy = nullptr);

// The Ritz step of the mixed form in one pass: U_r = B v_r and
// W_r = Z v_r - lambda_r U_r (r < nr) from the double-float twins Bt, Zt of
// the first m rows of B and Z, v_r = V[r*ldv ...] (device), lambda on the
// device; sq[r] = |U_r|^2 and sq[nr + r] = |W_r|^2.  U is not renormalised:
// with B orthonormal to double-float precision |U_r| = 1 to ~1e-14.
pg_status ritz_df(long N, const double* Bt, const double* Zt, int m, const double* V, int ldv, const double* lam,
                  double* U, double* W, int nr, double* sq, RedScratch& rs, cudaStream_t st);

}  // namespace pg
