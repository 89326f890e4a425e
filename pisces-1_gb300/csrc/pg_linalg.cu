// Deterministic skinny FP64 kernels for the Davidson subspace (see pg_linalg.cuh).
//
// Every reduction runs in two launches: blocks of the first write partial
// sums (one per output), the second reduces the partials of each output with
// one warp, in a fixed order.  No atomics, no dependence on scheduling.
#include <algorithm>
#include <cstdint>
#include <mutex>

#include "pg_linalg.cuh"

namespace pg {

namespace {

constexpr int kT = 256;
constexpr int kTP = 32;     // points per shared-memory tile in k_gram
constexpr int kBatch = 8;   // global loads a thread keeps in flight
constexpr int kStreamBlocks = 4 * kRedBlocks;  // blocks of the streaming kernels (about one point per thread)

long chunk_for(long N, int blocks, int align) {
  long c = (N + blocks - 1) / blocks;
  c = (c + align - 1) / align * align;
  return c > 0 ? c : align;
}

// out[o] = sum_b partial[b*no + o] over nb partial rows; one warp per output,
// lanes stride over the rows, then a fixed shuffle tree.  inv_sqrt_out: also
// store 1/sqrt(out[o]) at out[no + o] (used to normalise vectors on device).
__global__ void __launch_bounds__(kT) k_reduce_partials(const double* __restrict__ partial, int nb, int no,
                                                        double* __restrict__ out, int sqrt_mode,
                                                        const int* __restrict__ skip) {
  pdl_wait();
  pdl_release();
  if (skip && *skip) return;
  const int warp = (blockIdx.x * kT + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= no) return;
  double s = 0;
  for (int b0 = 0; b0 < nb; b0 += 8 * 32) {  // eight independent loads in flight per lane
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int b = b0 + u * 32 + lane;
      v[u] = b < nb ? partial[(long)b * no + warp] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) s += v[u];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) {
    out[warp] = s;
    if (sqrt_mode) out[no + warp] = 1.0 / sqrt(s);
  }
}

__global__ void __launch_bounds__(kT) k_gram(long N, long chunk, const double* __restrict__ P, int na,
                                             const double* __restrict__ Q, int nb, double* __restrict__ partial,
                                             const int* __restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ double sm[];
  double* Ps = sm;                       // na x (kTP+1)
  double* Qs = sm + na * (kTP + 1);      // nb x (kTP+1)
  const int no = na * nb;
  double acc[kMaxGramOut / kT];
#pragma unroll
  for (int s = 0; s < kMaxGramOut / kT; ++s) acc[s] = 0;
  const long g_begin = blockIdx.x * chunk;
  const long g_end = g_begin + chunk < N ? g_begin + chunk : N;
  for (long g0 = g_begin; g0 < g_end; g0 += kTP) {
    const int cnt = g_end - g0 < kTP ? (int)(g_end - g0) : kTP;
    // rows 0..na-1 from P, na..na+nb-1 from Q (Qs follows Ps); batched loads
    const int tot = (na + nb) * kTP;
    for (int e0 = threadIdx.x; e0 < tot; e0 += kBatch * kT) {
      double v[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * kT;
        const int row = e / kTP, p = e % kTP;
        const double* src = row < na ? P + (long)row * N : Q + (long)(row - na) * N;
        v[u] = (e < tot && p < cnt) ? src[g0 + p] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * kT;
        if (e < tot) Ps[(e / kTP) * (kTP + 1) + e % kTP] = v[u];
      }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < kMaxGramOut / kT; ++s) {
      const int o = threadIdx.x + s * kT;
      if (o < no) {
        const double* pa = Ps + (o / nb) * (kTP + 1);
        const double* qb = Qs + (o % nb) * (kTP + 1);
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;  // four chains hide the DFMA latency
#pragma unroll
        for (int p = 0; p < kTP; p += 4) {
          a0 += pa[p] * qb[p];
          a1 += pa[p + 1] * qb[p + 1];
          a2 += pa[p + 2] * qb[p + 2];
          a3 += pa[p + 3] * qb[p + 3];
        }
        acc[s] += (a0 + a1) + (a2 + a3);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int s = 0; s < kMaxGramOut / kT; ++s) {
    const int o = threadIdx.x + s * kT;
    if (o < no) partial[(long)blockIdx.x * no + o] = acc[s];
  }
}

template <int NR>
__global__ void __launch_bounds__(kT) k_combine(long N, long chunk, const double* P, int na,
                                                const double* __restrict__ C, int ca, int cr, double cscale,
                                                const double* X,
                                                const double* __restrict__ alpha, int inv_sqrt, double* Y, int nr,
                                                double* __restrict__ partial, double* sq_out, unsigned* counter,
                                                const int* __restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ double sm[];
  double* Cs = sm;                 // na x nr
  __shared__ double al[NR];
  __shared__ double red[kT / 32][NR];
  for (int e = threadIdx.x; e < na * nr; e += kT) Cs[e] = cscale * C[(long)(e / nr) * ca + (long)(e % nr) * cr];
  if (threadIdx.x < nr) {
    double a = 0;
    if (alpha) a = inv_sqrt ? 1.0 / sqrt(alpha[threadIdx.x]) : alpha[threadIdx.x];
    al[threadIdx.x] = a;
  }
  __syncthreads();
  double sacc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) sacc[r] = 0;
  const long g_begin = blockIdx.x * chunk;
  const long g_end = g_begin + chunk < N ? g_begin + chunk : N;
  for (long g = g_begin + threadIdx.x; g < g_end; g += kT) {
    double acc[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r) acc[r] = (r < nr && X && alpha) ? al[r] * X[(long)r * N + g] : 0.0;
    // eight independent loads in flight before they are consumed
    for (int a0 = 0; a0 < na; a0 += kBatch) {
      double pv[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) pv[u] = a0 + u < na ? P[(long)(a0 + u) * N + g] : 0.0;
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        if (a0 + u >= na) break;
        const double* c = Cs + (a0 + u) * nr;
#pragma unroll
        for (int r = 0; r < NR; ++r)
          if (r < nr) acc[r] += pv[u] * c[r];
      }
    }
#pragma unroll
    for (int r = 0; r < NR; ++r)
      if (r < nr) {
        Y[(long)r * N + g] = acc[r];
        sacc[r] += acc[r] * acc[r];
      }
  }
  if (!partial) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    double v = sacc[r];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < nr) {
    double s = 0;
    for (int w = 0; w < kT / 32; ++w) s += red[w][threadIdx.x];
    partial[(long)blockIdx.x * nr + threadIdx.x] = s;
  }
  reduce_in_last_block(partial, nr, sq_out, 1, counter);
}

// ------------------------------------------------------------------------
// Double-float (two FP32 numbers, hi + lo) arithmetic for the mixed form's
// subspace products.  The FP32 pipe of this part retires ~67 TFLOP/s against
// ~1 TFLOP/s for FP64; a double-float multiply-accumulate costs ~11 FP32
// operations and keeps ~48 significant bits (Dekker 1971, Knuth TwoSum).

// x = hi + lo to about 2^-48 |x| (hi takes the top 24 mantissa bits; the
// remaining 29 are rounded to the 24 of lo), with integer operations only
// (the FP64 pipe is not touched).  |x| < 2^-126 flushes to zero.  |x| >=
// 2^128 and Inf give hi = +-Inf, NaN gives hi = NaN (lo = 0), so a
// non-finite input reaches the products and norms built from the pair.
__device__ __forceinline__ void df_split(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t h = (uint32_t)(b >> 32);
  const int e = (int)((h >> 20) & 0x7ff);
  const int ef = e - 1023 + 127;
  if (ef <= 0) {
    hi = 0.f;
    lo = 0.f;
    return;
  }
  const uint32_t sign = h & 0x80000000u;
  if (ef >= 255) {
    const bool nan = e == 0x7ff && (b & 0xfffffffffffffull) != 0;
    hi = __uint_as_float(nan ? 0x7fc00000u : (sign | 0x7f800000u));
    lo = 0.f;
    return;
  }
  hi = __uint_as_float(sign | ((uint32_t)ef << 23) | (uint32_t)((b >> 29) & 0x7fffffu));
  const uint32_t rem = (uint32_t)(b & 0x1fffffffu);  // the 29 mantissa bits below hi
  const int el = e - 1075 + 127;                      // exponent of one unit of rem
  float scale = el > 0 ? __uint_as_float((uint32_t)el << 23) : 0.f;
  const float l = __uint2float_rn(rem) * scale;
  lo = sign ? -l : l;
}

// (sh, sl) += a * b with a = (ah, al), b = (bh, bl)
__device__ __forceinline__ void df_fma(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  const float t = sh + p;
  const float bp = t - sh;
  const float err = (sh - (t - bp)) + (p - bp);
  sl += err + e;
  sh = t;
}

// Gram partials in double-float, written as double (hi + lo): same contract
// as k_gram.  A thread owns a kGA x kGB block of outputs (kGA rows of P
// against kGB rows of Q) for one slice of the points of each tile, so every
// point value it reads from shared memory feeds kGB or kGA products.  Tiles of
// tp points of all na + nb rows stream through kGStages shared-memory stages
// with cp.async (each thread converts the doubles it copied to (hi, lo) pairs
// in place once they land), keeping two tiles in flight behind the one being
// multiplied.  At the end the slices of each output block are summed in a
// fixed order.
constexpr int kGA = 4, kGB = 4, kGStages = 3;
constexpr int kGramSmemMax = 112 * 1024;

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_stages() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(kGStages - 2) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Tile geometry of k_gram_df: S slices per output block, tiles of tp = 2 S m
// points so that every slice takes exactly m point pairs of every tile (no
// lanes idle in the multiply loop), as many pairs as kGStages stages of
// (na + nb) rows allow in kGramSmemMax.
struct GramGeom {
  int ablk, nblk, S, m, tp;
  size_t smem;
};

inline GramGeom gram_geometry(int na, int nb) {
  GramGeom g;
  g.ablk = (na + kGA - 1) / kGA;
  g.nblk = g.ablk * ((nb + kGB - 1) / kGB);
  g.S = g.nblk <= kT ? kT / g.nblk : 1;
  const size_t per_pair_set = (size_t)kGStages * (na + nb) * 2 * g.S * 8;  // stage bytes per unit of m
  g.m = (int)std::max<size_t>(1, std::min<size_t>(8, kGramSmemMax / per_pair_set));
  g.tp = 2 * g.S * g.m;
  g.smem = std::max((size_t)g.m * per_pair_set, (size_t)g.S * g.nblk * kGA * kGB * 8);
  return g;
}

// kPair: N even and P, Q 16-byte aligned, so that consecutive point pairs
// are copied with 16-byte cp.async and converted two at a time.
// split_p / split_q: the rows of P / Q are already double-float "twins" (a
// float2 (hi, lo) per point, the layout the staging converts to), copied as
// they are and not converted again.
template <bool kPair>
__global__ void __launch_bounds__(kT, 2) k_gram_df(long N, long chunk, const double* __restrict__ P, int na,
                                                   const double* __restrict__ Q, int nb, int tp, int m, int S,
                                                   int ablk, int nblk, int split_p, int split_q,
                                                   double* __restrict__ partial, const int* __restrict__ skip) {
  pdl_wait();
  pdl_release();
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char gsm[];
  const int rows = na + nb;
  const int hp = tp >> 1;  // point pairs per tile row
  const int stage_elems = rows * tp;
  double* stage0 = reinterpret_cast<double*>(gsm);
  const long g_begin = blockIdx.x * chunk;
  const long g_end = g_begin + chunk < N ? g_begin + chunk : N;
  const int ntiles = g_end > g_begin ? (int)((g_end - g_begin + tp - 1) / tp) : 0;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int blk = tid / S, slice = tid - blk * S;
  const bool active = blk < nblk;
  const int a0 = (blk % ablk) * kGA, b0 = (blk / ablk) * kGB;
  int ra[kGA], rb[kGB];  // stage rows of this thread's outputs (clamped; extra outputs are discarded)
#pragma unroll
  for (int i = 0; i < kGA; ++i) ra[i] = (a0 + i < na ? a0 + i : na - 1) * hp;
#pragma unroll
  for (int j = 0; j < kGB; ++j) rb[j] = (na + (b0 + j < nb ? b0 + j : nb - 1)) * hp;
  float sh[kGA][kGB], sl[kGA][kGB];
#pragma unroll
  for (int i = 0; i < kGA; ++i)
#pragma unroll
    for (int j = 0; j < kGB; ++j) sh[i][j] = sl[i][j] = 0.f;

  // staging: warp w copies rows w, w + 8, ...; its lanes stride over the row
  auto issue = [&](int tile) {
    double* dst = stage0 + (size_t)(tile % kGStages) * stage_elems;
    const long g0 = g_begin + (long)tile * tp;
    const int cnt = g_end - g0 < tp ? (int)(g_end - g0) : tp;
    for (int row = warp; row < rows; row += kT / 32) {
      const double* src = (row < na ? P + (long)row * N : Q + (long)(row - na) * N) + g0;
      double* d = dst + (size_t)row * tp;
      if (kPair) {
        for (int q = lane; q < hp; q += 32) {
          const int p = 2 * q;
          if (p + 1 < cnt) {
            cp_async16(d + p, src + p);
          } else if (p < cnt) {
            cp_async8(d + p, src + p);
            d[p + 1] = 0.0;
          } else {
            d[p] = 0.0;
            d[p + 1] = 0.0;
          }
        }
      } else {
        for (int p = lane; p < tp; p += 32) {
          if (p < cnt) cp_async8(d + p, src + p);
          else d[p] = 0.0;
        }
      }
    }
  };
  for (int t = 0; t < kGStages - 1; ++t) {
    if (t < ntiles) issue(t);
    cp_async_commit();
  }
  for (int it = 0; it < ntiles; ++it) {
    cp_async_wait_stages();  // this thread's copies of tile `it` have landed
    double* cur = stage0 + (size_t)(it % kGStages) * stage_elems;
    // convert the points this thread copied, in place, to (hi, lo) pairs
    for (int row = warp; row < rows; row += kT / 32) {
      if (row < na ? split_p : split_q) continue;  // a twin row: already (hi, lo)
      double* d = cur + (size_t)row * tp;
      if (kPair) {
        for (int q = lane; q < hp; q += 32) {
          const double2 d2 = *reinterpret_cast<const double2*>(d + 2 * q);
          float h0, l0, h1, l1;
          df_split(d2.x, h0, l0);
          df_split(d2.y, h1, l1);
          *reinterpret_cast<float4*>(d + 2 * q) = make_float4(h0, l0, h1, l1);
        }
      } else {
        for (int p = lane; p < tp; p += 32) {
          float h, l;
          df_split(d[p], h, l);
          *reinterpret_cast<float2*>(d + p) = make_float2(h, l);
        }
      }
    }
    __syncthreads();  // tile `it` converted; everyone is done with tile it-1
    if (it + kGStages - 1 < ntiles) issue(it + kGStages - 1);
    cp_async_commit();
    if (active) {
      // m point pairs per slice (one 16-byte load per row each; zero points
      // past the tile's end add nothing)
      const float4* cur4 = reinterpret_cast<const float4*>(cur);
      for (int u = 0; u < m; ++u) {
        const int q = slice + u * S;
        float4 y[kGB];
#pragma unroll
        for (int j = 0; j < kGB; ++j) y[j] = cur4[rb[j] + q];
#pragma unroll
        for (int i = 0; i < kGA; ++i) {
          const float4 x = cur4[ra[i] + q];
#pragma unroll
          for (int j = 0; j < kGB; ++j) {
            df_fma(sh[i][j], sl[i][j], x.x, x.y, y[j].x, y[j].y);
            df_fma(sh[i][j], sl[i][j], x.z, x.w, y[j].z, y[j].w);
          }
        }
      }
    }
  }
  cp_async_wait_all();
  __syncthreads();
  // slices -> one partial per output, summed in slice order
  double* red = reinterpret_cast<double*>(gsm);
  if (active) {
#pragma unroll
    for (int i = 0; i < kGA; ++i)
#pragma unroll
      for (int j = 0; j < kGB; ++j)
        red[((size_t)slice * nblk + blk) * (kGA * kGB) + i * kGB + j] = (double)sh[i][j] + (double)sl[i][j];
  }
  __syncthreads();
  const int no = na * nb;
  for (int o = tid; o < no; o += kT) {
    const int a = o / nb, b = o - (o / nb) * nb;
    const int bo = a / kGA + (b / kGB) * ablk;
    const int k = (a % kGA) * kGB + (b % kGB);
    double acc = 0;
    for (int q = 0; q < S; ++q) acc += red[((size_t)q * nblk + bo) * (kGA * kGB) + k];
    partial[(long)blockIdx.x * no + o] = acc;
  }
}

// Combine in double-float: same contract as k_combine (coefficients and
// alpha are FP64 and split once per block; Y is written as double).
// kTwinIn: the rows of P are double-float twins (float2 (hi, lo) per point)
// and are read without converting; kTwinOut: each output is also written as
// its twin to Yt.  Compile-time flags: a runtime choice inside the unrolled
// loop doubles the registers of the kernel and halves its occupancy.  Up to 4
// outputs the kernel fits 64 registers (4 blocks per SM, no spills).
template <int NR, bool kTwinIn, bool kTwinOut>
__global__ void __launch_bounds__(kT, NR <= 4 ? 4 : 2) k_combine_df(long N, long chunk, const double* P, int na,
                                                   const double* __restrict__ C, int ca, int cr, double cscale,
                                                   const double* X, const double* __restrict__ alpha, int inv_sqrt,
                                                   double* Y, int nr, float2* Yt, double* __restrict__ partial,
                                                   double* sq_out, unsigned* counter, const int* __restrict__ skip) {
  pdl_wait();
  pdl_release();
  if (skip && *skip) return;
  extern __shared__ float smf[];
  float* Ch = smf;              // na x nr
  float* Cl = smf + na * nr;
  __shared__ float alh[NR], all[NR];
  __shared__ double red[kT / 32][NR];
  for (int e = threadIdx.x; e < na * nr; e += kT) {
    float h, l;
    df_split(cscale * C[(long)(e / nr) * ca + (long)(e % nr) * cr], h, l);
    Ch[e] = h;
    Cl[e] = l;
  }
  if (threadIdx.x < nr) {
    double a = 0;
    if (alpha) a = inv_sqrt ? 1.0 / sqrt(alpha[threadIdx.x]) : alpha[threadIdx.x];
    float h, l;
    df_split(a, h, l);
    alh[threadIdx.x] = h;
    all[threadIdx.x] = l;
  }
  __syncthreads();
  double sacc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) sacc[r] = 0;
  const bool keep = X && alpha;
  const long g_begin = blockIdx.x * chunk;
  const long g_end = g_begin + chunk < N ? g_begin + chunk : N;
  for (long g = g_begin + threadIdx.x; g < g_end; g += kT) {
    float sh[NR], sl[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      sh[r] = 0.f;
      sl[r] = 0.f;
      if (r < nr && keep) {
        float xh, xl;
        df_split(X[(long)r * N + g], xh, xl);
        df_fma(sh[r], sl[r], alh[r], all[r], xh, xl);
      }
    }
    for (int a0 = 0; a0 < na; a0 += kBatch) {
      double pv[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) pv[u] = a0 + u < na ? P[(long)(a0 + u) * N + g] : 0.0;
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        if (a0 + u >= na) break;
        float ph, pl;
        if (kTwinIn) {  // the 8 bytes are a float2 (hi, lo): hi in the low word
          ph = __int_as_float(__double2loint(pv[u]));
          pl = __int_as_float(__double2hiint(pv[u]));
        } else {
          df_split(pv[u], ph, pl);
        }
        const float* ch = Ch + (a0 + u) * nr;
        const float* cl = Cl + (a0 + u) * nr;
#pragma unroll
        for (int r = 0; r < NR; ++r)
          if (r < nr) df_fma(sh[r], sl[r], ph, pl, ch[r], cl[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < NR; ++r)
      if (r < nr) {
        const double y = (double)sh[r] + (double)sl[r];
        Y[(long)r * N + g] = y;
        // the accumulator pair is the output in double-float form already
        // (it and y = sh + sl agree to 2^-53 relative)
        if (kTwinOut) Yt[(long)r * N + g] = make_float2(sh[r], sl[r]);
        sacc[r] += y * y;
      }
  }
  if (!partial) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    double v = sacc[r];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < nr) {
    double s = 0;
    for (int w = 0; w < kT / 32; ++w) s += red[w][threadIdx.x];
    partial[(long)blockIdx.x * nr + threadIdx.x] = s;
  }
  reduce_in_last_block(partial, nr, sq_out, 1, counter);
}

// out[o] = sum of partial[b*no + o] over the nb rows, in a fixed order (k_reduce_partials)
pg_status reduce(const double* partial, int nb, int no, double* out, bool sqrt_mode, cudaStream_t st,
                 const int* skip = nullptr) {
  const int blocks = (no * 32 + kT - 1) / kT;
  PG_CUDA_TRY(launch_dependent(k_reduce_partials, dim3(blocks), dim3(kT), 0, st, partial, nb, no, out,
                               sqrt_mode ? 1 : 0, skip));
  return check_launch("k_reduce_partials");
}

}  // namespace

pg_status RedScratch::ensure() {
  if (!partial.p) PG_TRY(partial.alloc((size_t)kRedBlocks * kMaxGramOut));
  if (!counter.p) {
    PG_TRY(counter.alloc(1));
    PG_CUDA_TRY(cudaMemset(counter.p, 0, sizeof(unsigned)));
  }
  return PG_OK;
}

// Double-float twins of count doubles: t[i] = (hi, lo) of x[i] (df_split);
// with y, also y[i] = x[i] (a copy and its twin in one pass).
__global__ void __launch_bounds__(kT) k_split_twin(long count, const double* __restrict__ x, float2* __restrict__ t,
                                                   double* __restrict__ y) {
  pdl_wait();
  pdl_release();
  for (long i = blockIdx.x * (long)kT + threadIdx.x; i < count; i += (long)gridDim.x * kT) {
    const double v = x[i];
    float h, l;
    df_split(v, h, l);
    t[i] = make_float2(h, l);
    if (y) y[i] = v;
  }
}

// 16-byte copies of point pairs: every row start 16-byte aligned
inline bool pair_ok(long N, const double* P, const double* Q) {
  return N % 2 == 0 && ((uintptr_t)P % 16) == 0 && ((uintptr_t)Q % 16) == 0;
}

// Dynamic shared-memory opt-in, once per kernel (the largest size any call
// needs: 112 + 16 vectors of 33 doubles for the Gram kernels).
static pg_status opt_in_smem() {
  static const cudaError_t init = [] {  // thread-safe static initialisation
    const int big = (int)(sizeof(double) * (size_t)(128 + 16) * (kTP + 1));
    cudaError_t e = cudaFuncSetAttribute(k_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_gram_df<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGramSmemMax);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_gram_df<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGramSmemMax);
    return e;
  }();
  PG_CUDA_TRY(init);
  return PG_OK;
}

pg_status gram(long N, const double* P, int na, const double* Q, int nb, double* out, RedScratch& rs,
               cudaStream_t st, bool dfloat, const double* Pt, const double* Qt, const int* skip) {
  PG_ARG(na > 0 && nb > 0 && na * nb <= kMaxGramOut && na + nb <= 144, "gram: %d x %d outputs exceed the limits",
         na, nb);
  PG_TRY(rs.ensure());
  PG_TRY(opt_in_smem());
  const long chunk = chunk_for(N, kRedBlocks, kTP);
  const int blocks = (int)((N + chunk - 1) / chunk);
  if (dfloat) {
    const GramGeom gg = gram_geometry(na, nb);
    PG_ARG(gg.nblk <= kT, "gram: %d output blocks", gg.nblk);  // at most ~160 within the limits above
    const long dchunk = chunk_for(N, kRedBlocks, gg.tp);
    const int dblocks = (int)((N + dchunk - 1) / dchunk);
    const double* Ps = Pt ? Pt : P;
    const double* Qs = Qt ? Qt : Q;
    const int sp = Pt ? 1 : 0, sq = Qt ? 1 : 0;
    if (pair_ok(N, Ps, Qs))
      PG_CUDA_TRY(launch_dependent(k_gram_df<true>, dim3(dblocks), dim3(kT), gg.smem, st, N, dchunk, Ps, na, Qs, nb,
                                   gg.tp, gg.m, gg.S, gg.ablk, gg.nblk, sp, sq, rs.partial.p, skip));
    else
      PG_CUDA_TRY(launch_dependent(k_gram_df<false>, dim3(dblocks), dim3(kT), gg.smem, st, N, dchunk, Ps, na, Qs,
                                   nb, gg.tp, gg.m, gg.S, gg.ablk, gg.nblk, sp, sq, rs.partial.p, skip));
    PG_TRY(check_launch("k_gram_df"));
    return reduce(rs.partial.p, dblocks, na * nb, out, false, st, skip);
  } else {
    const size_t smem = sizeof(double) * (size_t)(na + nb) * (kTP + 1);
    k_gram<<<blocks, kT, smem, st>>>(N, chunk, P, na, Q, nb, rs.partial.p, skip);
    PG_TRY(check_launch("k_gram"));
  }
  return reduce(rs.partial.p, blocks, na * nb, out, false, st, skip);
}

pg_status combine(long N, const double* P, int na, const double* C, int ca, int cr, double cscale, const double* X,
                  const double* alpha, bool inv_sqrt, double* Y, int nr, double* sq, RedScratch& rs,
                  cudaStream_t st, bool dfloat, const double* Pt, double* Yt, const int* skip) {
  PG_ARG(nr > 0 && nr <= kMaxCombine && na >= 0 && na * nr <= 128 * kMaxCombine, "combine: bad sizes na=%d nr=%d",
         na, nr);
  PG_TRY(rs.ensure());
  PG_TRY(opt_in_smem());
  const long chunk = chunk_for(N, kStreamBlocks, kT);
  const int blocks = (int)((N + chunk - 1) / chunk);
  if (dfloat) {
    const size_t smem = sizeof(float) * 2 * (size_t)(na > 0 ? na : 1) * nr;
#define PG_COMBINE_DF3(NRV, TI, TO)                                                                                \
  PG_CUDA_TRY(launch_dependent(k_combine_df<NRV, TI, TO>, dim3(blocks), dim3(kT), smem, st, N, chunk, Pt ? Pt : P, na, \
                               C, ca, cr, cscale, X, alpha, inv_sqrt ? 1 : 0, Y, nr, reinterpret_cast<float2*>(Yt),  \
                               sq ? rs.partial.p : nullptr, sq, rs.counter.p, skip))
#define PG_COMBINE_DF(NRV)                                             \
  do {                                                                 \
    if (Pt && Yt) PG_COMBINE_DF3(NRV, true, true);                     \
    else if (Pt) PG_COMBINE_DF3(NRV, true, false);                     \
    else if (Yt) PG_COMBINE_DF3(NRV, false, true);                     \
    else PG_COMBINE_DF3(NRV, false, false);                            \
  } while (0)
    if (nr <= 1) PG_COMBINE_DF(1);
    else if (nr <= 2) PG_COMBINE_DF(2);
    else if (nr <= 4) PG_COMBINE_DF(4);
    else if (nr <= 8) PG_COMBINE_DF(8);
    else PG_COMBINE_DF(16);
#undef PG_COMBINE_DF
#undef PG_COMBINE_DF3
    PG_TRY(check_launch("k_combine_df"));
  } else {
    const size_t smem = sizeof(double) * (size_t)(na > 0 ? na : 1) * nr;
#define PG_COMBINE(NRV) \
  k_combine<NRV><<<blocks, kT, smem, st>>>(N, chunk, P, na, C, ca, cr, cscale, X, alpha, inv_sqrt ? 1 : 0, Y, nr, \
                                           sq ? rs.partial.p : nullptr, sq, rs.counter.p, skip)
    if (nr <= 1) PG_COMBINE(1);
    else if (nr <= 2) PG_COMBINE(2);
    else if (nr <= 4) PG_COMBINE(4);
    else if (nr <= 8) PG_COMBINE(8);
    else PG_COMBINE(16);
#undef PG_COMBINE
    PG_TRY(check_launch("k_combine"));
  }
  return PG_OK;  // with sq, the kernel's last block has reduced the norms
}

// FP32 -> FP64 with integer operations (exact for normal numbers and zero;
// FP32 subnormals flush to a signed zero; Inf and NaN are kept): keeps the
// conversion off the FP64 pipe, which retires about two operations per SM
// per clock on this part.
__device__ __forceinline__ double f32_to_f64_int(float v) {
  const uint32_t u = __float_as_uint(v);
  const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xffu, mt = u & 0x7fffffu;
  uint32_t hi = sign | ((e + 896u) << 20) | (mt >> 3);
  uint32_t lo = mt << 29;
  hi = e == 0 ? sign : hi;
  lo = e == 0 ? 0u : lo;
  hi = e == 255 ? (sign | 0x7ff00000u | (mt >> 3) | (mt ? 0x80000u : 0u)) : hi;
  lo = e == 255 ? 0u : lo;
  return __hiloint2double((int)hi, (int)lo);
}

// The Ritz step of the mixed form in one pass: U_r = B v_r and
// W_r = Z v_r - lambda_r U_r in double-float from the twins of the m rows of
// B and Z (v_r = column r of V, leading dimension ldv), written as FP64, and
// |U_r|^2, |W_r|^2 (squares summed in FP32 per thread, in FP64 across threads)
// reduced by the last block into out[r] and out[nr + r].  Two FP64 additions
// per output and point (the pairs to FP64); the rest runs on the FP32 pipe.
template <int NR>
__global__ void __launch_bounds__(kT, NR <= 4 ? 3 : 2) k_ritz_df(long N, long chunk, const double* Bt, const double* Zt,
                                                               int m, const double* __restrict__ V, int ldv,
                                                               const double* __restrict__ lam, double* U, double* W,
                                                               int nr, double* __restrict__ partial, double* out,
                                                               unsigned* counter) {
  pdl_wait();
  pdl_release();
  extern __shared__ float smf[];
  float* Ch = smf;  // m x nr
  float* Cl = smf + m * nr;
  __shared__ float nlh[NR], nll[NR];
  __shared__ double red[kT / 32][2 * NR];
  for (int e = threadIdx.x; e < m * nr; e += kT) {
    float h, l;
    df_split(V[(long)(e / nr) + (long)(e % nr) * ldv], h, l);
    Ch[e] = h;
    Cl[e] = l;
  }
  if (threadIdx.x < nr) {
    float h, l;
    df_split(-lam[threadIdx.x], h, l);
    nlh[threadIdx.x] = h;
    nll[threadIdx.x] = l;
  }
  __syncthreads();
  float su[NR], sw[NR];  // about one point per thread: FP32 sums of the squares
#pragma unroll
  for (int r = 0; r < NR; ++r) su[r] = sw[r] = 0.f;
  const long g_begin = blockIdx.x * chunk;
  const long g_end = g_begin + chunk < N ? g_begin + chunk : N;
  for (long g = g_begin + threadIdx.x; g < g_end; g += kT) {
    float uh[NR], ul[NR], zh[NR], zl[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r) uh[r] = ul[r] = zh[r] = zl[r] = 0.f;
    for (int a0 = 0; a0 < m; a0 += kBatch / 2) {
      double pb[kBatch / 2], pz[kBatch / 2];
#pragma unroll
      for (int u = 0; u < kBatch / 2; ++u) {
        pb[u] = a0 + u < m ? Bt[(long)(a0 + u) * N + g] : 0.0;
        pz[u] = a0 + u < m ? Zt[(long)(a0 + u) * N + g] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kBatch / 2; ++u) {
        if (a0 + u >= m) break;
        // the 8 bytes are a float2 (hi, lo): hi in the low word
        const float bh = __int_as_float(__double2loint(pb[u])), bl = __int_as_float(__double2hiint(pb[u]));
        const float qh = __int_as_float(__double2loint(pz[u])), ql = __int_as_float(__double2hiint(pz[u]));
        const float* ch = Ch + (a0 + u) * nr;
        const float* cl = Cl + (a0 + u) * nr;
#pragma unroll
        for (int r = 0; r < NR; ++r)
          if (r < nr) {
            df_fma(uh[r], ul[r], bh, bl, ch[r], cl[r]);
            df_fma(zh[r], zl[r], qh, ql, ch[r], cl[r]);
          }
      }
    }
#pragma unroll
    for (int r = 0; r < NR; ++r)
      if (r < nr) {
        df_fma(zh[r], zl[r], nlh[r], nll[r], uh[r], ul[r]);  // W = Z v - lambda U
        const double u = f32_to_f64_int(uh[r]) + f32_to_f64_int(ul[r]);
        const double w = f32_to_f64_int(zh[r]) + f32_to_f64_int(zl[r]);
        U[(long)r * N + g] = u;
        W[(long)r * N + g] = w;
        // the pair's sum in FP32 (after the cancellation in W its low part
        // need not be small against its high part), then its square
        const float uf = uh[r] + ul[r], wf = zh[r] + zl[r];
        su[r] = fmaf(uf, uf, su[r]);
        sw[r] = fmaf(wf, wf, sw[r]);
      }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    // sums of 16 lanes in FP32 (2^-22 relative at most), the last step and
    // everything after it in FP64: few operations on the FP64 pipe
    float af = su[r], bf = sw[r];
    for (int o = 16; o > 1; o >>= 1) {
      af += __shfl_down_sync(0xffffffffu, af, o);
      bf += __shfl_down_sync(0xffffffffu, bf, o);
    }
    double a = f32_to_f64_int(af), b = f32_to_f64_int(bf);
    a += __shfl_down_sync(0xffffffffu, a, 1);
    b += __shfl_down_sync(0xffffffffu, b, 1);
    if (lane == 0) {
      red[warp][r] = a;
      red[warp][NR + r] = b;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * nr) {
    const int o = threadIdx.x < nr ? threadIdx.x : NR + threadIdx.x - nr;
    double t = 0;
    for (int w = 0; w < kT / 32; ++w) t += red[w][o];
    partial[(long)blockIdx.x * 2 * nr + threadIdx.x] = t;
  }
  reduce_in_last_block(partial, 2 * nr, out, 0, counter);
}

pg_status ritz_df(long N, const double* Bt, const double* Zt, int m, const double* V, int ldv, const double* lam,
                  double* U, double* W, int nr, double* sq, RedScratch& rs, cudaStream_t st) {
  PG_ARG(m > 0 && nr > 0 && nr <= kMaxCombine && m * nr <= 128 * kMaxCombine && Bt && Zt,
         "ritz_df: bad sizes m=%d nr=%d", m, nr);
  PG_TRY(rs.ensure());
  const long chunk = chunk_for(N, kStreamBlocks, kT);
  const int blocks = (int)((N + chunk - 1) / chunk);
  const size_t smem = sizeof(float) * 2 * (size_t)m * nr;
#define PG_RITZ_DF(NRV)                                                                                           \
  PG_CUDA_TRY(launch_dependent(k_ritz_df<NRV>, dim3(blocks), dim3(kT), smem, st, N, chunk, Bt, Zt, m, V, ldv, lam, U, \
                               W, nr, rs.partial.p, sq, rs.counter.p))
  if (nr <= 1) PG_RITZ_DF(1);
  else if (nr <= 2) PG_RITZ_DF(2);
  else if (nr <= 4) PG_RITZ_DF(4);
  else if (nr <= 8) PG_RITZ_DF(8);
  else PG_RITZ_DF(16);
#undef PG_RITZ_DF
  return check_launch("k_ritz_df");
}

pg_status split_twin(long count, const double* x, double* t, cudaStream_t st, double* copy) {
  if (count <= 0) return PG_OK;
  const long b = (count + kT - 1) / kT;
  PG_CUDA_TRY(launch_dependent(k_split_twin, dim3((unsigned)(b < 152L * 8 ? b : 152L * 8)), dim3(kT), 0, st, count, x,
                               reinterpret_cast<float2*>(t), copy));
  return check_launch("k_split_twin");
}


// The reduction scratch of the public block products: one per calling
// thread and device (a buffer allocated on one device is not used on another).
constexpr int kScratchDevices = 64;
pg_status thread_scratch(RedScratch** out) {
  static thread_local RedScratch rs[kScratchDevices];
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev));
  PG_ARG(dev >= 0 && dev < kScratchDevices, "block products: device %d out of range", dev);
  *out = &rs[dev];
  return PG_OK;
}

}  // namespace pg

extern "C" pg_status pg_block_gram(long n, const double* P, int np, const double* Q, int nq, double* out,
                                   int precision, void* stream) {
  PG_ARG(n > 0 && P && Q && out && np > 0 && nq > 0, "pg_block_gram: bad arguments");
  PG_ARG(precision == PG_FP64 || precision == PG_MIXED, "pg_block_gram: unknown precision");
  pg::RedScratch* rs = nullptr;
  PG_TRY(pg::thread_scratch(&rs));
  return pg::gram(n, P, np, Q, nq, out, *rs, pg::as_stream(stream), precision == PG_MIXED);
}

extern "C" pg_status pg_block_combine(long n, const double* P, int np, const double* C, int ny, double* Y,
                                      int precision, void* stream) {
  PG_ARG(n > 0 && P && C && Y && np > 0 && ny > 0, "pg_block_combine: bad arguments");
  PG_ARG(precision == PG_FP64 || precision == PG_MIXED, "pg_block_combine: unknown precision");
  pg::RedScratch* rs = nullptr;
  PG_TRY(pg::thread_scratch(&rs));
  return pg::combine(n, P, np, C, ny, 1, 1.0, nullptr, nullptr, false, Y, ny, nullptr, *rs, pg::as_stream(stream),
                     precision == PG_MIXED);
}

extern "C" pg_status pg_split_twin(long n, const double* x, double* twin, void* stream) {
  PG_ARG(n > 0 && x && twin && x != twin, "pg_split_twin: bad arguments");
  return pg::split_twin(n, x, twin, pg::as_stream(stream));
}

extern "C" pg_status pg_block_gram_twin(long n, const double* Pt, int np, const double* Qt, int nq, double* out,
                                        void* stream) {
  PG_ARG(n > 0 && Pt && Qt && out && np > 0 && nq > 0, "pg_block_gram_twin: bad arguments");
  pg::RedScratch* rs = nullptr;
  PG_TRY(pg::thread_scratch(&rs));
  return pg::gram(n, Pt, np, Qt, nq, out, *rs, pg::as_stream(stream), true, Pt, Qt);
}

extern "C" pg_status pg_block_combine_twin(long n, const double* Pt, int np, const double* C, int ny, double* Y,
                                           double* Yt, void* stream) {
  PG_ARG(n > 0 && Pt && C && Y && np > 0 && ny > 0, "pg_block_combine_twin: bad arguments");
  pg::RedScratch* rs = nullptr;
  PG_TRY(pg::thread_scratch(&rs));
  return pg::combine(n, Pt, np, C, ny, 1, 1.0, nullptr, nullptr, false, Y, ny, nullptr, *rs, pg::as_stream(stream),
                     true, Pt, Yt);
}

// ---------------------------------------------------------------------------
// pg_block_gram_noalloc: pg_block_gram for callers that may not allocate
// device memory.  The per-block partial sums live in a fixed file-scope
// device array instead of a cudaMalloc'd buffer; the kernels and the
// reduction order are pg_block_gram's, so the results are bit-identical.
namespace {

constexpr int kNoAllocMaxOut = 256;  // np * nq limit of this entry point
constexpr long kNoAllocPartials = (long)pg::kRedBlocks * kNoAllocMaxOut;  // 75,776 doubles = 592 KiB

// Nothing here needs to start at zero: each call writes every partial it
// reads back.  One array per device, shared by every caller of the entry point.
__device__ __align__(256) double g_noalloc_partial[kNoAllocPartials];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_m;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

}  // namespace

extern "C" pg_status pg_block_gram_noalloc(long n, const double* P, int np, const double* Q, int nq, double* out,
                                           int precision, void* stream) {
  using namespace pg;
  PG_ARG(n > 0 && P && Q && out && np > 0 && nq > 0, "pg_block_gram_noalloc: bad arguments");
  PG_ARG(precision == PG_FP64 || precision == PG_MIXED, "pg_block_gram_noalloc: unknown precision");
  PG_ARG((long)np * nq <= kNoAllocMaxOut,
         "pg_block_gram_noalloc: %d x %d = %ld outputs exceed this entry point's fixed scratch (at most %d "
         "outputs; use pg_block_gram)",
         np, nq, (long)np * nq, kNoAllocMaxOut);
  PG_ARG(np + nq <= 144, "pg_block_gram_noalloc: np + nq = %d exceeds 144", np + nq);
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev));
  PG_ARG(dev >= 0 && dev < kNoAllocMaxDevices, "pg_block_gram_noalloc: device %d out of range", dev);
  double* partial = nullptr;
  {
    // first call on a device: the address of the scratch array in this
    // device's context (no allocation; done before any stream capture)
    std::lock_guard<std::mutex> l(g_noalloc_m);
    if (!g_noalloc_ptr[dev]) {
      void* addr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_partial);
      if (e != cudaSuccess || !addr) {
        set_error("pg_block_gram_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return PG_CUDA;
      }
      g_noalloc_ptr[dev] = static_cast<double*>(addr);
    }
    partial = g_noalloc_ptr[dev];
  }
  PG_TRY(opt_in_smem());
  cudaStream_t st = as_stream(stream);
  const int no = np * nq;
  if (precision == PG_MIXED) {
    const GramGeom gg = gram_geometry(np, nq);
    PG_ARG(gg.nblk <= kT, "pg_block_gram_noalloc: %d output blocks", gg.nblk);
    const long chunk = chunk_for(n, pg::kRedBlocks, gg.tp);
    const int blocks = (int)((n + chunk - 1) / chunk);
    if (pair_ok(n, P, Q))
      k_gram_df<true><<<blocks, kT, gg.smem, st>>>(n, chunk, P, np, Q, nq, gg.tp, gg.m, gg.S, gg.ablk, gg.nblk, 0,
                                                    0, partial, nullptr);
    else
      k_gram_df<false><<<blocks, kT, gg.smem, st>>>(n, chunk, P, np, Q, nq, gg.tp, gg.m, gg.S, gg.ablk, gg.nblk, 0,
                                                     0, partial, nullptr);
    PG_TRY(check_launch("k_gram_df"));
    return reduce(partial, blocks, no, out, false, st);
  }
  const long chunk = chunk_for(n, pg::kRedBlocks, kTP);
  const int blocks = (int)((n + chunk - 1) / chunk);
  const size_t smem = sizeof(double) * (size_t)(np + nq) * (kTP + 1);
  k_gram<<<blocks, kT, smem, st>>>(n, chunk, P, np, Q, nq, partial, nullptr);
  PG_TRY(check_launch("k_gram"));
  return reduce(partial, blocks, no, out, false, st);
}
