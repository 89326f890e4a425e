// Y = H X, mixed form: kinetic contractions on the 5th-generation tensor
// cores (tcgen05, TF32 inputs, FP32 accumulation in tensor memory) as
// split-precision products, V*X and the accumulation into Y in FP64.
//
// Each axis contraction is a batched GEMM.  With the "columns" c of an axis
// being all points of the other two axes and all vectors, the transposed
// product  D[c, i] = sum_b X[b, c] * T[i, b]  has M = columns (128 per tile),
// N = n_axis (padded to 16) and K = n_axis (padded to 8): A is a 128-column
// tile of X^T, B is the kinetic matrix, which stays in shared memory for the
// whole (persistent) kernel when it fits (n <= 112); larger n (up to 256)
// runs K in chunks, restaging each chunk of B per tile.  Both are split into
// TF32 high and low parts, D = Ah*Bh + Ah*Bl + Al*Bh (error ~2^-21 relative per term; Al*Bl dropped),
// accumulated in FP32 in TMEM.  X is split on the fly from FP64 with integer
// operations only (the FP64 pipe is two orders of magnitude slower on this
// part).  Three passes: Y = V X + Tx.X, Y += Ty.X, Y += Tz.X; X stays L2
// resident between passes for the grids of the eigensolve workloads.
//
// Operand layout in shared memory: no-swizzle K-major core matrices
// (8 rows x 16 bytes); K-adjacent core matrices 128 B apart (leading byte
// offset), 8-row groups kpad/4*128 B apart (stride byte offset).
// One thread issues the MMAs and commits them to an mbarrier; every wait is
// bounded and a timeout is reported through an error word.
#include <algorithm>
#include <cstdint>

#include "pg_solve.cuh"

namespace {

constexpr int kThreads = 512;  // 16 warps: the A fill and the epilogue each take one round of loads at 64^3
constexpr int kTileM = 128;
constexpr int kMaxN = 256;  // n_axis limit: the MMA N extent (rows of the axis matrix, padded to 16)
constexpr int kBatch = 16;  // global loads a thread keeps in flight while filling A

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// FP64 -> (hi, lo) TF32 pair with integer operations: truncate to FP32,
// round the mantissa to 10 bits for hi, lo = the exact FP32 remainder
// (rounded to TF32 by the tensor core).  Values below 2^-126 flush to zero;
// |x| >= 2^128 and Inf give hi = +-Inf, NaN gives hi = NaN (lo = 0), so a
// non-finite input reaches the product.
__device__ __forceinline__ void split_tf32(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t h = (uint32_t)(b >> 32);
  const int ex = (int)((h >> 20) & 0x7ff);
  const int e = ex - 1023 + 127;
  if (e >= 255) {
    const bool nan = ex == 0x7ff && (b & 0xfffffffffffffull) != 0;
    hi = __uint_as_float(nan ? 0x7fc00000u : ((h & 0x80000000u) | 0x7f800000u));
    lo = 0.f;
    return;
  }
  uint32_t f = 0;
  if (e > 0) f = (h & 0x80000000u) | ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7fffffu);
  const uint32_t hb = (f + 0x1000u) & 0xffffe000u;
  const float xf = __uint_as_float(f);
  hi = __uint_as_float(hb);
  lo = xf - hi;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  for (long it = 0; it < (1L << 26); ++it) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(bar), "r"(phase)
                 : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* out) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) out[j] = __uint_as_float(r[j]);
}

struct AxisMap {
  int n;          // length of the contracted axis
  long stride;    // element stride along the axis
  long ncols;     // columns: N * nvec / n
};

// No staging area: the x-axis epilogue writes straight from the TMEM rows.
constexpr uint32_t kNoStage = 0xffffffffu;
constexpr uint32_t kStageWarpBytes = 32 * 16 * 4;  // one warp's 32 x 16 accumulator chunk

// x-axis (AXIS 0) epilogue of one 16-output chunk through shared memory.  Lane
// L holds the accumulator row of column c0w + L, a grid line along x whose
// outputs i0 .. i0+15 are consecutive doubles, while neighbouring lanes' lines
// are nx doubles apart.  The rows go to a 32 x 16 block, XOR-swizzled by row
// pair so that both the row writes and the column-pair reads hit 32 distinct
// banks; each global load or store below then covers 16 consecutive outputs of
// two lines (two 128-byte segments) instead of one output of 32 lines.
// gshift_own: lane L's vector offset (grid point = address - gshift), passed
// to the lanes that handle its line.
__device__ __forceinline__ void epilogue_x16(const float (&d)[16], float* stg, int lane, long c0w, long ncols,
                                             int i0, int n, int nx, long gshift_own, int mode,
                                             const double* __restrict__ X, double* __restrict__ Y,
                                             const double* __restrict__ v) {
  const int sw = (lane >> 1) & 15;
#pragma unroll
  for (int j = 0; j < 16; ++j) stg[lane * 16 + (j ^ sw)] = d[j];
  __syncwarp();
  const int j = lane & 15, half = lane >> 4;
  const int i = i0 + j;
  // 16 rounds in two halves of 8: mode 2 keeps two loads per round in flight,
  // and 16 rounds of them do not fit the 128 registers of the launch
#pragma unroll
  for (int h = 0; h < 16; h += 8) {
    double prev[8];
    float val[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int it = h + u;
      const int r = 2 * it + half;  // row (line) handled in this round; (r >> 1) & 15 == it
      val[u] = stg[r * 16 + (j ^ it)];
      const long gs = (long)__shfl_sync(0xffffffffu, (long long)gshift_own, r);
      const long c = c0w + r;
      const long a = (long)nx * c + i;
      prev[u] = 0.0;
      if (c < ncols && i < n) {
        if (mode == 2) prev[u] = v[a - gs] * X[a];
        else if (mode == 1) prev[u] = Y[a];
      }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const long c = c0w + 2 * (h + u) + half;
      if (c < ncols && i < n) Y[(long)nx * c + i] = prev[u] + (double)val[u];
    }
  }
  __syncwarp();  // the block is rewritten by the warp's next chunk
}

// base address (element index into X/Y) of column c, and the grid point of
// its first element, for each axis
template <int AXIS>
__device__ __forceinline__ long col_base(long c, int nx, int ny, long N) {
  if (AXIS == 0) return (long)nx * c;
  if (AXIS == 1) {
    const long q = c / nx;
    return (c - q * nx) + (long)nx * ny * q;
  }
  const long plane = (long)nx * ny;
  const long vv = c / plane;
  return (c - vv * plane) + N * vv;
}

// Fill the A operand of one tile: columns c0 .. c0+127 at K values k0 ..
// k0+kc-1, split into TF32 hi/lo halves in the K-major core-matrix layout.
// Lane L takes row m = 8 g + (L >> 2) and K index 4 q + (L & 3) of core
// matrix (g, q), so one warp store fills one 8 x 4 core matrix: 128
// contiguous bytes, no bank conflicts.  One warp load reads 8 lines x 32 bytes
// (AXIS 0: four consecutive K of eight grid lines) or 4 rows x 64 bytes (AXIS
// 1, 2: eight consecutive columns at four K), every sector fully used.  Warp
// wi of 16 / RG owns the row groups g = wi, wi + 16 / RG, ..., so each lane's
// column bases are computed once per tile; kBatch loads per thread are in
// flight before they are split and stored.
template <int AXIS, int RG>
__device__ __forceinline__ void fill_a(int wi, int lane, const double* __restrict__ X, long c0, long ncols, int k0,
                                       int kc, int n, long stride, int nx, int ny, long N, unsigned char* sAh,
                                       unsigned char* sAl) {
  static_assert(kBatch % RG == 0, "a load batch covers whole row-group rounds");
  constexpr int kWarps = (kTileM / 8) / RG;  // warps sharing the fill
  const int kq = kc >> 2;                    // core matrices along K
  long base[RG];
  bool cv[RG];
#pragma unroll
  for (int r = 0; r < RG; ++r) {
    const long c = c0 + 8 * (wi + r * kWarps) + (lane >> 2);
    cv[r] = c < ncols;
    base[r] = cv[r] ? (AXIS == 0 ? (long)nx * c : col_base<AXIS>(c, nx, ny, N)) : 0;
  }
  const int kl = lane & 3;
  for (int t0 = 0; t0 < RG * kq; t0 += kBatch) {
    const int q0 = t0 / RG;
    double xv[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int q = q0 + u / RG, r = u % RG;
      const int kk = k0 + 4 * q + kl;
      xv[u] = (q < kq && kk < n && cv[r]) ? X[base[r] + (long)kk * stride] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int q = q0 + u / RG, r = u % RG;
      if (q < kq) {
        float h, l;
        split_tf32(xv[u], h, l);
        const uint32_t off = (uint32_t)(((wi + r * kWarps) * kq + q) * 128 + lane * 4);
        *(float*)(sAh + off) = h;
        *(float*)(sAl + off) = l;
      }
    }
  }
}

}  // namespace

namespace pg {
// One launch serves up to kMaxTcJobs solves on the same grid: job j owns the
// tiles [tile0_j, tile0_{j+1}) of the launch, with its own X, Y and V.
constexpr int kMaxTcJobs = 16;
static_assert(kMaxTcJobs == kMaxBatchJobs, "batcher and kernel job tables differ");
struct TcJob {
  const double* x;
  double* y;
  const double* v;
  long ncols;  // columns of this job: N * nvec / n_axis
  long tile0;  // first tile of this job in the launch
};
struct TcJobs {
  TcJob j[kMaxTcJobs];
  int n;
  long ntiles;
};
}  // namespace pg

namespace {

using pg::TcJob;
using pg::TcJobs;

template <int AXIS>
__global__ void __launch_bounds__(kThreads, 1)
    k_hx_tc(int nx, int ny, int nz, AxisMap am, int npad, int kc, int nch, uint32_t tmem_cols,
            const float* __restrict__ t_hi, const float* __restrict__ t_lo, const __grid_constant__ TcJobs jobs,
            int mode, uint32_t stage_off, int* __restrict__ err) {
  // mode 0: Y = D;  1: Y += D;  2: Y = V X + D   (D = the axis contraction)
  // stage_off (AXIS 0): byte offset of the 16 warps' epilogue blocks in the
  // dynamic shared memory (it may overlap the A tile, free by then), or
  // kNoStage
  // K is processed in nch chunks of kc (one chunk for n <= 112): per chunk the
  // A tile and the B chunk are staged, multiplied into the same accumulator,
  // and the shared memory is reused once those MMAs have completed.
  extern __shared__ __align__(1024) unsigned char smem[];
  const int n = am.n;
  const uint32_t b_bytes = (uint32_t)npad * kc * 4;  // one K chunk of one half of B
  const uint32_t a_bytes = (uint32_t)kTileM * kc * 4;
  unsigned char* sBh = smem;
  unsigned char* sBl = smem + b_bytes;
  unsigned char* sAh = smem + 2 * b_bytes;
  unsigned char* sAl = sAh + a_bytes;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(8) uint64_t mbar_b;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x;
  const long N = (long)nx * ny * nz;
  const long ntiles = jobs.ntiles;

  // B (the kinetic matrix, rows = output index i, K = b): both halves are
  // operand images in global memory, one per K chunk, brought in by bulk
  // copies; with a single chunk B is loaded once and stays resident
  auto load_b = [&](int ch) {  // one thread
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_u32(&mbar_b)), "r"(2 * b_bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sBh)),
                 "l"(t_hi + (size_t)ch * npad * kc), "r"(b_bytes), "r"(smem_u32(&mbar_b))
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sBl)),
                 "l"(t_lo + (size_t)ch * npad * kc), "r"(b_bytes), "r"(smem_u32(&mbar_b))
                 : "memory");
  };
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_b)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    load_b(0);  // overlaps the first A fill
  }
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // the prologue above reads only the grid's constant operand images; X, Y
  // and V may still be written by the kernel ahead (programmatic launch)
  pg::pdl_wait();
  pg::pdl_release();
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(npad >> 3) << 17) |
                         ((uint32_t)(kTileM >> 4) << 24);
  const uint32_t lbo = 128, sbo = (uint32_t)(kc >> 2) * 128;
  const int warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3;      // TMEM lanes 32*quarter .. +31
  const int group = warp >> 2;       // which 16-column chunks this warp reads (every kThreads/128-th)
  uint32_t phase = 0, b_phase = 0;
  bool ok = true;
  bool b_ready = false;   // single chunk: B resident
  bool first = true;      // the first chunk's B load was issued above

  for (long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    int jb = 0;
    while (jb + 1 < jobs.n && tile >= jobs.j[jb + 1].tile0) ++jb;
    const double* __restrict__ X = jobs.j[jb].x;
    double* __restrict__ Y = jobs.j[jb].y;
    const double* __restrict__ v = jobs.j[jb].v;
    const long ncols = jobs.j[jb].ncols;
    const long c0 = (tile - jobs.j[jb].tile0) * kTileM;
    for (int ch = 0; ch < nch; ++ch) {
      const int k0 = ch * kc;
      if (nch > 1 && !first && tid == 0) load_b(ch);  // the previous chunk's MMAs have completed
      first = false;
      // ---- A operand: 128 columns x kc, split into TF32 hi/lo
      static_assert(kThreads / 32 == kTileM / 8, "one row group of the A tile per warp");
      fill_a<AXIS, 1>(warp, lane, X, c0, ncols, k0, kc, n, am.stride, nx, ny, N, sAh, sAl);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      bool bok = true;
      if (nch > 1 || !b_ready) {  // this chunk's B images have landed
        bok = mbar_wait(smem_u32(&mbar_b), b_phase);
        b_phase ^= 1u;
        b_ready = true;
      }
      if (!__syncthreads_and(bok ? 1 : 0)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (tid == 0) {
        const uint32_t ah = smem_u32(sAh), al = smem_u32(sAl), bh = smem_u32(sBh), bl = smem_u32(sBl);
        for (int kk = 0; kk < kc / 8; ++kk) {
          const uint32_t off = (uint32_t)kk * 256;  // 8 K-elements = two core matrices
          const uint64_t dah = smem_desc(ah + off, lbo, sbo), dal = smem_desc(al + off, lbo, sbo);
          const uint64_t dbh = smem_desc(bh + off, lbo, sbo), dbl = smem_desc(bl + off, lbo, sbo);
          const uint32_t acc = (ch > 0 || kk > 0) ? 1u : 0u;
          // small terms first, then the leading product
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                       " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                       "l"(dal), "l"(dbh), "r"(idesc), "r"(acc));
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                       " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                       "l"(dah), "l"(dbl), "r"(idesc), "r"(1u));
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                       " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                       "l"(dah), "l"(dbh), "r"(idesc), "r"(1u));
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(&mbar)));
      }
      const bool waited = mbar_wait(smem_u32(&mbar), phase);
      phase ^= 1u;
      if (!__syncthreads_and(waited ? 1 : 0)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    if (!ok) break;
    // ---- epilogue: thread (quarter, lane) owns column c = c0 + 32*quarter + lane
    const int m = 32 * quarter + lane;
    const long c = c0 + m;
    const bool cvalid = c < ncols;
    const long base = cvalid ? col_base<AXIS>(c, nx, ny, N) : 0;
    const long gshift = cvalid ? (c / (N / n)) * N : 0;  // vector offset: grid point = address - gshift
    // one 16-row chunk per warp and round: 16 loads in flight, then the stores
    for (int ck = group; ck * 16 < npad; ck += kThreads / 128) {
      float d[16];
      tmem_ld16(tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(ck * 16), d);
      if (AXIS == 0 && stage_off != kNoStage) {
        float* stg = reinterpret_cast<float*>(smem + stage_off + (uint32_t)warp * kStageWarpBytes);
        epilogue_x16(d, stg, lane, c0 + 32 * quarter, ncols, ck * 16, n, nx, gshift, mode, X, Y, v);
      } else if (cvalid) {
        double prev[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int i = ck * 16 + j;
          const long a = base + (long)i * am.stride;
          prev[j] = 0.0;
          if (i < n) {
            if (mode == 2) prev[j] = v[a - gshift] * X[a];
            else if (mode == 1) prev[j] = Y[a];
          }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int i = ck * 16 + j;
          if (i < n) Y[base + (long)i * am.stride] = prev[j] + (double)d[j];
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // A buffers and the accumulator are free for the next tile
  }
  if (!ok && tid == 0) atomicExch(err, 1);
  if (tid < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
}


// Pipelined form of k_hx_tc for CTAs that own several tiles and a single K
// chunk (n <= 112).  Warps 0-7 (producers) fill the A tile of tile i+1 while
// warps 8-15 (consumers) drain the accumulator of tile i; thread 0 issues the
// MMAs.  Two TMEM accumulators alternate between tiles:
//   mbar_mma[k]  completes when the MMAs into accumulator k are done (A is
//                then free for the next fill, and the accumulator readable);
//   mbar_free[k] completes when the eight consumer warps have read
//                accumulator k (it may then take the tile after next).
// Every wait is bounded; a timeout raises `abort` in shared memory, every
// role leaves its loop, and the error word is set.
constexpr int kPipeThreads = 512;
constexpr int kProducers = 256;

// OR of f over the kProducers producer threads (named barrier 1): every
// producer takes the same branch afterwards.
__device__ __forceinline__ int producers_any(int f) {
  int r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n selp.s32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"(f), "n"(kProducers)
      : "memory");
  return r;
}

template <int AXIS>
__global__ void __launch_bounds__(kPipeThreads, 1)
    k_hx_tc_pipe(int nx, int ny, int nz, AxisMap am, int npad, int kc, uint32_t tmem_cols,
                 const float* __restrict__ t_hi, const float* __restrict__ t_lo,
                 const __grid_constant__ TcJobs jobs, int mode, uint32_t stage_off, int* __restrict__ err) {
  // stage_off (AXIS 0): byte offset of the eight consumer warps' epilogue
  // blocks, after the A tile (which the producers refill meanwhile), or
  // kNoStage
  extern __shared__ __align__(1024) unsigned char smem[];
  const int n = am.n;
  const uint32_t b_bytes = (uint32_t)npad * kc * 4;
  const uint32_t a_bytes = (uint32_t)kTileM * kc * 4;
  unsigned char* sBh = smem;
  unsigned char* sBl = smem + b_bytes;
  unsigned char* sAh = smem + 2 * b_bytes;
  unsigned char* sAl = sAh + a_bytes;
  __shared__ __align__(8) uint64_t mbar_b, mbar_mma[2], mbar_free[2];
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const long N = (long)nx * ny * nz;
  const long ntiles = jobs.ntiles;
  if (tid == 0) {
    abort_flag = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_b)));
    for (int k = 0; k < 2; ++k) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_mma[k])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 8;" ::"r"(smem_u32(&mbar_free[k])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_u32(&mbar_b)), "r"(2 * b_bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sBh)),
                 "l"(t_hi), "r"(b_bytes), "r"(smem_u32(&mbar_b))
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sBl)),
                 "l"(t_lo), "r"(b_bytes), "r"(smem_u32(&mbar_b))
                 : "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(2 * tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // the prologue above reads only the grid's constant operand images; X, Y
  // and V may still be written by the kernel ahead (programmatic launch)
  pg::pdl_wait();
  pg::pdl_release();
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(npad >> 3) << 17) |
                         ((uint32_t)(kTileM >> 4) << 24);
  const uint32_t lbo = 128, sbo = (uint32_t)(kc >> 2) * 128;
  auto fail = [&]() { atomicExch(&abort_flag, 1); };

  if (tid < kProducers) {
    // ---------------------------------------------------------------- producers
    bool b_ready = false;
    long i = 0;
    for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int k = (int)(i & 1);
      // the MMAs of the previous tile have read A (every producer waits, then
      // all producers agree on whether to go on)
      int bad = 0;
      if (i >= 1 && !mbar_wait(smem_u32(&mbar_mma[(i - 1) & 1]), (uint32_t)(((i - 1) >> 1) & 1))) bad = 1;
      if (producers_any(bad | *(volatile int*)&abort_flag)) {
        fail();
        break;
      }
      int jb = 0;
      while (jb + 1 < jobs.n && tile >= jobs.j[jb + 1].tile0) ++jb;
      const double* __restrict__ X = jobs.j[jb].x;
      const long ncols = jobs.j[jb].ncols;
      const long c0 = (tile - jobs.j[jb].tile0) * kTileM;
      static_assert(kProducers / 32 == kTileM / 8 / 2, "two row groups of the A tile per producer warp");
      fill_a<AXIS, 2>(warp, lane, X, c0, ncols, 0, kc, n, am.stride, nx, ny, N, sAh, sAl);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("bar.sync 1, %0;" ::"n"(kProducers) : "memory");  // the A tile is complete
      if (tid == 0) {
        bool ok = true;
        if (!b_ready) ok = b_ready = mbar_wait(smem_u32(&mbar_b), 0);
        // the consumers have read this accumulator's previous tile (i - 2)
        if (ok && i >= 2) ok = mbar_wait(smem_u32(&mbar_free[k]), (uint32_t)(((i - 2) >> 1) & 1));
        if (!ok || *(volatile int*)&abort_flag) {
          fail();
        } else {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t ah = smem_u32(sAh), al = smem_u32(sAl), bh = smem_u32(sBh), bl = smem_u32(sBl);
          const uint32_t acc = tmem + (uint32_t)k * tmem_cols;
          for (int kk = 0; kk < kc / 8; ++kk) {
            const uint32_t off = (uint32_t)kk * 256;
            const uint64_t dah = smem_desc(ah + off, lbo, sbo), dal = smem_desc(al + off, lbo, sbo);
            const uint64_t dbh = smem_desc(bh + off, lbo, sbo), dbl = smem_desc(bl + off, lbo, sbo);
            asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                         " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(acc),
                         "l"(dal), "l"(dbh), "r"(idesc), "r"(kk > 0 ? 1u : 0u));
            asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                         " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(acc),
                         "l"(dah), "l"(dbl), "r"(idesc), "r"(1u));
            asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                         " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(acc),
                         "l"(dah), "l"(dbh), "r"(idesc), "r"(1u));
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar_mma[k])));
        }
      }
    }
  } else {
    // ---------------------------------------------------------------- consumers
    const int cw = warp - kProducers / 32;  // consumer warp 0..7
    const int quarter = warp & 3;           // TMEM lanes 32*quarter .. +31
    const int group = cw >> 2;              // which 16-row chunks this warp reads
    long i = 0;
    for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int k = (int)(i & 1);
      if (!mbar_wait(smem_u32(&mbar_mma[k]), (uint32_t)((i >> 1) & 1))) fail();
      if (*(volatile int*)&abort_flag) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      int jb = 0;
      while (jb + 1 < jobs.n && tile >= jobs.j[jb + 1].tile0) ++jb;
      const double* __restrict__ X = jobs.j[jb].x;
      double* __restrict__ Y = jobs.j[jb].y;
      const double* __restrict__ v = jobs.j[jb].v;
      const long ncols = jobs.j[jb].ncols;
      const long c0 = (tile - jobs.j[jb].tile0) * kTileM;
      const int m = 32 * quarter + lane;
      const long c = c0 + m;
      const bool cvalid = c < ncols;
      const long base = cvalid ? col_base<AXIS>(c, nx, ny, N) : 0;
      const long gshift = cvalid ? (c / (N / n)) * N : 0;
      const uint32_t acc = tmem + (uint32_t)k * tmem_cols;
      for (int ck = group; ck * 16 < npad; ck += 2) {
        float d[16];
        tmem_ld16(acc + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(ck * 16), d);
        if (AXIS == 0 && stage_off != kNoStage) {
          float* stg = reinterpret_cast<float*>(smem + stage_off + (uint32_t)cw * kStageWarpBytes);
          epilogue_x16(d, stg, lane, c0 + 32 * quarter, ncols, ck * 16, n, nx, gshift, mode, X, Y, v);
        } else if (cvalid) {
          double prev[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int r = ck * 16 + j;
            const long a = base + (long)r * am.stride;
            prev[j] = 0.0;
            if (r < n) {
              if (mode == 2) prev[j] = v[a - gshift] * X[a];
              else if (mode == 1) prev[j] = Y[a];
            }
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int r = ck * 16 + j;
            if (r < n) Y[base + (long)r * am.stride] = prev[j] + (double)d[j];
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&mbar_free[k])) : "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (abort_flag && tid == 0) atomicExch(err, 1);
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * tmem_cols));
}

}  // namespace

namespace pg {

static int g_num_sms = 0;

// One axis contraction on the tensor cores for a list of jobs on the same
// grid: Y_j (mode) D_j with D_j = A x_axis X_j, A given as TF32 hi/lo halves
// (n_axis x n_axis, row-major).  Each job covers nvec_j vectors.
pg_status tc_axis_jobs(const pg_grid* g, int a, const float* Ahi, const float* Alo, const double* const* v,
                       const double* const* x, double* const* y, const int* nvec, int njobs, int mode,
                       cudaStream_t st, int ctas, int form) {
  PG_ARG(njobs > 0 && njobs <= kMaxTcJobs, "tc_axis: %d jobs (at most %d)", njobs, kMaxTcJobs);
  if (g->n[a] > kMaxN) {
    set_error("mixed form supports n <= %d per axis (got %d)", kMaxN, g->n[a]);
    return PG_UNSUPPORTED;
  }
  // once per process (thread-safe static initialisation): SM count and the
  // dynamic shared-memory opt-in of the three axis kernels, set to the most
  // the device allows beside each kernel's static shared memory
  static int g_max_dyn = 0;
  static const cudaError_t init = [] {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (g_num_sms <= 0) g_num_sms = 148;
    const void* fns[6] = {(const void*)k_hx_tc<0>,      (const void*)k_hx_tc<1>,      (const void*)k_hx_tc<2>,
                          (const void*)k_hx_tc_pipe<0>, (const void*)k_hx_tc_pipe<1>, (const void*)k_hx_tc_pipe<2>};
    int lim = optin;
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) {
      cudaFuncAttributes fa;
      e = cudaFuncGetAttributes(&fa, fns[k]);
      if (e == cudaSuccess) lim = std::min(lim, optin - (int)fa.sharedSizeBytes);
    }
    for (int k = 0; k < 6 && e == cudaSuccess; ++k)
      e = cudaFuncSetAttribute(fns[k], cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    g_max_dyn = lim;
    return e;
  }();
  PG_CUDA_TRY(init);
  const long N = g->N;
  const int n = g->n[a];
  AxisMap am;
  am.n = n;
  am.stride = a == 0 ? 1 : (a == 1 ? g->n[0] : (long)g->n[0] * g->n[1]);
  am.ncols = 0;
  TcJobs jobs;
  jobs.n = njobs;
  long tiles = 0;
  for (int j = 0; j < njobs; ++j) {
    jobs.j[j].x = x[j];
    jobs.j[j].y = y[j];
    jobs.j[j].v = v ? v[j] : nullptr;
    jobs.j[j].ncols = N / n * nvec[j];
    jobs.j[j].tile0 = tiles;
    tiles += (jobs.j[j].ncols + kTileM - 1) / kTileM;
  }
  jobs.ntiles = tiles;
  const int npad = pg::tc_npad(n);
  const int kpad = pg::tc_kpad(n);
  const int kc = pg::tc_kchunk(n);           // K chunk (the grid's operand images use the same split)
  const int nch = (kpad + kc - 1) / kc;
  uint32_t cols = 32;
  while (cols < (uint32_t)npad) cols <<= 1;
  const size_t smem = (size_t)2 * npad * kc * 4 + (size_t)2 * kTileM * kc * 4;
  if ((long)smem > (long)g_max_dyn) {
    set_error("tc_axis: %zu bytes of shared memory needed, the device allows %d", smem, g_max_dyn);
    return PG_UNSUPPORTED;
  }
  // one persistent CTA of kThreads per SM, or the tuned count
  const long cap = ctas > 0 && ctas < g_num_sms ? ctas : g_num_sms;
  const int grid = (int)(tiles < cap ? tiles : cap);
  int* err = g->tc_err.p;
  const size_t a_region = (size_t)2 * kTileM * kc * 4, b_region = (size_t)2 * npad * kc * 4;
  // several tiles per CTA: the pipelined form overlaps them (form 0), or as tuned
  const bool pipe = nch == 1 && (form == 2 || (form == 0 && tiles > cap));
  if (pipe) {
    // x-axis epilogue blocks of the eight consumer warps after the A tile
    const size_t stage = (size_t)(kPipeThreads - kProducers) / 32 * kStageWarpBytes;
    const bool staged = a == 0 && smem + stage <= (size_t)g_max_dyn;
    const uint32_t stage_off = staged ? (uint32_t)smem : kNoStage;
    const size_t smem_p = staged ? smem + stage : smem;
    switch (a) {
      case 0:
        PG_CUDA_TRY(launch_dependent(k_hx_tc_pipe<0>, dim3(grid), dim3(kPipeThreads), smem_p, st, g->n[0], g->n[1],
                                     g->n[2], am, npad, kc, cols, Ahi, Alo, jobs, mode, stage_off, err));
        break;
      case 1:
        PG_CUDA_TRY(launch_dependent(k_hx_tc_pipe<1>, dim3(grid), dim3(kPipeThreads), smem_p, st, g->n[0], g->n[1],
                                     g->n[2], am, npad, kc, cols, Ahi, Alo, jobs, mode, stage_off, err));
        break;
      default:
        PG_CUDA_TRY(launch_dependent(k_hx_tc_pipe<2>, dim3(grid), dim3(kPipeThreads), smem_p, st, g->n[0], g->n[1],
                                     g->n[2], am, npad, kc, cols, Ahi, Alo, jobs, mode, stage_off, err));
    }
    return check_launch("k_hx_tc_pipe");
  }
  // x-axis epilogue blocks of all 16 warps: in the A tile (free once a tile's
  // MMAs have completed) when it is large enough, else after it
  const size_t stage = (size_t)kThreads / 32 * kStageWarpBytes;
  uint32_t stage_off = kNoStage;
  size_t smem_t = smem;
  if (a == 0) {
    if (a_region >= stage) {
      stage_off = (uint32_t)b_region;
    } else if (smem + stage <= (size_t)g_max_dyn) {
      stage_off = (uint32_t)smem;
      smem_t = smem + stage;
    }
  }
  switch (a) {
    case 0:
      PG_CUDA_TRY(launch_dependent(k_hx_tc<0>, dim3(grid), dim3(kThreads), smem_t, st, g->n[0], g->n[1], g->n[2], am,
                                   npad, kc, nch, cols, Ahi, Alo, jobs, mode, stage_off, err));
      break;
    case 1:
      PG_CUDA_TRY(launch_dependent(k_hx_tc<1>, dim3(grid), dim3(kThreads), smem_t, st, g->n[0], g->n[1], g->n[2], am,
                                   npad, kc, nch, cols, Ahi, Alo, jobs, mode, stage_off, err));
      break;
    default:
      PG_CUDA_TRY(launch_dependent(k_hx_tc<2>, dim3(grid), dim3(kThreads), smem_t, st, g->n[0], g->n[1], g->n[2], am,
                                   npad, kc, nch, cols, Ahi, Alo, jobs, mode, stage_off, err));
  }
  return check_launch("k_hx_tc");
}

pg_status tc_axis(const pg_grid* g, int a, const float* Ahi, const float* Alo, const double* v, const double* x,
                  double* y, int nvec, int mode, cudaStream_t st) {
  return tc_axis_jobs(g, a, Ahi, Alo, v ? &v : nullptr, &x, &y, &nvec, 1, mode, st, 0, 0);
}

bool fused_hx_ok(const pg_grid* g);
bool f16_hx_ok(const pg_grid* g);
pg_status hx_f16(const pg_grid* g, const double* v, const double* x, double* y, int nvec, const HxParams& p,
                 cudaStream_t st, bool unit);
pg_status hx_f16_jobs(const pg_grid* g, const double* const* v, const double* const* x, double* const* y,
                      const int* nvec, int njobs, const HxParams& p, cudaStream_t st, bool unit);
pg_status hx_fused(const pg_grid* g, const double* v, const double* x, double* y, int nvec, const HxParams& p,
                   cudaStream_t st);
pg_status hx_fused_jobs(const pg_grid* g, const double* const* v, const double* const* x, double* const* y,
                        const int* nvec, int njobs, const HxParams& p, cudaStream_t st);

// Mixed H*X of several solves on the same grid in one launch (fused) or one
// launch per axis, with the launch parameters tuned for the whole block.
pg_status hx_mixed_batch(const pg_grid* g, const double* const* v, const double* const* x, double* const* y,
                         const int* nvec, int njobs, cudaStream_t st, bool unit) {
  int total = 0;
  for (int j = 0; j < njobs; ++j) total += nvec[j];
  HxParams p = hx_params(g, total);
  if (p.kind == 3) {
    bool aligned = true;
    for (int j = 0; j < njobs; ++j) aligned = aligned && (nvec[j] == 0 || ((uintptr_t)x[j] & 15u) == 0);
    if (aligned) return hx_f16_jobs(g, v, x, y, nvec, njobs, p, st, unit);
    p.kind = fused_hx_ok(g) ? 2 : 1;
  }
  if (p.kind == 2) return hx_fused_jobs(g, v, x, y, nvec, njobs, p, st);
  for (int a = 0; a < 3; ++a)
    PG_TRY(tc_axis_jobs(g, a, g->t_hi[a].p, g->t_lo[a].p, v, x, y, nvec, njobs, a == 0 ? 2 : 1, st, p.ctas, p.form));
  return PG_OK;
}

// Y = H X: the fused kernel (pg_hx_fused.cu) or the three axis passes
// Y = V X + Tx.X, Y += Ty.X, Y += Tz.X, as hx_params chooses.
// The tensor-core completion waits report a timeout through g->tc_err; with
// check, the call waits for the stream and returns PG_DEVICE_TIMEOUT if one
// occurred (the eigensolver checks the word at its own synchronisation points).
pg_status hx_mixed(const pg_grid* g, const double* v, const double* x, double* y, int nvec, cudaStream_t st,
                   bool check, bool unit) {
  HxParams p = hx_params(g, nvec);
  if (p.kind == 3 && ((uintptr_t)x & 15u) != 0) p.kind = fused_hx_ok(g) ? 2 : 1;  // bulk copies need alignment
  if (p.kind == 3) {
    PG_TRY(hx_f16(g, v, x, y, nvec, p, st, unit));
    return check ? check_tc_error(g, st) : PG_OK;
  }
  if (p.kind == 2) {
    PG_TRY(hx_fused(g, v, x, y, nvec, p, st));
    return check ? check_tc_error(g, st) : PG_OK;
  }
  if (g->hx_kernel == 2 || g->hx_kernel == 3) {
    set_error("pg_hx: the fused mixed H*X kernel does not take this grid");
    return PG_UNSUPPORTED;
  }
  for (int a = 0; a < 3; ++a)
    PG_TRY(tc_axis_jobs(g, a, g->t_hi[a].p, g->t_lo[a].p, &v, &x, &y, &nvec, 1, a == 0 ? 2 : 1, st, p.ctas,
                        p.form));
  return check ? check_tc_error(g, st) : PG_OK;
}

pg_status check_tc_error(const pg_grid* g, cudaStream_t st) {
  int herr = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&herr, g->tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  PG_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    set_error("pg_hx: tensor-core completion wait timed out");
    return PG_DEVICE_TIMEOUT;
  }
  return PG_OK;
}

}  // namespace pg
