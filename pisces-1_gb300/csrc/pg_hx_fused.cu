// Y = H X, mixed form, as one persistent tensor-core kernel with two kinds of
// work item (the x and y contractions of one grid plane; the z contraction of
// 128 grid lines), so that each vector's X and the partial sums stay in L2
// between the two passes and HBM sees X read once and Y written once.
//
// H = V + Tx (+) Ty (+) Tz on the x-fastest grid (src/mtx.cpp:22-109).  For
// one vector u:
//   xy item (u, k): plane P[i, j] = X[u][i + nx j + nx ny k] (nx x ny);
//       D[i, j] = sum_i' Tx[i, i'] P[i', j] + sum_j' P[i, j'] Ty[j, j']
//     both contractions accumulate into ONE TMEM tile D (lanes i, columns j):
//       x: A = Tx (M = i, K = i'),       B = P as rows j, K = i'  (the plane
//          in memory order: B[j][i'] = P[i', j])
//       y: A = P as rows i, K = j' (the plane transposed while it is staged),
//          B = Ty (N = j, K = j')
//     epilogue: W = D in FP32, into the low word of each point's Y slot;
//   z item (u, t): 128 consecutive plane points p = 128 t .. 128 t + 127,
//       D[p, k] = sum_k' X[u][p + nx ny k'] Tz[k, k'],
//     epilogue: Y = V X + (W + D), one FP64 multiply-add per point.
// The z epilogue of vector u reads W, so it waits (bounded) until all xy
// items of u have finished; its operand fill and MMAs do not wait.
//
// Work order (one global ticket counter), with a lag L of two vectors:
// XY(0), XY(1), XY(2), Z(0), XY(3), Z(1), ..., XY(b-1), Z(b-3), Z(b-2),
// Z(b-1).  A z item's dependencies always hold lower
// tickets, and every ticket is held by a running CTA, so the waits end
// whatever the number of resident CTAs.
//
// Precision as the three-pass kernels (pg_hx_tc.cu): split-TF32 products
// Ah Bh + Ah Bl + Al Bh accumulated in FP32 in TMEM; the x + y and z sums
// add in FP32 (their own precision) and V X in FP64.  The FP64 pipe of this
// part retires about two FMAs per SM per clock, so the epilogues use two
// FP64 instructions per point (one conversion, one multiply-add), not five.
//
// Staged fill (where shared memory has room, n <= 64 per axis): the raw
// FP64 rows of the next work item are bulk-copied (cp.async.bulk, one row per
// copy, rows padded so that the producers' shared-memory reads are free of
// bank conflicts) into a staging buffer while the current item is converted
// and multiplied; the producers then convert from shared memory instead of
// waiting on global loads in register batches.
//
// Shared memory (no-swizzle K-major core matrices, as pg_hx_tc.cu): the
// kinetic matrices (resident; one image when the axes share one matrix),
// the plane in both orientations, and the z tile (over the plane images).
// An A operand image is read as 128 rows whatever its true row count; the
// rows past its end fall on the images that follow it and only feed TMEM
// lanes the epilogue ignores.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>

#include "pg_solve.cuh"

namespace {

constexpr int kTile = 128;  // MMA M: TMEM lanes
constexpr int kMaxJobs = 16;
constexpr int kBatch = 12;  // operand loads a producer thread keeps in flight per fill round

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// FP64 -> (hi, lo) TF32 pair with integer operations (as pg_hx_tc.cu):
// hi = the FP32 truncation rounded to 10 mantissa bits, lo = the FP32
// remainder; |x| < 2^-126 flushes to zero, Inf/NaN and |x| >= 2^128 give a
// non-finite hi.
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
  hi = __uint_as_float(hb);
  lo = __uint_as_float(f) - hi;
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

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d),
               "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// L2 prefetch of bytes [p, p + n), rounded inward to 16-byte boundaries.
__device__ __forceinline__ void prefetch_l2(const void* p, long n) {
  const uintptr_t a = ((uintptr_t)p + 15) & ~(uintptr_t)15;
  const uintptr_t e = ((uintptr_t)p + (uintptr_t)n) & ~(uintptr_t)15;
  if (e > a)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((uint32_t)(e - a)) : "memory");
}

}  // namespace

namespace pg {

struct FusedJob {
  const double* x;
  double* y;
  const double* v;
  int nvec;
  int vec0;  // first vector of this job in the launch's vector list
};
struct FusedJobs {
  FusedJob j[kMaxJobs];
  int n;
  int nvec;  // vectors of all jobs
};

struct FusedGeom {
  int nx, ny, nz;
  int kx, ky, kz;    // K extents (padded to 8)
  int npy, npz;      // MMA N extents (padded to 16)
  int nzt;           // z items per vector
  int lag;           // vectors between a vector's xy items and its z items
  uint32_t tx_hi, tx_lo, ty_hi, ty_lo, tz_hi, tz_lo;  // byte offsets in dynamic shared memory
  uint32_t pn_hi, pn_lo, pt_hi, pt_lo, z_hi, z_lo;
  uint32_t acc_cols;  // TMEM columns per accumulator
  int staged;         // 1: raw rows of the next item are bulk-copied into the staging buffer
  uint32_t stg;       // byte offset of the staging buffer
  uint32_t stg_pxy;   // its row pitch for a plane (bytes; row j holds X[0..nx) of grid line j)
  uint32_t stg_pz;    // its row pitch for a z tile (bytes; row k holds the tile's points of plane k)
};

constexpr int kMaxConst = 6;
struct FusedConst {  // distinct kinetic operand images, bulk-copied once per CTA
  const float* src[kMaxConst];
  uint32_t dst[kMaxConst];
  uint32_t bytes[kMaxConst];
  int n;
  uint32_t total;
};

constexpr int kFusedMaxVec = 1024;
struct FusedCounters {
  unsigned ticket;
  unsigned finished;
  unsigned done[kFusedMaxVec];  // finished xy items per vector
};

}  // namespace pg

namespace {

using pg::FusedConst;
using pg::FusedCounters;
using pg::FusedGeom;
using pg::FusedJobs;

struct Item {
  int kind;  // 0: xy plane, 1: z tile, -1: none
  int u;     // vector in the launch's list
  int idx;   // plane k or z tile t
};

// Ticket -> work item.  Order: XY(0) .. XY(L-1), then XY(s), Z(s-L) for s =
// L .. b-1, then the remaining Z blocks (L = lag: the z items of a vector
// come L vectors after its xy items, so their dependencies are long done).
__device__ __forceinline__ Item decode(unsigned t, int nvec, int nz, int nzt, int lag) {
  const unsigned ps = (unsigned)(nz + nzt);
  if (t >= (unsigned)nvec * ps) return Item{-1, 0, 0};
  const int L = lag < nvec ? lag : nvec;
  const unsigned head = (unsigned)L * nz;
  if (t < head) return Item{0, (int)(t / nz), (int)(t % nz)};
  unsigned r = t - head;
  const unsigned mid = (unsigned)(nvec - L) * ps;
  if (r < mid) {
    const unsigned s = r / ps, w = r - s * ps;
    if (w < (unsigned)nz) return Item{0, L + (int)s, (int)w};
    return Item{1, (int)s, (int)(w - nz)};
  }
  r -= mid;
  return Item{1, nvec - L + (int)(r / nzt), (int)(r % nzt)};
}

__device__ __forceinline__ void vec_ptrs(const FusedJobs& J, int u, long N, const double*& x, double*& y,
                                         const double*& v) {
  int j = 0;
  while (j + 1 < J.n && u >= J.j[j + 1].vec0) ++j;
  const long off = (long)(u - J.j[j].vec0) * N;
  x = J.j[j].x + off;
  y = J.j[j].y + off;
  v = J.j[j].v;
}

// Warp roles of the kernel (one CTA per SM, 16 warps: four per SM
// sub-partition, 128 registers each):
//   warps 0-6   producers: take tickets, fill the operand images of item i
//               (from L2: the X data of item i+1 is prefetched meanwhile);
//   warps 7-14  epilogue: drain the accumulator of item i-2 or i-1 (two TMEM
//               accumulators alternate), two warps per TMEM lane quarter;
//   warp 15     lane 0 issues the MMAs of item i-1.
// Hand-over through mbarriers: full (producers -> issuer, images written),
// empty (MMA completion -> producers, images free), acc_full[b] (MMA
// completion and the issuer -> epilogue), acc_empty[b] (epilogue -> issuer).
// Each role decides with one leader thread and broadcasts over a named
// barrier, so a role's threads always take the same branch; every wait is
// bounded and also ends when another role has given up (s_abort).
constexpr int kProdWarps = 7;
constexpr int kEpiWarps = 8;
constexpr int kIssueWarp = kProdWarps + kEpiWarps;
constexpr int kThreadsAll = (kIssueWarp + 1) * 32;
constexpr int kRing = 8;  // tickets in flight in one CTA: at most five (fill .. epilogue)

// xy item: the plane of vector u at z index k into both images.  Producer
// warp w fills core matrices cm = w, w + 7, ... of the natural image (rows
// j, K = i; cm = gj * kx/4 + qi): lane L takes row j = 8 gj + L/4 and i =
// 4 qi + L%4, so a warp load reads 8 grid lines x 32 bytes and its store
// fills one 128-byte core matrix; the same value goes to the transposed
// image (rows i, K = j).  (gj, qi) advance by 7 core matrices per step
// without a division.  The loads of the first round are issued before
// ready() returns (ready waits until the images are free), so their latency
// overlaps that wait.
template <class Src, class Ready>
__device__ __forceinline__ void fill_plane(const FusedGeom& G, Src&& P, unsigned char* smem, int pw, int lane,
                                           Ready&& ready) {
  const int kq = G.kx >> 2;
  const int ncm = (G.npy >> 3) * kq;
  const int kyq32 = (G.ky >> 2) * 32;
  const int lj = lane >> 2, li = lane & 3;
  const int pt_lane = (lj >> 2) * 32 + li * 4 + (lj & 3);  // transposed-image offset of the lane in its block
  float* pnh = reinterpret_cast<float*>(smem + G.pn_hi);
  float* pnl = reinterpret_cast<float*>(smem + G.pn_lo);
  float* pth = reinterpret_cast<float*>(smem + G.pt_hi);
  float* ptl = reinterpret_cast<float*>(smem + G.pt_lo);
  const int rounds = (ncm + kProdWarps * kBatch - 1) / (kProdWarps * kBatch);
  int gj = pw / kq, qi = pw - (pw / kq) * kq;  // of cm = pw
  for (int r = 0; r < rounds; ++r) {
    const int c0 = pw + r * kProdWarps * kBatch;
    double xv[kBatch];
    int sgj = gj, sqi = qi;
#pragma unroll
    for (int b = 0; b < kBatch; ++b) {
      const int j = 8 * gj + lj, i = 4 * qi + li;
      xv[b] = (c0 + kProdWarps * b < ncm && j < G.ny && i < G.nx) ? P(i, j) : 0.0;
      qi += kProdWarps;
      while (qi >= kq) qi -= kq, ++gj;
    }
    if (r == 0) ready();
    gj = sgj, qi = sqi;
#pragma unroll
    for (int b = 0; b < kBatch; ++b) {
      const int cm = c0 + kProdWarps * b;
      if (cm < ncm) {
        float h, l;
        split_tf32(xv[b], h, l);
        pnh[cm * 32 + lane] = h;
        pnl[cm * 32 + lane] = l;
        if (8 * gj + lj < G.ky) {
          const int off = (qi >> 1) * kyq32 + (qi & 1) * 16 + gj * 64 + pt_lane;
          pth[off] = h;
          ptl[off] = l;
        }
      }
      qi += kProdWarps;
      while (qi >= kq) qi -= kq, ++gj;
    }
  }
  if (rounds == 0) ready();
}

// z item: grid points p0 .. p0 + 127 of every plane (rows), K = z index
// (cm = g * kz/4 + q).  Lane L takes row 8 g + L/4 and K 4 q + L%4: a warp
// load reads four runs of eight consecutive points.
template <class Src, class Ready>
__device__ __forceinline__ void fill_ztile(const FusedGeom& G, Src&& X, long p0, long nxny, unsigned char* smem,
                                           int pw, int lane, Ready&& ready) {
  const int kq = G.kz >> 2;
  const int ncm = (kTile / 8) * kq;
  const int lj = lane >> 2, li = lane & 3;
  float* zh = reinterpret_cast<float*>(smem + G.z_hi);
  float* zl = reinterpret_cast<float*>(smem + G.z_lo);
  const int rounds = (ncm + kProdWarps * kBatch - 1) / (kProdWarps * kBatch);
  int g = pw / kq, q = pw - (pw / kq) * kq;
  for (int r = 0; r < rounds; ++r) {
    const int c0 = pw + r * kProdWarps * kBatch;
    double xv[kBatch];
#pragma unroll
    for (int b = 0; b < kBatch; ++b) {
      const long p = p0 + 8 * g + lj;
      const int k = 4 * q + li;
      xv[b] = (c0 + kProdWarps * b < ncm && p < nxny && k < G.nz) ? X(p - p0, k) : 0.0;
      q += kProdWarps;
      while (q >= kq) q -= kq, ++g;
    }
    if (r == 0) ready();
#pragma unroll
    for (int b = 0; b < kBatch; ++b) {
      const int cm = c0 + kProdWarps * b;
      if (cm < ncm) {
        float h, l;
        split_tf32(xv[b], h, l);
        zh[cm * 32 + lane] = h;
        zl[cm * 32 + lane] = l;
      }
    }
  }
  if (rounds == 0) ready();
}

// One thread: prefetch the X data of an item into L2 (the fill then reads L2).
__device__ __forceinline__ void prefetch_item(const FusedGeom& G, const FusedJobs& J, const Item& it, long N,
                                              long nxny) {
  if (it.kind < 0) return;
  const double *x, *v;
  double* y;
  vec_ptrs(J, it.u, N, x, y, v);
  if (it.kind == 0) {
    prefetch_l2(x + nxny * it.idx, nxny * 8);
  } else {
    const long p0 = (long)it.idx * kTile;
    const long np = std::min((long)kTile, nxny - p0);
    for (int k = 0; k < G.nz; ++k) prefetch_l2(x + p0 + nxny * k, np * 8);
  }
}

// The lanes of one warp: bulk-copy the raw rows of an item into the staging
// buffer, completing on mbarrier bar (lane 0 sets the byte count first).
// Rows: a plane's ny grid lines (nx doubles each), or a z tile's nz planes
// (up to 128 points each).  Every address and size is a multiple of 16
// bytes (the launch checks nx even and X 16-byte aligned).
__device__ __forceinline__ void stage_item(const FusedGeom& G, const FusedJobs& J, const Item& it, long N, long nxny,
                                           unsigned char* smem, uint32_t bar, int lane) {
  if (it.kind < 0) return;
  const double *x, *v;
  double* y;
  vec_ptrs(J, it.u, N, x, y, v);
  int rows;
  uint32_t row_bytes, pitch;
  const double* src;
  long src_stride;
  if (it.kind == 0) {
    rows = G.ny;
    row_bytes = (uint32_t)G.nx * 8u;
    pitch = G.stg_pxy;
    src = x + nxny * it.idx;
    src_stride = G.nx;
  } else {
    const long p0 = (long)it.idx * kTile;
    rows = G.nz;
    row_bytes = (uint32_t)std::min((long)kTile, nxny - p0) * 8u;
    pitch = G.stg_pz;
    src = x + p0;
    src_stride = nxny;
  }
  if (lane == 0) {
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(bar), "r"((uint32_t)rows * row_bytes)
                 : "memory");
  }
  __syncwarp();
  const uint32_t dst0 = smem_u32(smem + G.stg);
  for (int r = lane; r < rows; r += 32)
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     dst0 + (uint32_t)r * pitch),
                 "l"(src + src_stride * r), "r"(row_bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Bounded wait that also gives up once another role has raised the abort flag.
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t phase, volatile int* abort) {
  for (long it = 0; it < (1L << 26); ++it) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(bar), "r"(phase)
                 : "memory");
    if (ok) return true;
    if (*abort) return false;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* out) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) out[j] = __uint_as_float(r[j]);
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

__global__ void __launch_bounds__(kThreadsAll, 1)
    k_hx_fused(const __grid_constant__ FusedGeom G, const __grid_constant__ FusedConst C,
               const __grid_constant__ FusedJobs J, FusedCounters* __restrict__ cnt, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar_t, mbar_full, mbar_empty, mbar_acc_full[2], mbar_acc_empty[2], mbar_stg;
  __shared__ uint32_t tmem_base;
  __shared__ unsigned ring[kRing];
  __shared__ int s_abort, s_prod_ok, s_epi_ok, s_last, s_stg_issued;
  volatile int* abort = &s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long nxny = (long)G.nx * G.ny;
  const long N = nxny * G.nz;
  const int nvec = J.nvec;

  if (tid == 0) {
    s_abort = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_t)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar_full)), "r"(kProdWarps * 32));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_empty)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_stg)));
    s_stg_issued = 0;
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(smem_u32(&mbar_acc_full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_acc_empty[b])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_u32(&mbar_t)), "r"(C.total)
                 : "memory");
    for (int c = 0; c < C.n; ++c)
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_u32(smem + C.dst[c])),
                   "l"(C.src[c]), "r"(C.bytes[c]), "r"(smem_u32(&mbar_t))
                   : "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(2 * G.acc_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // the prologue read only the grid's constant images; X, Y, V and the
  // counters may still be in use by the kernel ahead (programmatic launch)
  pg::pdl_wait();
  pg::pdl_release();
  const uint32_t tmem = tmem_base;
  if (tid == 0) ring[0] = atomicAdd(&cnt->ticket, 1u);
  __syncthreads();

  if (warp < kProdWarps) {
    // ------------------------------------------------------------ producers
    const int ptid = tid;  // 0 .. 32 kProdWarps - 1
    const uint32_t bar_stg = smem_u32(&mbar_stg);
    if (G.staged && warp == 0) {
      const Item it0 = decode(ring[0], nvec, G.nz, G.nzt, G.lag);
      stage_item(G, J, it0, N, nxny, smem, bar_stg, lane);
      if (lane == 0 && it0.kind >= 0) s_stg_issued = 1;
    }
    for (int i = 0;; ++i) {
      // ring[i] was written before the previous item's barrier; the leader
      // takes the ticket after it now, so its X data is in L2 by its turn
      const Item it = decode(ring[i % kRing], nvec, G.nz, G.nzt, G.lag);
      if (ptid == 0) {
        const unsigned t1 = atomicAdd(&cnt->ticket, 1u);
        ring[(i + 1) % kRing] = t1;
        if (!G.staged) prefetch_item(G, J, decode(t1, nvec, G.nz, G.nzt, G.lag), N, nxny);
      }
      if (G.staged && it.kind >= 0) {
        // this item's rows are in the staging buffer once its copies land
        if (ptid == 0) {
          const int ok = mbar_wait_or_abort(bar_stg, (uint32_t)(i & 1), abort);
          if (!ok) *abort = 1;
          s_prod_ok = ok;
        }
        named_sync(1, kProdWarps * 32);
        if (!s_prod_ok) break;
      }
      // the images are free once the previous item's MMAs are done
      auto ready = [&]() {
        if (ptid == 0) {
          const int ok = i == 0 || mbar_wait_or_abort(smem_u32(&mbar_empty), (uint32_t)((i - 1) & 1), abort);
          if (!ok) *abort = 1;
          s_prod_ok = ok;
        }
        named_sync(1, kProdWarps * 32);
      };
      const double *x, *v;
      double* y;
      if (it.kind >= 0) vec_ptrs(J, it.u, N, x, y, v);
      const unsigned char* stg = smem + G.stg;
      if (it.kind == 0) {
        const double* P = x + nxny * it.idx;
        if (G.staged)
          fill_plane(G, [&](int i, int j) { return *reinterpret_cast<const double*>(stg + j * G.stg_pxy + i * 8); },
                     smem, warp, lane, ready);
        else
          fill_plane(G, [&](int i, int j) { return P[i + (long)G.nx * j]; }, smem, warp, lane, ready);
      } else if (it.kind == 1) {
        const long p0 = (long)it.idx * kTile;
        if (G.staged)
          fill_ztile(G, [&](long q, int k) { return *reinterpret_cast<const double*>(stg + k * G.stg_pz + q * 8); },
                     p0, nxny, smem, warp, lane, ready);
        else
          fill_ztile(G, [&](long q, int k) { return x[p0 + q + nxny * k]; }, p0, nxny, smem, warp, lane, ready);
      } else {
        ready();
      }
      if (!s_prod_ok) break;
      if (it.kind >= 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (G.staged && it.kind >= 0) {
        // every producer has read the staging buffer (and fenced those reads
        // against the async proxy): the MMAs may start, and the next item's
        // copies may overwrite the buffer
        named_sync(1, kProdWarps * 32);
        mbar_arrive(smem_u32(&mbar_full));
        if (warp == 0) {
          const Item nx_it = decode(ring[(i + 1) % kRing], nvec, G.nz, G.nzt, G.lag);
          stage_item(G, J, nx_it, N, nxny, smem, bar_stg, lane);
          if (lane == 0 && nx_it.kind >= 0) s_stg_issued = i + 2;
        }
        continue;
      }
      mbar_arrive(smem_u32(&mbar_full));
      if (it.kind < 0) break;
    }
  } else if (warp < kIssueWarp) {
    // ------------------------------------------------------------- epilogue
    const int quarter = warp & 3, half = (warp - kProdWarps) >> 2;
    const bool leader = warp == kProdWarps && lane == 0;
    for (int i = 0;; ++i) {
      const int b = i & 1;
      // ring[i] was written before the producers' arrival for item i - 1,
      // which the wait for item i - 1 below has seen
      const Item it = decode(ring[i % kRing], nvec, G.nz, G.nzt, G.lag);
      const double *x = nullptr, *v = nullptr;
      double* y = nullptr;
      if (it.kind >= 0) vec_ptrs(J, it.u, N, x, y, v);
      const int i0 = 32 * quarter + lane;
      const long pl = nxny * (it.kind == 0 ? it.idx : 0);
      const long p = (long)(it.kind == 1 ? it.idx : 0) * kTile + i0;
      if (leader) {
        int ok = 1;
        if (it.kind == 1) {
          // every plane of the vector has its W in Y (bounded wait, ~2 s)
          const unsigned long long t0 = globaltimer_ns();
          while (*(volatile unsigned*)&cnt->done[it.u] < (unsigned)G.nz) {
            if (*abort || globaltimer_ns() - t0 > 2000000000ull) {
              ok = 0;
              break;
            }
            __nanosleep(128);
          }
          __threadfence();
        }
        if (ok) ok = mbar_wait_or_abort(smem_u32(&mbar_acc_full[b]), (uint32_t)((i >> 1) & 1), abort);
        if (!ok) *abort = 1;
        s_epi_ok = ok;
      }
      named_sync(2, kEpiWarps * 32);
      if (!s_epi_ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (it.kind < 0) break;
      const uint32_t acc = tmem + (uint32_t)b * G.acc_cols + ((uint32_t)(32 * quarter) << 16);
      if (it.kind == 0) {
        // the x + y sums of the plane, FP32, into the low word of each point's
        // Y slot (the z item of the same points reads them, then overwrites
        // the slot with the result)
        for (int c = half; c < (G.npy >> 4); c += 2) {
          float d[16];
          tmem_ld16(acc + (uint32_t)(16 * c), d);
          if (i0 < G.nx) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int j = 16 * c + q;
              if (j < G.ny)  // the whole 8-byte slot: full sectors, no fetch of Y before the write
                reinterpret_cast<uint2*>(y)[pl + i0 + (long)G.nx * j] = make_uint2(__float_as_uint(d[q]), 0u);
            }
          }
        }
      } else {
        // Y = V X + (Kxy + Kz): the partial sums add in FP32 (the accumulators'
        // own precision) and V X joins in one FP64 multiply-add
        const float* yw = reinterpret_cast<const float*>(y);
        for (int c = half; c < (G.npz >> 3); c += 2) {
          double vv[8], xx[8];
          float w[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int k = 8 * c + q;
            const bool in = p < nxny && k < G.nz;
            const long a = p + nxny * k;
            vv[q] = in ? v[a] : 0.0;
            xx[q] = in ? __ldcs(x + a) : 0.0;  // last uses of X and W: evict first, V stays
            w[q] = in ? __ldcs(yw + 2 * a) : 0.f;
          }
          float d[8];
          tmem_ld8(acc + (uint32_t)(8 * c), d);
          if (p < nxny) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int k = 8 * c + q;
              if (k < G.nz) __stcs(y + p + nxny * k, fma(vv[q], xx[q], (double)(w[q] + d[q])));
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      named_sync(2, kEpiWarps * 32);
      if (leader) {
        if (it.kind == 0) {
          // this plane's W is in Y: count it for the z items of vector u
          __threadfence();
          atomicAdd(&cnt->done[it.u], 1u);
        }
        mbar_arrive(smem_u32(&mbar_acc_empty[b]));
      }
    }
  } else if (lane == 0) {
    // --------------------------------------------------------------- issuer
    const uint32_t idesc_xy = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(G.npy >> 3) << 17) |
                              ((uint32_t)(kTile >> 4) << 24);
    const uint32_t idesc_z = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(G.npz >> 3) << 17) |
                             ((uint32_t)(kTile >> 4) << 24);
    const uint32_t sb = smem_u32(smem);
    const uint32_t sbo_x = (uint32_t)(G.kx >> 2) * 128, sbo_y = (uint32_t)(G.ky >> 2) * 128,
                   sbo_z = (uint32_t)(G.kz >> 2) * 128;
    // descriptors of K step 0; step kk adds kk * 256 bytes to the address field
    const uint64_t d_txh = smem_desc(sb + G.tx_hi, 128, sbo_x), d_txl = smem_desc(sb + G.tx_lo, 128, sbo_x);
    const uint64_t d_pnh = smem_desc(sb + G.pn_hi, 128, sbo_x), d_pnl = smem_desc(sb + G.pn_lo, 128, sbo_x);
    const uint64_t d_pth = smem_desc(sb + G.pt_hi, 128, sbo_y), d_ptl = smem_desc(sb + G.pt_lo, 128, sbo_y);
    const uint64_t d_tyh = smem_desc(sb + G.ty_hi, 128, sbo_y), d_tyl = smem_desc(sb + G.ty_lo, 128, sbo_y);
    const uint64_t d_zh = smem_desc(sb + G.z_hi, 128, sbo_z), d_zl = smem_desc(sb + G.z_lo, 128, sbo_z);
    const uint64_t d_tzh = smem_desc(sb + G.tz_hi, 128, sbo_z), d_tzl = smem_desc(sb + G.tz_lo, 128, sbo_z);
    bool ok = mbar_wait_or_abort(smem_u32(&mbar_t), 0, abort);
    int last_commit = -1;
    for (int i = 0; ok; ++i) {
      const int b = i & 1;
      ok = mbar_wait_or_abort(smem_u32(&mbar_full), (uint32_t)(i & 1), abort);
      if (ok && i >= 2) ok = mbar_wait_or_abort(smem_u32(&mbar_acc_empty[b]), (uint32_t)(((i - 2) >> 1) & 1), abort);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const Item it = decode(ring[i % kRing], nvec, G.nz, G.nzt, G.lag);
      if (it.kind < 0) {
        mbar_arrive(smem_u32(&mbar_acc_full[b]));
        mbar_arrive(smem_u32(&mbar_acc_full[b]));
        break;
      }
      const uint32_t acc = tmem + (uint32_t)b * G.acc_cols;
      if (it.kind == 0) {
        for (int kk = 0; kk < G.kx / 8; ++kk) {  // x: A = Tx, B = plane (rows j)
          const uint64_t o = (uint64_t)kk * 16;
          mma_tf32(acc, d_txl + o, d_pnh + o, idesc_xy, kk > 0 ? 1u : 0u);
          mma_tf32(acc, d_txh + o, d_pnl + o, idesc_xy, 1u);
          mma_tf32(acc, d_txh + o, d_pnh + o, idesc_xy, 1u);
        }
        for (int kk = 0; kk < G.ky / 8; ++kk) {  // y: A = plane (rows i), B = Ty
          const uint64_t o = (uint64_t)kk * 16;
          mma_tf32(acc, d_ptl + o, d_tyh + o, idesc_xy, 1u);
          mma_tf32(acc, d_pth + o, d_tyl + o, idesc_xy, 1u);
          mma_tf32(acc, d_pth + o, d_tyh + o, idesc_xy, 1u);
        }
      } else {
        for (int kk = 0; kk < G.kz / 8; ++kk) {  // z: A = 128 lines, B = Tz
          const uint64_t o = (uint64_t)kk * 16;
          mma_tf32(acc, d_zl + o, d_tzh + o, idesc_z, kk > 0 ? 1u : 0u);
          mma_tf32(acc, d_zh + o, d_tzl + o, idesc_z, 1u);
          mma_tf32(acc, d_zh + o, d_tzh + o, idesc_z, 1u);
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar_empty)));
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar_acc_full[b])));
      mbar_arrive(smem_u32(&mbar_acc_full[b]));  // orders the issuer's reads before the epilogue's
      last_commit = i;
    }
    if (!ok) {
      *abort = 1;
      // MMAs still in flight get a bounded wait before the tensor memory is released
      if (last_commit >= 0) mbar_wait(smem_u32(&mbar_empty), (uint32_t)(last_commit & 1));
      mbar_wait(smem_u32(&mbar_t), 0);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // a staging copy issued for an item that an aborted loop never consumed
  // lands before the CTA leaves (bounded wait; s_stg_issued = last item + 1)
  if (tid == 0 && G.staged && s_abort && s_stg_issued > 0)
    mbar_wait(smem_u32(&mbar_stg), (uint32_t)((s_stg_issued - 1) & 1));
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * G.acc_cols));
  if (tid == 0) {
    if (s_abort) atomicExch(err, 1);
    __threadfence();
    s_last = atomicAdd(&cnt->finished, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last) {
    // the last CTA to finish: every other CTA has stopped taking tickets and
    // counting planes, so the counters go back to zero for the next launch
    for (int u = tid; u < nvec; u += kThreadsAll) cnt->done[u] = 0;
    if (tid == 0) {
      cnt->ticket = 0;
      cnt->finished = 0;
    }
    __threadfence();
  }
}

}  // namespace

namespace pg {

namespace {

struct FusedPlan {
  bool ok = false;
  FusedGeom G{};
  FusedConst C{};
  size_t smem = 0;
  char why[160] = "";
};

int g_fused_sms = 0;
int g_fused_max_dyn = 0;

cudaError_t fused_init() {
  static const cudaError_t init = [] {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_fused_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_hx_fused);
    if (e == cudaSuccess) {
      g_fused_max_dyn = optin - (int)fa.sharedSizeBytes;
      e = cudaFuncSetAttribute(k_hx_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, g_fused_max_dyn);
    }
    if (g_fused_sms <= 0) g_fused_sms = 148;
    return e;
  }();
  return init;
}

bool same_matrix(const pg_grid* g, int a, int b) {
  return g->n[a] == g->n[b] && g->t[a] == g->t[b];
}

FusedPlan plan_fused(const pg_grid* g) {
  FusedPlan P;
  const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
  auto no = [&](const char* why) {
    snprintf(P.why, sizeof(P.why), "%s", why);
    return P;
  };
  if (nx > kTile) return no("nx > 128 (TMEM lanes)");
  for (int a = 0; a < 3; ++a)
    if (tc_kchunk(g->n[a]) != tc_kpad(g->n[a])) return no("an axis needs K chunks (n > 112)");
  FusedGeom& G = P.G;
  G.nx = nx;
  G.ny = ny;
  G.nz = nz;
  G.kx = tc_kpad(nx);
  G.ky = tc_kpad(ny);
  G.kz = tc_kpad(nz);
  G.npy = tc_npad(ny);
  G.npz = tc_npad(nz);
  if (G.npy > 256 || G.npz > 256) return no("N > 256");
  G.nzt = (int)(((long)nx * ny + kTile - 1) / kTile);
  G.lag = 2;
  const int npx = tc_npad(nx);
  const uint32_t sz_t[3] = {(uint32_t)npx * G.kx * 4, (uint32_t)G.npy * G.ky * 4, (uint32_t)G.npz * G.kz * 4};
  const uint32_t sz_pt = (uint32_t)G.kx * G.ky * 4;   // rows i (kx), K = j
  const uint32_t sz_pn = (uint32_t)G.npy * G.kx * 4;  // rows j (npy), K = i
  const uint32_t sz_z = (uint32_t)kTile * G.kz * 4;
  uint32_t cur = 0;
  G.pt_hi = cur;
  G.pt_lo = cur + sz_pt;
  cur += 2 * sz_pt;
  G.tx_hi = cur;
  G.tx_lo = cur + sz_t[0];
  cur += 2 * sz_t[0];
  G.pn_hi = cur;
  G.pn_lo = cur + sz_pn;
  cur += 2 * sz_pn;
  FusedConst& C = P.C;
  C.n = 0;
  C.total = 0;
  auto add_const = [&](const float* src, uint32_t dst, uint32_t bytes) {
    C.src[C.n] = src;
    C.dst[C.n] = dst;
    C.bytes[C.n] = bytes;
    C.total += bytes;
    ++C.n;
  };
  add_const(g->t_hi[0].p, G.tx_hi, sz_t[0]);
  add_const(g->t_lo[0].p, G.tx_lo, sz_t[0]);
  if (same_matrix(g, 1, 0)) {
    G.ty_hi = G.tx_hi;
    G.ty_lo = G.tx_lo;
  } else {
    G.ty_hi = cur;
    G.ty_lo = cur + sz_t[1];
    cur += 2 * sz_t[1];
    add_const(g->t_hi[1].p, G.ty_hi, sz_t[1]);
    add_const(g->t_lo[1].p, G.ty_lo, sz_t[1]);
  }
  if (same_matrix(g, 2, 0)) {
    G.tz_hi = G.tx_hi;
    G.tz_lo = G.tx_lo;
  } else if (same_matrix(g, 2, 1)) {
    G.tz_hi = G.ty_hi;
    G.tz_lo = G.ty_lo;
  } else {
    G.tz_hi = cur;
    G.tz_lo = cur + sz_t[2];
    cur += 2 * sz_t[2];
    add_const(g->t_hi[2].p, G.tz_hi, sz_t[2]);
    add_const(g->t_lo[2].p, G.tz_lo, sz_t[2]);
  }
  // the z tile over the plane images where they are large enough
  if (sz_z <= 2 * sz_pt) {
    G.z_hi = G.pt_hi;
  } else {
    G.z_hi = cur;
    cur += sz_z;
  }
  if (sz_z <= 2 * sz_pn) {
    G.z_lo = G.pn_hi;
  } else {
    G.z_lo = cur;
    cur += sz_z;
  }
  // A operands are read as 128 rows
  uint32_t total = cur;
  total = std::max(total, G.tx_hi + (uint32_t)kTile * G.kx * 4);
  total = std::max(total, G.tx_lo + (uint32_t)kTile * G.kx * 4);
  total = std::max(total, G.pt_hi + (uint32_t)kTile * G.ky * 4);
  total = std::max(total, G.pt_lo + (uint32_t)kTile * G.ky * 4);
  P.smem = total;
  if ((long)P.smem > (long)g_fused_max_dyn) return no("operand images exceed shared memory");
  // staging buffer for the next item's raw rows, where it fits (row pitches:
  // a multiple of 16 bytes, 32 resp. 64 bytes past a multiple of 128, so
  // that the producers' reads of eight rows resp. four rows take the minimum
  // number of shared-memory wavefronts)
  G.staged = 0;
  if (nx % 2 == 0) {
    G.stg_pxy = (uint32_t)((nx * 8 + 127) / 128 * 128 + 32);
    G.stg_pz = (uint32_t)(kTile * 8 + 64);
    G.stg = (total + 127u) / 128u * 128u;
    const size_t with = (size_t)G.stg + std::max((size_t)ny * G.stg_pxy, (size_t)nz * G.stg_pz);
    if ((long)with <= (long)g_fused_max_dyn) {
      G.staged = 1;
      P.smem = with;
    }
  }
  uint32_t cols = 32;
  while (cols < (uint32_t)std::max(G.npy, G.npz)) cols <<= 1;
  G.acc_cols = cols;
  P.ok = true;
  return P;
}

}  // namespace

// The counter block of the fused kernel for the calling stream: one per
// stream (launches on one stream are ordered, and the last CTA of a launch
// resets its block), keyed by the stream's process-unique id.
static pg_status fused_counters(const pg_grid* g, cudaStream_t st, FusedCounters** out) {
  unsigned long long id = 0;
  PG_CUDA_TRY(cudaStreamGetId(st, &id));
  std::lock_guard<std::mutex> l(g->fused_m);
  auto it = g->fused_cnt.find(id);
  if (it == g->fused_cnt.end()) {
    if (g->fused_cnt.size() >= 256) {
      set_error("fused H*X: more than 256 streams used on one grid");
      return PG_UNSUPPORTED;
    }
    std::unique_ptr<DevBuf<unsigned>> b(new DevBuf<unsigned>());
    PG_TRY(b->alloc(sizeof(FusedCounters) / sizeof(unsigned)));
    PG_CUDA_TRY(cudaMemset(b->p, 0, sizeof(FusedCounters)));
    it = g->fused_cnt.emplace(id, std::move(b)).first;
  }
  *out = reinterpret_cast<FusedCounters*>(it->second->p);
  return PG_OK;
}

bool fused_hx_ok(const pg_grid* g) {
  if (fused_init() != cudaSuccess) return false;
  return plan_fused(g).ok;
}

// Mixed H*X of up to kMaxJobs vector blocks on the same grid in one launch
// of the fused kernel (the caller has checked fused_hx_ok).
pg_status hx_fused_jobs(const pg_grid* g, const double* const* v, const double* const* x, double* const* y,
                        const int* nvec, int njobs, const HxParams& hp, cudaStream_t st) {
  PG_ARG(njobs > 0 && njobs <= kMaxJobs, "fused H*X: %d jobs (at most %d)", njobs, kMaxJobs);
  PG_CUDA_TRY(fused_init());
  FusedPlan P = plan_fused(g);
  if (!P.ok) {
    set_error("fused H*X not available on this grid: %s", P.why);
    return PG_UNSUPPORTED;
  }
  if (hp.lag > 0) P.G.lag = hp.lag;
  // bulk copies need 16-byte aligned rows: every block of X must start on a
  // 16-byte boundary (nx even makes every row and tile offset a multiple)
  for (int j = 0; j < njobs; ++j)
    if (nvec[j] > 0 && ((uintptr_t)x[j] & 15u) != 0) P.G.staged = 0;
  if (g->N % 2 != 0) P.G.staged = 0;
  FusedCounters* cnt = nullptr;
  PG_TRY(fused_counters(g, st, &cnt));
  FusedJobs J;
  memset(&J, 0, sizeof(J));
  int total = 0;
  for (int j = 0; j < njobs; ++j) {
    PG_ARG(nvec[j] >= 0, "fused H*X: negative vector count");
    J.j[J.n].x = x[j];
    J.j[J.n].y = y[j];
    J.j[J.n].v = v[j];
    J.j[J.n].nvec = nvec[j];
    J.j[J.n].vec0 = total;
    total += nvec[j];
    if (nvec[j] > 0) ++J.n;
  }
  if (total == 0) return PG_OK;
  PG_ARG(total <= kFusedMaxVec, "fused H*X: %d vectors in one launch (at most %d)", total, kFusedMaxVec);
  J.nvec = total;
  const long items = (long)total * (P.G.nz + P.G.nzt);
  const int cap = hp.ctas > 0 && hp.ctas < g_fused_sms ? hp.ctas : g_fused_sms;
  const int grid = (int)std::min<long>(items, cap);
  PG_CUDA_TRY(launch_dependent(k_hx_fused, dim3(grid), dim3(kThreadsAll), P.smem, st, P.G, P.C, J, cnt, g->tc_err.p));
  return check_launch("k_hx_fused");
}

pg_status hx_fused(const pg_grid* g, const double* v, const double* x, double* y, int nvec, const HxParams& hp,
                   cudaStream_t st) {
  for (int v0 = 0; v0 < nvec; v0 += kFusedMaxVec) {
    const int nb = std::min(kFusedMaxVec, nvec - v0);
    const double* xs = x + (long)v0 * g->N;
    double* ys = y + (long)v0 * g->N;
    PG_TRY(hx_fused_jobs(g, &v, &xs, &ys, &nb, 1, hp, st));
  }
  return PG_OK;
}

// The tuned launch parameters (tune_hx.py measures every candidate on a
// GB300 per cubic grid size and block size and keeps the fastest); the
// build turns the table into this include.
struct TunedEntry {
  int n, nvec, kind, lag, ctas, form;
};
static const TunedEntry kTuned[] = {
#include "pg_hx_tuned.inc"
    {0, 0, 0, 0, 0, 0}};

bool f16_hx_ok(const pg_grid* g);
void f16_plan_text(const pg_grid* g, const HxParams& p, char* buf, int len);

HxParams hx_params(const pg_grid* g, int nvec) {
  const bool fused_ok = fused_hx_ok(g);
  const bool f16_ok = f16_hx_ok(g);
  HxParams p{f16_ok ? 3 : (fused_ok ? 2 : 1), 2, 0, 0};
  if (g->n[0] == g->n[1] && g->n[1] == g->n[2]) {
    // the entry of this grid size with the nearest block size
    const TunedEntry* best = nullptr;
    for (const TunedEntry* e = kTuned; e->n; ++e)
      if (e->n == g->n[0] && (!best || std::abs(e->nvec - nvec) < std::abs(best->nvec - nvec))) best = e;
    if (best) p = HxParams{best->kind, best->lag, best->ctas, best->form};
  }
  if (g->hx_kernel) p.kind = g->hx_kernel;
  if (g->hx_lag) p.lag = g->hx_lag;
  if (g->hx_ctas) p.ctas = g->hx_ctas;
  if (g->hx_form) p.form = g->hx_form;
  if (p.kind == 3 && !f16_ok && g->hx_kernel != 3) p.kind = fused_ok ? 2 : 1;
  if (p.kind == 2 && !fused_ok && g->hx_kernel != 2) p.kind = 1;
  return p;
}

// Text description of the mixed-form H*X plan of a grid for blocks of nvec vectors.
void hx_plan_text(const pg_grid* g, int nvec, char* buf, int len) {
  if (fused_init() != cudaSuccess) {
    snprintf(buf, (size_t)len, "three axis passes (k_hx_tc): device query failed");
    return;
  }
  const FusedPlan P = plan_fused(g);
  const HxParams p = hx_params(g, nvec);
  if (p.kind == 3) {
    f16_plan_text(g, p, buf, len);
    return;
  }
  if (p.kind == 2 && P.ok)
    snprintf(buf, (size_t)len,
             "fused (k_hx_fused): xy planes %dx%d + z tiles of 128 lines (%d per vector, lag %d vectors), "
             "K %d/%d/%d, %s, %zu B shared memory, %d constant images, %u TMEM columns x 2, %d CTAs",
             P.G.nx, P.G.ny, P.G.nzt, p.lag, P.G.kx, P.G.ky, P.G.kz,
             P.G.staged ? "rows bulk-copied to a staging buffer" : "rows loaded from L2", P.smem, P.C.n / 2,
             P.G.acc_cols,
             p.ctas > 0 && p.ctas < g_fused_sms ? p.ctas : g_fused_sms);
  else
    snprintf(buf, (size_t)len, "three axis passes (k_hx_tc): %s form, %d CTAs%s%s",
             p.form == 1 ? "serial" : (p.form == 2 ? "pipelined" : "automatic"),
             p.ctas > 0 && p.ctas < g_fused_sms ? p.ctas : g_fused_sms, P.ok ? "" : "; fused kernel: ",
             P.ok ? "" : P.why);
}

}  // namespace pg

extern "C" pg_status pg_grid_set_hx_kernel(pg_grid* g, int kind) {
  PG_ARG(g, "pg_grid_set_hx_kernel: null grid");
  PG_ARG(kind >= 0 && kind <= 3, "pg_grid_set_hx_kernel: kind must be 0, 1, 2 or 3 (got %d)", kind);
  if (kind == 3 && !pg::f16_hx_ok(g)) {
    char why[256];
    pg::HxParams p{3, 2, 0, 0};
    pg::f16_plan_text(g, p, why, sizeof(why));
    pg::set_error("pg_grid_set_hx_kernel: %s", why);
    return PG_UNSUPPORTED;
  }
  if (kind == 2 && !pg::fused_hx_ok(g)) {
    char why[256];
    pg::hx_plan_text(g, 1, why, sizeof(why));
    pg::set_error("pg_grid_set_hx_kernel: %s", why);
    return PG_UNSUPPORTED;
  }
  g->hx_kernel = kind;
  return PG_OK;
}

extern "C" pg_status pg_grid_set_hx_params(pg_grid* g, int kind, int lag, int ctas, int form) {
  PG_ARG(g, "pg_grid_set_hx_params: null grid");
  PG_ARG(lag >= 0 && lag <= 64 && ctas >= 0 && ctas <= 4096 && form >= 0 && form <= 2,
         "pg_grid_set_hx_params: lag %d, ctas %d or form %d out of range", lag, ctas, form);
  PG_TRY(pg_grid_set_hx_kernel(g, kind));
  g->hx_lag = lag;
  g->hx_ctas = ctas;
  g->hx_form = form;
  return PG_OK;
}

extern "C" pg_status pg_grid_hx_plan(const pg_grid* g, char* text, int len) {
  return pg_grid_hx_plan_for(g, 1, text, len);
}

extern "C" pg_status pg_grid_hx_plan_for(const pg_grid* g, int nvec, char* text, int len) {
  PG_ARG(g && text && len > 0 && nvec > 0, "pg_grid_hx_plan: bad arguments");
  pg::hx_plan_text(g, nvec, text, len);
  return PG_OK;
}
