// Y = H X, mixed form with an FP16 split: one persistent tensor-core kernel
// with the work items of the fused kernel (pg_hx_fused.cu: the x and y
// contractions of one grid plane into one TMEM tile; the z contraction of 128
// grid lines; a ticket queue that keeps each vector's X and partial sums in
// L2 between the two), for grids of at most 96 points per axis whose axes
// share one kinetic matrix.
//
// H = V + Tx (+) Ty (+) Tz on the x-fastest grid (src/mtx.cpp:22-109).
//
// Operands.  Each item's raw FP64 values are copied by the tensor memory
// accelerator into a staging buffer while the item before it is converted
// and multiplied: boxes 16 values (128 bytes) wide with the 128-byte swizzle
// (16-byte chunk c of box row r lands at chunk c ^ (r mod 8)), six to eight
// copies per item; the producers read eight consecutive rows at a time, so
// the swizzle puts their reads in distinct banks.  The
// producer warps convert them to an FP16 high part and remainder scaled by a
// power of two 2^s per item, so that hi + lo holds about 22 significant
// bits, the precision of the TF32 split of the other kernels: the item's
// largest |x| lands in [2^14, 2^15) (s from the largest FP64 exponent of its
// staged values, found by a pass over them); where the caller knows every
// value lies in [-1, 1] (the Davidson's orthonormal basis vectors) s = 14
// without the pass.  The kinetic matrices are kept as FP16 images of T 2^tau
// (pg_grid.t16_*).  D = Ah Bh + Ah Bl + Al Bh accumulates in FP32 in TMEM and
// the epilogue multiplies by 2^-(s + tau), exactly.
//
// One plane image serves both contractions of an xy item: stored with rows
// j and K = i (8 x 8 FP16 core matrices, no swizzle), it is the K-major B
// operand of the x contraction (A = Tx, K = i) and the MN-major A operand of
// the y contraction (M = i, K = j; B = Ty).  The z tile's image holds 8
// planes x 8 points per core matrix: the MN-major A operand of the z
// contraction (M = point, K = plane; B = Tz).  So each value is converted
// once and stored as one 16-byte row of a core matrix, from 64 contiguous
// staging bytes.
//
// Epilogues as the fused kernel: the x + y sums go, as FP32, to the low word
// of each point's Y slot; the z epilogue writes Y = fma(V, X, W + Kz), with
// V X in FP64 (one FP64 operation per point: W + Kz is converted with
// integer operations).
//
// Every wait is bounded; a timeout sets the grid's error word (pg_hx reports
// PG_DEVICE_TIMEOUT) and the kernel drains its copies and MMAs and returns.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>

#include "pg_tc16.cuh"

namespace {

constexpr int kMaxJobs = 8;  // jobs of one launch (each carries two tensor maps); more go to further launches
constexpr int kF16MaxVec = 1024;

}  // namespace

namespace pg {

struct F16Job {
  CUtensorMap txy;  // X of the job as (x, y, plane of all its vectors), boxes 16 x ny x 1
  CUtensorMap tz;   // X of the job as (plane point, plane of all its vectors), boxes 16 x nz
  const double* x;
  double* y;
  const double* v;
  int nvec;
  int vec0;
};
struct F16Jobs {
  F16Job j[kMaxJobs];
  int n;
  int nvec;
};

struct F16Geom {
  int nx, ny, nz;
  int kx, ky, kz;     // K extents padded to 16
  int npy, npz;       // MMA N extents padded to 16
  int nzt;            // z items per vector
  int lag;            // vectors between a vector's xy items and its z items
  int tau;            // the kinetic images hold T 2^tau
  int unit_bound;     // 1: every value of X lies in [-1, 1]; a fixed scale 2^14, no maximum pass
  uint32_t t_hi, t_lo;            // the kinetic image (shared by the three axes)
  uint32_t t_bytes;               // bytes of one kinetic image as copied
  uint32_t op_hi, op_lo;          // operand images of the current item
  uint32_t stg;                   // staging buffer (1024-byte aligned)
  uint32_t reg_xy, reg_z;         // bytes of one 16-value-wide box region: 128 ny, 128 nz (rounded to 1024)
  uint32_t acc_cols;              // TMEM columns per accumulator
  int acc_shift;                  // log2 of the accumulators (2 or 4) the epilogue may lag behind by
};

struct F16Counters {
  unsigned ticket;
  unsigned finished;
  unsigned done[kF16MaxVec];  // finished xy items per vector
};

}  // namespace pg

namespace {

using pg::F16Counters;
using pg::F16Geom;
using pg::F16Jobs;

struct Item {
  int kind;  // 0: xy plane, 1: z tile, -1: none
  int u;     // vector in the launch's list
  int idx;   // plane k or z tile t
};

// Ticket -> work item, as the fused kernel: XY(0) .. XY(L-1), then XY(s),
// Z(s-L) for s = L .. b-1, then the remaining Z blocks.
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

__device__ __forceinline__ int job_of(const F16Jobs& J, int u) {
  int j = 0;
  while (j + 1 < J.n && u >= J.j[j + 1].vec0) ++j;
  return j;
}

__device__ __forceinline__ void vec_ptrs(const F16Jobs& J, int u, long N, const double*& x, double*& y,
                                         const double*& v) {
  const int j = job_of(J, u);
  const long off = (long)(u - J.j[j].vec0) * N;
  x = J.j[j].x + off;
  y = J.j[j].y + off;
  v = J.j[j].v;
}

// The lanes of one warp: the tensor copies of an item into the staging buffer,
// completing on mbarrier bar.  An xy item: ceil(nx / 16) boxes of 16 x ny
// values (plane idx of its vector), one region each; a z item: eight boxes
// of 16 points x nz planes.  Values past the grid (the last box of a row,
// the last tile) arrive as zeros; every box counts in full.  x coordinates
// are multiples of 16 values.
__device__ __forceinline__ void stage_item(const F16Geom& G, const F16Jobs& J, const Item& it, long nxny,
                                           unsigned char* smem, uint32_t bar, int lane) {
  if (it.kind < 0) return;
  const int jb = job_of(J, it.u);
  const int ul = it.u - J.j[jb].vec0;
  const int nbox = it.kind == 0 ? (G.nx + 15) / 16 : kTile / 16;
  const uint32_t box_bytes = 128u * (uint32_t)(it.kind == 0 ? G.ny : G.nz);
  if (lane == 0) {
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(bar), "r"((uint32_t)nbox * box_bytes)
                 : "memory");
  }
  __syncwarp();
  const uint32_t dst0 = smem_u32(smem + G.stg);
  // one box per lane
  if (it.kind == 0) {
    const void* map = &J.j[jb].txy;
    const int zc = ul * G.nz + it.idx;
    for (int b = lane; b < nbox; b += 32)
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
          "[%5];" ::"r"(dst0 + (uint32_t)b * G.reg_xy),
          "l"(map), "r"(16 * b), "r"(0), "r"(zc), "r"(bar)
          : "memory");
  } else {
    const void* map = &J.j[jb].tz;
    const int p0 = it.idx * kTile;
    const int yc = ul * G.nz;
    for (int b = lane; b < nbox; b += 32)
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
          "[%4];" ::"r"(dst0 + (uint32_t)b * G.reg_z),
          "l"(map), "r"(p0 + 16 * b), "r"(yc), "r"(bar)
          : "memory");
  }
}

__global__ void __launch_bounds__(kThreadsAll, 1)
    k_hx_f16(const __grid_constant__ F16Geom G, const unsigned short* __restrict__ t_hi,
             const unsigned short* __restrict__ t_lo, const __grid_constant__ F16Jobs J, F16Counters* __restrict__ cnt,
             int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar_t, mbar_full, mbar_empty, mbar_acc_full[kMaxAcc], mbar_acc_empty[kMaxAcc], mbar_stg;
  __shared__ uint32_t tmem_base;
  __shared__ unsigned ring[kRing];
  __shared__ int sig[kRing];  // item scale exponents, by ticket slot
  __shared__ int s_emax[kProdWarps];
  __shared__ int s_abort, s_prod_ok, s_epi_ok, s_last, s_stg_issued;
  volatile int* abort = &s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long nxny = (long)G.nx * G.ny;
  const long N = nxny * G.nz;
  const int nvec = J.nvec;

  if (tid == 0) {
    s_abort = 0;
    s_stg_issued = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_t)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar_full)), "r"(kProdWarps * 32));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_empty)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_stg)));
    for (int b = 0; b < kMaxAcc; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(smem_u32(&mbar_acc_full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_acc_empty[b])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // the kinetic image (the grid's constant data) while the kernel ahead finishes
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_u32(&mbar_t)), "r"(2u * G.t_bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(smem + G.t_hi)),
                 "l"(t_hi), "r"(G.t_bytes), "r"(smem_u32(&mbar_t))
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(smem + G.t_lo)),
                 "l"(t_lo), "r"(G.t_bytes), "r"(smem_u32(&mbar_t))
                 : "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(G.acc_cols << G.acc_shift));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  pg::pdl_wait();
  pg::pdl_release();
  const uint32_t tmem = tmem_base;
  if (tid == 0) ring[0] = atomicAdd(&cnt->ticket, 1u);
  __syncthreads();

  if (warp < kProdWarps) {
    // ------------------------------------------------------------ producers
    const int ptid = tid;
    const uint32_t bar_stg = smem_u32(&mbar_stg);
    const unsigned char* stg = smem + G.stg;
    if (warp == 0) {
      const Item it0 = decode(ring[0], nvec, G.nz, G.nzt, G.lag);
      stage_item(G, J, it0, nxny, smem, bar_stg, lane);
      if (lane == 0 && it0.kind >= 0) s_stg_issued = 1;
    }
    for (int i = 0;; ++i) {
      const Item it = decode(ring[i % kRing], nvec, G.nz, G.nzt, G.lag);
      if (ptid == 0) ring[(i + 1) % kRing] = atomicAdd(&cnt->ticket, 1u);
      if (it.kind < 0) {
        // no more work: hand the issuer its stop item once the images are free
        if (ptid == 0) {
          const int ok = i == 0 || mbar_wait_or_abort(smem_u32(&mbar_empty), (uint32_t)((i - 1) & 1), abort);
          if (!ok) *abort = 1;
        }
        mbar_arrive(smem_u32(&mbar_full));
        break;
      }
      // the item's rows have landed
      if (ptid == 0) {
        const int ok = mbar_wait_or_abort(bar_stg, (uint32_t)(i & 1), abort);
        if (!ok) *abort = 1;
        s_prod_ok = ok;
      }
      named_sync(1, kProdWarps * 32);
      if (!s_prod_ok) break;
      const int ntask = it.kind == 0 ? (G.kx >> 3) * G.npy : 16 * G.kz;
      // the item's scale: its largest exponent over the producers
      if (!G.unit_bound) {
        int em = max_exponent(stg, ntask, it.kind, G, ptid);
        em = (int)__reduce_max_sync(0xffffffffu, (unsigned)em);
        if (lane == 0) s_emax[warp] = em;
      }
      // the images are free once the previous item's MMAs are done
      if (ptid == 0) {
        const int ok = i == 0 || mbar_wait_or_abort(smem_u32(&mbar_empty), (uint32_t)((i - 1) & 1), abort);
        if (!ok) *abort = 1;
        s_prod_ok = ok;
      }
      named_sync(1, kProdWarps * 32);
      if (!s_prod_ok) break;
      int emax = 1023;  // |x| <= 1
      if (!G.unit_bound) {
        emax = 0;
#pragma unroll
        for (int w = 0; w < kProdWarps; ++w) emax = s_emax[w] > emax ? s_emax[w] : emax;
      }
      // largest |x| < 2^(emax - 1022): scaled below 2^15.  The epilogue's
      // factor 2^-(s + tau) must be a normal FP32 number; blocks whose values
      // all lie below about 2^-100 (or above 2^100) are scaled less and lose
      // what FP32 cannot hold, as the TF32 split of the other kernels does.
      int s = (emax == 0 || emax == 0x7ff) ? 0 : 1037 - emax;
      s = s > 126 - G.tau ? 126 - G.tau : (s < -127 - G.tau ? -127 - G.tau : s);
      if (ptid == 0) sig[i % kRing] = s;
      unsigned char* ohi = smem + G.op_hi;
      unsigned char* olo = smem + G.op_lo;
      TaskIter ti(ptid, it.kind == 0 ? G.npy : G.kz);
      const int sb = s - 896;
      // two tasks per turn: their loads and conversions overlap
      int t = ptid;
      for (; t + kProdWarps * 32 < ntask; t += 2 * kProdWarps * 32) {
        const Task k0 = task_of(G, it.kind, ti);
        ti.next();
        const Task k1 = task_of(G, it.kind, ti);
        ti.next();
        double v0[8], v1[8];
        load8(stg, k0, v0);
        load8(stg, k1, v1);
        uint4 h0, l0, h1, l1;
        split8(v0, sb, h0, l0);
        split8(v1, sb, h1, l1);
        *reinterpret_cast<uint4*>(ohi + k0.dst) = h0;
        *reinterpret_cast<uint4*>(olo + k0.dst) = l0;
        *reinterpret_cast<uint4*>(ohi + k1.dst) = h1;
        *reinterpret_cast<uint4*>(olo + k1.dst) = l1;
      }
      if (t < ntask) {
        const Task k = task_of(G, it.kind, ti);
        double v[8];
        load8(stg, k, v);
        uint4 h, l;
        split8(v, sb, h, l);
        *reinterpret_cast<uint4*>(ohi + k.dst) = h;
        *reinterpret_cast<uint4*>(olo + k.dst) = l;
      }
      // the staging reads and image writes are done (and fenced against the
      // async proxy): the next item's copies may start, the MMAs may read
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      named_sync(1, kProdWarps * 32);
      // the MMAs may start now; warp 0 then issues the next item's copies
      mbar_arrive(smem_u32(&mbar_full));
      if (warp == 0) {
        const Item nx_it = decode(ring[(i + 1) % kRing], nvec, G.nz, G.nzt, G.lag);
        stage_item(G, J, nx_it, nxny, smem, bar_stg, lane);
        if (lane == 0 && nx_it.kind >= 0) s_stg_issued = i + 2;
      }
    }
  } else if (warp < kIssueWarp) {
    // ------------------------------------------------------------- epilogue
    const int quarter = warp & 3, part = (warp - kProdWarps) >> 2;  // warps of one lane quarter share its columns
    const bool leader = warp == kProdWarps && lane == 0;
    for (int i = 0;; ++i) {
      const int b = i & ((1 << G.acc_shift) - 1);
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
        if (ok) ok = mbar_wait_or_abort(smem_u32(&mbar_acc_full[b]), (uint32_t)((i >> G.acc_shift) & 1), abort);
        if (!ok) *abort = 1;
        s_epi_ok = ok;
      }
      named_sync(2, kEpiWarps * 32);
      if (!s_epi_ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (it.kind < 0) break;
      const float unscale = exp2i(-(sig[i % kRing] + G.tau));
      const uint32_t acc = tmem + (uint32_t)b * G.acc_cols + ((uint32_t)(32 * quarter) << 16);
      if (it.kind == 0) {
        // the x + y sums of the plane, FP32, into the low word of each
        // point's Y slot (the z item of the same points reads them)
        for (int c = part; c < (G.npy >> 4); c += kEpiParts) {
          float d[16];
          tmem_ld16(acc + (uint32_t)(16 * c), d);
          if (i0 < G.nx) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int j = 16 * c + q;
              if (j < G.ny)  // the whole 8-byte slot: full sectors, no fetch of Y before the write
                reinterpret_cast<uint2*>(y)[pl + i0 + (long)G.nx * j] = make_uint2(__float_as_uint(d[q] * unscale), 0u);
            }
          }
        }
      } else {
        // Y = V X + (Kxy + Kz): the partial sums add in FP32 and V X joins in
        // one FP64 multiply-add (the FP32 sum converted with integer operations)
        const float* yw = reinterpret_cast<const float*>(y);
        for (int c = part; c < (G.npz >> 4); c += kEpiParts) {
          double vv[16], xx[16];
          float w[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int k = 16 * c + q;
            const bool in = p < nxny && k < G.nz;
            const long a = p + nxny * k;
            vv[q] = in ? v[a] : 0.0;
            xx[q] = in ? __ldcs(x + a) : 0.0;  // last uses of X and W: evict first, V stays
            w[q] = in ? __ldcs(yw + 2 * a) : 0.f;
          }
          float d[16];
          tmem_ld16(acc + (uint32_t)(16 * c), d);
          if (p < nxny) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int k = 16 * c + q;
              if (k < G.nz) __stcs(y + p + nxny * k, fma(vv[q], xx[q], f32_to_f64(fmaf(d[q], unscale, w[q]))));
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      named_sync(2, kEpiWarps * 32);
      if (leader) {
        if (it.kind == 0) {
          __threadfence();
          atomicAdd(&cnt->done[it.u], 1u);
        }
        mbar_arrive(smem_u32(&mbar_acc_empty[b]));
      }
    }
  } else if (lane == 0) {
    // --------------------------------------------------------------- issuer
    // kind::f16, FP16 A and B, FP32 D; bit 15: A MN-major
    const uint32_t id_x = (1u << 4) | ((uint32_t)(G.npy >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
    const uint32_t id_y = id_x | (1u << 15);
    const uint32_t id_z = (1u << 4) | (1u << 15) | ((uint32_t)(G.npz >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
    const uint32_t sb = smem_u32(smem);
    const uint32_t kq_x = (uint32_t)(G.kx >> 3) * 128u;  // row-group stride of the plane / x-kinetic image
    const uint32_t kq_y = (uint32_t)(G.ky >> 3) * 128u;
    const uint32_t kq_z = (uint32_t)(G.kz >> 3) * 128u;
    // K-major images: LBO = next 8 K values (128 B), SBO = next 8 rows.
    // MN-major images: LBO = next 8 K values, SBO = next 8 M values.
    const uint64_t d_th = smem_desc(sb + G.t_hi, 128, kq_x), d_tl = smem_desc(sb + G.t_lo, 128, kq_x);
    const uint64_t d_tyh = smem_desc(sb + G.t_hi, 128, kq_y), d_tyl = smem_desc(sb + G.t_lo, 128, kq_y);
    const uint64_t d_tzh = smem_desc(sb + G.t_hi, 128, kq_z), d_tzl = smem_desc(sb + G.t_lo, 128, kq_z);
    const uint64_t d_pbh = smem_desc(sb + G.op_hi, 128, kq_x), d_pbl = smem_desc(sb + G.op_lo, 128, kq_x);
    const uint64_t d_pah = smem_desc(sb + G.op_hi, kq_x, 128), d_pal = smem_desc(sb + G.op_lo, kq_x, 128);
    const uint64_t d_zh = smem_desc(sb + G.op_hi, 16 * 128, 128), d_zl = smem_desc(sb + G.op_lo, 16 * 128, 128);
    bool ok = mbar_wait_or_abort(smem_u32(&mbar_t), 0, abort);
    int last_commit = -1;
    for (int i = 0; ok; ++i) {
      const int b = i & ((1 << G.acc_shift) - 1);
      ok = mbar_wait_or_abort(smem_u32(&mbar_full), (uint32_t)(i & 1), abort);
      const int nacc = 1 << G.acc_shift;
      if (ok && i >= nacc)
        ok = mbar_wait_or_abort(smem_u32(&mbar_acc_empty[b]), (uint32_t)(((i - nacc) >> G.acc_shift) & 1), abort);
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
        for (int kk = 0; kk < G.kx / 16; ++kk) {  // x: A = Tx (K = i), B = plane rows j
          const uint64_t o = (uint64_t)kk * 16;    // 256 bytes: two core matrices along K
          mma_f16(acc, d_tl + o, d_pbh + o, id_x, kk > 0 ? 1u : 0u);
          mma_f16(acc, d_th + o, d_pbl + o, id_x, 1u);
          mma_f16(acc, d_th + o, d_pbh + o, id_x, 1u);
        }
        for (int kk = 0; kk < G.ky / 16; ++kk) {  // y: A = plane, M = i, K = j (MN-major); B = Ty
          const uint64_t oa = (uint64_t)kk * 2 * (kq_x >> 4), ob = (uint64_t)kk * 16;
          mma_f16(acc, d_pal + oa, d_tyh + ob, id_y, 1u);
          mma_f16(acc, d_pah + oa, d_tyl + ob, id_y, 1u);
          mma_f16(acc, d_pah + oa, d_tyh + ob, id_y, 1u);
        }
      } else {
        for (int kk = 0; kk < G.kz / 16; ++kk) {  // z: A = 128 lines, M = point, K = plane (MN-major); B = Tz
          const uint64_t oa = (uint64_t)kk * 2 * 16 * (128 >> 4), ob = (uint64_t)kk * 16;
          mma_f16(acc, d_zl + oa, d_tzh + ob, id_z, kk > 0 ? 1u : 0u);
          mma_f16(acc, d_zh + oa, d_tzl + ob, id_z, 1u);
          mma_f16(acc, d_zh + oa, d_tzh + ob, id_z, 1u);
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar_empty)));
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar_acc_full[b])));
      mbar_arrive(smem_u32(&mbar_acc_full[b]));
      last_commit = i;
    }
    if (!ok) {
      *abort = 1;
      if (last_commit >= 0) mbar_wait(smem_u32(&mbar_empty), (uint32_t)(last_commit & 1));
      mbar_wait(smem_u32(&mbar_t), 0);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // a staging copy issued for an item that an aborted loop never consumed
  // lands before the CTA leaves (bounded wait)
  if (tid == 0 && s_abort && s_stg_issued > 0) mbar_wait(smem_u32(&mbar_stg), (uint32_t)((s_stg_issued - 1) & 1));
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(G.acc_cols << G.acc_shift));
  if (tid == 0) {
    if (s_abort) atomicExch(err, 1);
    __threadfence();
    s_last = atomicAdd(&cnt->finished, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last) {
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

struct F16Plan {
  bool ok = false;
  F16Geom G{};
  size_t smem = 0;
  char why[160] = "";
};

int g_f16_sms = 0;
int g_f16_max_dyn = 0;

cudaError_t f16_init() {
  static const cudaError_t init = [] {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_f16_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_hx_f16);
    if (e == cudaSuccess) {
      g_f16_max_dyn = optin - (int)fa.sharedSizeBytes;
      e = cudaFuncSetAttribute(k_hx_f16, cudaFuncAttributeMaxDynamicSharedMemorySize, g_f16_max_dyn);
    }
    if (g_f16_sms <= 0) g_f16_sms = 148;
    return e;
  }();
  return init;
}

F16Plan plan_f16(const pg_grid* g) {
  F16Plan P;
  const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
  auto no = [&](const char* why) {
    snprintf(P.why, sizeof(P.why), "%s", why);
    return P;
  };
  if (!g->t16_hi[0].p) return no("no FP16 kinetic images (an axis has more than 128 points)");
  if (nx > 96 || ny > 96 || nz > 96) return no("an axis has more than 96 points");
  if (nx % 2 != 0) return no("odd nx (bulk copies need 16-byte rows)");
  for (int a = 1; a < 3; ++a)
    if (g->n[a] != nx || g->t[a] != g->t[0]) return no("the axes do not share one kinetic matrix");
  F16Geom& G = P.G;
  G.nx = nx;
  G.ny = ny;
  G.nz = nz;
  G.kx = tc16_kpad(nx);
  G.ky = tc16_kpad(ny);
  G.kz = tc16_kpad(nz);
  G.npy = tc_npad(ny);
  G.npz = tc_npad(nz);
  G.nzt = (int)(((long)nx * ny + kTile - 1) / kTile);
  G.lag = 2;
  G.tau = g->t16_scale;
  const uint32_t npx = (uint32_t)tc_npad(nx);
  // the kinetic image: npx rows as copied, read as 128 rows by the x
  // contraction (the slot is 128 rows long)
  G.t_bytes = npx * (uint32_t)G.kx * 2u;
  const uint32_t t_slot = (uint32_t)kTile * (uint32_t)G.kx * 2u;
  uint32_t cur = 0;
  G.t_hi = cur;
  cur += t_slot;
  G.t_lo = cur;
  cur += t_slot;
  // operand images: the plane (npy x kx) plus the y contraction's overread,
  // or the z tile (128 x kz)
  const uint32_t plane = (uint32_t)G.npy * (uint32_t)G.kx * 2u + kOverread;
  const uint32_t ztile = (uint32_t)kTile * (uint32_t)G.kz * 2u;
  const uint32_t op = (std::max(plane, ztile) + 127u) / 128u * 128u;
  G.op_hi = cur;
  cur += op;
  G.op_lo = cur;
  cur += op;
  // staging: box regions of 128-byte rows, 1024-byte aligned (the swizzle
  // atom); ceil(nx / 16) regions of ny rows, or eight regions of nz rows
  G.stg = (cur + 1023u) / 1024u * 1024u;
  G.reg_xy = (uint32_t)(128 * ny + 1023) / 1024u * 1024u;
  G.reg_z = (uint32_t)(128 * nz + 1023) / 1024u * 1024u;
  cur = G.stg + std::max((uint32_t)((nx + 15) / 16) * G.reg_xy, (uint32_t)(kTile / 16) * G.reg_z);
  P.smem = cur;
  if ((long)P.smem > (long)g_f16_max_dyn) return no("operand images and staging exceed shared memory");
  uint32_t cols = 32;
  while (cols < (uint32_t)std::max(G.npy, G.npz)) cols <<= 1;
  G.acc_cols = cols;
  // as many accumulators as tensor memory holds (at most four), so that a
  // long z epilogue does not hold up the next items' MMAs
  G.acc_shift = cols * 4 <= 512 ? 2 : 1;
  P.ok = true;
  return P;
}

}  // namespace

// Work counters of the FP16 kernel, one block per stream (as the fused kernel's).
static pg_status f16_counters(const pg_grid* g, cudaStream_t st, F16Counters** out) {
  unsigned long long id = 0;
  PG_CUDA_TRY(cudaStreamGetId(st, &id));
  std::lock_guard<std::mutex> l(g->fused_m);
  const unsigned long long key = id ^ 0x8000000000000000ull;  // beside the fused kernel's blocks
  auto it = g->fused_cnt.find(key);
  if (it == g->fused_cnt.end()) {
    if (g->fused_cnt.size() >= 512) {
      set_error("FP16 H*X: more than 256 streams used on one grid");
      return PG_UNSUPPORTED;
    }
    std::unique_ptr<DevBuf<unsigned>> b(new DevBuf<unsigned>());
    PG_TRY(b->alloc(sizeof(F16Counters) / sizeof(unsigned)));
    PG_CUDA_TRY(cudaMemset(b->p, 0, sizeof(F16Counters)));
    it = g->fused_cnt.emplace(key, std::move(b)).first;
  }
  *out = reinterpret_cast<F16Counters*>(it->second->p);
  return PG_OK;
}

bool f16_hx_ok(const pg_grid* g) {
  if (f16_init() != cudaSuccess) return false;
  return plan_f16(g).ok;
}

void f16_plan_text(const pg_grid* g, const HxParams& p, char* buf, int len) {
  if (f16_init() != cudaSuccess) {
    snprintf(buf, (size_t)len, "FP16 split (k_hx_f16): device query failed");
    return;
  }
  const F16Plan P = plan_f16(g);
  if (!P.ok) {
    snprintf(buf, (size_t)len, "FP16 split (k_hx_f16): not available: %s", P.why);
    return;
  }
  snprintf(buf, (size_t)len,
           "FP16 split (k_hx_f16): xy planes %dx%d + z tiles of 128 lines (%d per vector, lag %d vectors), "
           "K %d/%d/%d, rows bulk-copied to a staging buffer, %zu B shared memory, %u TMEM columns x %d, %d CTAs",
           P.G.nx, P.G.ny, P.G.nzt, p.lag > 0 ? p.lag : P.G.lag, P.G.kx, P.G.ky, P.G.kz, P.smem, P.G.acc_cols,
           1 << P.G.acc_shift,
           p.ctas > 0 && p.ctas < g_f16_sms ? p.ctas : g_f16_sms);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependence on the driver library).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// The two tensor maps of a job: X (nvec vectors of the grid) as a 3-D
// (x, y, plane) tensor with boxes of 16 x ny x 1, and as a 2-D (plane point,
// plane) tensor with boxes of 16 x nz; FP64, 128-byte swizzle, zeros past
// the edges.
static pg_status encode_maps(const pg_grid* g, const double* x, int nvec, CUtensorMap* txy, CUtensorMap* tz);

pg_status encode_job_maps(const pg_grid* g, const double* x, int nvec, CUtensorMap* txy, CUtensorMap* tz) {
  static_assert(sizeof(CUtensorMap) == sizeof(pg_grid::TensorMapPair::xy), "tensor map size");
  const std::pair<const void*, int> key(x, nvec);
  {
    std::lock_guard<std::mutex> l(g->fused_m);
    auto it = g->tmaps.find(key);
    if (it != g->tmaps.end()) {
      memcpy(txy, it->second.xy, sizeof(CUtensorMap));
      memcpy(tz, it->second.z, sizeof(CUtensorMap));
      return PG_OK;
    }
  }
  PG_TRY(encode_maps(g, x, nvec, txy, tz));
  std::lock_guard<std::mutex> l(g->fused_m);
  if (g->tmaps.size() >= 4096) g->tmaps.clear();
  pg_grid::TensorMapPair& e = g->tmaps[key];
  memcpy(e.xy, txy, sizeof(CUtensorMap));
  memcpy(e.z, tz, sizeof(CUtensorMap));
  return PG_OK;
}

static pg_status encode_maps(const pg_grid* g, const double* x, int nvec, CUtensorMap* txy, CUtensorMap* tz) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) {
    set_error("FP16 H*X: cuTensorMapEncodeTiled is not available");
    return PG_UNSUPPORTED;
  }
  const cuuint64_t nx = (cuuint64_t)g->n[0], ny = (cuuint64_t)g->n[1], nz = (cuuint64_t)g->n[2];
  const cuuint32_t one[3] = {1, 1, 1};
  {
    const cuuint64_t dims[3] = {nx, ny, nz * (cuuint64_t)nvec};
    const cuuint64_t strides[2] = {nx * 8, nx * ny * 8};
    const cuuint32_t box[3] = {16, (cuuint32_t)ny, 1};
    const CUresult r = enc(txy, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(x), dims, strides, box, one,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      set_error("FP16 H*X: tensor map (planes) rejected: driver error %d", (int)r);
      return PG_CUDA;
    }
  }
  {
    const cuuint64_t dims[2] = {nx * ny, nz * (cuuint64_t)nvec};
    const cuuint64_t strides[1] = {nx * ny * 8};
    const cuuint32_t box[2] = {16, (cuuint32_t)nz};
    const CUresult r = enc(tz, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(x), dims, strides, box, one,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      set_error("FP16 H*X: tensor map (z tiles) rejected: driver error %d", (int)r);
      return PG_CUDA;
    }
  }
  return PG_OK;
}

// Mixed H*X of vector blocks on the same grid, up to kMaxJobs per launch of
// the FP16 kernel (the caller has checked f16_hx_ok); X 16-byte aligned.
pg_status hx_f16_jobs(const pg_grid* g, const double* const* v, const double* const* x, double* const* y,
                      const int* nvec, int njobs, const HxParams& hp, cudaStream_t st, bool unit) {
  PG_ARG(njobs > 0, "FP16 H*X: no jobs");
  if (njobs > kMaxJobs) {
    PG_TRY(hx_f16_jobs(g, v, x, y, nvec, kMaxJobs, hp, st, unit));
    return hx_f16_jobs(g, v + kMaxJobs, x + kMaxJobs, y + kMaxJobs, nvec + kMaxJobs, njobs - kMaxJobs, hp, st, unit);
  }
  PG_CUDA_TRY(f16_init());
  F16Plan P = plan_f16(g);
  if (!P.ok) {
    set_error("FP16 H*X not available on this grid: %s", P.why);
    return PG_UNSUPPORTED;
  }
  if (hp.lag > 0) P.G.lag = hp.lag;
  P.G.unit_bound = unit ? 1 : 0;
  for (int j = 0; j < njobs; ++j)
    PG_ARG(nvec[j] == 0 || ((uintptr_t)x[j] & 15u) == 0, "FP16 H*X: X must be 16-byte aligned");
  F16Counters* cnt = nullptr;
  PG_TRY(f16_counters(g, st, &cnt));
  F16Jobs J;
  memset(&J, 0, sizeof(J));
  int total = 0;
  for (int j = 0; j < njobs; ++j) {
    PG_ARG(nvec[j] >= 0, "FP16 H*X: negative vector count");
    if (nvec[j] > 0) PG_TRY(encode_job_maps(g, x[j], nvec[j], &J.j[J.n].txy, &J.j[J.n].tz));
    J.j[J.n].x = x[j];
    J.j[J.n].y = y[j];
    J.j[J.n].v = v[j];
    J.j[J.n].nvec = nvec[j];
    J.j[J.n].vec0 = total;
    total += nvec[j];
    if (nvec[j] > 0) ++J.n;
  }
  if (total == 0) return PG_OK;
  PG_ARG(total <= kF16MaxVec, "FP16 H*X: %d vectors in one launch (at most %d)", total, kF16MaxVec);
  J.nvec = total;
  const long items = (long)total * (P.G.nz + P.G.nzt);
  const int cap = hp.ctas > 0 && hp.ctas < g_f16_sms ? hp.ctas : g_f16_sms;
  const int grid = (int)std::min<long>(items, cap);
  PG_CUDA_TRY(launch_dependent(k_hx_f16, dim3(grid), dim3(kThreadsAll), P.smem, st, P.G,
                               (const unsigned short*)g->t16_hi[0].p, (const unsigned short*)g->t16_lo[0].p, J, cnt,
                               g->tc_err.p));
  return check_launch("k_hx_f16");
}

pg_status hx_f16(const pg_grid* g, const double* v, const double* x, double* y, int nvec, const HxParams& hp,
                 cudaStream_t st, bool unit) {
  for (int v0 = 0; v0 < nvec; v0 += kF16MaxVec) {
    const int nb = std::min(kF16MaxVec, nvec - v0);
    const double* xs = x + (long)v0 * g->N;
    double* ys = y + (long)v0 * g->N;
    PG_TRY(hx_f16_jobs(g, &v, &xs, &ys, &nb, 1, hp, st, unit));
  }
  return PG_OK;
}

}  // namespace pg
