// The kinetic preconditioner of the mixed form, R <- (T - sigma_v)^-1 R for a
// block of vectors, as one persistent tensor-core kernel with an FP16 split,
// for grids whose three axes have the same n <= 96 (one eigenbasis).
//
// T = Tx (+) Ty (+) Tz with T_a = Q diag(d_a) Q^T on every axis (the DST-I for
// the sine DVR, the real Fourier basis for the periodic FFT kinetic term), so
//   (T - sigma)^-1 = (Q (x) Q (x) Q) D^-1 (Q (x) Q (x) Q)^T,
//   D(i,j,k) = dx_i + dy_j + dz_k - sigma, |D| kept at least `floor`.
// Three kinds of work items per vector, each two chained contractions:
//   XF, plane k of R:     W1 = Q^T P Q      (x, then y forward)
//   ZS, 128 grid lines:   W2 = Q D^-1 Q^T L  (z forward, the diagonal, z backward)
//   XB, plane k of W2:    R  = Q P Q^T      (x, then y backward)
// A ZS item of a vector starts once every XF plane of the vector is in W1, an
// XB item once every ZS tile of the vector is in W2 (per-vector completion
// counters, bounded waits); the ticket order (XF(s), ZS(s - L), XB(s - 2L) for
// steps s) gives each item's dependencies smaller tickets, so the smallest
// unfinished ticket can always proceed.
//
// Per item, as the FP16 H*X kernel (pg_hx_f16.cu): the item's rows are copied
// by the tensor memory accelerator into a staging buffer while the previous
// item is in flight, the producers scale them by 2^s (the largest |x| into
// [2^14, 2^15): an XF item's from a pass over its staged values, ZS and XB
// items' from the largest exponent the previous phase wrote into the
// vector's W1 or W2) and split them into FP16 high parts and remainders, and
// the first MMA (hi.hi + hi.lo + lo.hi, FP32 in TMEM) contracts one axis.
// The epilogue warps read that result from TMEM (one row per lane), multiply
// by 2^-(tau + 4) (and, in a ZS item, by 1 / D), split it again and write it
// as the K-major A operand of the second MMA: into a region of its own where
// shared memory allows (the producers then convert the next item meanwhile),
// else over the item's operand image.  The second MMA contracts the next
// axis; the epilogue multiplies by the inverse of the product of the scales
// (a power of two) and writes FP64.  The factor 2^-4 keeps the intermediate below 2^15:
// an orthonormal transform grows no entry by more than sqrt(n) < 16, and in a
// ZS item 2^-ef bounds 1 / |D| <= 1 / floor.
//
// Every wait is bounded; a timeout sets the grid's error word and the kernel
// drains its copies and MMAs and returns.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>

#include "pg_tc16.cuh"

namespace {

constexpr int kKinMaxVec = 32;  // vectors of one launch; more go to further launches

}  // namespace

namespace pg {

struct KinGeom {
  int nx, ny, nz;
  int kx, ky, kz;     // K extents padded to 16 (also the padded N extents)
  int npy, npz;
  int nzt;            // ZS items per vector
  int lag;            // steps between a vector's XF, ZS and XB items
  int tau;            // the eigenbasis images hold Q 2^tau
  int ef;             // 1 / |D| <= 2^ef
  float floor;        // least |D|
  uint32_t qf_hi, qf_lo, qb_hi, qb_lo;  // forward (Q^T) and backward (Q) images; the same offsets when Q^T = Q
  uint32_t q_bytes;                     // bytes of one image as copied
  int q_sym;
  uint32_t op_hi, op_lo;  // the item's operand image
  uint32_t mid_hi, mid_lo;  // the second MMA's A image: its own region where shared memory allows, else op_*
  int mid_sep;
  uint32_t stg;           // staging buffer (1024-byte aligned)
  uint32_t reg_xy, reg_z; // bytes of one 16-value-wide box region (rounded to 1024)
  uint32_t acc_cols;      // TMEM columns per accumulator
  int acc_shift;          // log2 of the accumulators
  int nvec;
};

struct KinArgs {
  CUtensorMap r_xy;   // R as planes (boxes 16 x ny x 1)
  CUtensorMap w1_z;   // W1 as grid lines (boxes 16 points x nz)
  CUtensorMap w2_xy;  // W2 as planes
  double* r;
  double* w1;
  double* w2;
  const double* sigma;  // per vector
  const double* d[3];   // eigenvalues per axis
};

struct KinCounters {
  unsigned ticket;
  unsigned finished;
  unsigned done_xf[kKinMaxVec];  // XF planes in W1, per vector
  unsigned done_zs[kKinMaxVec];  // ZS tiles in W2, per vector
  unsigned exp_w1[kKinMaxVec];   // largest FP64 exponent (biased) in W1, per vector
  unsigned exp_w2[kKinMaxVec];   // the same in W2
};

}  // namespace pg

namespace {

using pg::KinArgs;
using pg::KinCounters;
using pg::KinGeom;

constexpr int kXF = 0, kZS = 1, kXB = 2;

struct KItem {
  int kind;  // kXF, kZS, kXB; -1: none
  int u;     // vector
  int idx;   // plane or tile
};

// Ticket -> item: steps s = 0, 1, ... hold XF(s) (nz planes), ZS(s - L) (nzt
// tiles) and XB(s - 2L) (nz planes), each where the vector exists.
__device__ __forceinline__ KItem kdecode(unsigned t, int nvec, int nz, int nzt, int L) {
  for (int s = 0; s < nvec + 2 * L; ++s) {
    if (s < nvec) {
      if (t < (unsigned)nz) return KItem{kXF, s, (int)t};
      t -= nz;
    }
    if (s >= L && s - L < nvec) {
      if (t < (unsigned)nzt) return KItem{kZS, s - L, (int)t};
      t -= nzt;
    }
    if (s >= 2 * L && s - 2 * L < nvec) {
      if (t < (unsigned)nz) return KItem{kXB, s - 2 * L, (int)t};
      t -= nz;
    }
  }
  return KItem{-1, 0, 0};
}

__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Warp 0 of the producers: wait (lane 0, bounded) until the item's input is
// complete, then issue its tensor copies into the staging buffer, completing
// on bar.  Returns false if the wait gave up.
__device__ __forceinline__ bool kstage(const KinGeom& G, const KinArgs& A, const KItem& it, KinCounters* cnt,
                                       unsigned char* smem, uint32_t bar, int lane, volatile int* abort,
                                       int* exp_out) {
  if (it.kind < 0) return true;
  int ok = 1;
  if (lane == 0 && it.kind != kXF) {
    const volatile unsigned* c = it.kind == kZS ? &cnt->done_xf[it.u] : &cnt->done_zs[it.u];
    const unsigned need = it.kind == kZS ? (unsigned)G.nz : (unsigned)G.nzt;
    const unsigned long long t0 = globaltimer_ns();
    while (*c < need) {
      if (*abort || globaltimer_ns() - t0 > 2000000000ull) {
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    // the item's scale comes from the largest exponent of the whole input vector
    __threadfence();
    *exp_out = (int)*(it.kind == kZS ? (volatile unsigned*)&cnt->exp_w1[it.u] : (volatile unsigned*)&cnt->exp_w2[it.u]);
  }
  ok = __shfl_sync(0xffffffffu, ok, 0);
  if (!ok) return false;
  if (it.kind != kXF) {
    // the other CTAs' generic stores, then this warp's tensor copies
    __threadfence();
    fence_proxy_async_global();
  }
  const bool xy = it.kind != kZS;
  const int nbox = xy ? (G.nx + 15) / 16 : kTile / 16;
  const uint32_t box_bytes = 128u * (uint32_t)(xy ? G.ny : G.nz);
  if (lane == 0) {
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(bar), "r"((uint32_t)nbox * box_bytes)
                 : "memory");
  }
  __syncwarp();
  const uint32_t dst0 = smem_u32(smem + G.stg);
  if (xy) {
    const void* map = it.kind == kXF ? &A.r_xy : &A.w2_xy;
    const int zc = it.u * G.nz + it.idx;
    for (int b = lane; b < nbox; b += 32)
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
          "[%5];" ::"r"(dst0 + (uint32_t)b * G.reg_xy),
          "l"(map), "r"(16 * b), "r"(0), "r"(zc), "r"(bar)
          : "memory");
  } else {
    const void* map = &A.w1_z;
    const int p0 = it.idx * kTile;
    const int yc = it.u * G.nz;
    for (int b = lane; b < nbox; b += 32)
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
          "[%4];" ::"r"(dst0 + (uint32_t)b * G.reg_z),
          "l"(map), "r"(p0 + 16 * b), "r"(yc), "r"(bar)
          : "memory");
  }
  return true;
}

// Sixteen FP32 values (one TMEM row segment) -> two 16-byte rows of FP16 high
// parts and two of remainders, stored at byte offsets o0 and o1 of the two
// images.
__device__ __forceinline__ void split16_store(const float* a, unsigned char* hi, unsigned char* lo, uint32_t o0,
                                              uint32_t o1) {
  uint32_t h[8], l[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const __half2 hh = __floats2half2_rn(a[2 * q], a[2 * q + 1]);
    const float2 hf = __half22float2(hh);
    const __half2 ll = __floats2half2_rn(a[2 * q] - hf.x, a[2 * q + 1] - hf.y);
    h[q] = *reinterpret_cast<const uint32_t*>(&hh);
    l[q] = *reinterpret_cast<const uint32_t*>(&ll);
  }
  *reinterpret_cast<uint4*>(hi + o0) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4*>(hi + o1) = make_uint4(h[4], h[5], h[6], h[7]);
  *reinterpret_cast<uint4*>(lo + o0) = make_uint4(l[0], l[1], l[2], l[3]);
  *reinterpret_cast<uint4*>(lo + o1) = make_uint4(l[4], l[5], l[6], l[7]);
}

__global__ void __launch_bounds__(kThreadsAll, 1)
    k_kin_f16(const __grid_constant__ KinGeom G, const unsigned short* __restrict__ qf_hi,
              const unsigned short* __restrict__ qf_lo, const unsigned short* __restrict__ qb_hi,
              const unsigned short* __restrict__ qb_lo, const __grid_constant__ KinArgs A,
              KinCounters* __restrict__ cnt, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar_q, mbar_full, mbar_empty, mbar_mid, mbar_acc_full[kMaxAcc],
      mbar_acc_empty[kMaxAcc], mbar_stg;
  __shared__ uint32_t tmem_base;
  __shared__ unsigned ring[kRing];
  __shared__ int sig[kRing];  // item scale exponents, by ticket slot
  __shared__ int s_emax[kProdWarps];
  __shared__ int s_vexp[kRing];  // ZS and XB items: largest exponent of the input vector, by ticket slot
  __shared__ float s_d[3][kTile];  // eigenvalues per axis, zero past n
  __shared__ int s_abort, s_prod_ok, s_epi_ok, s_last, s_stg_issued;
  volatile int* abort = &s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long nxny = (long)G.nx * G.ny;
  const int nvec = G.nvec;

  if (tid == 0) {
    s_abort = 0;
    s_stg_issued = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_q)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar_full)), "r"(kProdWarps * 32));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_empty)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_mid)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_stg)));
    for (int b = 0; b < kMaxAcc; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(smem_u32(&mbar_acc_full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar_acc_empty[b])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // the eigenbasis images (the grid's constant data) while the kernel ahead finishes
    const int nimg = G.q_sym ? 2 : 4;
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_u32(&mbar_q)), "r"((uint32_t)nimg * G.q_bytes)
                 : "memory");
    const unsigned short* src[4] = {qf_hi, qf_lo, qb_hi, qb_lo};
    const uint32_t dst[4] = {G.qf_hi, G.qf_lo, G.qb_hi, G.qb_lo};
    for (int m = 0; m < nimg; ++m)
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_u32(smem + dst[m])),
                   "l"(src[m]), "r"(G.q_bytes), "r"(smem_u32(&mbar_q))
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
  for (int e = tid; e < 3 * kTile; e += kThreadsAll) {
    const int a = e / kTile, i = e % kTile;
    const int n = a == 0 ? G.nx : (a == 1 ? G.ny : G.nz);
    s_d[a][i] = i < n ? (float)A.d[a][i] : 0.f;
  }
  if (tid == 0) ring[0] = atomicAdd(&cnt->ticket, 1u);
  __syncthreads();

  if (warp < kProdWarps) {
    // ------------------------------------------------------------ producers
    const int ptid = tid;
    const uint32_t bar_stg = smem_u32(&mbar_stg);
    const unsigned char* stg = smem + G.stg;
    if (warp == 0) {
      const KItem it0 = kdecode(ring[0], nvec, G.nz, G.nzt, G.lag);
      const bool ok = kstage(G, A, it0, cnt, smem, bar_stg, lane, abort, &s_vexp[0]);
      if (lane == 0) {
        if (!ok) *abort = 1;
        else if (it0.kind >= 0) s_stg_issued = 1;
      }
    }
    for (int i = 0;; ++i) {
      const KItem it = kdecode(ring[i % kRing], nvec, G.nz, G.nzt, G.lag);
      if (ptid == 0) ring[(i + 1) % kRing] = atomicAdd(&cnt->ticket, 1u);
      if (it.kind < 0) {
        // no more work: hand the issuer its stop item once the image is free
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
      const int ck = it.kind == kZS ? 1 : 0;  // conversion tasks: z tile or plane
      const int ntask = ck == 0 ? (G.kx >> 3) * G.npy : 16 * G.kz;
      if (it.kind == kXF) {  // the item's scale: its largest exponent over the producers
        int em = max_exponent(stg, ntask, ck, G, ptid);
        em = (int)__reduce_max_sync(0xffffffffu, (unsigned)em);
        if (lane == 0) s_emax[warp] = em;
      }
      // the image is free once the previous item's second MMA is done
      if (ptid == 0) {
        const int ok = i == 0 || mbar_wait_or_abort(smem_u32(&mbar_empty), (uint32_t)((i - 1) & 1), abort);
        if (!ok) *abort = 1;
        s_prod_ok = ok;
      }
      named_sync(1, kProdWarps * 32);
      if (!s_prod_ok) break;
      int emax = 0;
      if (it.kind == kXF) {
#pragma unroll
        for (int w = 0; w < kProdWarps; ++w) emax = s_emax[w] > emax ? s_emax[w] : emax;
      } else {
        emax = s_vexp[i % kRing];
      }
      // largest |x| < 2^(emax - 1022): scaled below 2^15; the factors of both
      // epilogues, 2^-(s + tau - 4 [- ef]), stay normal FP32 numbers
      int s = (emax == 0 || emax == 0x7ff) ? 0 : 1037 - emax;
      const int s_lo = -123 - G.tau + G.ef, s_hi = 126 - G.tau;
      s = s > s_hi ? s_hi : (s < s_lo ? s_lo : s);
      if (ptid == 0) sig[i % kRing] = s;
      unsigned char* ohi = smem + G.op_hi;
      unsigned char* olo = smem + G.op_lo;
      TaskIter ti(ptid, ck == 0 ? G.npy : G.kz);
      const int sb = s - 896;
      int t = ptid;
      for (; t + kProdWarps * 32 < ntask; t += 2 * kProdWarps * 32) {
        const Task k0 = task_of(G, ck, ti);
        ti.next();
        const Task k1 = task_of(G, ck, ti);
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
        const Task k = task_of(G, ck, ti);
        double v[8];
        load8(stg, k, v);
        uint4 h, l;
        split8(v, sb, h, l);
        *reinterpret_cast<uint4*>(ohi + k.dst) = h;
        *reinterpret_cast<uint4*>(olo + k.dst) = l;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      named_sync(1, kProdWarps * 32);
      mbar_arrive(smem_u32(&mbar_full));
      if (warp == 0) {
        const KItem nx_it = kdecode(ring[(i + 1) % kRing], nvec, G.nz, G.nzt, G.lag);
        const bool ok = kstage(G, A, nx_it, cnt, smem, bar_stg, lane, abort, &s_vexp[(i + 1) % kRing]);
        if (lane == 0) {
          if (!ok) *abort = 1;
          else if (nx_it.kind >= 0) s_stg_issued = i + 2;
        }
      }
    }
  } else if (warp < kIssueWarp) {
    // ------------------------------------------------------------- epilogue
    const int quarter = warp & 3, part = (warp - kProdWarps) >> 2;  // warps of one lane quarter share its columns
    const bool leader = warp == kProdWarps && lane == 0;
    const int r = 32 * quarter + lane;  // TMEM lane: x index (planes) or line of the tile
    unsigned char* mhi = smem + G.mid_hi;
    unsigned char* mlo = smem + G.mid_lo;
    for (int i = 0;; ++i) {
      const int b = i & ((1 << G.acc_shift) - 1);
      const KItem it = kdecode(ring[i % kRing], nvec, G.nz, G.nzt, G.lag);
      if (leader) {
        const int ok = mbar_wait_or_abort(smem_u32(&mbar_acc_full[b]), 0u, abort);
        if (!ok) *abort = 1;
        s_epi_ok = ok;
      }
      named_sync(2, kEpiWarps * 32);
      if (!s_epi_ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (it.kind < 0) break;
      const int s = sig[i % kRing];
      const bool zs = it.kind == kZS;
      const uint32_t acc = tmem + (uint32_t)b * G.acc_cols + ((uint32_t)(32 * quarter) << 16);
      const int ncol = zs ? G.npz : G.npy;  // columns of both results
      const int kq = (zs ? G.kz : G.ky) >> 3;  // core matrices along K of the second A image
      // ---- first result -> the second MMA's A image (K-major, row r)
      {
        const long p = zs ? (long)it.idx * kTile + r : 0;
        const bool valid = zs ? p < nxny : r < G.nx;
        float dxy = 0.f, sg = 0.f;
        if (zs && valid) {
          const int ii = (int)(p % G.nx), jj = (int)(p / G.nx);
          dxy = s_d[0][ii] + s_d[1][jj];
          sg = (float)A.sigma[it.u];
        }
        const float f = exp2i(-(G.tau + 4 + (zs ? G.ef : 0)));
        const uint32_t row = (uint32_t)(r >> 3) * (uint32_t)kq * 128u + (uint32_t)(r & 7) * 16u;
        for (int c = part; c < (ncol >> 4); c += kEpiParts) {
          float d[16];
          tmem_ld16(acc + (uint32_t)(16 * c), d);
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            float a = valid ? d[q] * f : 0.f;
            if (zs) {  // the diagonal in FP32 (it sets the convergence rate only)
              float den = (dxy + s_d[2][16 * c + q]) - sg;
              if (fabsf(den) < G.floor) den = den < 0.f ? -G.floor : G.floor;
              a = __fdividef(a, den);
            }
            d[q] = a;
          }
          split16_store(d, mhi, mlo, row + (uint32_t)(2 * c) * 128u, row + (uint32_t)(2 * c + 1) * 128u);
        }
        // K octets past the result's columns (none: the N and K extents are both padded to 16)
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      named_sync(2, kEpiWarps * 32);
      if (leader) {
        mbar_arrive(smem_u32(&mbar_mid));
        const int ok = mbar_wait_or_abort(smem_u32(&mbar_acc_full[b]), 1u, abort);
        if (!ok) *abort = 1;
        s_epi_ok = ok;
      }
      named_sync(2, kEpiWarps * 32);
      if (!s_epi_ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // ---- second result -> FP64, and the largest FP64 exponent written
      // (W1 and W2: the scale of the next phase's items)
      {
        const float unscale = exp2i(-(s + G.tau - 4 - (zs ? G.ef : 0)));
        uint32_t em = 0;
        auto track = [&em](float v) {
          const uint32_t e = (__float_as_uint(v) >> 23) & 0xffu;
          const uint32_t e64 = e == 0 ? 0u : (e == 255 ? 0x7ffu : e + 896u);
          em = e64 > em ? e64 : em;
        };
        if (zs) {
          const long p = (long)it.idx * kTile + r;
          double* out = A.w2 + (long)it.u * nxny * G.nz;
          for (int c = part; c < (G.npz >> 4); c += kEpiParts) {
            float d[16];
            tmem_ld16(acc + (uint32_t)(16 * c), d);
            if (p < nxny) {
#pragma unroll
              for (int q = 0; q < 16; ++q) {
                const int k = 16 * c + q;
                if (k < G.nz) {
                  const float v = d[q] * unscale;
                  track(v);
                  out[p + nxny * k] = f32_to_f64(v);
                }
              }
            }
          }
        } else {
          double* out = (it.kind == kXF ? A.w1 : A.r) + (long)it.u * nxny * G.nz + nxny * it.idx;
          for (int c = part; c < (G.npy >> 4); c += kEpiParts) {
            float d[16];
            tmem_ld16(acc + (uint32_t)(16 * c), d);
            if (r < G.nx) {
#pragma unroll
              for (int q = 0; q < 16; ++q) {
                const int j = 16 * c + q;
                if (j < G.ny) {
                  const float v = d[q] * unscale;
                  track(v);
                  out[r + (long)G.nx * j] = f32_to_f64(v);
                }
              }
            }
          }
        }
        if (it.kind != kXB) {
          em = __reduce_max_sync(0xffffffffu, em);
          if (lane == 0 && em > 0) atomicMax(zs ? &cnt->exp_w2[it.u] : &cnt->exp_w1[it.u], em);
        }
      }
      // W1 and W2 are read next by other CTAs' tensor copies: every writer
      // orders its stores before the async proxy, the leader's fence and
      // counter below release them, kstage acquires them (with a proxy fence
      // before the copies)
      if (it.kind != kXB) fence_proxy_async_global();
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      named_sync(2, kEpiWarps * 32);
      if (leader) {
        if (it.kind != kXB) {
          __threadfence();
          atomicAdd(it.kind == kXF ? &cnt->done_xf[it.u] : &cnt->done_zs[it.u], 1u);
        }
        mbar_arrive(smem_u32(&mbar_acc_empty[b]));
      }
    }
  } else if (lane == 0) {
    // --------------------------------------------------------------- issuer
    // kind::f16, FP16 A and B, FP32 D; bit 15: A MN-major
    const uint32_t id_xy = (1u << 4) | ((uint32_t)(G.npy >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
    const uint32_t id_z1 = (1u << 4) | (1u << 15) | ((uint32_t)(G.npz >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
    const uint32_t id_z2 = (1u << 4) | ((uint32_t)(G.npz >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
    const uint32_t sb = smem_u32(smem);
    const uint32_t kq_x = (uint32_t)(G.kx >> 3) * 128u;
    const uint32_t kq_y = (uint32_t)(G.ky >> 3) * 128u;
    const uint32_t kq_z = (uint32_t)(G.kz >> 3) * 128u;
    // K-major images: LBO = next 8 K values (128 B), SBO = next 8 rows
    const uint64_t d_qfh = smem_desc(sb + G.qf_hi, 128, kq_x), d_qfl = smem_desc(sb + G.qf_lo, 128, kq_x);
    const uint64_t d_qbh = smem_desc(sb + G.qb_hi, 128, kq_x), d_qbl = smem_desc(sb + G.qb_lo, 128, kq_x);
    const uint64_t d_pbh = smem_desc(sb + G.op_hi, 128, kq_x), d_pbl = smem_desc(sb + G.op_lo, 128, kq_x);
    // z tile (MN-major A): LBO = next 8 planes, SBO = next 8 points
    const uint64_t d_zh = smem_desc(sb + G.op_hi, 16 * 128, 128), d_zl = smem_desc(sb + G.op_lo, 16 * 128, 128);
    // the second A image: K-major, 128 rows
    const uint64_t d_mxh = smem_desc(sb + G.mid_hi, 128, kq_y), d_mxl = smem_desc(sb + G.mid_lo, 128, kq_y);
    const uint64_t d_mzh = smem_desc(sb + G.mid_hi, 128, kq_z), d_mzl = smem_desc(sb + G.mid_lo, 128, kq_z);
    // the eigenbasis as a B operand (rows = output index, K = input index)
    const uint64_t d_qfyh = smem_desc(sb + G.qf_hi, 128, kq_y), d_qfyl = smem_desc(sb + G.qf_lo, 128, kq_y);
    const uint64_t d_qbyh = smem_desc(sb + G.qb_hi, 128, kq_y), d_qbyl = smem_desc(sb + G.qb_lo, 128, kq_y);
    const uint64_t d_qfzh = smem_desc(sb + G.qf_hi, 128, kq_z), d_qfzl = smem_desc(sb + G.qf_lo, 128, kq_z);
    const uint64_t d_qbzh = smem_desc(sb + G.qb_hi, 128, kq_z), d_qbzl = smem_desc(sb + G.qb_lo, 128, kq_z);
    bool ok = mbar_wait_or_abort(smem_u32(&mbar_q), 0, abort);
    uint32_t last_bar = 0, last_parity = 0;  // the barrier and phase of the last commit
    for (int i = 0; ok; ++i) {
      const int b = i & ((1 << G.acc_shift) - 1);
      ok = mbar_wait_or_abort(smem_u32(&mbar_full), (uint32_t)(i & 1), abort);
      const int nacc = 1 << G.acc_shift;
      if (ok && i >= nacc)
        ok = mbar_wait_or_abort(smem_u32(&mbar_acc_empty[b]), (uint32_t)(((i - nacc) >> G.acc_shift) & 1), abort);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const KItem it = kdecode(ring[i % kRing], nvec, G.nz, G.nzt, G.lag);
      if (it.kind < 0) {
        mbar_arrive(smem_u32(&mbar_acc_full[b]));
        mbar_arrive(smem_u32(&mbar_acc_full[b]));
        break;
      }
      const uint32_t acc = tmem + (uint32_t)b * G.acc_cols;
      const bool fw = it.kind == kXF;
      // first MMA
      if (it.kind != kZS) {
        const uint64_t ah = fw ? d_qfh : d_qbh, al = fw ? d_qfl : d_qbl;
        for (int kk = 0; kk < G.kx / 16; ++kk) {  // x: A = Q (rows i', K = i), B = plane rows j
          const uint64_t o = (uint64_t)kk * 16;
          mma_f16(acc, al + o, d_pbh + o, id_xy, kk > 0 ? 1u : 0u);
          mma_f16(acc, ah + o, d_pbl + o, id_xy, 1u);
          mma_f16(acc, ah + o, d_pbh + o, id_xy, 1u);
        }
      } else {
        for (int kk = 0; kk < G.kz / 16; ++kk) {  // z: A = 128 lines (M = point, K = plane), B = Q^T
          const uint64_t oa = (uint64_t)kk * 2 * 16 * (128 >> 4), ob = (uint64_t)kk * 16;
          mma_f16(acc, d_zl + oa, d_qfzh + ob, id_z1, kk > 0 ? 1u : 0u);
          mma_f16(acc, d_zh + oa, d_qfzl + ob, id_z1, 1u);
          mma_f16(acc, d_zh + oa, d_qfzh + ob, id_z1, 1u);
        }
      }
      // with its own region for the second A image, the operand image is free
      // for the next item once the first MMA has read it
      if (G.mid_sep)
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(&mbar_empty)));
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar_acc_full[b])));
      mbar_arrive(smem_u32(&mbar_acc_full[b]));
      last_bar = smem_u32(&mbar_acc_full[b]);
      last_parity = 0;
      // the epilogue has turned the first result into the second A image
      ok = mbar_wait_or_abort(smem_u32(&mbar_mid), (uint32_t)(i & 1), abort);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (it.kind != kZS) {
        const uint64_t bh = fw ? d_qfyh : d_qbyh, bl = fw ? d_qfyl : d_qbyl;
        for (int kk = 0; kk < G.ky / 16; ++kk) {  // y: A = first result (rows i', K = j), B = Q (rows j', K = j)
          const uint64_t o = (uint64_t)kk * 16;
          mma_f16(acc, d_mxl + o, bh + o, id_xy, kk > 0 ? 1u : 0u);
          mma_f16(acc, d_mxh + o, bl + o, id_xy, 1u);
          mma_f16(acc, d_mxh + o, bh + o, id_xy, 1u);
        }
      } else {
        for (int kk = 0; kk < G.kz / 16; ++kk) {  // z back: A = scaled result (rows point, K = k'), B = Q
          const uint64_t o = (uint64_t)kk * 16;
          mma_f16(acc, d_mzl + o, d_qbzh + o, id_z2, kk > 0 ? 1u : 0u);
          mma_f16(acc, d_mzh + o, d_qbzl + o, id_z2, 1u);
          mma_f16(acc, d_mzh + o, d_qbzh + o, id_z2, 1u);
        }
      }
      if (!G.mid_sep)
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(&mbar_empty)));
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar_acc_full[b])));
      mbar_arrive(smem_u32(&mbar_acc_full[b]));
      last_bar = smem_u32(&mbar_acc_full[b]);
      last_parity = 1;
    }
    if (!ok) {
      *abort = 1;
      // the MMAs already issued finish before the CTA leaves (bounded waits;
      // a commit tracks every earlier MMA of the thread)
      if (last_bar) mbar_wait(last_bar, last_parity);
      mbar_wait(smem_u32(&mbar_q), 0);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
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
    for (int u = tid; u < nvec; u += kThreadsAll) {
      cnt->done_xf[u] = 0;
      cnt->done_zs[u] = 0;
      cnt->exp_w1[u] = 0;
      cnt->exp_w2[u] = 0;
    }
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

struct KinPlan {
  bool ok = false;
  KinGeom G{};
  size_t smem = 0;
  char why[160] = "";
};

int g_kin_sms = 0;
int g_kin_max_dyn = 0;

cudaError_t kin_init() {
  static const cudaError_t init = [] {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_kin_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_kin_f16);
    if (e == cudaSuccess) {
      g_kin_max_dyn = optin - (int)fa.sharedSizeBytes;
      e = cudaFuncSetAttribute(k_kin_f16, cudaFuncAttributeMaxDynamicSharedMemorySize, g_kin_max_dyn);
    }
    if (g_kin_sms <= 0) g_kin_sms = 148;
    return e;
  }();
  return init;
}

KinPlan plan_kin(const pg_grid* g) {
  KinPlan P;
  const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
  auto no = [&](const char* why) {
    snprintf(P.why, sizeof(P.why), "%s", why);
    return P;
  };
  if (!g->q16f_hi.p) return no("no FP16 eigenbasis images (the axes differ in n, or n > 128)");
  if (nx > 96) return no("an axis has more than 96 points");
  if (nx % 2 != 0) return no("odd nx (bulk copies need 16-byte rows)");
  if (ny != nx || nz != nx) return no("the axes differ in n");
  KinGeom& G = P.G;
  G.nx = nx;
  G.ny = ny;
  G.nz = nz;
  G.kx = tc16_kpad(nx);
  G.ky = tc16_kpad(ny);
  G.kz = tc16_kpad(nz);
  G.npy = tc_npad(ny);
  G.npz = tc_npad(nz);
  G.nzt = (int)(((long)nx * ny + kTile - 1) / kTile);
  G.lag = 1;
  G.tau = g->q16_scale;
  G.q_sym = g->q16_sym ? 1 : 0;
  const uint32_t npx = (uint32_t)tc_npad(nx);
  G.q_bytes = npx * (uint32_t)G.kx * 2u;
  // each image slot is 128 rows long: the x contraction reads 128 rows of A
  const uint32_t q_slot = (uint32_t)kTile * (uint32_t)G.kx * 2u;
  uint32_t cur = 0;
  G.qf_hi = cur;
  cur += q_slot;
  G.qf_lo = cur;
  cur += q_slot;
  if (G.q_sym) {
    G.qb_hi = G.qf_hi;
    G.qb_lo = G.qf_lo;
  } else {
    G.qb_hi = cur;
    cur += q_slot;
    G.qb_lo = cur;
    cur += q_slot;
  }
  // the operand image: a plane (npy x kx, plus the overread of a 128-row
  // A read), a z tile (128 x kz), or the second A image (128 x k)
  const uint32_t plane = (uint32_t)G.npy * (uint32_t)G.kx * 2u + kOverread;
  const uint32_t ztile = (uint32_t)kTile * (uint32_t)std::max(G.ky, G.kz) * 2u;
  const uint32_t op = (std::max(plane, ztile) + 127u) / 128u * 128u;
  G.op_hi = cur;
  cur += op;
  G.op_lo = cur;
  cur += op;
  G.reg_xy = (uint32_t)(128 * ny + 1023) / 1024u * 1024u;
  G.reg_z = (uint32_t)(128 * nz + 1023) / 1024u * 1024u;
  const uint32_t stg_bytes = std::max((uint32_t)((nx + 15) / 16) * G.reg_xy, (uint32_t)(kTile / 16) * G.reg_z);
  // the second A image (128 rows): in a region of its own if that fits, so
  // that the producers convert the next item while the second MMA runs
  const uint32_t mid = (uint32_t)kTile * (uint32_t)std::max(G.ky, G.kz) * 2u;
  const uint32_t sep_end = (cur + 2 * mid + 1023u) / 1024u * 1024u + stg_bytes;
  G.mid_sep = (long)sep_end <= (long)g_kin_max_dyn ? 1 : 0;
  if (G.mid_sep) {
    G.mid_hi = cur;
    cur += mid;
    G.mid_lo = cur;
    cur += mid;
  } else {
    G.mid_hi = G.op_hi;
    G.mid_lo = G.op_lo;
  }
  G.stg = (cur + 1023u) / 1024u * 1024u;
  cur = G.stg + stg_bytes;
  P.smem = cur;
  if ((long)P.smem > (long)g_kin_max_dyn) return no("images and staging exceed shared memory");
  uint32_t cols = 32;
  while (cols < (uint32_t)std::max(G.npy, G.npz)) cols <<= 1;
  G.acc_cols = cols;
  G.acc_shift = cols * 4 <= 512 ? 2 : 1;
  P.ok = true;
  return P;
}

}  // namespace

// Work counters of the preconditioner kernel, one block per stream.
static pg_status kin_counters(const pg_grid* g, cudaStream_t st, KinCounters** out) {
  unsigned long long id = 0;
  PG_CUDA_TRY(cudaStreamGetId(st, &id));
  std::lock_guard<std::mutex> l(g->fused_m);
  const unsigned long long key = id ^ 0x4000000000000000ull;  // beside the H*X kernels' blocks
  auto it = g->fused_cnt.find(key);
  if (it == g->fused_cnt.end()) {
    if (g->fused_cnt.size() >= 768) {
      set_error("FP16 preconditioner: more than 256 streams used on one grid");
      return PG_UNSUPPORTED;
    }
    std::unique_ptr<DevBuf<unsigned>> b(new DevBuf<unsigned>());
    PG_TRY(b->alloc(sizeof(KinCounters) / sizeof(unsigned)));
    PG_CUDA_TRY(cudaMemset(b->p, 0, sizeof(KinCounters)));
    it = g->fused_cnt.emplace(key, std::move(b)).first;
  }
  *out = reinterpret_cast<KinCounters*>(it->second->p);
  return PG_OK;
}

bool kin_f16_ok(const pg_grid* g) {
  if (kin_init() != cudaSuccess) return false;
  return plan_kin(g).ok;
}

void kin_f16_plan_text(const pg_grid* g, char* buf, int len) {
  if (kin_init() != cudaSuccess) {
    snprintf(buf, (size_t)len, "FP16 split (k_kin_f16): device query failed");
    return;
  }
  const KinPlan P = plan_kin(g);
  if (!P.ok) {
    snprintf(buf, (size_t)len, "FP16 split (k_kin_f16): not available: %s", P.why);
    return;
  }
  snprintf(buf, (size_t)len,
           "FP16 split (k_kin_f16): XF planes, ZS tiles of 128 lines (%d per vector), XB planes, lag 3 steps "
           "(1 for one or two vectors), intermediate image %s, %zu B shared memory, %u TMEM columns x %d, %d CTAs",
           P.G.nzt, P.G.mid_sep ? "separate" : "over the operand image", P.smem, P.G.acc_cols,
           1 << P.G.acc_shift, g_kin_sms);
}

// R <- (T - sigma_v)^-1 R for the k vectors of R (contiguous, 16-byte
// aligned), with W1 and W2 k vectors of scratch each; sigma on the device.
pg_status kin_f16(const pg_grid* g, double* R, double* w1, double* w2, int k, const double* sigma, double floor,
                  cudaStream_t st) {
  PG_ARG(k >= 0 && R && w1 && w2 && sigma && floor > 0.0, "FP16 preconditioner: bad arguments");
  if (k == 0) return PG_OK;
  PG_CUDA_TRY(kin_init());
  KinPlan P = plan_kin(g);
  if (!P.ok) {
    set_error("FP16 preconditioner not available on this grid: %s", P.why);
    return PG_UNSUPPORTED;
  }
  PG_ARG((((uintptr_t)R | (uintptr_t)w1 | (uintptr_t)w2) & 15u) == 0,
         "FP16 preconditioner: R, W1 and W2 must be 16-byte aligned");
  int e = 0;
  std::frexp(1.0 / floor, &e);  // 1 / floor = m 2^e, m in [0.5, 1)
  P.G.ef = std::max(0, std::min(e, 60));
  P.G.floor = (float)floor;
  KinCounters* cnt = nullptr;
  PG_TRY(kin_counters(g, st, &cnt));
  const long N = g->N;
  for (int v0 = 0; v0 < k; v0 += kKinMaxVec) {
    const int nb = std::min(kKinMaxVec, k - v0);
    KinArgs A;
    memset(&A, 0, sizeof(A));
    CUtensorMap unused;
    PG_TRY(encode_job_maps(g, R + (long)v0 * N, nb, &A.r_xy, &unused));
    PG_TRY(encode_job_maps(g, w1, nb, &unused, &A.w1_z));
    PG_TRY(encode_job_maps(g, w2, nb, &A.w2_xy, &unused));
    A.r = R + (long)v0 * N;
    A.w1 = w1;
    A.w2 = w2;
    A.sigma = sigma + v0;
    for (int a = 0; a < 3; ++a) A.d[a] = g->d_dev[a].p;
    P.G.nvec = nb;
    // steps between a vector's phases: three keep enough independent planes
    // in flight that ZS and XB items seldom wait (measured at 48-96 points,
    // 2-8 vectors); with one or two vectors the order matters little
    P.G.lag = nb >= 3 ? 3 : 1;
    const long items = (long)nb * (2 * P.G.nz + P.G.nzt);
    const int grid = (int)std::min<long>(items, g_kin_sms);
    const unsigned short* qbh = g->q16_sym ? g->q16f_hi.p : g->q16b_hi.p;
    const unsigned short* qbl = g->q16_sym ? g->q16f_lo.p : g->q16b_lo.p;
    PG_CUDA_TRY(launch_dependent(k_kin_f16, dim3(grid), dim3(kThreadsAll), P.smem, st, P.G, g->q16f_hi.p,
                                 g->q16f_lo.p, qbh, qbl, A, cnt, g->tc_err.p));
    PG_TRY(check_launch("k_kin_f16"));
  }
  return PG_OK;
}

}  // namespace pg
