// Device pieces shared by the FP16-split tensor-core kernels (the mixed H*X
// of pg_hx_f16.cu and the kinetic preconditioner of pg_kin_f16.cu): warp
// roles, mbarrier and tcgen05 wrappers, the FP64 -> FP16 operand split, and
// the conversion tasks that turn staged rows into core-matrix images.
//
// Warp roles of a CTA: kProdWarps producer warps (operand conversion; warp 0
// also issues the tensor copies), kEpiWarps epilogue warps (kEpiParts per
// TMEM lane quarter, each taking every kEpiParts-th block of 16 columns), one
// issuer warp whose lane 0 launches the MMAs.
//
// Staged rows: an xy item's plane arrives as ceil(nx / 16) box regions of ny
// rows of 16 doubles, a z item's 128 grid lines as eight box regions of nz
// rows of 16 points; every row is 128 bytes with the 128-byte swizzle.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <cstdint>

#include "pg_solve.cuh"

namespace pg {
// cuTensorMapEncodeTiled through the runtime's driver entry point
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();
// X (nvec vectors of the grid) as a 3-D (x, y, plane) tensor with boxes of
// 16 x ny x 1 and as a 2-D (plane point, plane) tensor with boxes of 16 x nz;
// FP64, 128-byte swizzle, zeros past the edges
pg_status encode_job_maps(const pg_grid* g, const double* x, int nvec, CUtensorMap* txy, CUtensorMap* tz);
}  // namespace pg

namespace {

constexpr int kTile = 128;  // MMA M: TMEM lanes, z-tile points
constexpr int kProdWarps = 7;
constexpr int kEpiWarps = 8;
constexpr int kEpiParts = kEpiWarps / 4;  // epilogue warps per TMEM lane quarter
static_assert(kEpiWarps % 4 == 0, "the epilogue covers the four TMEM lane quarters evenly");
constexpr int kIssueWarp = kProdWarps + kEpiWarps;
constexpr int kThreadsAll = (kIssueWarp + 1) * 32;
constexpr int kRing = 8;  // tickets in flight in one CTA
constexpr uint32_t kOverread = 2048;  // bytes past a plane image the y contraction's 128-row A read may touch
constexpr int kMaxAcc = 4;  // TMEM accumulators in rotation

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok)
               : "r"(bar), "r"(phase)
               : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  for (long it = 0; it < (1L << 26); ++it)
    if (mbar_try(bar, phase)) return true;
  return false;
}

// Bounded wait that also gives up once another role has raised the abort flag.
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t phase, volatile int* abort) {
  for (long it = 0; it < (1L << 26); ++it) {
    if (mbar_try(bar, phase)) return true;
    if (*abort) return false;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
               "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
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

// 2^e as FP32 for -126 <= e <= 127.
__device__ __forceinline__ float exp2i(int e) {
  e = e < -126 ? -126 : (e > 127 ? 127 : e);
  return __uint_as_float((uint32_t)(e + 127) << 23);
}

// FP64 x 2^s -> FP32 with 32-bit integer operations (the mantissa
// truncated to 23 bits, 2^-24 relative); sb = s - 896 (the exponent rebias).
// Below 2^-126 gives a signed zero; Inf and NaN stay non-finite (the scale
// keeps finite values below 2^15).
__device__ __forceinline__ float f64_scaled_to_f32(double x, int sb) {
  const uint32_t h = (uint32_t)__double2hiint(x), l = (uint32_t)__double2loint(x);
  const uint32_t e = (h >> 20) & 0x7ffu;
  const uint32_t man = __funnelshift_l(l, h, 3) & 0x7fffffu;
  const int ef = (int)e + sb;
  uint32_t f = (h & 0x80000000u) | ((uint32_t)ef << 23) | man;
  f = ef > 0 ? f : (h & 0x80000000u);
  f = e == 0x7ffu ? ((h & 0x80000000u) | 0x7f800000u | (man | l ? 0x400000u : 0u)) : f;
  return __uint_as_float(f);
}

// FP32 -> FP64 with integer operations: exact for normal numbers and zero;
// FP32 subnormals flush to a signed zero; Inf and NaN are kept.  (The FP64
// pipe of this part retires about two operations per SM per clock, so the z
// epilogue keeps one FP64 operation per point, the multiply-add.)
__device__ __forceinline__ double f32_to_f64(float v) {
  const uint32_t u = __float_as_uint(v);
  const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  uint32_t hi = sign | ((e + 896u) << 20) | (m >> 3);
  uint32_t lo = m << 29;
  hi = e == 0 ? sign : hi;
  lo = e == 0 ? 0u : lo;
  hi = e == 255 ? (sign | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u)) : hi;
  lo = e == 255 ? 0u : lo;
  return __hiloint2double((int)hi, (int)lo);
}

// Eight FP64 values (scaled by 2^s, sb = s - 896) -> eight FP16 high parts
// and eight FP16 remainders, as two 16-byte rows.
__device__ __forceinline__ void split8(const double* v, int sb, uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float a = f64_scaled_to_f32(v[2 * q], sb), b = f64_scaled_to_f32(v[2 * q + 1], sb);
    const __half2 hh = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(hh);
    const __half2 ll = __floats2half2_rn(a - hf.x, b - hf.y);
    h[q] = *reinterpret_cast<const uint32_t*>(&hh);
    l[q] = *reinterpret_cast<const uint32_t*>(&ll);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}


// Conversion tasks of an item: one 16-byte row of a core matrix each, from
// eight staged doubles (zero for rows past the data).
//   xy: task (j, q) (j < npy, q: i-octet < kx/8): core matrix (j/8, q) of
//       the plane image, its row j%8 = X[j][8q .. 8q+7], staged in box q/2,
//       row j, chunks 4 (q%2) .. +3 (swizzled).  Eight consecutive tasks are
//       eight consecutive rows j of one core matrix: their reads fall in
//       distinct banks and their stores fill 128 contiguous bytes.
//   z:  task (k, m) (k < kz, m: point octet < 16): core matrix (k/8 along K,
//       m along M) at (k/8 * 16 + m) * 128, its row k%8 = the tile's points
//       8m .. 8m+7 of plane k, staged in box m/2, row k.
struct Task {
  int row;       // staged row (j or k), or -1 for a zero row
  uint32_t src;  // byte offset of the staged row's first 16-byte chunk within the box region set
  int chunk0;    // its first chunk, 0 or 4
  uint32_t dst;  // byte offset of the image row
};

template <class Geom>
__device__ __forceinline__ Task task_xy(const Geom& G, int j, int q) {
  Task k;
  k.row = j < G.ny ? j : -1;
  k.src = (uint32_t)(q >> 1) * G.reg_xy + (uint32_t)(j < G.ny ? j : 0) * 128u;
  k.chunk0 = 4 * (q & 1);
  k.dst = (uint32_t)((j >> 3) * (G.kx >> 3) + q) * 128u + (uint32_t)(j & 7) * 16u;
  return k;
}

template <class Geom>
__device__ __forceinline__ Task task_z(const Geom& G, int k, int m) {
  Task r;
  r.row = k < G.nz ? k : -1;
  r.src = (uint32_t)(m >> 1) * G.reg_z + (uint32_t)(k < G.nz ? k : 0) * 128u;
  r.chunk0 = 4 * (m & 1);
  r.dst = (uint32_t)((k >> 3) * 16 + m) * 128u + (uint32_t)(k & 7) * 16u;
  return r;
}

// The eight staged doubles of a task (chunk c of staged row r sits at chunk
// c ^ (r mod 8): the 128-byte swizzle).
__device__ __forceinline__ void load8(const unsigned char* stg, const Task& k, double* v) {
  if (k.row < 0) {
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = 0.0;
    return;
  }
  const int sw = k.row & 7;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const double2 d = *reinterpret_cast<const double2*>(stg + k.src + (uint32_t)(((k.chunk0 + e) ^ sw) << 4));
    v[2 * e] = d.x;
    v[2 * e + 1] = d.y;
  }
}

// The tasks of one producer thread, t = ptid, ptid + 224, ...: a task index
// t = major * rows + row (rows = npy for xy, kz for z) kept as the pair
// (row, major), advanced without a division.
struct TaskIter {
  int row, major, rows;
  __device__ __forceinline__ TaskIter(int t, int rows_) : row(t % rows_), major(t / rows_), rows(rows_) {}
  __device__ __forceinline__ void next() {
    row += kProdWarps * 32;
    while (row >= rows) row -= rows, ++major;
  }
};

template <class Geom>
__device__ __forceinline__ Task task_of(const Geom& G, int kind, const TaskIter& ti) {
  return kind == 0 ? task_xy(G, ti.row, ti.major) : task_z(G, ti.row, ti.major);
}

// Largest FP64 biased exponent among the staged values of an item's tasks.
template <class Geom>
__device__ __forceinline__ int max_exponent(const unsigned char* stg, int ntask, int kind, const Geom& G,
                                            int ptid) {
  uint32_t emax = 0;
  TaskIter ti(ptid, kind == 0 ? G.npy : G.kz);
  // two tasks per turn: their loads are in flight together
  int t = ptid;
  for (; t + kProdWarps * 32 < ntask; t += 2 * kProdWarps * 32) {
    const Task k0 = task_of(G, kind, ti);
    ti.next();
    const Task k1 = task_of(G, kind, ti);
    ti.next();
    double v[16];
    load8(stg, k0, v);
    load8(stg, k1, v + 8);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const uint32_t e = (uint32_t)__double2hiint(v[q]) >> 20 & 0x7ffu;
      emax = e > emax ? e : emax;
    }
  }
  if (t < ntask) {
    const Task k = task_of(G, kind, ti);
    double v[8];
    load8(stg, k, v);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint32_t e = (uint32_t)__double2hiint(v[q]) >> 20 & 0x7ffu;
      emax = e > emax ? e : emax;
    }
  }
  return (int)emax;
}

}  // namespace
