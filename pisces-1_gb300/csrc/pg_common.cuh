// Shared helpers of libpisces_gb300: status/error text, CUDA checks, grid handle.
#pragma once

#include <cuda_runtime.h>
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "pisces_gb300.h"

namespace pg {

// Last error text, per calling thread.
void set_error(const char* fmt, ...);
const char* last_error();

// On failure the runtime's last-error slot is cleared as well, so that a
// failed call is not reported again by the next launch check.
#define PG_CUDA_TRY(expr)                                                                  \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      cudaGetLastError();                                                                  \
      ::pg::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(e_)); \
      return PG_CUDA;                                                                      \
    }                                                                                      \
  } while (0)

#define PG_TRY(expr)                  \
  do {                                \
    pg_status s_ = (expr);            \
    if (s_ != PG_OK) return s_;       \
  } while (0)

#define PG_ARG(cond, ...)             \
  do {                                \
    if (!(cond)) {                    \
      ::pg::set_error(__VA_ARGS__);   \
      return PG_BAD_ARG;              \
    }                                 \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Kernel launches issued by this library (every launch site calls check_launch).
void count_launch();
// Device allocations made by this library (every cudaMalloc goes through DevBuf).
void count_device_alloc();

// Launch-status check after a kernel launch.
inline pg_status check_launch(const char* what) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("launch of %s failed: %s", what, cudaGetErrorString(e));
    return PG_CUDA;
  }
  return PG_OK;
}

// Device buffer owned by RAII (cudaMalloc/cudaFree).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  pg_status alloc(size_t count) {
    release();
    if (count == 0) return PG_OK;
    count_device_alloc();
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      set_error("cudaMalloc of %zu bytes failed", count * sizeof(T));
      return PG_OOM;
    }
    n = count;
    return PG_OK;
  }
  // Grow-only: keeps the buffer if it already holds count elements (a
  // long-lived owner then allocates, and frees, only while it grows).
  pg_status ensure(size_t count) { return n >= count && p ? PG_OK : alloc(count); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// Programmatic dependent launch.  A kernel launched by launch_dependent may
// be scheduled before the kernel ahead of it in the stream has finished; it
// must call pdl_wait() before it touches global memory (the wait returns once
// that kernel has completed and its writes are visible; in a kernel launched
// normally it returns at once).  pdl_release() lets the next dependent launch
// be scheduled; it is issued right after the wait.  A dependent is scheduled
// only when every block of the kernel ahead has released or exited, i.e. when
// all of them are resident, so the early launch cannot take the resources
// that kernel still needs.  What it saves is the gap between the end of one
// kernel and the start of the next.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                    Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Grow-only page-locked host buffer: copies between it and the device are
// asynchronous (a pageable source or target makes cudaMemcpyAsync stage
// through a driver buffer, and a device-to-host copy wait for the stream).
template <typename T>
struct HostPinned {
  T* p = nullptr;
  size_t n = 0;
  HostPinned() = default;
  HostPinned(const HostPinned&) = delete;
  HostPinned& operator=(const HostPinned&) = delete;
  ~HostPinned() { release(); }
  pg_status ensure(size_t count) {
    if (p && n >= count) return PG_OK;
    release();
    if (cudaMallocHost(&p, count * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      set_error("cudaMallocHost of %zu bytes failed", count * sizeof(T));
      return PG_OOM;
    }
    n = count;
    return PG_OK;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
};

// Byte offset of element (r, k) of a tensor-core operand tile in shared
// memory: no-swizzle K-major core matrices of 8 rows x 16 bytes (4 FP32/TF32
// values), K-adjacent core matrices 128 bytes apart, 8-row groups kpad/4 *
// 128 bytes apart.  The grid keeps its kinetic matrices in this layout
// (rows padded to 16, K to 8) so that a kernel copies them in one piece.
inline __host__ __device__ unsigned tc_kmajor_off(int r, int k, int kpad) {
  return (unsigned)(((r >> 3) * (kpad >> 2) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
}
// The same for FP16 operands: core matrices of 8 rows x 8 values (16
// bytes), K padded to 16 (one MMA K step).
inline __host__ __device__ unsigned tc16_kmajor_off(int r, int k, int kpad16) {
  return (unsigned)(((r >> 3) * (kpad16 >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
inline __host__ __device__ int tc16_kpad(int n) { return (n + 15) / 16 * 16; }
inline __host__ __device__ int tc_npad(int n) { return (n + 15) / 16 * 16; }
inline __host__ __device__ int tc_kpad(int n) { return (n + 7) / 8 * 8; }
// K chunk of the tensor-core contraction: the B chunk (npad x kc) and the A
// tile (128 x kc), both as TF32 hi/lo, must fit 220 KB of shared memory;
// n <= 112 gives one chunk (kc = kpad).  The operand images are stored as
// ceil(kpad / kc) consecutive chunk images of npad x kc.
inline __host__ __device__ int tc_kchunk(int n) {
  const int npad = tc_npad(n), kpad = tc_kpad(n);
  const int kc_max = (220 * 1024 / (8 * (npad + 128))) / 8 * 8;
  const int nch = (kpad + kc_max - 1) / kc_max;
  return ((kpad + nch - 1) / nch + 7) / 8 * 8;
}

}  // namespace pg

// The grid handle: sizes, host copies of the 1-D data and device kinetic matrices.
struct pg_grid {
  int dvrtype = 2;                 // 2: sine DVR; 3: periodic FFT kinetic (as dense circulant matrices)
  int n[3];
  double L[3];
  long N;
  int device;
  std::vector<double> x[3];        // grid points per axis
  std::vector<double> t[3];        // full symmetric kinetic matrices, n x n row-major (host)
  pg::DevBuf<double> t_dev[3];     // same, FP64, on the device
  // TF32-rounded high part and the TF32-rounded remainder T - hi, each as
  // tensor-core operand images (tc_kmajor_off layout, one tc_npad x tc_kchunk
  // image per K chunk)
  pg::DevBuf<float> t_hi[3];
  pg::DevBuf<float> t_lo[3];
  // FP16 high part and remainder of T * 2^t16_scale (one power of two for
  // all axes, chosen so that the largest entry lies in [2^14, 2^15)), as
  // tc16_kmajor_off images (rows padded to 16, K to 16); built for n <= 128
  pg::DevBuf<unsigned short> t16_hi[3];
  pg::DevBuf<unsigned short> t16_lo[3];
  int t16_scale = 0;
  pg::DevBuf<double> x_dev[3];     // grid points on the device
  pg::DevBuf<int> tc_err;          // set by the tensor-core H*X kernels if a completion wait times out
  // eigenbasis of the kinetic matrices (the orthonormal DST-I, symmetric),
  // for the kinetic preconditioner: FP64, TF32 hi/lo, and the eigenvalues
  pg::DevBuf<double> q_dev[3];
  // forward transform Q^T (q_*) and backward transform Q (qb_*): FP64 and
  // operand images, as t_hi / t_lo; the same matrix for the symmetric DST-I
  pg::DevBuf<float> q_hi[3], q_lo[3];
  pg::DevBuf<double> qb_dev[3];
  pg::DevBuf<float> qb_hi[3], qb_lo[3];
  pg::DevBuf<double> d_dev[3];
  // FP16 high part and remainder of Q^T 2^q16_scale (forward, q16f_*) and of
  // Q 2^q16_scale (backward, q16b_*) as tc16_kmajor_off images, for the FP16
  // kinetic preconditioner; built when every axis has the same n <= 128
  // (one eigenbasis for the three axes).  q16_sym: Q^T = Q (the DST-I), the
  // backward images are not stored.
  pg::DevBuf<unsigned short> q16f_hi, q16f_lo, q16b_hi, q16b_lo;
  int q16_scale = 0;
  bool q16_sym = false;
  std::vector<double> ekin[3];     // FFT grids: plane-wave energies per axis (Tdiag)
  // random start columns (Randm11 from seed 1; the same values for every
  // solve on this grid), generated once and grown on demand
  mutable std::mutex start_m;
  mutable pg::DevBuf<double> start_rand;
  // mixed H*X kernel choice (0 automatic, 1 three axis passes, 2 fused) and
  // the fused kernel's work counters, one block per stream id
  int hx_kernel = 0;
  int pc_kernel = 0;  // mixed kinetic preconditioner: 0 automatic (FP16 kernel where it applies), 1 axis passes
  int hx_lag = 0, hx_ctas = 0, hx_form = 0;  // overrides of the tuned launch parameters (0: tuned)
  mutable std::mutex fused_m;
  mutable std::map<unsigned long long, std::unique_ptr<pg::DevBuf<unsigned>>> fused_cnt;
  // tensor maps of the FP16 kernels' vector blocks by (address, vectors): a
  // map depends only on those and the grid's shape, so a solve's blocks are
  // encoded once (under fused_m)
  struct TensorMapPair {
    alignas(64) unsigned char xy[128];
    alignas(64) unsigned char z[128];
  };
  mutable std::map<std::pair<const void*, int>, TensorMapPair> tmaps;
};

namespace pg {
// Launch parameters of the mixed-form H*X for one grid shape and block size:
// from the tuned table (pg_hx_tuned.inc, written by tune_hx.py), else the
// built-in rules, then the grid's overrides.
struct HxParams {
  int kind;  // 1: three axis passes (k_hx_tc), 2: fused (k_hx_fused)
  int lag;   // fused: vectors between a vector's xy items and its z items
  int ctas;  // CTAs per launch (0: one per SM)
  int form;  // three passes: 0 automatic, 1 serial, 2 pipelined (one K chunk only)
};
HxParams hx_params(const pg_grid* g, int nvec);
// Single-axis contraction Y = A x_axis X for nvec vectors, A an n_axis x
// n_axis matrix given in both FP64 and split-TF32 form; mode 0: Y = A X,
// mode 1: Y += A X.  FP64 or tensor-core arithmetic per precision.
pg_status axis_apply(const pg_grid* g, int axis, const double* A64, const float* Ahi, const float* Alo,
                     const double* x, double* y, int nvec, int mode, int precision, cudaStream_t st);
// H*X without the public call's synchronous status check (pg_hx.cu); the
// caller checks check_tc_error() at its own synchronisation points.
// unit: every value of X is known to lie in [-1, 1] (the Davidson's
// orthonormal basis vectors), which lets the FP16-split kernel use a fixed
// operand scale.
pg_status hx(const pg_grid* g, const double* v, const double* x, double* y, int nvec, int precision,
             cudaStream_t st, bool unit = false);
pg_status check_tc_error(const pg_grid* g, cudaStream_t st);
}  // namespace pg
