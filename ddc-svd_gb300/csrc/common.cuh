// common.cuh -- shared device/host infrastructure of libddcsvd (sm_103a).
//
// * bounded grid barrier for cooperative persistent kernels: every spin has a
//   wall-clock limit (%globaltimer); on expiry the kernel records
//   DDCSVD_ERR_TIMEOUT in the device status word and unwinds -- no trap, no
//   endless loop;
// * warp / block reductions;
// * launch bookkeeping (kernel launch counter for the C-ABI accounting).
#pragma once

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include <algorithm>
#include <stdio.h>

#include "../../include/ddcsvd.h"

namespace ddcsvd {

// Wall-clock limit of one device-side wait (ns).  Generous against the
// microsecond-scale steps between barriers, short enough that a wedged
// kernel returns promptly with a status instead of holding the GPU.
constexpr unsigned long long kWaitLimitNs = 4000000000ull;

// Device status word layout: [0] = error code (0 = ok), [1] = detail.
struct DevStatus {
  int code;
  int detail;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile_int(const int* p) {
  return *reinterpret_cast<const volatile int*>(p);
}

__device__ __forceinline__ void set_error(DevStatus* st, int code, int detail) {
  if (atomicCAS(&st->code, 0, code) == 0) st->detail = detail;
}

// Barrier state: one per cooperative launch, zeroed before the launch.
struct GridBarrier {
  unsigned count;
  unsigned gen;
};

// Grid-wide barrier for a cooperative launch of `nblocks` CTAs.  Returns
// false (in every thread of the CTA) if the status word holds an error or
// the wait exceeded kWaitLimitNs; callers then leave their loops.
__device__ __forceinline__ bool grid_sync(GridBarrier* bar, unsigned nblocks, DevStatus* st,
                                          int where) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = ld_volatile_int(&st->code) == 0;
    if (ok) {
      unsigned g = ld_acquire(&bar->gen);
      __threadfence();
      unsigned arrived = atomicAdd(&bar->count, 1u);
      if (arrived == nblocks - 1) {
        bar->count = 0;
        __threadfence();
        atomicAdd(&bar->gen, 1u);
      } else {
        unsigned long long t0 = global_ns();
        while (ld_acquire(&bar->gen) == g) {
          if (ld_volatile_int(&st->code) != 0) {
            ok = 0;
            break;
          }
          if (global_ns() - t0 > kWaitLimitNs) {
            set_error(st, DDCSVD_ERR_TIMEOUT, where);
            ok = 0;
            break;
          }
          __nanosleep(32);
        }
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_prod(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v *= __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; `red` must hold blockDim.x/32 elements.  All threads get
// the result.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  T r = 0;
  for (int i = 0; i < nw; i++) r += red[i];
  return r;
}

__host__ __device__ constexpr inline int ceil_div(int a, int b) { return (a + b - 1) / b; }
__host__ __device__ constexpr inline long long round_up(long long a, long long b) {
  return (a + b - 1) / b * b;
}

// ------------------------------------------------------------------ host side
extern long long g_launch_count;  // kernels launched by this library
inline void count_launch(long long k = 1) { __atomic_fetch_add(&g_launch_count, k, __ATOMIC_RELAXED); }

void set_last_error(const char* fmt, ...);

#define DDC_CUDA_TRY(expr)                                                          \
  do {                                                                              \
    cudaError_t _e = (expr);                                                        \
    if (_e != cudaSuccess) {                                                        \
      ::ddcsvd::set_last_error("%s:%d %s -> %s", __FILE__, __LINE__, #expr,         \
                               cudaGetErrorString(_e));                             \
      return DDCSVD_ERR_CUDA;                                                       \
    }                                                                               \
  } while (0)

#define DDC_TRY(expr)              \
  do {                             \
    int _s = (expr);               \
    if (_s != DDCSVD_OK) return _s; \
  } while (0)

}  // namespace ddcsvd
