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

// Device status word: error code (0 = ok) and detail, written by kernels;
// the two limits below are written by the host before each call
// (ddcsvd_set_limits) and only read on the device.
struct __align__(16) DevStatus {
  int code;
  int detail;
  unsigned wait_us;  // wall-clock limit of one device-side wait in microseconds (0: kWaitLimitNs)
  unsigned extra;    // fault injection: arrivals that the first grid barrier of a cooperative
                     // launch waits for beyond its own CTAs (0 in normal use; > 0 makes that
                     // barrier's waits run out, which tests the timeout path)
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

__device__ __forceinline__ uint4 ld_status(const DevStatus* st) {
  uint4 v;
  asm volatile("ld.volatile.global.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(st)
               : "memory");
  return v;
}

__device__ __forceinline__ void set_error(DevStatus* st, int code, int detail) {
  if (atomicCAS(&st->code, 0, code) == 0) st->detail = detail;
}

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// Barrier state: one per cooperative launch, zeroed before the launch.
struct GridBarrier {
  unsigned count;  // arrivals so far in this launch (only ever grows)
  unsigned gen;    // unused, kept for layout
};

// Grid-wide barrier for a cooperative launch of `nblocks` CTAs.  Returns
// false (in every thread of the CTA) if the status word holds an error or
// the wait exceeded its limit (st->wait_us, else kWaitLimitNs); callers then
// leave their loops.
//
// The arrival counter is never reset inside a launch: barrier k of the launch
// is complete once it reaches (k + 1) * nblocks, and because no CTA can arrive
// at barrier k + 1 before barrier k is complete, the value returned by a CTA's
// own arrival tells it which barrier it is in.  That costs one atomic round
// trip per CTA plus the polls, with no second "release" write on the critical
// path.  The status word is read alongside the arrival and then every 32 polls.
__device__ __forceinline__ bool grid_sync(GridBarrier* bar, unsigned nblocks, DevStatus* st,
                                          int where) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint4 s = ld_status(st);
    const int code = (int)s.x;
    const unsigned old = atom_add_acq_rel(&bar->count, 1u);
    const unsigned round = old / nblocks;
    const unsigned target = (round + 1u) * nblocks + (round == 0u ? s.w : 0u);
    const unsigned long long limit = s.z ? 1000ull * s.z : kWaitLimitNs;
    int ok = code == 0;
    if (ok && old + 1u != target) {
      unsigned polls = 0;
      unsigned long long t0 = 0;
      while ((int)(ld_acquire(&bar->count) - target) < 0) {
        if ((++polls & 31u) == 0) {
          if (ld_volatile_int(&st->code) != 0) {
            ok = 0;
            break;
          }
          const unsigned long long now = global_ns();
          if (t0 == 0) {
            t0 = now;
          } else if (now - t0 > limit) {
            set_error(st, DDCSVD_ERR_TIMEOUT, where);
            ok = 0;
            break;
          }
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Optional phase trace for kernel tuning: a build with -DDDCSVD_PHASE_TRACE
// records %globaltimer at DDC_MARK points of one CTA into a device array that
// ddcsvd_trace_read() copies out.  Without the macro the marks compile to
// nothing.
#ifdef DDCSVD_PHASE_TRACE
// the translation unit that uses the marks defines g_phase_trace[128 * 16]
#define DDC_MARK(cond, row, slot)                                                        \
  do {                                                                                   \
    if ((cond) && threadIdx.x == 0 && (row) < 128) g_phase_trace[(row) * 16 + (slot)] = global_ns(); \
  } while (0)
#else
#define DDC_MARK(cond, row, slot) \
  do {                            \
  } while (0)
#endif

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

// ---- compensated (float-float) sums
// A value hi + lo with |lo| <= ulp(hi)/2, built from error-free transforms
// (Knuth's two-sum, the FMA product error).  Sums of squares carried this way
// keep about 44 significant bits using only FP32 instructions: on GB300 the
// FP64 pipe is narrow and its latency sits on the critical path of every
// Householder step, so the panel kernels avoid it.  The _rn intrinsics keep
// the compiler from contracting or reassociating the error terms.
struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  const float t = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  const float hi = __fadd_rn(s, t);
  return FF{hi, __fsub_rn(t, __fsub_rn(hi, s))};
}

// a + x * x with the product's rounding error kept
__device__ __forceinline__ FF ff_add_sq(FF a, float x) {
  const float p = __fmul_rn(x, x);
  const float pe = __fmaf_rn(x, x, -p);
  return ff_add(a, FF{p, pe});
}

__device__ __forceinline__ FF warp_sum_ff(FF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    FF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    // order the operands by lane so that both partners compute the same sum
    v = ((threadIdx.x & o) == 0) ? ff_add(v, w) : ff_add(w, v);
  }
  return v;
}

// Householder parameters (reference convention alpha = -sign(x0) ||x||,
// sign(0) = +1) from x0 and a compensated (float-float) ||tail||^2, in FP32
// only.  The input matrix is scaled so that max|a| lies in [2^-40, 2^40] (or is left
// alone when it already does), so x0^2 + t2 neither overflows nor loses
// anything that matters against ||A||.  sqrt of the rounded pair and the two
// quotients are correctly rounded FP32 operations: alpha is within one ulp
// of the FP64 result.
__device__ __forceinline__ void householder_ff(float x0, FF t2, float* alpha, float* tau, float* scale) {
  const FF n2 = ff_add_sq(t2, x0);
  const float nrm = sqrtf(__fadd_rn(n2.hi, n2.lo));
  if (nrm == 0.f) {
    *alpha = 0.f;
    *tau = 0.f;
    *scale = 0.f;
    return;
  }
  const float ax = fabsf(x0);
  const float sg = x0 < 0.f ? -1.f : 1.f;
  *alpha = -sg * nrm;
  *tau = (nrm + ax) / nrm;
  *scale = sg / (ax + nrm);  // 1 / (x0 - alpha)
}

// 2^k with max|a| * 2^k in [0.5, 1) when max|a| is outside [2^-40, 2^40], else 1
__device__ __forceinline__ float range_scale(unsigned bits) {
  const float a = __uint_as_float(bits);
  if (!(a > 0.f) || isinf(a) || (a >= 0x1p-40f && a <= 0x1p40f)) return 1.f;
  int ex = 0;
  frexpf(a, &ex);
  return ldexpf(1.f, max(-126, min(126, -ex)));
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
