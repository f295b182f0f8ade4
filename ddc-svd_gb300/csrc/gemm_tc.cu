// gemm_tc.cu -- tcgen05 tensor-core GEMM in split TF32 for sm_103a.
//
//   C (M x N, col-major) = beta * C + alpha * A B,   A: M x K, B: K x N,
//   both operands K-major in global memory (row r of A at A + r*lda, column
//   n of B at B + n*ldb, K contiguous).
//
// FP32 accuracy from TF32 tensor cores.  Each FP32 operand x is split into
// TF32 parts (round-to-nearest) and the products of the parts are summed in
// FP32 in TMEM:
//   2 parts (GEMM_TF32X3): x = h + l, h*h' + h*l' + l*h'      ~2^-21 relative
//   3 parts (GEMM_TF32X6): x = h + m + l,
//                          h*h' + h*m' + m*h' + m*m' + h*l' + l*h'  below FP32
// (smallest products are issued first).
//
// A persistent CTA (one per SM) computes 128 x BN tiles (BN = 128, 64 or 32)
// one after another, 10 warps:
//   warp 0      TMA producer: raw FP32 K-slabs (32 wide, 128-byte swizzle)
//               of A and B into a shared-memory ring (3 stages for two
//               parts, 2 for three);
//   warps 2-9   split each landed slab in place into its TF32 parts (part 0
//               overwrites the raw copy), then release it to the MMA;
//   warp 1      TMEM allocation and the single MMA-issuing thread:
//               tcgen05.mma.kind::tf32 over 4 K-steps x (3 or 6) products
//               per slab into one of two TMEM slab accumulators (fresh per
//               slab); tcgen05.commit frees the stage and the accumulator;
//   warps 2-9   drain each slab accumulator with tcgen05.ld (lane = row;
//               two warps per TMEM lane quarter, each half of the columns)
//               into FP32 registers with round-to-nearest adds -- the tensor
//               core's own accumulation over many MMAs loses ~2-3 bits
//               against FP32 FMA chains -- and finally update C (coalesced
//               along columns of col-major C, or 32-column chunks through
//               shared memory and one TMA store / reduce-add each).
// The stage ring and the accumulator pair run on across tiles, so one tile's
// epilogue overlaps the next tile's loads.  Split-K slices write FP32
// partials that a second kernel reduces in a fixed order (deterministic).
//
// Every mbarrier wait is bounded by wall-clock time; on expiry the CTA
// records DDCSVD_ERR_TIMEOUT, skips its stores, waits (bounded) for its own
// TMA copies in flight and frees its TMEM before returning.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <string.h>

#include "async.cuh"
#include "internal.hpp"

namespace ddcsvd {

void splitk_reduce(ddcsvd_context* ctx, int M, int N, int ksplit, const float* partial, float alpha,
                   float beta, float* C, int ldc, bool trans);

namespace tc {

constexpr int BM = 128;
constexpr int BK = 32;  // FP32 elements per slab row: 128 bytes = one swizzle span
constexpr int THREADS = 320;  // producer warp, MMA warp, 8 split / drain / epilogue warps
constexpr int kWorkers = THREADS - 64;
// Each 32-wide K slab is accumulated in a fresh TMEM buffer and drained by
// the epilogue warps into FP32 registers: the tensor core's own accumulation
// error grows with the number of MMAs it chains (measured: ~linear in K;
// draining every 4 slabs raised the 4096^2 SVD residual from 1.3e-6 to
// 3.7e-6), so every slab is drained and added in FP32 round-to-nearest.
constexpr unsigned long long kTcWaitNs = 2000000000ull;

// Bounded wait for the phase of the given parity.  Returns false when the CTA
// aborts (another role gave up, or this wait ran out of time).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          DevStatus* st, int where) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (global_ns() - t0 > kTcWaitNs) {
      *abort_flag = 1;
      set_error(st, DDCSVD_ERR_TIMEOUT, where);
      return false;
    }
  }
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle,
// 8-row core groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);  // start address
  d |= (uint64_t)(16 >> 4) << 16;           // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset
  d |= (uint64_t)1 << 46;                   // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;                   // 128-byte swizzle
  return d;
}

// Instruction descriptor: D = FP32, A = B = TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// In-place split of a raw FP32 tile into NP TF32 parts: raw -> part 0, the
// others into part buffers 1 (and 2), all in the same (swizzled) positions.
template <int NP>
__device__ __forceinline__ void split_tile(float4* raw, float4* p1, float4* p2, int n16, int t, int nt) {
  for (int q = t; q < n16; q += nt) {
    const float4 v = raw[q];
    float x[4] = {v.x, v.y, v.z, v.w}, h[4], m[4], l[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      h[c] = __uint_as_float(to_tf32(x[c]));
      const float r = x[c] - h[c];
      m[c] = __uint_as_float(to_tf32(r));
      if (NP == 3) l[c] = __uint_as_float(to_tf32(r - m[c]));
    }
    raw[q] = make_float4(h[0], h[1], h[2], h[3]);
    p1[q] = make_float4(m[0], m[1], m[2], m[3]);
    if (NP == 3) p2[q] = make_float4(l[0], l[1], l[2], l[3]);
  }
}

struct TcParams {
  int M, N;
  int a_koff, b_koff;  // K coordinate of the first slab in the A / B maps
  int nslab;           // slabs of 32 along K in total
  int per_split;       // slabs per K slice
  int ksplit;          // K slices
  int tiles_m, tiles_n;
  float* C;
  int ldc;
  float alpha, beta;
  float* partial;  // split-K partials (M x N per slice, ld M) or null
  int trans;       // store C transposed: element (r, c) at C[c + r * ldc]
  int tma_epi;     // 0: per-thread C update; 1: TMA store (beta 0); 2: TMA reduce-add (beta 1)
  DevStatus* st;
};

// Shared memory: the stage ring, then two epilogue chunk buffers of BM x 32
// FP32, then the barriers.
template <int BN, int NP>
struct Layout {
  static constexpr int A_BYTES = BM * BK * 4;
  static constexpr int B_BYTES = BN * BK * 4;
  static constexpr int STAGE = NP * (A_BYTES + B_BYTES);
  static constexpr int STAGES = (NP == 2) ? 3 : 2;
  static constexpr int EPI_CHUNK = 32;                  // columns per epilogue chunk
  static constexpr int EPI_BYTES = BM * EPI_CHUNK * 4;  // one chunk buffer
  static constexpr int EPI_OFF = STAGES * STAGE;
  static constexpr int BAR_OFF = EPI_OFF + 2 * EPI_BYTES;
  static constexpr int SMEM = BAR_OFF + 1024 + 256;     // + alignment and barriers
  static constexpr int TMEM_COLS = 2 * BN;              // two slab accumulators
};

// phase marks (trace builds): CTA 0, one row per slab of the CTA (first 128)
#ifdef DDCSVD_PHASE_TRACE
__device__ unsigned long long g_gemm_trace[128 * 16];
#define GMARK(cond, g, slot)                                                        \
  do {                                                                              \
    if ((cond) && blockIdx.x == 0 && (g) < 128) g_gemm_trace[(g) * 16 + (slot)] = global_ns(); \
  } while (0)
#else
#define GMARK(cond, g, slot) \
  do {                       \
  } while (0)
#endif

// AND of `v` over the 256 threads of warps 2-9 (named barrier 2); every one of
// them must call it.
__device__ __forceinline__ bool epi_vote(bool v) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.b32 p, %1, 0;\n\t"
      "bar.red.and.pred q, 2, 256, p;\n\t"
      "selp.s32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((int)v)
      : "memory");
  return r != 0;
}

// Persistent: each CTA takes work items (K slice, N tile, M tile; M fastest)
// blockIdx.x, blockIdx.x + gridDim.x, ...  The stage ring and the two slab
// accumulators continue across items, indexed by this CTA's running slab
// count, so the producer and the MMA issuer run ahead into the next item
// while the split/epilogue warps write the previous one out.
template <int BN, int NP>
__global__ void __launch_bounds__(THREADS, 1)
    tc_gemm_split_tf32_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                              const __grid_constant__ CUtensorMap tmC, TcParams p) {
  using L = Layout<BN, NP>;
  constexpr int STAGES = L::STAGES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(round_up(reinterpret_cast<uintptr_t>(smem_raw), 1024));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::BAR_OFF);
  uint64_t* full = bars;
  uint64_t* conv = bars + STAGES;
  uint64_t* empty = bars + 2 * STAGES;
  uint64_t* accf = bars + 3 * STAGES;      // [2] slab accumulator ready
  uint64_t* acce = bars + 3 * STAGES + 2;  // [2] slab accumulator drained
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3 * STAGES + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&conv[s], kWorkers);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], kWorkers);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(L::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const int items = p.tiles_m * p.tiles_n * p.ksplit;
  // work item w: m tile, n tile, K slice, first slab and slab count
  auto item = [&](int w, int& m0, int& n0, int& z, int& s_begin, int& nsl) {
    const int mt = w % p.tiles_m, rest = w / p.tiles_m;
    const int nt = rest % p.tiles_n;
    z = rest / p.tiles_n;
    m0 = mt * BM;
    n0 = nt * BN;
    s_begin = z * p.per_split;
    nsl = max(0, min(p.nslab, s_begin + p.per_split) - s_begin);
  };
  // stage layout: A parts 0..NP-1, then B parts 0..NP-1 (part 0 = raw -> hi)
  auto a_part = [&](int s, int k) { return smem + s * L::STAGE + k * L::A_BYTES; };
  auto b_part = [&](int s, int k) { return smem + s * L::STAGE + NP * L::A_BYTES + k * L::B_BYTES; };

  if (warp == 0) {
    if (lane == 0) {
      int gi = 0;  // this CTA's running slab count
      bool go = true;
      for (int w = blockIdx.x; w < items && go; w += gridDim.x) {
        int m0, n0, z, s_begin, nsl;
        item(w, m0, n0, z, s_begin, nsl);
        for (int i = 0; i < nsl; i++, gi++) {
          const int s = gi % STAGES;
          if (gi >= STAGES && !mbar_wait(&empty[s], ((gi / STAGES) - 1) & 1, abort_flag, p.st, 901)) {
            go = false;
            break;
          }
          GMARK(true, gi, 0);
          mbar_arrive_expect_tx(&full[s], L::A_BYTES + L::B_BYTES);
          const int sl = s_begin + i;
          tma_load_2d(a_part(s, 0), &tmA, p.a_koff + sl * BK, m0, &full[s]);
          tma_load_2d(b_part(s, 0), &tmB, p.b_koff + sl * BK, n0, &full[s]);
        }
      }
      // make sure no copy of ours is still landing before the CTA may exit
      for (int j = max(0, gi - STAGES); j < gi; j++) {
        const int s = j % STAGES;
        const unsigned long long t0 = global_ns();
        while (!mbar_try_wait(&full[s], (j / STAGES) & 1) && global_ns() - t0 < kTcWaitNs) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(BM, BN);
      int gi = 0;
      bool go = true;
      for (int w = blockIdx.x; w < items && go; w += gridDim.x) {
        int m0, n0, z, s_begin, nsl;
        item(w, m0, n0, z, s_begin, nsl);
        for (int i = 0; i < nsl; i++, gi++) {
          const int s = gi % STAGES, b = gi & 1;
          if (!mbar_wait(&conv[s], (gi / STAGES) & 1, abort_flag, p.st, 902) ||
              (gi >= 2 && !mbar_wait(&acce[b], ((gi >> 1) - 1) & 1, abort_flag, p.st, 905))) {
            go = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          GMARK(true, gi, 3);
          const uint32_t d = tmem + (uint32_t)(b * BN);
#pragma unroll
          for (int kk = 0; kk < BK / 8; kk++) {
            const uint32_t off = kk * 32;  // 8 TF32 elements = 32 bytes along K
            uint64_t da[NP], db[NP];
#pragma unroll
            for (int k = 0; k < NP; k++) {
              da[k] = smem_desc_sw128(smem_u32(a_part(s, k)) + off);
              db[k] = smem_desc_sw128(smem_u32(b_part(s, k)) + off);
            }
            const uint32_t first = kk > 0 ? 1u : 0u;  // each slab starts a fresh partial sum
            if (NP == 3) {  // l*h, h*l, m*m, m*h, h*m, h*h
              mma_tf32(d, da[2], db[0], idesc, first);
              mma_tf32(d, da[0], db[2], idesc, 1u);
              mma_tf32(d, da[1], db[1], idesc, 1u);
              mma_tf32(d, da[1], db[0], idesc, 1u);
              mma_tf32(d, da[0], db[1], idesc, 1u);
              mma_tf32(d, da[0], db[0], idesc, 1u);
            } else {  // l*h, h*l, h*h
              mma_tf32(d, da[1], db[0], idesc, first);
              mma_tf32(d, da[0], db[1], idesc, 1u);
              mma_tf32(d, da[0], db[0], idesc, 1u);
            }
          }
          mma_commit(&empty[s]);
          mma_commit(&accf[b]);
          GMARK(true, gi, 4);
        }
      }
    }
  } else {
    // warps 2-9: split landed slabs; drain each slab's partial sum from TMEM
    // into round-to-nearest FP32 registers (the tensor core's own accumulation
    // across many MMAs is less accurate than FP32 FMA chains); write each
    // finished item out.  Two warps share each TMEM lane quarter (warp % 4):
    // warps 2-5 hold the tile's first BN/2 columns, warps 6-9 the others.
    constexpr int HALF = BN / 2;
    const int ct = threadIdx.x - 64;
    const int q = warp & 3;         // TMEM lane quarter this warp may access
    const int h = (warp - 2) >> 2;  // column half
    const uint32_t lane_base = (uint32_t)(q * 32) << 16;
    const int rl = q * 32 + lane;  // row of the tile this thread holds
    float acc[HALF];
    bool ok = true;
    int gi = 0;
    // Every decision below is made alike by all 256 threads: tcgen05.ld is
    // warp-collective and the epilogue's named barriers count all eight warps,
    // so a wait that one lane gave up on is given up by its whole warp
    // (__all_sync), and each item's epilogue starts only after a vote of the
    // eight warps (bar.red.and on barrier 2).
    auto drain = [&](int g) {  // slab g of this CTA
      const int b = g & 1;
      if (!__all_sync(0xffffffffu, mbar_wait(&accf[b], (g >> 1) & 1, abort_flag, p.st, 904))) {
        ok = false;
        return;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      GMARK(ct == 0, g, 5);
#pragma unroll
      for (int c0 = 0; c0 < HALF; c0 += 16) {
        uint32_t r[16];
        tmem_ld16(tmem + lane_base + (uint32_t)(b * BN + h * HALF + c0), r);
#pragma unroll
        for (int jj = 0; jj < 16; jj++) acc[c0 + jj] += __uint_as_float(r[jj]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&acce[b]);
      GMARK(ct == 0, g, 6);
    };
    for (int w = blockIdx.x; w < items && ok; w += gridDim.x) {
      int m0, n0, z, s_begin, nsl;
      item(w, m0, n0, z, s_begin, nsl);
#pragma unroll
      for (int c = 0; c < HALF; c++) acc[c] = 0.f;
      for (int i = 0; i < nsl && ok; i++, gi++) {
        const int s = gi % STAGES;
        if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (gi / STAGES) & 1, abort_flag, p.st, 903))) {
          ok = false;
          break;
        }
        GMARK(ct == 0, gi, 1);
        split_tile<NP>(reinterpret_cast<float4*>(a_part(s, 0)), reinterpret_cast<float4*>(a_part(s, 1)),
                       reinterpret_cast<float4*>(a_part(s, NP - 1)), L::A_BYTES / 16, ct, kWorkers);
        split_tile<NP>(reinterpret_cast<float4*>(b_part(s, 0)), reinterpret_cast<float4*>(b_part(s, 1)),
                       reinterpret_cast<float4*>(b_part(s, NP - 1)), L::B_BYTES / 16, ct, kWorkers);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&conv[s]);
        GMARK(ct == 0, gi, 2);
        if (i >= 1) drain(gi - 1);
      }
      if (ok && nsl >= 1) drain(gi - 1);
      ok = epi_vote(ok && !*abort_flag);
      if (!ok) break;
      if (nsl < 1) continue;
      // ---------------- epilogue of this item: registers -> C
      GMARK(ct == 0, gi - 1, 7);
      const int row = m0 + rl;
      const int ch0 = n0 + h * HALF;  // first column this thread holds
      if (p.tma_epi && !p.partial) {
        // alpha * acc through the two shared-memory chunk buffers of BM x 32 and
        // one TMA store or reduce-add per chunk: with BN >= 64 each half fills
        // its own buffer with 32 of its columns per round; with BN = 32 the
        // halves share buffer 0.  A round refills the buffers only after the
        // previous round's copies have read them.
        constexpr bool OWN = HALF >= L::EPI_CHUNK;
        constexpr int ROUNDS = OWN ? HALF / L::EPI_CHUNK : 1;
        constexpr int COLS = OWN ? L::EPI_CHUNK : HALF;  // columns per thread per round
        float* buf = reinterpret_cast<float*>(smem + L::EPI_OFF + (OWN ? h : 0) * L::EPI_BYTES);
        const int cofs = OWN ? 0 : h * HALF;  // column offset inside a shared buffer
#pragma unroll
        for (int r = 0; r < ROUNDS; r++) {
          if (ct == 0) bulk_wait_read_0();
          asm volatile("bar.sync 1, 256;" ::: "memory");
#pragma unroll
          for (int c = 0; c < COLS; c++) buf[(cofs + c) * BM + rl] = p.alpha * acc[r * COLS + c];
          fence_proxy_async_smem();
          asm volatile("bar.sync 1, 256;" ::: "memory");
          if (ct == 0) {
            for (int hb = 0; hb < (OWN ? 2 : 1); hb++) {
              const int col = n0 + (OWN ? hb * HALF + r * L::EPI_CHUNK : 0);
              if (col >= p.N) continue;
              const float* src = reinterpret_cast<const float*>(smem + L::EPI_OFF + hb * L::EPI_BYTES);
              if (p.tma_epi == 2) tma_reduce_add_2d(&tmC, src, m0, col);
              else tma_store_2d(&tmC, src, m0, col);
            }
            bulk_commit();
          }
        }
      } else if (row < p.M) {
#pragma unroll
        for (int c0 = 0; c0 < HALF; c0 += 16) {
          if (p.partial) {
#pragma unroll
            for (int jj = 0; jj < 16; jj++) {
              const int col = ch0 + c0 + jj;
              if (col < p.N) p.partial[(size_t)z * p.M * p.N + row + (size_t)col * p.M] = acc[c0 + jj];
            }
          } else {
            // 16 independent loads of C in flight, then the 16 updates
            const size_t rs = p.trans ? (size_t)p.ldc : 1, cs = p.trans ? 1 : (size_t)p.ldc;
            float old[16];
#pragma unroll
            for (int jj = 0; jj < 16; jj++) {
              const int col = ch0 + c0 + jj;
              old[jj] = (p.beta != 0.f && col < p.N) ? p.C[row * rs + col * cs] : 0.f;
            }
#pragma unroll
            for (int jj = 0; jj < 16; jj++) {
              const int col = ch0 + c0 + jj;
              if (col < p.N) p.C[row * rs + col * cs] = p.beta * old[jj] + p.alpha * acc[c0 + jj];
            }
          }
        }
      }
      GMARK(ct == 0, gi - 1, 8);
    }
    // every TMA store / reduce-add of this CTA completes before its shared memory goes away
    if (ct == 0) bulk_wait_all();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------- host side
using EncodeFn = PFN_cuTensorMapEncodeTiled_v12000;

static EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(ptr);
    else
      cudaGetLastError();
  }
  return fn;
}

// 2-D map over a K-major operand: `rows` rows of `kext` FP32 elements,
// row stride `ld` elements; box = 32 (K) x box_rows, 128-byte swizzle.
static int make_map(CUtensorMap* map, const float* base, long long kext, long long rows, long long ld,
                    int box_rows) {
  EncodeFn enc = encode_fn();
  if (!enc) {
    set_last_error("cuTensorMapEncodeTiled unavailable");
    return DDCSVD_ERR_UNSUPPORTED;
  }
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((ld * 4) & 15)) {
    set_last_error("tensor-core operand not 16-byte aligned");
    return DDCSVD_ERR_ARG;
  }
  cuuint64_t dims[2] = {(cuuint64_t)kext, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_last_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return DDCSVD_ERR_CUDA;
  }
  return DDCSVD_OK;
}

// 2-D map over the column-major output C (rows innermost), box BM x BN, no
// swizzle: target of the TMA store / reduce-add epilogue.
static int make_map_c(CUtensorMap* map, const float* C, long long M, long long N, long long ldc, int bn) {
  EncodeFn enc = encode_fn();
  if (!enc) return DDCSVD_ERR_UNSUPPORTED;
  cuuint64_t dims[2] = {(cuuint64_t)M, (cuuint64_t)N};
  cuuint64_t strides[1] = {(cuuint64_t)(ldc * 4)};
  cuuint32_t box[2] = {(cuuint32_t)BM, (cuuint32_t)bn};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(C), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? DDCSVD_OK : DDCSVD_ERR_CUDA;
}

template <int BN, int NP>
static int launch(ddcsvd_context* ctx, int M, int N, int K, const float* A, long long lda, int a_koff,
                  const float* B, long long ldb, int b_koff, float* C, int ldc, float alpha, float beta,
                  Arena* scratch, bool trans) {
  using L = Layout<BN, NP>;
  CUtensorMap ma, mb;
  DDC_TRY(make_map(&ma, A, (long long)a_koff + K, M, lda, BM));
  DDC_TRY(make_map(&mb, B, (long long)b_koff + K, N, ldb, BN));
  static_assert(L::SMEM <= 232448, "tensor-core GEMM shared memory exceeds the opt-in limit");
  static bool attr_set = false;
  if (!attr_set) {
    DDC_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_split_tf32_kernel<BN, NP>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, L::SMEM));
    attr_set = true;
  }
  TcParams p;
  p.M = M;
  p.N = N;
  p.a_koff = a_koff;
  p.b_koff = b_koff;
  p.nslab = ceil_div(K, BK);
  p.C = C;
  p.ldc = ldc;
  p.alpha = alpha;
  p.beta = beta;
  p.trans = trans ? 1 : 0;
  p.st = ctx->d_status;
  const int tiles = ceil_div(M, BM) * ceil_div(N, BN);
  int ksplit = 1;
  if (scratch && !scratch->plan && tiles < ctx->num_sms && p.nslab >= 8) {
    ksplit = std::min(std::max(1, ctx->tune[TK_SPLITK_MAX]), std::max(1, (2 * ctx->num_sms) / tiles));
    ksplit = std::min(ksplit, p.nslab / 4);
    while (ksplit > 1 && (size_t)ksplit * M * N * sizeof(float) > scratch->cap) ksplit--;
  }
  p.per_split = ceil_div(p.nslab, ksplit);
  ksplit = ceil_div(p.nslab, p.per_split);
  p.ksplit = ksplit;
  p.tiles_m = ceil_div(M, BM);
  p.tiles_n = ceil_div(N, BN);
  p.partial = (ksplit > 1) ? reinterpret_cast<float*>(scratch->base) : nullptr;
  // C update through TMA stores (beta 0) or reduce-adds (beta 1) of 32-column chunks
  CUtensorMap mc;
  memset(&mc, 0, sizeof(mc));
  p.tma_epi = 0;
  if (!trans && ksplit == 1 && (beta == 0.f || beta == 1.f) && (reinterpret_cast<uintptr_t>(C) & 15) == 0 &&
      (ldc % 4) == 0 && make_map_c(&mc, C, M, N, ldc, L::EPI_CHUNK) == DDCSVD_OK)
    p.tma_epi = (beta == 0.f) ? 1 : 2;
  // persistent: one CTA per SM (the shared-memory footprint allows no more), items spread over them
  const int items = p.tiles_m * p.tiles_n * ksplit;
  const int grid = std::max(1, std::min(items, ctx->num_sms));
  tc_gemm_split_tf32_kernel<BN, NP><<<grid, THREADS, L::SMEM, ctx->stream>>>(ma, mb, mc, p);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  if (ksplit > 1) splitk_reduce(ctx, M, N, ksplit, p.partial, alpha, beta, C, ldc, trans);
  return DDCSVD_OK;
}

}  // namespace tc

bool tc_available(ddcsvd_context* ctx) {
  (void)ctx;
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return major == 10 && minor == 3 && tc::encode_fn() != nullptr;
}

size_t gemm_tc_scratch_bytes(GemmKind kind, int M, int N, int K) {
  (void)kind;
  (void)K;
  return std::min((size_t)16 * M * N, (size_t)2 * 256 * 128 * 128) * sizeof(float) + 4096;
}

static int tc_dispatch(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K, const float* A, long long lda,
                       int a_koff, const float* B, long long ldb, int b_koff, float* C, int ldc, float alpha,
                       float beta, Arena* scratch, bool trans) {
  if (kind != GEMM_TF32X3 && kind != GEMM_TF32X6) {
    set_last_error("split-BF16 tensor-core GEMM is not implemented");
    return DDCSVD_ERR_UNSUPPORTED;
  }
  if (M <= 0 || N <= 0) return DDCSVD_OK;
  if ((a_koff & 3) || (b_koff & 3)) return DDCSVD_ERR_ARG;
  const bool bn64 = (N <= 64) || ctx->tune[TK_TC_BN] == 64;
  const bool bn32 = (N <= 32);  // e.g. the W1 products of the 32-column QR panels
  if (kind == GEMM_TF32X6) {
    if (bn32)
      return tc::launch<32, 3>(ctx, M, N, K, A, lda, a_koff, B, ldb, b_koff, C, ldc, alpha, beta, scratch, trans);
    if (bn64)
      return tc::launch<64, 3>(ctx, M, N, K, A, lda, a_koff, B, ldb, b_koff, C, ldc, alpha, beta, scratch, trans);
    return tc::launch<128, 3>(ctx, M, N, K, A, lda, a_koff, B, ldb, b_koff, C, ldc, alpha, beta, scratch, trans);
  }
  if (bn32)
    return tc::launch<32, 2>(ctx, M, N, K, A, lda, a_koff, B, ldb, b_koff, C, ldc, alpha, beta, scratch, trans);
  if (bn64)
    return tc::launch<64, 2>(ctx, M, N, K, A, lda, a_koff, B, ldb, b_koff, C, ldc, alpha, beta, scratch, trans);
  return tc::launch<128, 2>(ctx, M, N, K, A, lda, a_koff, B, ldb, b_koff, C, ldc, alpha, beta, scratch, trans);
}

int gemm_tc_kmajor(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K, const float* A, long long lda,
                   int a_koff, const float* B, long long ldb, int b_koff, float* C, int ldc, float alpha,
                   float beta, Arena* scratch) {
  return tc_dispatch(ctx, kind, M, N, K, A, lda, a_koff, B, ldb, b_koff, C, ldc, alpha, beta, scratch, false);
}

int gemm_tc_kmajor_t(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K, const float* A, long long lda,
                     int a_koff, const float* B, long long ldb, int b_koff, float* Ct, int ldct, float alpha,
                     float beta, Arena* scratch) {
  return tc_dispatch(ctx, kind, M, N, K, A, lda, a_koff, B, ldb, b_koff, Ct, ldct, alpha, beta, scratch, true);
}

// Strided-operand entry used by gemm(): only the K-major layouts map onto the
// tensor-core kernel directly; callers with other layouts pack first.
int gemm_tc(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K1, Mat A1, Mat B1, int K2, Mat A2,
            Mat B2, float alpha, float beta, float* C, int ldc, Arena* scratch) {
  if (K2 > 0 && A2.p) {
    set_last_error("two-term tensor-core GEMM must be packed by the caller");
    return DDCSVD_ERR_ARG;
  }
  if (A1.cs != 1 || B1.rs != 1) {
    set_last_error("tensor-core GEMM needs K-major operands");
    return DDCSVD_ERR_ARG;
  }
  return gemm_tc_kmajor(ctx, kind, M, N, K1, A1.p, A1.rs, 0, B1.p, B1.cs, 0, C, ldc, alpha, beta, scratch);
}

}  // namespace ddcsvd

#ifdef DDCSVD_PHASE_TRACE
extern "C" int ddcsvd_gemm_trace_read(unsigned long long* out) {
  return (int)cudaMemcpyFromSymbol(out, ddcsvd::tc::g_gemm_trace, sizeof(ddcsvd::tc::g_gemm_trace));
}
#endif
