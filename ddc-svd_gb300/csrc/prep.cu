// prep.cu -- host-side preparation of the bidiagonal stages (2-4).
//
// After stage 1 the bidiagonal (a few KB) is read back once.  On the host it
// is split into unreduced blocks at negligible superdiagonal entries
// (per output matrix, "group"), the D&C forest (one tree per block) and the
// vector-stage layout (compact per-block scratch, 32 x 32 finalize tiles,
// per-group output pointers) are built, and everything goes back to the
// device in one copy.  The same code serves one SVD (one group) and a batch
// (one group per problem).
#include <string.h>

#include <vector>

#include "internal.hpp"
#include "prep.hpp"

namespace ddcsvd {

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

PrepBounds prep_bounds(const std::vector<int>& gn) {
  PrepBounds B;
  long long N = 0, store = 0, tiles = 0;
  for (int n : gn) {
    N += n;
    store += (long long)n * n;
    const long long t = (n + 31) / 32;
    tiles += t * t + n;
  }
  const size_t G = gn.size();
  size_t o = 0;
  o = align256(o + sizeof(double) * N);       // b1
  o = align256(o + sizeof(double) * N);       // b2
  o = align256(o + sizeof(long long) * N);    // base
  o = align256(o + sizeof(int) * 3 * N);      // blo, bhi, grp
  o = align256(o + sizeof(int) * 4 * G);      // g_lo, g_n, g_ldx, g_ldy
  o = align256(o + sizeof(void*) * 2 * G);    // g_X, g_Y
  o = align256(o + sizeof(int4) * tiles);     // tiles
  o = align256(o + sizeof(int) * dc_max_ints((int)N));
  B.blob_bytes = o + 256;
  B.store = store;
  B.N = (int)N;
  return B;
}

// Blob sections that depend on the block starts (not on the bidiagonal's
// values): forest, per-row block bounds, compact block bases, tiles, group
// tables and node tables; b1 / b2 keep their fixed offsets at the front.
int prep_layout(ddcsvd_context* ctx, const std::vector<int>& gn, const std::vector<GroupOut>& out,
                const std::vector<int>& starts, char* hblob, char* dblob, Prep* P) {
  const int G = (int)gn.size();
  int N = 0;
  for (int n : gn) N += n;
  std::vector<int> g_lo(G), blo(N), bhi(N), grp(N);
  {
    int off = 0;
    for (int g = 0; g < G; g++) {
      g_lo[g] = off;
      for (int i = 0; i < gn[g]; i++) grp[off + i] = g;
      off += gn[g];
    }
  }
  // ---- D&C forest over all blocks
  dc_build_host(N, starts, P->H, ctx->tune[TK_DC_TERMS]);
  // ---- compact block storage, per-row block bounds and finalize tiles
  std::vector<long long> base(N);
  std::vector<int4> tiles;
  long long store = 0;
  for (size_t s = 0; s + 1 < starts.size(); s++) {
    const int lo = starts[s], hi = starts[s + 1], nb = hi - lo;
    for (int i = lo; i < hi; i++) {
      base[i] = store;
      blo[i] = lo;
      bhi[i] = hi;
    }
    store += (long long)nb * nb;
    for (int k0 = 0; k0 < nb; k0 += 32)
      for (int i0 = 0; i0 < nb; i0 += 32) tiles.push_back(make_int4(lo, nb, k0, i0));
  }
  // ---- blob (same layout on host and device); b1, b2 first
  size_t o = 0;
  auto put = [&](const void* src, size_t bytes) {
    const size_t at = o;
    if (bytes) memcpy(hblob + at, src, bytes);
    o = align256(o + bytes);
    return at;
  };
  const size_t o_b1 = o;
  o = align256(o + sizeof(double) * N);
  const size_t o_b2 = o;
  o = align256(o + sizeof(double) * N);
  const size_t o_base = put(base.data(), sizeof(long long) * N);
  const size_t o_blo = o;
  memcpy(hblob + o, blo.data(), sizeof(int) * N);
  memcpy(hblob + o + sizeof(int) * N, bhi.data(), sizeof(int) * N);
  memcpy(hblob + o + 2 * sizeof(int) * N, grp.data(), sizeof(int) * N);
  o = align256(o + sizeof(int) * 3 * N);
  std::vector<int> gi(4 * G);
  std::vector<float*> gp(2 * G);
  for (int g = 0; g < G; g++) {
    gi[g] = g_lo[g];
    gi[G + g] = gn[g];
    gi[2 * G + g] = out[g].ldx;
    gi[3 * G + g] = out[g].ldy;
    gp[g] = out[g].X;
    gp[G + g] = out[g].Y;
  }
  const size_t o_gi = put(gi.data(), sizeof(int) * 4 * G);
  const size_t o_gp = put(gp.data(), sizeof(float*) * 2 * G);
  const size_t o_tiles = put(tiles.data(), sizeof(int4) * tiles.size());
  const size_t o_ints = put(P->H.ints.data(), sizeof(int) * P->H.ints.size());
  P->used = o;
  P->o_b1 = o_b1;
  P->o_b2 = o_b2;
  P->starts = starts;
  P->N = N;
  P->store = store;
  P->b1 = reinterpret_cast<const double*>(dblob + o_b1);
  P->b2 = reinterpret_cast<const double*>(dblob + o_b2);
  P->dints = reinterpret_cast<const int*>(dblob + o_ints);
  VecLayout& L = P->L;
  L.base = reinterpret_cast<const long long*>(dblob + o_base);
  L.blo = reinterpret_cast<const int*>(dblob + o_blo);
  L.bhi = L.blo + N;
  L.grp = L.blo + 2 * N;
  L.g_lo = reinterpret_cast<const int*>(dblob + o_gi);
  L.g_n = L.g_lo + G;
  L.g_ldx = L.g_lo + 2 * G;
  L.g_ldy = L.g_lo + 3 * G;
  L.g_X = reinterpret_cast<float* const*>(dblob + o_gp);
  L.g_Y = L.g_X + G;
  L.tiles = reinterpret_cast<const int4*>(dblob + o_tiles);
  L.ntiles = (int)tiles.size();
  P->single_block = (starts.size() == 2);
  P->laid_out = true;
  return DDCSVD_OK;
}

int prep_build(ddcsvd_context* ctx, const std::vector<int>& gn, const std::vector<GroupOut>& out, double* a64,
               double* b64, double eps, bool keep_last, char* hblob, char* dblob, Prep* P) {
  const int G = (int)gn.size();
  int N = 0;
  for (int n : gn) N += n;
  // ---- split each group, collect block starts (global)
  std::vector<int> starts;
  std::vector<int> blo(N), bhi(N);
  int off = 0;
  std::vector<int> st;
  for (int g = 0; g < G; g++) {
    const int n = gn[g];
    st.clear();
    const double keep = (keep_last && n > 0) ? b64[off + n - 1] : 0.0;
    split_bidiagonal(n, a64 + off, b64 + off, eps, st, blo.data() + off, bhi.data() + off);
    if (keep_last && n > 0) b64[off + n - 1] = keep;
    for (size_t i = 0; i + 1 < st.size(); i++) starts.push_back(off + st[i]);
    off += n;
  }
  starts.push_back(N);
  // ---- layout (reused when prep_layout already ran for the same blocks)
  if (!(P->laid_out && P->starts == starts)) DDC_TRY(prep_layout(ctx, gn, out, starts, hblob, dblob, P));
  memcpy(hblob + P->o_b1, a64, sizeof(double) * N);
  memcpy(hblob + P->o_b2, b64, sizeof(double) * N);
  DDC_CUDA_TRY(cudaMemcpyAsync(dblob, hblob, P->used, cudaMemcpyHostToDevice, ctx->stream));
  return DDCSVD_OK;
}

}  // namespace ddcsvd
