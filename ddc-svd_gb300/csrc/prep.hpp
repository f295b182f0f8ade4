// prep.hpp -- layout of the bidiagonal stages shared by prep.cu, twisted.cu
// and the pipelines.
#pragma once

#include <vector>

#include "internal.hpp"

namespace ddcsvd {

// Per-slot / per-group description of the vector stage.  A group is one
// output matrix (the single SVD, or one problem of a batch); a block is an
// unreduced piece of a group's bidiagonal.  Vector k (slot k) lives in block
// [lo, hi) of group g; its scratch arrays use the compact block layout
// element i at base + (i - lo) * nb + (k - lo), nb = hi - lo.
struct VecLayout {
  const int* blo;
  const int* bhi;
  const int* grp;
  const long long* base;  // storage offset of the slot's block
  const int* g_lo;        // first slot of the group
  const int* g_n;         // slots in the group
  float* const* g_X;      // group outputs: X column r at g_X + r * g_ldx
  const int* g_ldx;
  float* const* g_Y;
  const int* g_ldy;
  const int4* tiles;  // finalize tiles: (block lo, nb, k0, i0)
  int ntiles;
};

struct GroupOut {
  float* X;
  int ldx;
  float* Y;
  int ldy;
};

struct PrepBounds {
  size_t blob_bytes;
  long long store;
  int N;
};

struct Prep {
  DcHost H;
  VecLayout L;
  const double* b1;
  const double* b2;
  const int* dints;
  long long store;
  size_t used;
  size_t o_b1 = 0, o_b2 = 0;  // blob offsets of the bidiagonal
  int N;
  bool single_block;
  bool laid_out = false;      // prep_layout ran for `starts`
  std::vector<int> starts;
};

PrepBounds prep_bounds(const std::vector<int>& group_sizes);

// a64 / b64: host copies of the groups' bidiagonals, concatenated (b64 has one
// entry per row; the last entry of a group is its coupling to an extra
// column, kept only when keep_last).  b64 is split in place.  hblob must hold
// prep_bounds().blob_bytes (pinned), dblob the same on the device.
int prep_build(ddcsvd_context* ctx, const std::vector<int>& group_sizes, const std::vector<GroupOut>& out,
               double* a64, double* b64, double eps, bool keep_last, char* hblob, char* dblob, Prep* P);

// Everything of the blob but the bidiagonal's values, for the given block
// starts (ascending, ending with N).  A caller that expects no split inside
// a group can run it with the group boundaries while stage 1 is still on the
// GPU; prep_build then reuses it when the splits agree (else lays out anew).
int prep_layout(ddcsvd_context* ctx, const std::vector<int>& group_sizes, const std::vector<GroupOut>& out,
                const std::vector<int>& starts, char* hblob, char* dblob, Prep* P);

}  // namespace ddcsvd
