// plan.cuh -- the column-tiled CSR layout ("plan") used by the tiled event kernels.
//
// For a CSR matrix of shape m x n the output columns are cut into n_tiles tiles of
// tile_w columns.  Every row's column indices are regrouped by tile; the group of
// row r for tile t (a "segment") holds tile-local uint16 indices (col - t*tile_w) and
// is padded to a multiple of 8 entries with pad indices in [tile_w, tile_w + 32): entry slot
// e of chunk c holds tile_w + 8 * (c & 3) + e.  Every kernel's `< tile_w` test skips them, a
// gather from a shared-memory tile with 32 zeros past it adds nothing, and unpredicated
// shared-memory adds land on 32 dummy words past the tile, spread over 32 banks so that the
// lanes of one add instruction rarely meet on one word.  So every segment is a whole
// number of 16-byte chunks starting on a 16-byte boundary (a valid bulk-copy source).
// Heterogeneous weights are permuted along (float32, zero padding, same positions:
// chunk c holds weights [8c, 8c + 8), 32 bytes).
//
// Memory of one plan (all inside one caller-provided device allocation):
//   seg_off[m][T+1]     uint32  absolute chunk index: segment t of row r is chunks
//                               [seg_off[r][t], seg_off[r][t+1]) of idx (8 entries each)
//   idx[entries]        uint16
//   w[entries]          float32 (heterogeneous plans only)
//   meta[4]             uint32  meta[0] != 0 when no row holds a column twice (checked for rows of
//                               up to kPlanDupCheckMax entries, longer rows count as not checked
//                               and clear it); meta[1] = the longest row's length; meta[2] = the
//                               fixed-point exponent k of a fixed-weight plan (weights stored as
//                               int32 w * 2^k), written by bp_csr_plan_fix_weights
// Row r's chunks start at entry align8(indptr[r]) + (8*T + 8) * r, a bound that needs no
// prefix sum (row r needs at most nnz_r + 7*T padded entries and the gap to row r + 1 is at
// least nnz_r + 8*T + 1).  Chunk indices are 32-bit: a plan holds fewer than 2^32 chunks.
#pragma once

#include "common.cuh"

namespace bp {

constexpr int kPlanMaxTiles = 4000;  // plan build keeps 3 x n_tiles words in 48 KB of shared memory
constexpr int kPlanMaxTileW = 65472;  // local indices and the pad values (below tile_w + 32) are uint16
constexpr int kPlanPadSpan = 32;       // pad values tile_w + 8 * (chunk & 3) + slot: 32 distinct
constexpr int kChunkEntries = 8;      // entries per 16-byte chunk
constexpr int kPlanDupCheckMax = 4096;  // rows up to this length are checked for repeated columns

// Byte offsets of the arrays inside the plan memory.
struct PlanLayout {
  size_t off_seg, off_idx, off_w, off_meta, total;
  uint64_t entries, chunks;
};

inline PlanLayout plan_layout(int64_t m, int64_t nnz, int32_t n_tiles, bool heter) {
  PlanLayout L;
  const uint64_t per_row = 8ull * (uint64_t)n_tiles + 8ull;
  L.entries = align_up((size_t)nnz, 8) + per_row * (uint64_t)m + 8;
  L.chunks = L.entries / 8;
  L.off_seg = 0;
  L.off_idx = align_up(sizeof(uint32_t) * (size_t)m * (size_t)(n_tiles + 1), 256);
  L.off_w = L.off_idx + align_up(sizeof(uint16_t) * (size_t)L.entries, 256);
  L.off_meta = L.off_w + (heter ? align_up(sizeof(float) * (size_t)L.entries, 256) : 0);
  L.total = L.off_meta + 256;
  return L;
}

struct PlanView {
  const uint32_t* seg_off;
  const uint16_t* idx;
  const float* w;
  const uint32_t* meta;
  int64_t m, n;
  int32_t tile_w, n_tiles;
};

inline PlanView plan_view(const bp_csr_plan* p) {
  PlanLayout L = plan_layout(p->m, p->nnz, p->n_tiles, p->heter != 0);
  const char* base = static_cast<const char*>(p->mem);
  PlanView v;
  v.seg_off = reinterpret_cast<const uint32_t*>(base + L.off_seg);
  v.idx = reinterpret_cast<const uint16_t*>(base + L.off_idx);
  v.w = p->heter ? reinterpret_cast<const float*>(base + L.off_w) : nullptr;
  v.meta = reinterpret_cast<const uint32_t*>(base + L.off_meta);
  v.m = p->m;
  v.n = p->n;
  v.tile_w = p->tile_w;
  v.n_tiles = p->n_tiles;
  return v;
}

}  // namespace bp
