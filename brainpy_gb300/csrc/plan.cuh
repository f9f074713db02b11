// plan.cuh -- the column-tiled CSR layout ("plan") used by the tiled event kernels.
//
// For a CSR matrix of shape m x n the output columns are cut into n_tiles tiles of
// tile_w columns.  Every row's column indices are regrouped by tile; the group of
// row r for tile t (a "segment") holds tile-local uint16 indices (col - t*tile_w) and
// is padded with 0xFFFF to a multiple of 4 entries, so that each segment starts on an
// 8-byte boundary and is read in 8-byte chunks.  Heterogeneous weights are permuted
// along (float32, zero padding, same positions).
//
// Memory of one plan (all inside one caller-provided device allocation):
//   row_start[m]        uint64  first entry of row r in idx[] (a multiple of 4)
//   tile_off[m][T+1]    uint32  segment t of row r is idx[row_start + tile_off[t] .. + tile_off[t+1])
//   idx[entries]        uint16
//   w[entries]          float32 (heterogeneous plans only)
// Row r owns entries [row_start[r], row_start[r] + 4*ceil(len_r/4) + 4*T + 4), a bound that
// needs no prefix sum: row_start[r] = align4(indptr[r]) + (4*T + 4) * r.
#pragma once

#include "common.cuh"

namespace bp {

constexpr int kPlanMaxTiles = 4000;  // plan build keeps 3 x n_tiles words in 48 KB of shared memory
constexpr int kPlanMaxTileW = 65535;  // local indices are uint16, 0xFFFF is the pad value
constexpr uint16_t kPadIndex = 0xFFFF;

// Byte offsets of the arrays inside the plan memory.
struct PlanLayout {
  size_t off_row_start, off_tile_off, off_idx, off_w, total;
  uint64_t entries;
};

inline PlanLayout plan_layout(int64_t m, int64_t nnz, int32_t n_tiles, bool heter) {
  PlanLayout L;
  uint64_t per_row = 4ull * (uint64_t)n_tiles + 4ull;
  L.entries = align_up((size_t)nnz, 4) + per_row * (uint64_t)m + 4;
  L.off_row_start = 0;
  L.off_tile_off = align_up(sizeof(uint64_t) * (size_t)m, 256);
  L.off_idx = L.off_tile_off + align_up(sizeof(uint32_t) * (size_t)m * (size_t)(n_tiles + 1), 256);
  L.off_w = L.off_idx + align_up(sizeof(uint16_t) * (size_t)L.entries, 256);
  L.total = L.off_w + (heter ? align_up(sizeof(float) * (size_t)L.entries, 256) : 0);
  return L;
}

struct PlanView {
  const uint64_t* row_start;
  const uint32_t* tile_off;
  const uint16_t* idx;
  const float* w;
  int64_t m, n;
  int32_t tile_w, n_tiles;
};

inline PlanView plan_view(const bp_csr_plan* p) {
  PlanLayout L = plan_layout(p->m, p->nnz, p->n_tiles, p->heter != 0);
  const char* base = static_cast<const char*>(p->mem);
  PlanView v;
  v.row_start = reinterpret_cast<const uint64_t*>(base + L.off_row_start);
  v.tile_off = reinterpret_cast<const uint32_t*>(base + L.off_tile_off);
  v.idx = reinterpret_cast<const uint16_t*>(base + L.off_idx);
  v.w = p->heter ? reinterpret_cast<const float*>(base + L.off_w) : nullptr;
  v.m = p->m;
  v.n = p->n;
  v.tile_w = p->tile_w;
  v.n_tiles = p->n_tiles;
  return v;
}

}  // namespace bp
