// sort.cuh - cell-key sort of the neighbour search: a stable LSD radix sort
// of 32-bit cell keys with 32-bit payloads, and the cell-start table.
//
// Replaces the reference's GridIndex construction (atomic count, prefix sum,
// atomic fill; source/tit/geom/search/grid_search.hpp:58-84) with a stable
// sort, so the order of particles inside a cell is a pure function of the
// previous order and the results are run-to-run deterministic.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tg {

constexpr int kRadixBits = 8;
constexpr int kRadixBins = 1 << kRadixBits;
constexpr int kSortThreads = 256;             // 8 warps
constexpr int kSortItems = 8;                 // per thread
constexpr int kSortTile = kSortThreads * kSortItems;

// Scratch needed by radix_sort for n keys (bytes): per-tile histograms.
size_t radix_sort_scratch_bytes(int64_t n);

// Sort (keys, vals) by the low key_bits of keys, stable.  keys_a/vals_a hold
// the input (identity_vals: the payload is 0..n-1 and vals_a is not read);
// the result lands in (keys_a, vals_a) or (keys_b, vals_b), as returned
// through *result_in_b.  Each pass issues three kernels; *launches counts
// them.  With n_dev, the count is *n_dev (read on the device, at most n):
// the launches are sized for n and the tiles past the count do nothing.
cudaError_t radix_sort(uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b,
                       uint32_t* vals_b, int64_t n, int key_bits,
                       bool identity_vals, void* scratch, bool* result_in_b,
                       cudaStream_t stream, int64_t* launches,
                       const uint32_t* n_dev = nullptr);

// Re-sort of keys whose previous sorted order is known: keys[i] is the new
// key of the particle at slot i of the previous order, prev[i] the key that
// slot held when that order was sorted.  The particles whose key changed
// (movers) are compacted and radix-sorted alone; the others keep their
// relative order, and both runs are merged by rank.  The result equals the
// stable sort of keys (ties in slot order), as radix_sort gives it: out_keys
// the sorted keys, out_perm the slot of each.  Four kernels and the movers'
// radix passes.  The scratch holds a completion counter that must be zero
// before the first near_sort (near_sort_reset; every near_sort leaves it
// zero).
size_t near_sort_scratch_bytes(int64_t n);
cudaError_t near_sort_reset(void* scratch, int64_t n, cudaStream_t stream);
cudaError_t near_sort(const uint32_t* keys, const uint32_t* prev, int64_t n,
                      int key_bits, uint32_t* out_keys, uint32_t* out_perm,
                      void* scratch, cudaStream_t stream, int64_t* launches);

// cell_start[c] = first sorted index whose key >= c, for c in
// [0, total_cells]; cell_start[total_cells] = n.  Every cell searches the
// sorted keys (used by the no-allocation density pass, whose scratch is
// static).  The scratch holds (total_cells + 256) / 256 + 2 words.  Two
// kernels.
cudaError_t build_cell_table(const uint32_t* sorted_keys, int64_t n,
                             uint32_t total_cells, uint32_t* cell_start,
                             void* scratch, cudaStream_t stream,
                             int64_t* launches);

// The same table in one pass over the sorted keys: each sorted index writes
// the starts of the cells between its key and the previous one, and long
// empty stretches are filled by whole blocks from a list.  Writes each entry
// once; the scratch holds that list (cell_fill_scratch_bytes).  A memset and
// two kernels.
size_t cell_fill_scratch_bytes(uint32_t total_keys);
cudaError_t build_cell_table_fill(const uint32_t* sorted_keys, int64_t n,
                                  uint32_t total_keys, uint32_t* cell_start,
                                  void* scratch, int sm_count, cudaStream_t stream,
                                  int64_t* launches);

}  // namespace tg
