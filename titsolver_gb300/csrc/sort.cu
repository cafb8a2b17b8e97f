// sort.cu - stable LSD radix sort of cell keys and the cell-start table.
//
// One pass per 8-bit digit, three kernels per pass:
//   upsweep   per-tile digit histograms (tile = 256 threads x 8 keys),
//             stored digit-major: hist[digit * ntiles + tile]
//   rowscan   one block per digit: exclusive scan of its row over tiles,
//             and the row total
//   downsweep each tile ranks its keys stably (warp __match_any_sync per
//             item, items in tile order) and scatters them to
//             digit_base + row_scan + warp offset + rank
// Keys of one warp are loaded warp-striped (item i of lane l sits at
// warp_base + 32 i + l), so processing items in order, lanes in order, keeps
// the input order within equal digits.  No kernel waits on another block.
#include "sort.cuh"

namespace tg {
namespace {

constexpr int kWarps = kSortThreads / 32;

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__global__ void __launch_bounds__(kSortThreads)
    k_radix_upsweep(const uint32_t* __restrict__ keys, int64_t n, int shift,
                    uint32_t* __restrict__ hist, int ntiles,
                    const uint32_t* __restrict__ n_dev) {
  __shared__ uint32_t s_hist[kRadixBins];
  if (n_dev != nullptr) {
    n = *n_dev;  // count known on the device only
    if (static_cast<int64_t>(blockIdx.x) * kSortTile >= n) return;
  }
  for (int i = threadIdx.x; i < kRadixBins; i += blockDim.x) s_hist[i] = 0;
  __syncthreads();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kSortTile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    const int64_t idx = base + warp * (32 * kSortItems) + it * 32 + lane;
    if (idx < n) {
      const uint32_t d = (keys[idx] >> shift) & (kRadixBins - 1);
      atomicAdd(&s_hist[d], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kRadixBins; i += blockDim.x) {
    hist[static_cast<int64_t>(i) * ntiles + blockIdx.x] = s_hist[i];
  }
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v,
                                                         uint32_t* s_warp,
                                                         uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nwarps ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nwarps) s_warp[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  const uint32_t warp_excl = warp > 0 ? s_warp[warp - 1] : 0u;
  *total = s_warp[nwarps - 1];
  __syncthreads();
  return warp_excl + x - v;
}

__global__ void __launch_bounds__(256)
    k_radix_rowscan(uint32_t* __restrict__ hist, int ntiles,
                    uint32_t* __restrict__ row_total,
                    const uint32_t* __restrict__ n_dev) {
  __shared__ uint32_t s_warp[32];
  uint32_t* row = hist + static_cast<int64_t>(blockIdx.x) * ntiles;
  // With a count known on the device only, the tiles past it hold no keys
  // (and their histograms were not written).
  const int used = n_dev != nullptr
                       ? static_cast<int>((static_cast<int64_t>(*n_dev) + kSortTile - 1) / kSortTile)
                       : ntiles;
  uint32_t carry = 0;
  for (int base = 0; base < used; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const uint32_t v = i < used ? row[i] : 0u;
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(v, s_warp, &tot);
    if (i < used) row[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) row_total[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads)
    k_radix_downsweep(const uint32_t* __restrict__ keys_in,
                      const uint32_t* __restrict__ vals_in,
                      uint32_t* __restrict__ keys_out,
                      uint32_t* __restrict__ vals_out, int64_t n, int shift,
                      const uint32_t* __restrict__ row_scan,
                      const uint32_t* __restrict__ row_total, int ntiles,
                      const uint32_t* __restrict__ n_dev) {
  __shared__ uint32_t s_base[kRadixBins];
  if (n_dev != nullptr) n = *n_dev;
  // Tiles past a count known on the device only have nothing to move.
  if (static_cast<int64_t>(blockIdx.x) * kSortTile >= n) return;
  __shared__ uint32_t s_cnt[kWarps][kRadixBins];
  __shared__ uint32_t s_warp[32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // Digit bases: exclusive scan of the row totals (256 digits, 256 threads).
  {
    const uint32_t v = row_total[threadIdx.x];
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(v, s_warp, &tot);
    s_base[threadIdx.x] =
        ex + row_scan[static_cast<int64_t>(threadIdx.x) * ntiles + blockIdx.x];
  }
  for (int w = 0; w < kWarps; ++w) s_cnt[w][threadIdx.x] = 0;
  __syncthreads();

  const int64_t base =
      static_cast<int64_t>(blockIdx.x) * kSortTile + warp * (32 * kSortItems);
  uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
  int digit[kSortItems];
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    const int64_t idx = base + it * 32 + lane;
    const bool valid = idx < n;
    key[it] = valid ? keys_in[idx] : 0u;
    val[it] = valid ? (vals_in ? vals_in[idx] : static_cast<uint32_t>(idx)) : 0u;
    digit[it] = valid ? static_cast<int>((key[it] >> shift) & (kRadixBins - 1))
                      : kRadixBins;
    const uint32_t peers = __match_any_sync(0xffffffffu, digit[it]);
    uint32_t before = 0;
    if (valid) before = s_cnt[warp][digit[it]];
    __syncwarp();
    rank[it] = before + __popc(peers & lt);
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) s_cnt[warp][digit[it]] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // Exclusive prefix of the per-warp counts, per digit.
  {
    uint32_t run = 0;
    for (int w = 0; w < kWarps; ++w) {
      const uint32_t c = s_cnt[w][threadIdx.x];
      s_cnt[w][threadIdx.x] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    if (digit[it] < kRadixBins) {
      const uint32_t pos =
          s_base[digit[it]] + s_cnt[warp][digit[it]] + rank[it];
      keys_out[pos] = key[it];
      vals_out[pos] = val[it];
    }
  }
}

// cell_start[c] = lower_bound(keys, c) for every cell, in two passes:
//   k_coarse_bounds  one warp per block of kTableCells cells finds
//                    lower_bound(keys, first cell of the block) with 32-way
//                    probes (about log32(n) dependent loads)
//   k_cell_table     one thread per cell; the keys between the block's two
//                    coarse bounds are staged in shared memory (when they
//                    fit) and each thread searches there.
// Long runs of empty cells cost the same as full ones.
constexpr int kTableCells = 256;
constexpr int kTableStage = 2048;

__device__ __forceinline__ int64_t lower_bound_global(
    const uint32_t* __restrict__ keys, int64_t lo, int64_t hi, int64_t c) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (static_cast<int64_t>(__ldg(keys + mid)) < c) {
      lo = mid + 1;
    } else {
      hi = mid;
    }
  }
  return lo;
}

__global__ void __launch_bounds__(256)
    k_coarse_bounds(const uint32_t* __restrict__ keys, int64_t n,
                    int64_t nblocks, uint32_t* __restrict__ bounds) {
  const int64_t b = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (b > nblocks) return;  // whole warps exit together
  const int64_t c = b * kTableCells;
  int64_t lo = 0, hi = n;  // answer in [lo, hi]
  while (hi - lo > 32) {
    const int64_t step = (hi - lo) / 33;
    const int64_t probe = lo + step * (lane + 1);
    const bool ge = static_cast<int64_t>(__ldg(keys + probe)) >= c;
    const uint32_t mask = __ballot_sync(0xffffffffu, ge);
    if (mask == 0) {
      lo = lo + step * 32 + 1;
    } else {
      const int first = __ffs(mask) - 1;
      const int64_t new_hi = lo + step * (first + 1);
      lo = first == 0 ? lo : lo + step * first + 1;
      hi = new_hi;
    }
  }
  // At most 32 candidates left: one probe per lane.
  const int64_t probe = lo + lane;
  const bool ge = probe >= hi || static_cast<int64_t>(__ldg(keys + probe)) >= c;
  const uint32_t mask = __ballot_sync(0xffffffffu, ge);
  if (lane == 0) {
    bounds[b] = static_cast<uint32_t>(mask != 0 ? lo + (__ffs(mask) - 1) : hi);
  }
}

__global__ void __launch_bounds__(kTableCells)
    k_cell_table(const uint32_t* __restrict__ keys, int64_t n,
                 uint32_t total_cells, const uint32_t* __restrict__ bounds,
                 uint32_t* __restrict__ cell_start) {
  __shared__ uint32_t s_keys[kTableStage];
  const int64_t lo = bounds[blockIdx.x];
  const int64_t hi = bounds[blockIdx.x + 1];
  const int64_t cnt = hi - lo;
  const int64_t c = static_cast<int64_t>(blockIdx.x) * kTableCells + threadIdx.x;
  if (cnt <= kTableStage) {
    for (int64_t t = threadIdx.x; t < cnt; t += blockDim.x) {
      s_keys[t] = keys[lo + t];
    }
    __syncthreads();
    if (c > static_cast<int64_t>(total_cells)) return;
    int a = 0, b = static_cast<int>(cnt);
    while (a < b) {
      const int mid = (a + b) >> 1;
      if (static_cast<int64_t>(s_keys[mid]) < c) {
        a = mid + 1;
      } else {
        b = mid;
      }
    }
    cell_start[c] = static_cast<uint32_t>(lo + a);
  } else {
    if (c > static_cast<int64_t>(total_cells)) return;
    cell_start[c] = static_cast<uint32_t>(lower_bound_global(keys, lo, hi, c));
  }
}

// cell_start from the sorted keys in one pass: sorted index j starts every
// cell c with key[j-1] < c <= key[j] (j = n: the cells past the last key and
// the sentinel).  Who writes a run of cells depends on its length: up to
// kThreadRun cells the thread of j (a cell boundary inside the fluid, where a
// fluid key is followed by its cell's empty wall key), up to kBlockRun the
// whole warp, one run after another with consecutive lanes on consecutive
// cells, and longer runs (empty stretches of the grid, up to all the cells
// above the fluid) go to a list in chunks of at most kFillChunk cells, which
// k_fill_runs writes with one block per chunk.
constexpr int kThreadRun = 4;
constexpr int kBlockRun = 1024;
constexpr int kFillChunk = 16384;

struct FillRun {
  uint32_t lo, hi, value;  // cells [lo, hi] start at sorted index value
};

__global__ void __launch_bounds__(256)
    k_fill_starts(const uint32_t* __restrict__ keys, int64_t n, uint32_t total_keys,
                  uint32_t* __restrict__ cell_start, FillRun* __restrict__ runs,
                  uint32_t* __restrict__ run_count) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  // Every lane reaches the vote below, the ones past n with an empty run.
  int64_t lo = 1, hi = 0;
  if (j <= n) {
    lo = j == 0 ? 0 : static_cast<int64_t>(__ldg(keys + j - 1)) + 1;
    hi = j == n ? static_cast<int64_t>(total_keys) : __ldg(keys + j);
  }
  const int64_t len = hi - lo + 1;
  if (len > 0 && len <= kThreadRun) {
    for (int64_t c = lo; c <= hi; ++c) cell_start[c] = static_cast<uint32_t>(j);
  } else if (len >= kBlockRun) {
    const uint32_t chunks = static_cast<uint32_t>((len + kFillChunk - 1) / kFillChunk);
    const uint32_t r = atomicAdd(run_count, chunks);
    for (uint32_t q = 0; q < chunks; ++q) {
      const int64_t a = lo + static_cast<int64_t>(q) * kFillChunk;
      const int64_t b = min(hi, a + kFillChunk - 1);
      runs[r + q] = FillRun{static_cast<uint32_t>(a), static_cast<uint32_t>(b),
                            static_cast<uint32_t>(j)};
    }
  }
  unsigned mid = __ballot_sync(0xffffffffu, len > kThreadRun && len < kBlockRun);
  while (mid != 0u) {
    const int src = __ffs(mid) - 1;
    mid &= mid - 1u;
    const uint32_t lo_s = __shfl_sync(0xffffffffu, static_cast<uint32_t>(lo), src);
    const uint32_t len_s = __shfl_sync(0xffffffffu, static_cast<uint32_t>(len), src);
    const uint32_t val_s = __shfl_sync(0xffffffffu, static_cast<uint32_t>(j), src);
    for (uint32_t k = lane; k < len_s; k += 32u) cell_start[lo_s + k] = val_s;
  }
}

__global__ void __launch_bounds__(256)
    k_fill_runs(uint32_t* __restrict__ cell_start, const FillRun* __restrict__ runs,
                const uint32_t* __restrict__ run_count) {
  const uint32_t nr = *run_count;
  for (uint32_t r = blockIdx.x; r < nr; r += gridDim.x) {
    const FillRun f = runs[r];
    for (uint32_t c = f.lo + threadIdx.x; c <= f.hi && c >= f.lo; c += blockDim.x) {
      cell_start[c] = f.value;
    }
  }
}

}  // namespace

size_t cell_fill_scratch_bytes(uint32_t total_keys) {
  // Runs of at least kBlockRun cells are disjoint, so at most
  // (total_keys + 1) / kBlockRun of them, each split into at most
  // len / kFillChunk + 1 chunks: at most 2 (total_keys + 1) / kBlockRun
  // chunks, plus the counter.
  return 256 + sizeof(FillRun) * (2 * (static_cast<size_t>(total_keys) + 1) / kBlockRun + 2);
}

cudaError_t build_cell_table_fill(const uint32_t* sorted_keys, int64_t n,
                                  uint32_t total_keys, uint32_t* cell_start,
                                  void* scratch, int sm_count, cudaStream_t stream,
                                  int64_t* launches) {
  auto* count = static_cast<uint32_t*>(scratch);
  auto* runs = reinterpret_cast<FillRun*>(static_cast<unsigned char*>(scratch) + 256);
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  k_fill_starts<<<static_cast<unsigned>((n + 1 + 255) / 256), 256, 0, stream>>>(
      sorted_keys, n, total_keys, cell_start, runs, count);
  k_fill_runs<<<static_cast<unsigned>(8 * (sm_count > 0 ? sm_count : 152)), 256, 0, stream>>>(
      cell_start, runs, count);
  *launches += 2;
  return cudaGetLastError();
}

size_t radix_sort_scratch_bytes(int64_t n) {
  const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
  return static_cast<size_t>(kRadixBins) * (ntiles + 1) * sizeof(uint32_t) +
         256;
}

cudaError_t radix_sort(uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b,
                       uint32_t* vals_b, int64_t n, int key_bits,
                       bool identity_vals, void* scratch, bool* result_in_b,
                       cudaStream_t stream, int64_t* launches,
                       const uint32_t* n_dev) {
  *result_in_b = false;
  if (n <= 0) return cudaSuccess;
  const int ntiles = static_cast<int>((n + kSortTile - 1) / kSortTile);
  uint32_t* hist = static_cast<uint32_t*>(scratch);
  uint32_t* row_total = hist + static_cast<int64_t>(kRadixBins) * ntiles;
  const int passes = key_bits <= 0 ? 1 : (key_bits + kRadixBits - 1) / kRadixBits;
  uint32_t* ki = keys_a;
  uint32_t* vi = vals_a;
  uint32_t* ko = keys_b;
  uint32_t* vo = vals_b;
  for (int p = 0; p < passes; ++p) {
    const int shift = p * kRadixBits;
    k_radix_upsweep<<<ntiles, kSortThreads, 0, stream>>>(ki, n, shift, hist,
                                                         ntiles, n_dev);
    k_radix_rowscan<<<kRadixBins, 256, 0, stream>>>(hist, ntiles, row_total, n_dev);
    k_radix_downsweep<<<ntiles, kSortThreads, 0, stream>>>(
        ki, (p == 0 && identity_vals) ? nullptr : vi, ko, vo, n, shift, hist,
        row_total, ntiles, n_dev);
    *launches += 3;
    uint32_t* tk = ki;
    ki = ko;
    ko = tk;
    uint32_t* tv = vi;
    vi = vo;
    vo = tv;
  }
  *result_in_b = (passes % 2) == 1;
  return cudaGetLastError();
}

cudaError_t build_cell_table(const uint32_t* sorted_keys, int64_t n,
                             uint32_t total_cells, uint32_t* cell_start,
                             void* scratch, cudaStream_t stream,
                             int64_t* launches) {
  // Cells 0..total_cells inclusive, in blocks of kTableCells.
  const int64_t nblocks = (static_cast<int64_t>(total_cells) + kTableCells) / kTableCells;
  uint32_t* bounds = static_cast<uint32_t*>(scratch);
  const int64_t warps = nblocks + 1;  // bounds[0..nblocks]
  k_coarse_bounds<<<static_cast<unsigned>((warps * 32 + 255) / 256), 256, 0, stream>>>(
      sorted_keys, n, nblocks, bounds);
  k_cell_table<<<static_cast<unsigned>(nblocks), kTableCells, 0, stream>>>(
      sorted_keys, n, total_cells, bounds, cell_start);
  *launches += 2;
  return cudaGetLastError();
}

}  // namespace tg
