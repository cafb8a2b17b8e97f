// sort_near.cu - re-sort of cell keys between stages.
//
// Between two stages a particle moves a small fraction of a cell, so most
// keep their key.  With keys[i] the new key of the particle at slot i of the
// previous order and prev[i] the key that slot held when that order was
// sorted (prev is sorted), the particles with keys[i] == prev[i] (stayers)
// are already in order.  The others (movers) are compacted, in slot order,
// and radix-sorted alone (stable, so by (key, slot)); then every element's
// place in the stable order of all keys (ties in slot order) is
//   stayer s:  (stayers before s) + (movers m with (key_m, m) < (key_s, s))
//   mover m:   (its rank among the movers) + (stayers s with (key_s, s) <
//              (key_m, m))
// which is exactly where radix_sort of the whole array puts it.
//
// Kernels: mover flags per 32 slots with their exclusive scan (one kernel:
// each block scans its words and the last block to finish scans the block
// totals); the compaction; the movers' radix sort (their count is known on
// the device only); the stayers' scatter, each block searching the sorted
// movers once for its slot range and then in shared memory; the movers'
// scatter, each searching prev for its key's slot range.
#include "sort.cuh"

namespace tg {
namespace {

constexpr int kNsBlock = 256;        // threads of the per-slot kernels
constexpr int kScanBlock = 1024;     // words per block of the flag-count scan
constexpr int kMoverWindow = 2048;   // sorted movers a stayer block stages

__device__ __forceinline__ uint32_t lanemask_lt_ns() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Block-wide exclusive scan of one value per thread (blockDim.x a multiple
// of 32); the block total in *total.
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t* s_warp,
                                                    uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
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
    if (lane < nwarps) s_warp[lane] = w;
  }
  __syncthreads();
  const uint32_t before = warp > 0 ? s_warp[warp - 1] : 0u;
  *total = s_warp[nwarps - 1];
  __syncthreads();
  return before + x - v;
}

// Movers of each 32-slot word (mask) and the exclusive scan of their counts:
// block b takes words [b kScanBlock, (b + 1) kScanBlock), each warp 32 words
// read slot-coalesced (one ballot per word), and stores the scan within the
// block (prefix) and its total (bsum).  The block that finishes last (a
// counter, no waiting) turns bsum into the exclusive scan of the block
// totals, writes the movers' count to *total and resets the counter.  The
// movers before word w are prefix[w] + bsum[w / kScanBlock].
__global__ void __launch_bounds__(kScanBlock)
    k_ns_flags_scan(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ prev,
                    int64_t n, int64_t nwords, int64_t nblocks, uint32_t* __restrict__ mask,
                    uint32_t* __restrict__ prefix, uint32_t* bsum, uint32_t* __restrict__ total,
                    uint32_t* done) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w0 = static_cast<int64_t>(blockIdx.x) * kScanBlock + warp * 32;
  uint32_t my_mask = 0;
#pragma unroll 4
  for (int q = 0; q < 32; ++q) {
    const int64_t i = (w0 + q) * 32 + lane;
    const bool mover = i < n && __ldg(keys + i) != __ldg(prev + i);
    const uint32_t m = __ballot_sync(0xffffffffu, mover);
    if (lane == q) my_mask = m;
  }
  const int64_t w = w0 + lane;
  uint32_t tot;
  const uint32_t ex = block_scan_excl(static_cast<uint32_t>(__popc(my_mask)), s_warp, &tot);
  if (w < nwords) {
    mask[w] = my_mask;
    prefix[w] = ex;
  }
  if (threadIdx.x == 0) {
    bsum[blockIdx.x] = tot;
    __threadfence();
    s_last = atomicAdd(done, 1u) == gridDim.x - 1 ? 1u : 0u;
  }
  __syncthreads();
  if (s_last == 0u) return;
  __threadfence();
  uint32_t carry = 0;
  for (int64_t b0 = 0; b0 < nblocks; b0 += blockDim.x) {
    const int64_t b = b0 + threadIdx.x;
    const uint32_t v = b < nblocks ? __ldcg(bsum + b) : 0u;
    uint32_t t;
    const uint32_t e = block_scan_excl(v, s_warp, &t);
    if (b < nblocks) bsum[b] = carry + e;
    carry += t;
  }
  if (threadIdx.x == 0) {
    *total = carry;
    *done = 0u;
  }
}

// Movers before word w.
__device__ __forceinline__ uint32_t word_prefix(const uint32_t* __restrict__ prefix,
                                                const uint32_t* __restrict__ bsum, int64_t w) {
  return __ldg(prefix + w) + __ldg(bsum + (w / kScanBlock));
}

// Movers before slot x (x in [0, n]).
__device__ __forceinline__ uint32_t movers_before(const uint32_t* __restrict__ mask,
                                                  const uint32_t* __restrict__ prefix,
                                                  const uint32_t* __restrict__ bsum,
                                                  int64_t nwords, const uint32_t* total,
                                                  int64_t x) {
  const int64_t w = x >> 5;
  if (w >= nwords) return *total;
  const uint32_t below = (1u << (x & 31)) - 1u;
  return word_prefix(prefix, bsum, w) + static_cast<uint32_t>(__popc(__ldg(mask + w) & below));
}

// Movers in slot order: their keys and slots.
__global__ void __launch_bounds__(kNsBlock)
    k_ns_compact(const uint32_t* __restrict__ keys, int64_t n,
                 const uint32_t* __restrict__ mask, const uint32_t* __restrict__ prefix,
                 const uint32_t* __restrict__ bsum, uint32_t* __restrict__ mkey,
                 uint32_t* __restrict__ mslot) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t w = i >> 5;
  const uint32_t m = __ldg(mask + w);
  if (!((m >> (i & 31)) & 1u)) return;
  const uint32_t s =
      word_prefix(prefix, bsum, w) + static_cast<uint32_t>(__popc(m & lanemask_lt_ns()));
  mkey[s] = keys[i];
  mslot[s] = static_cast<uint32_t>(i);
}

// (k1, s1) < (k2, s2), lexicographic.
__device__ __forceinline__ bool pair_less(uint32_t k1, uint32_t s1, uint32_t k2, uint32_t s2) {
  return k1 < k2 || (k1 == k2 && s1 < s2);
}

// Sorted movers before (k, s): lower bound in [lo, hi).
__device__ __forceinline__ uint32_t movers_less(const uint32_t* __restrict__ mkey,
                                                const uint32_t* __restrict__ mslot,
                                                uint32_t lo, uint32_t hi, uint32_t k,
                                                uint32_t s) {
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (pair_less(__ldg(mkey + mid), __ldg(mslot + mid), k, s)) {
      lo = mid + 1;
    } else {
      hi = mid;
    }
  }
  return lo;
}

// Stayers: each block takes kNsBlock consecutive slots; its stayers' pairs
// lie between (prev[first], first) and (prev[last], last + 1), so one search
// of the sorted movers per end bounds the movers that can precede any of
// them, and the threads search that window in shared memory.
__global__ void __launch_bounds__(kNsBlock)
    k_ns_stayers(const uint32_t* __restrict__ prev, int64_t n,
                 const uint32_t* __restrict__ mask, const uint32_t* __restrict__ prefix,
                 const uint32_t* __restrict__ bsum, const uint32_t* __restrict__ total,
                 const uint32_t* __restrict__ mkey, const uint32_t* __restrict__ mslot,
                 uint32_t* __restrict__ out_keys, uint32_t* __restrict__ out_perm) {
  __shared__ uint32_t s_key[kMoverWindow], s_slot[kMoverWindow];
  __shared__ uint32_t s_lo, s_hi;
  const int64_t i0 = static_cast<int64_t>(blockIdx.x) * blockDim.x;
  const int64_t i1 = min(i0 + static_cast<int64_t>(blockDim.x), n);  // exclusive
  const uint32_t nm = *total;
  if (threadIdx.x == 0) {
    s_lo = movers_less(mkey, mslot, 0, nm, prev[i0], static_cast<uint32_t>(i0));
  } else if (threadIdx.x == 32) {
    s_hi = movers_less(mkey, mslot, 0, nm, prev[i1 - 1], static_cast<uint32_t>(i1));
  }
  __syncthreads();
  const uint32_t lo = s_lo, hi = s_hi;
  const bool staged = hi - lo <= static_cast<uint32_t>(kMoverWindow);
  if (staged) {
    for (uint32_t t = threadIdx.x; t < hi - lo; t += blockDim.x) {
      s_key[t] = __ldg(mkey + lo + t);
      s_slot[t] = __ldg(mslot + lo + t);
    }
  }
  __syncthreads();
  const int64_t i = i0 + threadIdx.x;
  if (i >= i1) return;
  const int64_t w = i >> 5;
  const uint32_t m = __ldg(mask + w);
  if ((m >> (i & 31)) & 1u) return;  // a mover
  const uint32_t k = prev[i];
  const uint32_t s = static_cast<uint32_t>(i);
  uint32_t before;
  if (staged) {
    uint32_t a = 0, b = hi - lo;
    while (a < b) {
      const uint32_t mid = (a + b) >> 1;
      if (pair_less(s_key[mid], s_slot[mid], k, s)) {
        a = mid + 1;
      } else {
        b = mid;
      }
    }
    before = lo + a;
  } else {
    before = movers_less(mkey, mslot, lo, hi, k, s);
  }
  const uint32_t stayers_before =
      s - (word_prefix(prefix, bsum, w) + static_cast<uint32_t>(__popc(m & lanemask_lt_ns())));
  const uint32_t pos = stayers_before + before;
  out_keys[pos] = k;
  out_perm[pos] = s;
}

// Movers: rank r among the sorted movers plus the stayers before (k, slot):
// those with keys below k (slots [0, lb) of prev, less the movers there) and
// those with key k at slots below the mover's (slots [lb, min(ub, slot))).
__global__ void __launch_bounds__(kNsBlock)
    k_ns_movers(const uint32_t* __restrict__ prev, int64_t n,
                const uint32_t* __restrict__ mask, const uint32_t* __restrict__ prefix,
                const uint32_t* __restrict__ bsum, int64_t nwords,
                const uint32_t* __restrict__ total,
                const uint32_t* __restrict__ mkey, const uint32_t* __restrict__ mslot,
                uint32_t* __restrict__ out_keys, uint32_t* __restrict__ out_perm) {
  const uint32_t nm = *total;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < nm;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const uint32_t k = mkey[r], slot = mslot[r];
    int64_t lo = 0, hi = n;
    while (lo < hi) {  // first slot with prev >= k
      const int64_t mid = (lo + hi) >> 1;
      if (__ldg(prev + mid) < k) {
        lo = mid + 1;
      } else {
        hi = mid;
      }
    }
    const int64_t lb = lo;
    hi = n;
    while (lo < hi) {  // first slot with prev > k
      const int64_t mid = (lo + hi) >> 1;
      if (__ldg(prev + mid) <= k) {
        lo = mid + 1;
      } else {
        hi = mid;
      }
    }
    const int64_t ub = lo;
    const int64_t cut = min(ub, static_cast<int64_t>(slot));
    const uint32_t mb_lb = movers_before(mask, prefix, bsum, nwords, total, lb);
    uint32_t stayers = static_cast<uint32_t>(lb) - mb_lb;
    if (cut > lb) {
      stayers += static_cast<uint32_t>(cut - lb) -
                 (movers_before(mask, prefix, bsum, nwords, total, cut) - mb_lb);
    }
    const uint32_t pos = static_cast<uint32_t>(r) + stayers;
    out_keys[pos] = k;
    out_perm[pos] = slot;
  }
}

struct NearLayout {
  int64_t nwords, nblocks;
  size_t off_mask, off_prefix, off_bsum, off_total, off_done, off_mk0, off_ms0, off_mk1,
      off_ms1, off_radix, bytes;
};

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t{255}; }

NearLayout near_layout(int64_t n) {
  NearLayout L{};
  L.nwords = (n + 31) / 32;
  L.nblocks = (L.nwords + kScanBlock - 1) / kScanBlock;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += align256(bytes);
    return at;
  };
  const size_t nn = static_cast<size_t>(n > 0 ? n : 1);
  L.off_mask = take(sizeof(uint32_t) * L.nwords);
  L.off_prefix = take(sizeof(uint32_t) * (L.nwords + 1));
  L.off_bsum = take(sizeof(uint32_t) * (L.nblocks + 1));
  L.off_total = take(sizeof(uint32_t));
  L.off_done = take(sizeof(uint32_t));
  L.off_mk0 = take(sizeof(uint32_t) * nn);
  L.off_ms0 = take(sizeof(uint32_t) * nn);
  L.off_mk1 = take(sizeof(uint32_t) * nn);
  L.off_ms1 = take(sizeof(uint32_t) * nn);
  L.off_radix = take(radix_sort_scratch_bytes(n));
  L.bytes = o;
  return L;
}

}  // namespace

size_t near_sort_scratch_bytes(int64_t n) { return near_layout(n).bytes; }

cudaError_t near_sort_reset(void* scratch, int64_t n, cudaStream_t stream) {
  const NearLayout L = near_layout(n);
  return cudaMemsetAsync(static_cast<unsigned char*>(scratch) + L.off_done, 0,
                         sizeof(uint32_t), stream);
}

cudaError_t near_sort(const uint32_t* keys, const uint32_t* prev, int64_t n,
                      int key_bits, uint32_t* out_keys, uint32_t* out_perm,
                      void* scratch, cudaStream_t stream, int64_t* launches) {
  if (n <= 0) return cudaSuccess;
  const NearLayout L = near_layout(n);
  auto* base = static_cast<unsigned char*>(scratch);
  auto* mask = reinterpret_cast<uint32_t*>(base + L.off_mask);
  auto* prefix = reinterpret_cast<uint32_t*>(base + L.off_prefix);
  auto* bsum = reinterpret_cast<uint32_t*>(base + L.off_bsum);
  auto* total = reinterpret_cast<uint32_t*>(base + L.off_total);
  auto* done = reinterpret_cast<uint32_t*>(base + L.off_done);
  auto* mk0 = reinterpret_cast<uint32_t*>(base + L.off_mk0);
  auto* ms0 = reinterpret_cast<uint32_t*>(base + L.off_ms0);
  auto* mk1 = reinterpret_cast<uint32_t*>(base + L.off_mk1);
  auto* ms1 = reinterpret_cast<uint32_t*>(base + L.off_ms1);
  const unsigned gslots = static_cast<unsigned>((n + kNsBlock - 1) / kNsBlock);
  k_ns_flags_scan<<<static_cast<unsigned>(L.nblocks), kScanBlock, 0, stream>>>(
      keys, prev, n, L.nwords, L.nblocks, mask, prefix, bsum, total, done);
  k_ns_compact<<<gslots, kNsBlock, 0, stream>>>(keys, n, mask, prefix, bsum, mk0, ms0);
  *launches += 2;
  bool in_b = false;
  cudaError_t e = radix_sort(mk0, ms0, mk1, ms1, n, key_bits, false, base + L.off_radix,
                             &in_b, stream, launches, total);
  if (e != cudaSuccess) return e;
  const uint32_t* mkey = in_b ? mk1 : mk0;
  const uint32_t* mslot = in_b ? ms1 : ms0;
  k_ns_stayers<<<gslots, kNsBlock, 0, stream>>>(prev, n, mask, prefix, bsum, total, mkey,
                                                 mslot, out_keys, out_perm);
  k_ns_movers<<<1216, kNsBlock, 0, stream>>>(prev, n, mask, prefix, bsum, L.nwords, total,
                                             mkey, mslot, out_keys, out_perm);
  *launches += 2;
  return cudaGetLastError();
}

}  // namespace tg
