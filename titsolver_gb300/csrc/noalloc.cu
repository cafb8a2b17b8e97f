// noalloc.cu - summation density of a point cloud that allocates nothing.
//
// For callers that cannot call cudaMalloc: code running where the device
// allocator is off limits (a host framework that owns every byte of device
// memory and forbids allocation inside its step callbacks, or a real-time loop
// that must never block in the allocator).  All scratch lives in one
// file-scope __device__ array of a fixed size (below); every GPU that loads
// this library holds it until the process exits.
//
// The array's name is only a host-side stand-in in host code; its device
// address comes from cudaGetSymbolAddress, taken once per device (with that
// device current) on the first call made on that device and kept for the
// life of the process (a device reset after that call is not supported).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "fluid.cuh"
#include "sort.cuh"

namespace tg {
namespace {

constexpr int64_t kMaxPoints = TG_NOALLOC_MAX_POINTS;
constexpr uint32_t kMaxCells = 1u << 17;  // keys: 2 per cell
constexpr int kMaxCellBits = 18;
constexpr int kMaxDevices = 64;

// Scratch layout (byte offsets into g_noalloc_scratch), each 256-aligned.
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t{255}; }
constexpr size_t kU32 = sizeof(uint32_t) * kMaxPoints;
constexpr size_t kOffKeysA = 0;
constexpr size_t kOffKeysB = kOffKeysA + align256(kU32);
constexpr size_t kOffValsA = kOffKeysB + align256(kU32);
constexpr size_t kOffValsB = kOffValsA + align256(kU32);
constexpr size_t kOffIds = kOffValsB + align256(kU32);
constexpr size_t kHistBytes =
    sizeof(uint32_t) * kRadixBins * ((kMaxPoints + kSortTile - 1) / kSortTile + 1) + 256;
constexpr size_t kOffHist = kOffIds + align256(kU32);
constexpr size_t kOffCells = kOffHist + align256(kHistBytes);
constexpr size_t kOffRecs = kOffCells + align256(sizeof(uint32_t) * (2 * kMaxCells + 1));
constexpr size_t kOffBounds = kOffRecs + align256(sizeof(Pos64_3) * kMaxPoints);
constexpr size_t kBoundsBytes = sizeof(uint32_t) * ((2 * kMaxCells + 256) / 256 + 2);
constexpr size_t kOffTank = kOffBounds + align256(kBoundsBytes);
constexpr size_t kOffIdBase = kOffTank + align256(sizeof(TankDev));
constexpr size_t kScratchBytes = kOffIdBase + 256;
static_assert(kBoundsBytes >= 4 * ((2 * kMaxCells + 256) / 256 + 2), "coarse bounds");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on the
// first call per device).
cudaError_t scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

// Bounding box and cell grid of the cloud, computed on the device: cells of
// at least the support radius (so neighbours lie within one cell), enlarged
// when needed so the grid has at most kMaxCells cells.
template<int D>
__global__ void __launch_bounds__(256)
    k_na_grid(const double* __restrict__ r, int64_t n, double h, double m,
              double unit_radius, double weight, TankDev* T,
              uint32_t* id_base) {
  __shared__ double s_lo[256][3], s_hi[256][3];
  double lo[3] = {INFINITY, INFINITY, INFINITY};
  double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const double x = r[i * D + k];
      lo[k] = fmin(lo[k], x);
      hi[k] = fmax(hi[k], x);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    s_lo[threadIdx.x][k] = lo[k];
    s_hi[threadIdx.x][k] = hi[k];
  }
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        s_lo[threadIdx.x][k] = fmin(s_lo[threadIdx.x][k], s_lo[threadIdx.x + s][k]);
        s_hi[threadIdx.x][k] = fmax(s_hi[threadIdx.x][k], s_hi[threadIdx.x + s][k]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double R = unit_radius * h;
  double cs = R * (1.0 + 1.0 / 65536.0);
  double ext[3];
  for (int k = 0; k < 3; ++k) {
    ext[k] = k < D ? (s_hi[0][k] - s_lo[0][k]) : 0.0;
    if (!(ext[k] >= 0.0) || !isfinite(ext[k])) ext[k] = 0.0;
  }
  // Grow the cells (doubling, bounded) until the grid fits; if it never
  // does (non-finite or astronomically spread input), use a single cell,
  // which is still exact (every point is a candidate of every other).
  bool fits = false;
  double nc[3] = {1.0, 1.0, 1.0};
  for (int it = 0; it < 2100 && !fits && isfinite(cs); ++it) {
    double cells = 1.0;
    for (int k = 0; k < D; ++k) {
      nc[k] = ceil((ext[k] + 2.0 * (R + cs)) / cs) + 1.0;
      cells *= nc[k];
    }
    fits = cells <= static_cast<double>(kMaxCells);
    if (!fits) cs *= 2.0;
  }
  TankDev t{};
  for (int k = 0; k < 3; ++k) {
    const bool use = fits && k < D;
    t.lo[k] = use ? s_lo[0][k] - (R + cs) : 0.0;
    t.nc[k] = use ? static_cast<int32_t>(nc[k]) : 1;
  }
  if (!fits) cs = 1.0;
  t.cs = cs;
  t.inv_cs = 1.0 / cs;
  t.cell_off = 0;
  t.h = h;
  t.hinv = 1.0 / h;
  t.radius2 = R * R;
  double hd = 1.0;
  for (int k = 0; k < D; ++k) hd *= t.hinv;
  t.w = weight * hd;
  t.wg = t.w * t.hinv;
  t.m = m;
  *T = t;
  *id_base = 0;
}

template<int D>
__global__ void __launch_bounds__(256)
    k_na_keys(const double* __restrict__ r, int64_t n, const TankDev* T,
              uint32_t* __restrict__ keys) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p[3] = {r[i * D], r[i * D + 1], D == 3 ? r[i * D + 2] : 0.0};
  int c[3] = {0, 0, 0};
  bool outside = false;
  cell_of<D>(*T, p, c, outside);
  keys[i] = key_of(flat_cell<D>(*T, c), false);
}

template<int D>
__global__ void __launch_bounds__(256)
    k_na_records(const double* __restrict__ r, const uint32_t* __restrict__ perm,
                 int64_t n, void* __restrict__ recs, uint32_t* __restrict__ ids) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint32_t s = perm[j];
  if constexpr (D == 2) {
    static_cast<Pos64_2*>(recs)[j] = Pos64_2{r[int64_t(s) * 2], r[int64_t(s) * 2 + 1]};
  } else {
    static_cast<Pos64_3*>(recs)[j] =
        Pos64_3{r[int64_t(s) * 3], r[int64_t(s) * 3 + 1], r[int64_t(s) * 3 + 2], 0.0};
  }
  ids[j] = s;
}

template<int D, int K>
cudaError_t run(unsigned char* base, int64_t n, const double* r, double h,
                double m, double* rho, int32_t* counts, uint64_t* hashes,
                cudaStream_t s) {
  auto* keys_a = reinterpret_cast<uint32_t*>(base + kOffKeysA);
  auto* keys_b = reinterpret_cast<uint32_t*>(base + kOffKeysB);
  auto* vals_a = reinterpret_cast<uint32_t*>(base + kOffValsA);
  auto* vals_b = reinterpret_cast<uint32_t*>(base + kOffValsB);
  auto* ids = reinterpret_cast<uint32_t*>(base + kOffIds);
  auto* cells = reinterpret_cast<uint32_t*>(base + kOffCells);
  auto* recs = base + kOffRecs;
  auto* T = reinterpret_cast<TankDev*>(base + kOffTank);
  auto* id_base = reinterpret_cast<uint32_t*>(base + kOffIdBase);
  const double pi = 3.14159265358979323846;
  const double area = 2.0 * std::sqrt(std::pow(pi, D)) / std::tgamma(D / 2.0);
  const double weight = 1.0 / (kernel_zero_moment(K, D) * area);
  const unsigned g = static_cast<unsigned>((n + 255) / 256);
  k_na_grid<D><<<1, 256, 0, s>>>(r, n, h, m, kernel_unit_radius(K), weight, T, id_base);
  k_na_keys<D><<<g, 256, 0, s>>>(r, n, T, keys_a);
  bool in_b = false;
  int64_t launches = 0;
  cudaError_t e = radix_sort(keys_a, vals_a, keys_b, vals_b, n, kMaxCellBits, true,
                             base + kOffHist, &in_b, s, &launches);
  if (e != cudaSuccess) return e;
  const uint32_t* sorted = in_b ? keys_b : keys_a;
  const uint32_t* perm = in_b ? vals_b : vals_a;
  e = build_cell_table(sorted, n, 2 * kMaxCells, cells, base + kOffBounds, s, &launches);
  if (e != cudaSuccess) return e;
  k_na_records<D><<<g, 256, 0, s>>>(r, perm, n, recs, ids);
  // One tank whose first cell (and first id) is 0: id_base doubles as the
  // tank cell-offset table.
  CloudArgs<D> a{recs, ids, sorted, cells, T, id_base, 1, n, 1, rho, counts, hashes,
                 id_base};
  k_sumdens<D, K, false><<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

template<int D>
cudaError_t dispatch(int kernel, unsigned char* base, int64_t n, const double* r,
                     double h, double m, double* rho, int32_t* counts,
                     uint64_t* hashes, cudaStream_t s) {
  switch (kernel) {
    case TG_KERNEL_CUBIC_SPLINE:
      return run<D, TG_KERNEL_CUBIC_SPLINE>(base, n, r, h, m, rho, counts, hashes, s);
    case TG_KERNEL_QUARTIC_SPLINE:
      return run<D, TG_KERNEL_QUARTIC_SPLINE>(base, n, r, h, m, rho, counts, hashes, s);
    case TG_KERNEL_QUINTIC_SPLINE:
      return run<D, TG_KERNEL_QUINTIC_SPLINE>(base, n, r, h, m, rho, counts, hashes, s);
    case TG_KERNEL_WENDLAND_C2:
      return run<D, TG_KERNEL_WENDLAND_C2>(base, n, r, h, m, rho, counts, hashes, s);
    case TG_KERNEL_WENDLAND_C4:
      return run<D, TG_KERNEL_WENDLAND_C4>(base, n, r, h, m, rho, counts, hashes, s);
    default:
      return run<D, TG_KERNEL_WENDLAND_C6>(base, n, r, h, m, rho, counts, hashes, s);
  }
}

}  // namespace
}  // namespace tg

extern "C" int tg_summation_density_noalloc(int32_t dim, int32_t kernel, int64_t n,
                                            const double* r, double h, double m,
                                            double* rho, int32_t* counts,
                                            uint64_t* hashes, void* stream) {
  if ((dim != 2 && dim != 3) || kernel < 0 || kernel > 5 || n < 0) {
    return TG_ERR_INVALID_ARGUMENT;
  }
  if (n > TG_NOALLOC_MAX_POINTS) return TG_ERR_CAPACITY;
  if (!(h > 0.0) || !std::isfinite(h) || !(m > 0.0) || !std::isfinite(m)) {
    return TG_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return TG_OK;
  if (r == nullptr || (rho == nullptr && counts == nullptr && hashes == nullptr)) {
    return TG_ERR_INVALID_ARGUMENT;
  }
  unsigned char* base = nullptr;
  if (tg::scratch_address(&base) != cudaSuccess) {
    cudaGetLastError();
    return TG_ERR_CUDA;
  }
  auto s = static_cast<cudaStream_t>(stream);
  const cudaError_t e =
      dim == 2 ? tg::dispatch<2>(kernel, base, n, r, h, m, rho, counts, hashes, s)
               : tg::dispatch<3>(kernel, base, n, r, h, m, rho, counts, hashes, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return TG_ERR_CUDA;
  }
  return TG_OK;
}
