// Photon radius count that allocates nothing.
//
// Some callers of this library cannot let it call cudaMalloc: cudaMalloc and
// cudaFree synchronize the whole device, which stalls a render loop running
// on other streams, and applications that hand out all device memory from
// their own pool at start-up (engines with a fixed memory budget) cannot let
// a library allocate on its own.  fr_radius_count_noalloc serves them: the
// caller passes device inputs and the device output, and every intermediate
// buffer of the query (the photon grid) lives in fixed file-scope device
// arrays below, sized for kNoAllocMaxPhotons photons.  Every GPU that loads
// the library holds these arrays (about 10.5 MB) until the process exits.
//
// All calls share the arrays: each call clears the bucket counts before it
// builds the grid, and calls that overlap on the GPU (on different streams or
// threads) race on the arrays and return wrong counts.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/friendsrender.h"
#include "fr_grid.cuh"
#include "fr_kernels.h"
#include "fr_layout.h"

namespace fr {
namespace {

constexpr int kNoAllocMaxPhotons = FR_NOALLOC_MAX_PHOTONS;
constexpr uint32_t kNoAllocTable = 1u << 19;  // buckets (a power of two)
constexpr int kNoAllocScanWords = 1024;       // scan block sums for kNoAllocTable + 1 entries
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float4 g_na_sorted[kNoAllocMaxPhotons];
static __device__ __align__(256) uint32_t g_na_key[kNoAllocMaxPhotons];
static __device__ __align__(256) uint32_t g_na_rank[kNoAllocMaxPhotons];
static __device__ __align__(256) uint32_t g_na_count[kNoAllocTable + 1];
static __device__ __align__(256) uint32_t g_na_start[kNoAllocTable + 1];
static __device__ __align__(256) uint32_t g_na_scan[kNoAllocScanWords];
static __device__ __align__(256) GridInfo g_na_grid;

__global__ void k_na_setup(float cell) {
  g_na_grid.cell = cell;
  g_na_grid.inv_cell = 1.0f / cell;
  g_na_grid.origin[0] = g_na_grid.origin[1] = g_na_grid.origin[2] = 0.0f;
  g_na_grid.r_sum = 0.0f;
  g_na_grid.r_count = 0;
}

// Bucket and rank of every photon (xyz triples).
__global__ void k_na_count(const float* __restrict__ xyz, int np) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float inv = g_na_grid.inv_cell;
  const float* p = xyz + 3 * (size_t)i;
  const uint32_t h = cell_hash(cell_of(p[0], 0.0f, inv), cell_of(p[1], 0.0f, inv), cell_of(p[2], 0.0f, inv),
                               kNoAllocTable - 1u);
  g_na_key[i] = h;
  g_na_rank[i] = atomicAdd(g_na_count + h, 1u);
}

__global__ void k_na_scatter(const float* __restrict__ xyz, int np) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float* p = xyz + 3 * (size_t)i;
  g_na_sorted[g_na_start[g_na_key[i]] + g_na_rank[i]] = make_float4(p[0], p[1], p[2], __uint_as_float((uint32_t)i));
}

// Device addresses of the arrays above, looked up once per device: in host
// code the array names are host-side stand-ins, not device addresses.
struct Scratch {
  bool ready = false;
  float4* sorted = nullptr;
  uint32_t *count = nullptr, *start = nullptr, *scan = nullptr;
  GridInfo* grid = nullptr;
};
Scratch g_scratch[kMaxDevices];
std::mutex g_scratch_mu;

thread_local char g_na_msg[256];

int na_fail(int code, const char* what, cudaError_t e) {
  std::snprintf(g_na_msg, sizeof(g_na_msg), "fr_radius_count_noalloc: %s: %s", what, cudaGetErrorString(e));
  return code;
}

// The scratch of the current device, which must be the stream's device: the
// arrays' addresses differ between devices.
int scratch_for_stream(cudaStream_t stream, Scratch** out) {
  int dev = 0, stream_dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(FR_ERR_CUDA, "cudaGetDevice", e);
  if ((e = cudaStreamGetDevice(stream, &stream_dev)) != cudaSuccess)
    return na_fail(FR_ERR_CUDA, "cudaStreamGetDevice", e);
  if (stream_dev != dev) {
    std::snprintf(g_na_msg, sizeof(g_na_msg),
                  "fr_radius_count_noalloc: the stream belongs to device %d but device %d is current", stream_dev,
                  dev);
    return FR_ERR_INVALID;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    std::snprintf(g_na_msg, sizeof(g_na_msg), "fr_radius_count_noalloc: device %d beyond the %d supported",
                  dev, kMaxDevices);
    return FR_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  Scratch& s = g_scratch[dev];
  if (!s.ready) {
    if ((e = cudaGetSymbolAddress((void**)&s.sorted, g_na_sorted)) != cudaSuccess ||
        (e = cudaGetSymbolAddress((void**)&s.count, g_na_count)) != cudaSuccess ||
        (e = cudaGetSymbolAddress((void**)&s.start, g_na_start)) != cudaSuccess ||
        (e = cudaGetSymbolAddress((void**)&s.scan, g_na_scan)) != cudaSuccess ||
        (e = cudaGetSymbolAddress((void**)&s.grid, g_na_grid)) != cudaSuccess)
      return na_fail(FR_ERR_CUDA, "cudaGetSymbolAddress", e);
    s.ready = true;
  }
  *out = &s;
  return FR_OK;
}

}  // namespace

int radius_count_noalloc(const float* hp_dev, int32_t nh, const float* photons_dev, int32_t np, float cell,
                         int32_t* counts_dev, cudaStream_t stream, const char** msg) {
  g_na_msg[0] = 0;
  *msg = g_na_msg;
  if (nh < 0 || np < 0 || !(cell > 0.0f) || !(cell <= 3.0e38f) || (nh && (!hp_dev || !counts_dev)) ||
      (np && !photons_dev)) {
    std::snprintf(g_na_msg, sizeof(g_na_msg), "fr_radius_count_noalloc: bad arguments");
    return FR_ERR_INVALID;
  }
  if (reinterpret_cast<uintptr_t>(hp_dev) % 16 != 0) {  // read as float4
    std::snprintf(g_na_msg, sizeof(g_na_msg), "fr_radius_count_noalloc: hp_dev is not 16-byte aligned");
    return FR_ERR_INVALID;
  }
  if (np > kNoAllocMaxPhotons) {
    std::snprintf(g_na_msg, sizeof(g_na_msg),
                  "fr_radius_count_noalloc: %d photons exceed the fixed scratch of %d photons", np,
                  kNoAllocMaxPhotons);
    return FR_ERR_INVALID;
  }
  if (nh == 0) return FR_OK;
  cudaError_t e;
  if (np == 0) {
    if ((e = cudaMemsetAsync(counts_dev, 0, sizeof(int32_t) * (size_t)nh, stream)) != cudaSuccess)
      return na_fail(FR_ERR_CUDA, "cudaMemsetAsync", e);
    return FR_OK;
  }
  Scratch* s = nullptr;
  int rc = scratch_for_stream(stream, &s);
  if (rc) return rc;
  ScanTemp st{};
  if (scan_temp_words(kNoAllocTable + 1, st) > (uint32_t)kNoAllocScanWords) {
    std::snprintf(g_na_msg, sizeof(g_na_msg), "fr_radius_count_noalloc: scan scratch too small");
    return FR_ERR_INVALID;
  }
  uint32_t* sw = s->scan;
  for (int l = 0; l < st.levels; ++l) {
    st.level[l] = sw;
    sw += st.level_n[l] + 1;
  }
  // The arrays keep the previous call's contents: clear the bucket counts.
  if ((e = cudaMemsetAsync(s->count, 0, sizeof(uint32_t) * (kNoAllocTable + 1), stream)) != cudaSuccess)
    return na_fail(FR_ERR_CUDA, "cudaMemsetAsync", e);
  k_na_setup<<<1, 1, 0, stream>>>(cell);
  const unsigned nb = (unsigned)((np + 255) / 256);
  k_na_count<<<nb, 256, 0, stream>>>(photons_dev, np);
  launch_scan(s->count, s->start, kNoAllocTable + 1, st, stream);
  k_na_scatter<<<nb, 256, 0, stream>>>(photons_dev, np);
  PhotonGrid g{};
  g.pos = s->sorted;
  g.cell_start = s->start;
  g.table = kNoAllocTable;
  launch_radius_count(reinterpret_cast<const float4*>(hp_dev), nh, g, s->grid, counts_dev, nullptr, 0, nullptr,
                      nullptr, stream);
  if ((e = cudaGetLastError()) != cudaSuccess) return na_fail(FR_ERR_CUDA, "kernel launch", e);
  return FR_OK;
}

}  // namespace fr
