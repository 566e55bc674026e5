// gb_common.cu -- host side of the shared infrastructure: the library's
// stream-ordered scratch pool and cached device properties.
#include <mutex>

#include "gb_common.cuh"

namespace gb {

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
cudaMemPool_t g_pools[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};

cudaError_t pool_for_current_device(cudaMemPool_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    // Keep freed blocks cached in the pool instead of returning them to the
    // driver at every synchronisation: scratch is small and reused per call.
    uint64_t threshold = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    if (e != cudaSuccess) return e;
    g_pools[dev] = pool;
  }
  *out = g_pools[dev];
  return cudaSuccess;
}
}  // namespace

cudaError_t scratch_alloc(void** ptr, size_t bytes, cudaStream_t stream) {
  cudaMemPool_t pool;
  cudaError_t e = pool_for_current_device(&pool);
  if (e != cudaSuccess) return e;
  if (bytes == 0) bytes = 256;
  return cudaMallocFromPoolAsync(ptr, bytes, pool, stream);
}

cudaError_t scratch_free(void* ptr, cudaStream_t stream) {
  if (!ptr) return cudaSuccess;
  return cudaFreeAsync(ptr, stream);
}

int device_sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_sm_count[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
    g_sm_count[dev] = n;
  }
  return g_sm_count[dev];
}

cudaError_t scan_tiles_alloc(ScanTiles* st, void** base, long long ntiles, cudaStream_t stream) {
  size_t bytes = (size_t)(ntiles + 1) * sizeof(unsigned long long);
  cudaError_t e = scratch_alloc(base, bytes, stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(*base, 0, bytes, stream);
  if (e != cudaSuccess) return e;
  st->ticket = reinterpret_cast<unsigned long long*>(*base);
  st->status = st->ticket + 1;
  return cudaSuccess;
}

}  // namespace gb

// Library identification for the host-side loader.
GB_EXPORT const char* awkward_gb300_version() { return "awkward_gb300 0.1 (sm_103a)"; }
