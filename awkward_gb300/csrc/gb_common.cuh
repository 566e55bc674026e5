// gb_common.cuh -- shared device/host infrastructure of libawkward_gb300.
//
//  * the error word: awkward's CUDA error protocol (src/awkward/_connect/cuda/
//    cuda_kernels/cuda_common.cu:31-33): a failing kernel does
//    atomicMin(err_code, invocation_index * 2^8 + message_index); the host
//    decodes it after synchronising (src/awkward/_connect/cuda/__init__.py:257-294).
//  * a stream-ordered scratch pool owned by the library (tile states, CTA
//    carries), never handed to the caller;
//  * warp / block scans and reductions over arbitrary (trivially copyable)
//    value types with an ordered, possibly non-commutative combine;
//  * a decoupled look-back over int64 tile aggregates with bounded spins.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define GB_ERROR_BITS 8
#define GB_NO_ERROR 0xffffffffffffffffULL
#define GB_EXPORT extern "C" __attribute__((visibility("default")))

// Library-internal failure codes.  They follow each kernel family's own
// message list (see awkward_gb300/_messages.py), so they never collide with
// awkward's message indices.
#define GB_MSG_TIMEOUT 32  // a bounded wait on the GPU gave up

namespace gb {

constexpr int kWarp = 32;

// ----------------------------------------------------------------- errors
__device__ __forceinline__ void raise_error(uint64_t* err, uint64_t inv, int code) {
  atomicMin(reinterpret_cast<unsigned long long*>(err),
            static_cast<unsigned long long>(inv * (1ull << GB_ERROR_BITS) + (uint64_t)code));
}

// ----------------------------------------------------------------- scratch
// Stream-ordered allocation from a per-device pool owned by the library.
cudaError_t scratch_alloc(void** ptr, size_t bytes, cudaStream_t stream);
cudaError_t scratch_free(void* ptr, cudaStream_t stream);
// SM count and the persistent-grid width of the current device (cached).
int device_sm_count();

// ----------------------------------------------------------------- shuffles
template <class V>
__device__ __forceinline__ V shfl_up(V v, int delta) {
  static_assert(sizeof(V) % 4 == 0, "shuffled types are multiples of 4 bytes");
  constexpr int W = sizeof(V) / 4;
  union U { V v; uint32_t w[W]; } u;
  u.v = v;
#pragma unroll
  for (int i = 0; i < W; i++) u.w[i] = __shfl_up_sync(0xffffffffu, u.w[i], delta);
  return u.v;
}
template <class V>
__device__ __forceinline__ V shfl_idx(V v, int src) {
  constexpr int W = sizeof(V) / 4;
  union U { V v; uint32_t w[W]; } u;
  u.v = v;
#pragma unroll
  for (int i = 0; i < W; i++) u.w[i] = __shfl_sync(0xffffffffu, u.w[i], src);
  return u.v;
}

// Inclusive warp scan in lane order (lane 0 earliest) with an ordered
// combine op(earlier, later) and its identity.
template <class V, class Op>
__device__ __forceinline__ V warp_inclusive_scan(V v, Op op, V identity) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    V o = shfl_up(v, d);
    if (lane >= d) v = op(o, v);
  }
  (void)identity;
  return v;
}

// Block-wide exclusive scan.  Returns the exclusive prefix of this thread
// (identity for thread 0) and the block total in *total.  `smem` must hold
// BLOCK/32 + 1 values.  Contains __syncthreads(); call from all threads.
template <int BLOCK, class V, class Op>
__device__ __forceinline__ V block_exclusive_scan(V v, Op op, V identity, V* smem, V* total) {
  constexpr int NW = BLOCK / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  V incl = warp_inclusive_scan(v, op, identity);
  if (lane == 31) smem[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    V w = lane < NW ? smem[lane] : identity;
    V wi = warp_inclusive_scan(w, op, identity);
    if (lane < NW) smem[lane] = wi;  // inclusive over warps
    if (lane == NW - 1) smem[NW] = wi;
  }
  __syncthreads();
  V warp_prefix = warp == 0 ? identity : smem[warp - 1];
  V excl = shfl_up(incl, 1);
  if (lane == 0) excl = identity;
  excl = op(warp_prefix, excl);
  *total = smem[NW];
  __syncthreads();
  return excl;
}

// ----------------------------------------------------------------- look-back
// Tile states of a single-pass scan of int64 tile aggregates.  Each 64-bit
// word packs (status << 62) | (value mod 2^62), status 0 = not yet
// published, 1 = aggregate of this tile only, 2 = inclusive prefix through
// this tile; values are read back sign-extended from 62 bits, so sums are
// exact while they stay in [-2^61, 2^61).  The array is zeroed (together
// with the ticket counter that precedes it) before the launch.
struct ScanTiles {
  unsigned long long* ticket;  // dynamic tile index counter
  unsigned long long* status;  // one word per tile
};

constexpr unsigned long long kLBValueMask = (1ull << 62) - 1;
constexpr uint32_t kSpinLimit = 1u << 22;  // x ~32-256 ns sleep: bounded at ~seconds

__device__ __forceinline__ void lb_publish(unsigned long long* w, unsigned long long status,
                                           unsigned long long value) {
  unsigned long long word = (status << 62) | (value & kLBValueMask);
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(w), "l"(word) : "memory");
}
__device__ __forceinline__ unsigned long long lb_load(const unsigned long long* w) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(w) : "memory");
  return v;
}

// Called by warp 0 of the block that owns `tile` (all 32 lanes).  Publishes
// `aggregate`, walks back over predecessors 32 at a time and returns the
// exclusive prefix of this tile (sum of all earlier aggregates).  A
// predecessor that does not publish within the spin limit is treated as 0
// and error `timeout_code` is raised, so the kernel always terminates.
__device__ __forceinline__ long long lookback_exclusive(const ScanTiles& st, long long tile,
                                                        long long aggregate, uint64_t inv,
                                                        uint64_t* err, int timeout_code,
                                                        uint32_t spin_limit = kSpinLimit) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) lb_publish(st.status, 2, (unsigned long long)aggregate);
    return 0;
  }
  if (lane == 0) lb_publish(st.status + tile, 1, (unsigned long long)aggregate);
  long long prefix = 0;
  long long base = tile - 1;
  bool timed_out = false;
  while (true) {
    long long p = base - lane;
    unsigned long long word = 2ull << 62;  // before tile 0: inclusive 0
    if (p >= 0) {
      uint32_t it = 0;
      uint32_t ns = 32;
      word = lb_load(st.status + p);
      while ((word >> 62) == 0) {
        if (++it > spin_limit) { timed_out = true; word = 2ull << 62; break; }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
        word = lb_load(st.status + p);
      }
    }
    unsigned status = (unsigned)(word >> 62);
    long long value = ((long long)(word << 2)) >> 2;
    unsigned incl_mask = __ballot_sync(0xffffffffu, status == 2);
    int stop = incl_mask ? __ffs(incl_mask) - 1 : 31;  // nearest inclusive predecessor
    long long contrib = lane <= stop ? value : 0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, d);
    prefix += contrib;
    if (incl_mask) break;
    base -= 32;
  }
  if (__any_sync(0xffffffffu, timed_out) && lane == 0) raise_error(err, inv, timeout_code);
  if (lane == 0) lb_publish(st.status + tile, 2, (unsigned long long)(prefix + aggregate));
  return prefix;
}

// Host helper: zeroed tile states for `ntiles` tiles from the scratch pool.
cudaError_t scan_tiles_alloc(ScanTiles* st, void** base, long long ntiles, cudaStream_t stream);

// ----------------------------------------------------------------- misc
template <class T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ bool ldg<bool>(const bool* p) {
  return __ldg(reinterpret_cast<const unsigned char*>(p)) != 0;
}

inline int ceil_div_int(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace gb
