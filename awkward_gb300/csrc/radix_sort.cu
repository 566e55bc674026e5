// radix_sort.cu -- stable LSD radix sort of (key, value) pairs, an int64
// exclusive scan and a lower-bound fill (see radix_sort.cuh).
//
// A pass sorts by one 8-bit digit in three launches:
//   upsweep    each tile of 2048 pairs counts its digits (warp-aggregated
//              shared-memory atomics) into counts[digit][tile];
//   scan       one exclusive scan over the digit-major counts gives every
//              (digit, tile) its first output position;
//   downsweep  each warp owns 256 consecutive pairs of its tile, 32 per step:
//              lanes holding the same digit find each other with
//              __match_any_sync, rank among themselves by lane order and add
//              to the warp's running count of that digit; the warps' counts
//              are then scanned in warp order.  The rank of a pair is thus its
//              order among equal digits in the input -- the pass is stable,
//              and so is the whole least-significant-digit-first sort.  The
//              tile is laid out in digit order in shared memory first, so the
//              global stores of each digit's run are contiguous.
#include "radix_sort.cuh"

namespace gb {
namespace {

constexpr int kRBlock = 256;
constexpr int kRWarps = kRBlock / 32;
constexpr int kRSteps = 8;                        // steps of 32 pairs per warp
constexpr int kRTile = kRBlock * kRSteps;         // 2048 pairs per tile
constexpr int kRWarpSpan = kRTile / kRWarps;      // 256 consecutive pairs per warp
constexpr int kRDigits = 256;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__global__ void __launch_bounds__(kRBlock)
    radix_upsweep(const unsigned long long* __restrict__ keys, long long n, int shift,
                  unsigned mask, long long* __restrict__ counts, long long ntiles) {
  __shared__ unsigned h[kRDigits];
  for (int b = threadIdx.x; b < kRDigits; b += kRBlock) h[b] = 0;
  __syncthreads();
  const long long tile = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long e0 = tile * kRTile + (long long)warp * kRWarpSpan;
#pragma unroll
  for (int j = 0; j < kRSteps; j++) {
    const long long e = e0 + j * 32 + lane;
    const bool valid = e < n;
    const unsigned d = valid ? (unsigned)(keys[e] >> shift) & mask : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&h[d], (unsigned)__popc(peers));
  }
  __syncthreads();
  for (int b = threadIdx.x; b <= (int)mask; b += kRBlock) counts[(long long)b * ntiles + tile] = h[b];
}

// Rank every pair of the tile among equal digits (warp-ordered counters, so
// input order is kept), place the tile in shared memory in digit order, then
// write each digit's run to its global position: consecutive threads store
// consecutive positions of the same digit run.
__global__ void __launch_bounds__(kRBlock)
    radix_downsweep(const unsigned long long* __restrict__ kin, const long long* __restrict__ vin,
                    unsigned long long* __restrict__ kout, long long* __restrict__ vout,
                    long long n, int shift, unsigned mask, const long long* __restrict__ starts,
                    long long ntiles) {
  __shared__ unsigned wcnt[kRWarps][kRDigits];
  __shared__ unsigned s_tstart[kRDigits];       // first tile slot of each digit
  __shared__ long long s_gbase[kRDigits];       // first global position of each digit (this tile)
  __shared__ unsigned long long s_key[kRTile];
  __shared__ unsigned short s_src[kRTile];      // tile position the slot's pair came from
  __shared__ unsigned s_scan[kRBlock / 32 + 1];
  const long long tile = blockIdx.x;
  const long long t0 = tile * kRTile;
  for (int i = threadIdx.x; i < kRWarps * kRDigits; i += kRBlock) (&wcnt[0][0])[i] = 0;
  for (int b = threadIdx.x; b <= (int)mask; b += kRBlock) s_gbase[b] = starts[(long long)b * ntiles + tile];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = warp * kRWarpSpan;
  unsigned long long key[kRSteps];
  unsigned rank[kRSteps];
  const unsigned lt = lanemask_lt();
#pragma unroll
  for (int j = 0; j < kRSteps; j++) {
    const long long e = t0 + w0 + j * 32 + lane;
    const bool valid = e < n;
    key[j] = valid ? kin[e] : 0ull;
    const unsigned d = valid ? (unsigned)(key[j] >> shift) & mask : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned before = 0;
    if (valid) before = wcnt[warp][d];
    rank[j] = before + __popc(peers & lt);
    __syncwarp();
    if (valid && (peers & lt) == 0) wcnt[warp][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: warps' counts -> exclusive warp offsets and the digit's tile total
  unsigned dtot = 0;
  for (int b = threadIdx.x; b < kRDigits; b += kRBlock) {
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < kRWarps; w++) {
      const unsigned c = b <= (int)mask ? wcnt[w][b] : 0u;
      if (b <= (int)mask) wcnt[w][b] = run;
      run += c;
    }
    dtot = run;  // kRBlock == kRDigits: one digit per thread
  }
  unsigned total;
  auto add = [](unsigned a, unsigned b) { return a + b; };
  const unsigned dstart = block_exclusive_scan<kRBlock>(dtot, add, 0u, s_scan, &total);
  s_tstart[threadIdx.x] = dstart;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kRSteps; j++) {
    const int te = w0 + j * 32 + lane;
    if (t0 + te < n) {
      const unsigned d = (unsigned)(key[j] >> shift) & mask;
      const unsigned slot = s_tstart[d] + wcnt[warp][d] + rank[j];
      s_key[slot] = key[j];
      s_src[slot] = (unsigned short)te;
    }
  }
  __syncthreads();
  const int cnt = (int)(n - t0 < kRTile ? n - t0 : kRTile);
  for (int i = threadIdx.x; i < cnt; i += kRBlock) {
    const unsigned long long k = s_key[i];
    const unsigned d = (unsigned)(k >> shift) & mask;
    const long long pos = s_gbase[d] + (i - (long long)s_tstart[d]);
    kout[pos] = k;
    vout[pos] = vin[t0 + s_src[i]];
  }
}

constexpr int kSBlock = 256;
constexpr int kSItems = 8;
constexpr int kSTile = kSBlock * kSItems;

__global__ void __launch_bounds__(kSBlock)
    scan_i64_kernel(const long long* in, long long* out, long long n, long long* total,
                    ScanTiles st, uint64_t inv, uint64_t* err) {
  __shared__ long long s_scan[kSBlock / 32 + 1];
  __shared__ long long s_tile;
  __shared__ long long s_prefix;
  if (threadIdx.x == 0) s_tile = (long long)atomicAdd(st.ticket, 1ull);
  __syncthreads();
  const long long tile = s_tile;
  const long long b0 = tile * kSTile + (long long)threadIdx.x * kSItems;
  long long v[kSItems];
  long long sum = 0;
#pragma unroll
  for (int i = 0; i < kSItems; i++) {
    v[i] = b0 + i < n ? in[b0 + i] : 0;
    sum += v[i];
  }
  long long tile_total;
  auto add = [](long long a, long long b) { return a + b; };
  long long excl = block_exclusive_scan<kSBlock>(sum, add, 0ll, s_scan, &tile_total);
  if (threadIdx.x < 32) {
    long long p = lookback_exclusive(st, tile, tile_total, inv, err, GB_MSG_TIMEOUT);
    if (threadIdx.x == 0) s_prefix = p;
  }
  __syncthreads();
  long long run = s_prefix + excl;
#pragma unroll
  for (int i = 0; i < kSItems; i++) {
    if (b0 + i < n) out[b0 + i] = run;
    run += v[i];
  }
  if (total != nullptr && b0 < n && b0 + kSItems >= n) *total = run;
}

__device__ __forceinline__ long long lower_bound_dev(const unsigned long long* keys, long long lo,
                                                     long long hi, unsigned long long x) {
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (keys[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

constexpr int kLBSpan = 1024;  // bounds filled by one CTA

__global__ void __launch_bounds__(256)
    lower_bound_kernel(const unsigned long long* __restrict__ keys, long long n,
                       long long* __restrict__ out, long long count) {
  __shared__ long long s_lo, s_hi;
  const long long j0 = (long long)blockIdx.x * kLBSpan;
  const long long j1 = j0 + kLBSpan < count ? j0 + kLBSpan : count;
  if (threadIdx.x == 0) s_lo = lower_bound_dev(keys, 0, n, (unsigned long long)j0);
  if (threadIdx.x == 32) s_hi = lower_bound_dev(keys, 0, n, (unsigned long long)j1);
  __syncthreads();
  const long long lo = s_lo, hi = s_hi;
  for (long long j = j0 + threadIdx.x; j < j1; j += blockDim.x)
    out[j] = lower_bound_dev(keys, lo, hi, (unsigned long long)j);
}

}  // namespace

cudaError_t exclusive_scan_i64(const long long* in, long long* out, long long n, long long* total,
                               uint64_t inv, uint64_t* err, cudaStream_t s) {
  if (n <= 0) {
    if (total != nullptr) return cudaMemsetAsync(total, 0, sizeof(long long), s);
    return cudaSuccess;
  }
  const long long ntiles = (n + kSTile - 1) / kSTile;
  ScanTiles st;
  void* base = nullptr;
  cudaError_t e = scan_tiles_alloc(&st, &base, ntiles, s);
  if (e != cudaSuccess) return e;
  scan_i64_kernel<<<(unsigned)ntiles, kSBlock, 0, s>>>(in, out, n, total, st, inv, err);
  e = cudaGetLastError();
  cudaError_t f = scratch_free(base, s);
  return e != cudaSuccess ? e : f;
}

cudaError_t fill_lower_bounds(const unsigned long long* sorted_keys, long long n, long long* out,
                              long long count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  lower_bound_kernel<<<(unsigned)((count + kLBSpan - 1) / kLBSpan), 256, 0, s>>>(sorted_keys, n,
                                                                                out, count);
  return cudaGetLastError();
}

cudaError_t radix_sort_pairs(const unsigned long long* keys_in, const long long* vals_in,
                             unsigned long long* keys_out, long long* vals_out, long long n,
                             int bits, uint64_t inv, uint64_t* err, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (bits <= 0) {
    // one distinct key: already sorted
    cudaError_t e = cudaMemcpyAsync(keys_out, keys_in, sizeof(long long) * (size_t)n,
                                    cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(vals_out, vals_in, sizeof(long long) * (size_t)n,
                          cudaMemcpyDeviceToDevice, s);
    return e;
  }
  const int passes = (bits + 7) / 8;
  const long long ntiles = (n + kRTile - 1) / kRTile;
  // ping-pong buffers arranged so that the last pass writes keys_out / vals_out
  void* scratch = nullptr;
  const size_t counts_words = (size_t)kRDigits * (size_t)ntiles;
  const size_t alt_words = passes > 1 ? (size_t)n : 0;
  cudaError_t e = scratch_alloc(&scratch, sizeof(long long) * (counts_words + 2 * alt_words), s);
  if (e != cudaSuccess) return e;
  long long* counts = static_cast<long long*>(scratch);
  unsigned long long* kalt = reinterpret_cast<unsigned long long*>(counts + counts_words);
  long long* valt = reinterpret_cast<long long*>(kalt + alt_words);
  const unsigned long long* ksrc = keys_in;
  const long long* vsrc = vals_in;
  for (int p = 0; p < passes && e == cudaSuccess; p++) {
    const int shift = 8 * p;
    const int nb = bits - shift < 8 ? bits - shift : 8;
    const unsigned mask = (1u << nb) - 1u;
    // the pass writing keys_out must be the last; the ones before alternate so
    // that it never reads and writes the same buffer
    const bool to_out = ((passes - 1 - p) % 2) == 0;
    unsigned long long* kdst = to_out ? keys_out : kalt;
    long long* vdst = to_out ? vals_out : valt;
    const long long nd = (long long)mask + 1;
    radix_upsweep<<<(unsigned)ntiles, kRBlock, 0, s>>>(ksrc, n, shift, mask, counts, ntiles);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = exclusive_scan_i64(counts, counts, nd * ntiles, nullptr, inv, err, s);
    if (e == cudaSuccess) {
      radix_downsweep<<<(unsigned)ntiles, kRBlock, 0, s>>>(ksrc, vsrc, kdst, vdst, n, shift, mask,
                                                           counts, ntiles);
      e = cudaGetLastError();
    }
    ksrc = kdst;
    vsrc = vdst;
  }
  cudaError_t f = scratch_free(scratch, s);
  return e != cudaSuccess ? e : f;
}

}  // namespace gb
