// broadcast.cu -- a ListArray broadcast to given offsets.
//
//   awkward_ListArray_broadcast_tooffsets  awkward_ListArray_broadcast_tooffsets.cpp:8-33
//
// List i must have exactly fromoffsets[i+1] - fromoffsets[i] elements; its
// elements j = starts[i] .. stops[i]-1 go to tocarry at the list's output
// position fromoffsets[i] - fromoffsets[0] (the CPU's running counter).  A CTA
// owns a tile of kTileLists lists: it validates them (error codes are the
// message order of awkward's CUDA kernel: 0 stops[i] > len(content), 1
// non-monotonic offsets, 2 count mismatch) and stages the tile's offsets, then
// each warp writes a contiguous share of the tile's output, a lane finding its
// list by a forward walk over the staged offsets.  No scan is needed: the
// output positions are the given offsets.
#include "list_tile.cuh"

using namespace gb;

namespace {

template <class C>
__global__ void __launch_bounds__(kTileBlock)
    broadcast_tooffsets_kernel(int64_t* __restrict__ tocarry, const int64_t* __restrict__ offsets,
                               long long nlists, const C* __restrict__ starts,
                               const C* __restrict__ stops, long long lencontent, uint64_t inv,
                               uint64_t* err) {
  __shared__ long long loc[kTileLists + 1];
  __shared__ long long s_start[kTileLists];
  __shared__ int s_bad;
  const long long l0 = (long long)blockIdx.x * kTileLists;
  const long long rem = nlists - l0;
  const int count = (int)(rem < kTileLists ? rem : kTileLists);
  const long long base = __ldg(offsets + l0);
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int i = threadIdx.x; i <= kTileLists; i += kTileBlock) {
    const int k = i < count ? i : count;
    loc[i] = __ldg(offsets + l0 + k) - base;
  }
  for (int r = threadIdx.x; r < count; r += kTileBlock) {
    const long long l = l0 + r;
    const long long start = (long long)starts[l], stop = (long long)stops[l];
    const long long cnt = __ldg(offsets + l + 1) - __ldg(offsets + l);
    int code = -1;
    if (start != stop && stop > lencontent) code = 0;
    else if (cnt < 0) code = 1;
    else if (stop - start != cnt) code = 2;
    if (code >= 0) {
      raise_error(err, inv, code);
      s_bad = 1;  // the tile's output positions are not usable
    }
    s_start[r] = start;
  }
  __syncthreads();
  if (s_bad) return;
  const long long out0 = base - __ldg(offsets);
  // never past the final total, whatever earlier (invalid) lists did to the offsets
  const long long limit = __ldg(offsets + nlists) - __ldg(offsets);
  constexpr int kWarps = kTileBlock / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long total = loc[count];
  const long long qa = total * warp / kWarps, qb = total * (warp + 1) / kWarps;
  if (qa >= qb) return;
  int lo = 0, hi = count;  // last r with loc[r] <= qa
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (loc[mid] <= qa) lo = mid;
    else hi = mid;
  }
  int r = lo;
  for (long long g = qa; g < qb; g += 32) {
    while (loc[r + 1] <= g) r++;
    const long long q = g + lane;
    if (q >= qb) continue;
    int rl = r;
    while (loc[rl + 1] <= q) rl++;
    const long long at = out0 + q;
    if (at >= 0 && at < limit) tocarry[at] = s_start[rl] + (q - loc[rl]);
  }
}

}  // namespace

#define GB_BROADCAST_TOOFFSETS(NAME, C)                                                        \
  GB_EXPORT int NAME(int64_t* tocarry, const int64_t* fromoffsets, int64_t offsetslength,      \
                     const C* fromstarts, const C* fromstops, int64_t lencontent,              \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {            \
    const long long n = offsetslength - 1;                                                     \
    if (n <= 0) return 0;                                                                      \
    broadcast_tooffsets_kernel<C><<<(unsigned)tile_count(n), kTileBlock, 0,                    \
                                    (cudaStream_t)stream>>>(tocarry, fromoffsets, n,           \
                                                            fromstarts, fromstops, lencontent, \
                                                            invocation_index, err_code);       \
    return (int)cudaGetLastError();                                                            \
  }
GB_BROADCAST_TOOFFSETS(awkward_ListArray32_broadcast_tooffsets_64, int32_t)
GB_BROADCAST_TOOFFSETS(awkward_ListArrayU32_broadcast_tooffsets_64, uint32_t)
GB_BROADCAST_TOOFFSETS(awkward_ListArray64_broadcast_tooffsets_64, int64_t)
