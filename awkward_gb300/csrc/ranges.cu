// ranges.cu -- `[..., start:stop:step]` on lists.
//
//   awkward_ListArray_getitem_next_range              awkward_ListArray_getitem_next_range.cpp:9-41
//   awkward_ListArray_getitem_next_range_carrylength  awkward_ListArray_getitem_next_range_carrylength.cpp:9-35
//   awkward_RegularArray_getitem_next_range           awkward_RegularArray_getitem_next_range.cpp:8-19
//
// Each list's slice is clipped against the list's length exactly as
// kernel-utils.cpp:7-39 (awkward_regularize_rangeslice) does; the number of
// kept positions is then computed in closed form instead of by stepping.
#include "list_tile.cuh"

using namespace gb;

namespace {

constexpr long long kSliceNone = 9223372036854775807LL;
constexpr int kMapBlock = 256;
inline int map_grid(long long n) {
  long long g = (n + kMapBlock - 1) / kMapBlock;
  long long cap = (long long)device_sm_count() * 16;
  return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

// kernel-utils.cpp:7-39
__device__ __forceinline__ void regularize_rangeslice(long long* start, long long* stop,
                                                      bool posstep, bool hasstart, bool hasstop,
                                                      long long length) {
  if (posstep) {
    if (!hasstart) *start = 0;
    else if (*start < 0) *start += length;
    if (*start < 0) *start = 0;
    if (*start > length) *start = length;
    if (!hasstop) *stop = length;
    else if (*stop < 0) *stop += length;
    if (*stop < 0) *stop = 0;
    if (*stop > length) *stop = length;
    if (*stop < *start) *stop = *start;
  } else {
    if (!hasstart) *start = length - 1;
    else if (*start < 0) *start += length;
    if (*start < -1) *start = -1;
    if (*start > length - 1) *start = length - 1;
    if (!hasstop) *stop = -1;
    else if (*stop < 0) *stop += length;
    if (*stop < -1) *stop = -1;
    if (*stop > length - 1) *stop = length - 1;
    if (*stop > *start) *stop = *start;
  }
}

// Kept positions of one list: first = regular start, count = number of j
// visited by `for (j = start; j < stop (or > stop); j += step)`.
__device__ __forceinline__ long long range_count(long long length, long long start,
                                                 long long stop, long long step,
                                                 long long* first) {
  long long rs = start, re = stop;
  regularize_rangeslice(&rs, &re, step > 0, start != kSliceNone, stop != kSliceNone, length);
  *first = rs;
  // |step| == 1 needs no division; otherwise a 32-bit one when the operands fit
  // (64-bit division is a long software sequence)
  long long span, astep;
  if (step > 0) {
    if (rs >= re) return 0;
    span = re - rs - 1;
    astep = step;
  } else if (step < 0) {
    if (rs <= re) return 0;
    span = rs - re - 1;
    astep = -step;
  } else {
    return 0;
  }
  if (astep == 1) return span + 1;
  if (span < (1ll << 32) && astep < (1ll << 32))
    return (long long)((unsigned)span / (unsigned)astep) + 1;
  return span / astep + 1;
}

template <class C>
__global__ void __launch_bounds__(kTileBlock)
    next_range_kernel(C* __restrict__ tooffsets, int64_t* __restrict__ tocarry,
                      const C* __restrict__ fromstarts, const C* __restrict__ fromstops,
                      long long n, long long start, long long stop, long long step, ScanTiles st,
                      uint64_t inv, uint64_t* err) {
  __shared__ TileSmem sm;
  __shared__ long long s_first[kTileLists];  // fromstarts[i] + regular start
  const long long tile = tile_claim(sm, st);
  const long long l0 = tile * kTileLists;
  long long cnt[kTileLPT];
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const int li = threadIdx.x * kTileLPT + r;
    const long long i = l0 + li;
    long long c = 0;
    if (i < n) {
      const long long fs = (long long)fromstarts[i];
      const long long length = (long long)fromstops[i] - fs;
      long long first;
      c = range_count(length, start, stop, step, &first);
      s_first[li] = fs + first;
    }
    cnt[r] = c;
  }
  const long long prefix = tile_scan(sm, st, tile, cnt, inv, err);
  const long long total = sm.total;
  for (int li = threadIdx.x; li < kTileLists; li += kTileBlock) {
    const long long i = l0 + li;
    if (i < n) tooffsets[i + 1] = (C)(prefix + sm.loc[li + 1]);
  }
  if (tile == 0 && threadIdx.x == 0) tooffsets[0] = 0;
  tile_for_each_slot(sm, total, [&](long long q, int r) {
    tocarry[prefix + q] = s_first[r] + (q - sm.loc[r]) * step;
  });
}

template <class C>
__global__ void next_range_carrylength_kernel(unsigned long long* __restrict__ carrylength,
                                              const C* __restrict__ fromstarts,
                                              const C* __restrict__ fromstops, long long n,
                                              long long start, long long stop, long long step) {
  __shared__ long long scan[kMapBlock / 32 + 1];
  long long s = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long first;
    s += range_count((long long)fromstops[i] - (long long)fromstarts[i], start, stop, step,
                     &first);
  }
  long long total;
  auto add = [](long long a, long long b) { return a + b; };
  block_exclusive_scan<kMapBlock>(s, add, 0ll, scan, &total);
  if (threadIdx.x == 0 && total) atomicAdd(carrylength, (unsigned long long)total);
}

__global__ void regular_next_range_kernel(int64_t* __restrict__ tocarry, long long regular_start,
                                          long long step, long long length, long long size,
                                          long long nextsize) {
  const long long total = length * nextsize;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long i = q / nextsize, j = q - i * nextsize;
    tocarry[q] = i * size + regular_start + j * step;
  }
}

}  // namespace

#define GB_NEXT_RANGE(NAME, C)                                                                  \
  GB_EXPORT int NAME(C* tooffsets, int64_t* tocarry, const C* fromstarts, const C* fromstops,   \
                     int64_t lenstarts, int64_t start, int64_t stop, int64_t step,              \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {             \
    cudaStream_t s = (cudaStream_t)stream;                                                      \
    if (lenstarts <= 0) return (int)cudaMemsetAsync(tooffsets, 0, sizeof(C), s);                \
    const long long nt = tile_count(lenstarts);                                                 \
    ScanTiles st;                                                                               \
    void* base = nullptr;                                                                       \
    cudaError_t e = scan_tiles_alloc(&st, &base, nt, s);                                        \
    if (e != cudaSuccess) return (int)e;                                                        \
    next_range_kernel<C><<<(unsigned)nt, kTileBlock, 0, s>>>(                                   \
        tooffsets, tocarry, fromstarts, fromstops, lenstarts, start, stop, step, st,            \
        invocation_index, err_code);                                                            \
    e = cudaGetLastError();                                                                     \
    cudaError_t f = scratch_free(base, s);                                                      \
    return (int)(e != cudaSuccess ? e : f);                                                     \
  }
GB_NEXT_RANGE(awkward_ListArray32_getitem_next_range_64, int32_t)
GB_NEXT_RANGE(awkward_ListArrayU32_getitem_next_range_64, uint32_t)
GB_NEXT_RANGE(awkward_ListArray64_getitem_next_range_64, int64_t)

#define GB_NEXT_RANGE_CARRYLENGTH(NAME, C)                                                     \
  GB_EXPORT int NAME(int64_t* carrylength, const C* fromstarts, const C* fromstops,            \
                     int64_t lenstarts, int64_t start, int64_t stop, int64_t step,             \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {            \
    (void)invocation_index;                                                                    \
    (void)err_code;                                                                            \
    cudaStream_t s = (cudaStream_t)stream;                                                     \
    cudaError_t e = cudaMemsetAsync(carrylength, 0, sizeof(int64_t), s);                       \
    if (e != cudaSuccess || lenstarts <= 0) return (int)e;                                     \
    next_range_carrylength_kernel<C><<<map_grid(lenstarts), kMapBlock, 0, s>>>(                \
        reinterpret_cast<unsigned long long*>(carrylength), fromstarts, fromstops, lenstarts,  \
        start, stop, step);                                                                    \
    return (int)cudaGetLastError();                                                            \
  }
GB_NEXT_RANGE_CARRYLENGTH(awkward_ListArray32_getitem_next_range_carrylength, int32_t)
GB_NEXT_RANGE_CARRYLENGTH(awkward_ListArrayU32_getitem_next_range_carrylength, uint32_t)
GB_NEXT_RANGE_CARRYLENGTH(awkward_ListArray64_getitem_next_range_carrylength, int64_t)

GB_EXPORT int awkward_RegularArray_getitem_next_range_64(int64_t* tocarry, int64_t regular_start,
                                                        int64_t step, int64_t length,
                                                        int64_t size, int64_t nextsize,
                                                        uint64_t invocation_index,
                                                        uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  const long long total = length * nextsize;
  if (total <= 0) return 0;
  regular_next_range_kernel<<<map_grid(total), kMapBlock, 0, (cudaStream_t)stream>>>(
      tocarry, regular_start, step, length, size, nextsize);
  return (int)cudaGetLastError();
}
