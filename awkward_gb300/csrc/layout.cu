// layout.cu -- list-layout conversions next to the reducer and getitem path.
//
//   awkward_ListArray{32,U32,64}_compact_offsets_64  awkward_ListArray_compact_offsets.cpp:7-23
//       ListArray (starts, stops) -> offsets: one single-pass scan over list
//       tiles (counts scanned in shared memory, tile prefix by decoupled
//       look-back), error 0 "stops[i] < starts[i]" raised by the first tile
//       that meets one (the CPU stops there; outputs past it are then not
//       defined, as awkward raises).
//   awkward_RegularArray_getitem_carry_64  awkward_RegularArray_getitem_carry.cpp:7-19
//   awkward_RegularArray_localindex_64     awkward_RegularArray_localindex.cpp:7-18
//   awkward_RegularArray_getitem_next_range_spreadadvanced_64  (.cpp:7-19)
//       elementwise over the lencarry*size (length*size) outputs, each thread
//       taking 8 consecutive outputs with one division.
//   awkward_localindex_64                          awkward_localindex.cpp:8-14
//   awkward_NumpyArray_reduce_adjust_starts_shifts_64  (.cpp:7-23)
//   awkward_ListArray*_getitem_next_range_counts_64    (.cpp:7-18): the total
//       telescopes to offsets[n] - offsets[0];
//   awkward_ListArray*_getitem_next_range_spreadadvanced_64  (.cpp:7-21): a
//       list-tile fill (tile of 1024 lists, counts scanned in shared memory).
#include "list_tile.cuh"

using namespace gb;

namespace {

template <class C>
__global__ void __launch_bounds__(kTileBlock)
    compact_offsets_kernel(int64_t* __restrict__ tooffsets, const C* __restrict__ starts,
                           const C* __restrict__ stops, long long length, ScanTiles st,
                           uint64_t inv, uint64_t* err) {
  __shared__ TileSmem sm;
  const long long tile = tile_claim(sm, st);
  const long long l0 = tile * kTileLists;
  long long cnt[kTileLPT];
  bool bad = false;
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const long long i = l0 + threadIdx.x * kTileLPT + r;
    cnt[r] = 0;
    if (i < length) {
      const C a = starts[i], b = stops[i];
      if (b < a) bad = true;
      cnt[r] = (long long)b - (long long)a;
    }
  }
  if (bad) raise_error(err, inv, 0);
  const long long prefix = tile_scan(sm, st, tile, cnt, inv, err);
  for (int li = threadIdx.x; li < kTileLists; li += kTileBlock) {
    const long long i = l0 + li;
    if (i < length) tooffsets[i + 1] = prefix + sm.loc[li + 1];
  }
  if (tile == 0 && threadIdx.x == 0) tooffsets[0] = 0;
}

constexpr int kPer = 8;  // consecutive outputs per thread

// out[q] for q < n, with i = q / size, j = q % size:
//   kLocal: j;  kCarry: from[i] * size + j;  kSpread: from[i].
enum RegularMode { kLocal = 0, kCarry = 1, kSpread = 2 };

template <int MODE>
__global__ void __launch_bounds__(256)
    regular_index_kernel(int64_t* __restrict__ out, const int64_t* __restrict__ from, long long n,
                         long long size) {
  for (long long q0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) * kPer; q0 < n;
       q0 += (long long)gridDim.x * blockDim.x * kPer) {
    long long i = q0 / size, j = q0 - i * size;
    long long f = MODE == kLocal ? 0 : from[i];
    const long long q1 = q0 + kPer < n ? q0 + kPer : n;
    for (long long q = q0; q < q1; q++) {
      out[q] = MODE == kLocal ? j : MODE == kCarry ? f * size + j : f;
      if (++j == size) {
        j = 0;
        i++;
        if (MODE != kLocal && q + 1 < q1) f = from[i];
      }
    }
  }
}

__global__ void __launch_bounds__(256) iota_kernel(int64_t* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = i;
}

// toptr[k] += shifts[toptr[k]] - starts[k] where toptr[k] >= 0.
__global__ void __launch_bounds__(256)
    adjust_starts_shifts_kernel(int64_t* __restrict__ toptr, long long n,
                                const int64_t* __restrict__ starts,
                                const int64_t* __restrict__ shifts) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const long long i = toptr[k];
    if (i >= 0) toptr[k] = i + shifts[i] - starts[k];
  }
}

template <class C>
__global__ void range_counts_kernel(int64_t* total, const C* __restrict__ offsets, long long n) {
  if (blockIdx.x == 0 && threadIdx.x == 0)
    *total = n > 0 ? (long long)offsets[n] - (long long)offsets[0] : 0;
}

// toadvanced[offsets[i] + j] = fromadvanced[i] for j < offsets[i+1] - offsets[i].
template <class C>
__global__ void __launch_bounds__(kTileBlock)
    range_spread_kernel(int64_t* __restrict__ toadvanced, const int64_t* __restrict__ fromadvanced,
                        const C* __restrict__ offsets, long long n) {
  __shared__ TileSmem sm;
  for (long long l0 = (long long)blockIdx.x * kTileLists; l0 < n;
       l0 += (long long)gridDim.x * kTileLists) {
    const long long total = stage_lists(
        sm, l0, n, [&](long long l) { return (long long)offsets[l + 1] - (long long)offsets[l]; });
    tile_for_each_slot(sm, total, [&](long long q, int r) {
      const long long i = l0 + r;
      toadvanced[(long long)offsets[i] + (q - sm.loc[r])] = fromadvanced[i];
    });
    __syncthreads();
  }
}

unsigned elementwise_grid(long long n) {
  long long g = (n + 256 * kPer - 1) / (256 * kPer);
  const long long cap = (long long)device_sm_count() * 16;
  if (g < 1) g = 1;
  return (unsigned)(g < cap ? g : cap);
}

}  // namespace

#define GB_COMPACT_OFFSETS(NAME, C)                                                              \
  GB_EXPORT int NAME(int64_t* tooffsets, const C* fromstarts, const C* fromstops, int64_t length, \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {             \
    cudaStream_t s = (cudaStream_t)stream;                                                       \
    if (length <= 0) return (int)cudaMemsetAsync(tooffsets, 0, sizeof(int64_t), s);              \
    const long long nt = tile_count(length);                                                     \
    ScanTiles st;                                                                                \
    void* base = nullptr;                                                                        \
    cudaError_t e = scan_tiles_alloc(&st, &base, nt, s);                                         \
    if (e != cudaSuccess) return (int)e;                                                         \
    compact_offsets_kernel<C><<<(unsigned)nt, kTileBlock, 0, s>>>(                               \
        tooffsets, fromstarts, fromstops, length, st, invocation_index, err_code);               \
    e = cudaGetLastError();                                                                      \
    cudaError_t f = scratch_free(base, s);                                                       \
    return (int)(e != cudaSuccess ? e : f);                                                      \
  }
GB_COMPACT_OFFSETS(awkward_ListArray32_compact_offsets_64, int32_t)
GB_COMPACT_OFFSETS(awkward_ListArrayU32_compact_offsets_64, uint32_t)
GB_COMPACT_OFFSETS(awkward_ListArray64_compact_offsets_64, int64_t)

GB_EXPORT int awkward_RegularArray_getitem_carry_64(int64_t* tocarry, const int64_t* fromcarry,
                                                    int64_t lencarry, int64_t size,
                                                    uint64_t invocation_index, uint64_t* err_code,
                                                    void* stream) {
  (void)invocation_index;
  (void)err_code;
  if (lencarry <= 0 || size <= 0) return (int)cudaSuccess;
  const long long n = (long long)lencarry * size;
  regular_index_kernel<kCarry><<<elementwise_grid(n), 256, 0, (cudaStream_t)stream>>>(
      tocarry, fromcarry, n, size);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_RegularArray_localindex_64(int64_t* toindex, int64_t size, int64_t length,
                                                 uint64_t invocation_index, uint64_t* err_code,
                                                 void* stream) {
  (void)invocation_index;
  (void)err_code;
  if (length <= 0 || size <= 0) return (int)cudaSuccess;
  const long long n = (long long)length * size;
  regular_index_kernel<kLocal><<<elementwise_grid(n), 256, 0, (cudaStream_t)stream>>>(
      toindex, nullptr, n, size);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_RegularArray_getitem_next_range_spreadadvanced_64(
    int64_t* toadvanced, const int64_t* fromadvanced, int64_t length, int64_t nextsize,
    uint64_t invocation_index, uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  if (length <= 0 || nextsize <= 0) return (int)cudaSuccess;
  const long long n = (long long)length * nextsize;
  regular_index_kernel<kSpread><<<elementwise_grid(n), 256, 0, (cudaStream_t)stream>>>(
      toadvanced, fromadvanced, n, nextsize);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_localindex_64(int64_t* toindex, int64_t length, uint64_t invocation_index,
                                    uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  if (length <= 0) return (int)cudaSuccess;
  iota_kernel<<<elementwise_grid(length), 256, 0, (cudaStream_t)stream>>>(toindex, length);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_NumpyArray_reduce_adjust_starts_shifts_64(
    int64_t* toptr, int64_t outlength, const int64_t* offsets, const int64_t* starts,
    const int64_t* shifts, uint64_t invocation_index, uint64_t* err_code, void* stream) {
  (void)offsets;
  (void)invocation_index;
  (void)err_code;
  if (outlength <= 0) return (int)cudaSuccess;
  adjust_starts_shifts_kernel<<<elementwise_grid(outlength), 256, 0, (cudaStream_t)stream>>>(
      toptr, outlength, starts, shifts);
  return (int)cudaGetLastError();
}

#define GB_RANGE_COUNTS(NAME, C)                                                             \
  GB_EXPORT int NAME(int64_t* total, const C* fromoffsets, int64_t lenstarts,               \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {         \
    (void)invocation_index;                                                                 \
    (void)err_code;                                                                         \
    range_counts_kernel<C><<<1, 32, 0, (cudaStream_t)stream>>>(total, fromoffsets, lenstarts); \
    return (int)cudaGetLastError();                                                         \
  }
GB_RANGE_COUNTS(awkward_ListArray32_getitem_next_range_counts_64, int32_t)
GB_RANGE_COUNTS(awkward_ListArrayU32_getitem_next_range_counts_64, uint32_t)
GB_RANGE_COUNTS(awkward_ListArray64_getitem_next_range_counts_64, int64_t)

#define GB_RANGE_SPREAD(NAME, C)                                                              \
  GB_EXPORT int NAME(int64_t* toadvanced, const int64_t* fromadvanced, const C* fromoffsets,  \
                     int64_t lenstarts, uint64_t invocation_index, uint64_t* err_code,        \
                     void* stream) {                                                          \
    (void)invocation_index;                                                                   \
    (void)err_code;                                                                           \
    if (lenstarts <= 0) return (int)cudaSuccess;                                              \
    const long long tiles = (lenstarts + kTileLists - 1) / kTileLists;                        \
    const long long cap = (long long)device_sm_count() * 16;                                  \
    range_spread_kernel<C><<<(unsigned)(tiles < cap ? tiles : cap), kTileBlock, 0,           \
                             (cudaStream_t)stream>>>(toadvanced, fromadvanced, fromoffsets,   \
                                                     lenstarts);                              \
    return (int)cudaGetLastError();                                                           \
  }
GB_RANGE_SPREAD(awkward_ListArray32_getitem_next_range_spreadadvanced_64, int32_t)
GB_RANGE_SPREAD(awkward_ListArrayU32_getitem_next_range_spreadadvanced_64, uint32_t)
GB_RANGE_SPREAD(awkward_ListArray64_getitem_next_range_spreadadvanced_64, int64_t)
