// jagged.cu -- jagged getitem kernels and the carries they feed.
//
//   awkward_ListArray_getitem_jagged_apply     awkward_ListArray_getitem_jagged_apply.cpp:8-56
//   awkward_ListArray_getitem_jagged_carrylen  awkward_ListArray_getitem_jagged_carrylen.cpp:8-18
//   awkward_ListArray_getitem_jagged_descend   awkward_ListArray_getitem_jagged_descend.cpp:8-31
//   awkward_ListArray_getitem_jagged_expand    awkward_ListArray_getitem_jagged_expand.cpp:8-32
//   awkward_ListArray_getitem_jagged_numvalid  awkward_ListArray_getitem_jagged_numvalid.cpp:8-30
//   awkward_ListArray_getitem_jagged_shrink    awkward_ListArray_getitem_jagged_shrink.cpp:8-46
//   awkward_RegularArray_getitem_jagged_expand awkward_RegularArray_getitem_jagged_expand.cpp:8-20
//   awkward_ListArray_localindex               awkward_ListArray_localindex.cpp:8-19
//
// Error codes are the indices of the messages in awkward's CUDA kernels of
// the same name (their `// message:` enum order).
#include <dlfcn.h>

#include <mutex>
#include <type_traits>

#include "list_tile.cuh"

using namespace gb;

namespace {

constexpr int kMapBlock = 256;
inline int map_grid(long long n) {
  long long g = (n + kMapBlock - 1) / kMapBlock;
  long long cap = (long long)device_sm_count() * 16;
  return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

// ------------------------------------------------------------------ apply
// errors: 0 jagged slice's stops[i] < starts[i]; 1 jagged slice's offsets
// extend beyond its content; 2 stops[i] < starts[i]; 3 stops[i] > len(content);
// 4 index out of range
//
// With W other than void the kernel also gathers the content at each carry
// into tocontent (array[index] in one pass; tocarry may then be null).
template <class C, class W = void>
__global__ void __launch_bounds__(kTileBlock)
    jagged_apply_kernel(int64_t* __restrict__ tooffsets, int64_t* __restrict__ tocarry,
                        const int64_t* __restrict__ slicestarts,
                        const int64_t* __restrict__ slicestops, long long n,
                        const int64_t* __restrict__ sliceindex, long long sliceinnerlen,
                        const C* __restrict__ fromstarts, const C* __restrict__ fromstops,
                        long long contentlen, ScanTiles st, uint64_t inv, uint64_t* err,
                        void* __restrict__ tocontent = nullptr,
                        const void* __restrict__ content = nullptr) {
  __shared__ TileSmem sm;
  __shared__ long long s_slice[kTileLists];
  __shared__ long long s_start[kTileLists];
  __shared__ long long s_count[kTileLists];
  const long long tile = tile_claim(sm, st);
  const long long l0 = tile * kTileLists;
  long long cnt[kTileLPT];
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const int li = threadIdx.x * kTileLPT + r;
    const long long i = l0 + li;
    long long c = 0;
    if (i < n) {
      const long long ss = slicestarts[i], se = slicestops[i];
      const long long start = (long long)fromstarts[i], stop = (long long)fromstops[i];
      bool ok = true;
      if (ss != se) {
        if (se < ss) { raise_error(err, inv, 0); ok = false; }
        else if (se > sliceinnerlen) { raise_error(err, inv, 1); ok = false; }
        else if (stop < start) { raise_error(err, inv, 2); ok = false; }
        else if (start != stop && stop > contentlen) { raise_error(err, inv, 3); ok = false; }
        if (ok) c = se - ss;
      }
      s_slice[li] = ss;
      s_start[li] = start;
      s_count[li] = stop - start;
    }
    cnt[r] = c;
  }
  const long long prefix = tile_scan(sm, st, tile, cnt, inv, err);
  const long long total = sm.total;
  for (int li = threadIdx.x; li < kTileLists; li += kTileBlock) {
    const long long i = l0 + li;
    if (i < n) tooffsets[i] = prefix + sm.loc[li];
    if (i == n) tooffsets[n] = prefix + total;  // only the tile holding list n-1 ... n
  }
  if (l0 + kTileLists == n && threadIdx.x == 0) tooffsets[n] = prefix + total;
  tile_for_each_slot(sm, total, [&](long long q, int r) {
    const long long j = s_slice[r] + (q - sm.loc[r]);
    long long idx = sliceindex[j];
    const long long count = s_count[r];
    if (idx < -count || idx >= count) {
      raise_error(err, inv, 4);
      return;
    }
    if (idx < 0) idx += count;
    const long long at = s_start[r] + idx;
    if constexpr (std::is_void<W>::value) {
      tocarry[prefix + q] = at;
    } else {
      if (at < 0 || at >= contentlen) {  // a start below zero; the CPU kernel does not check it
        raise_error(err, inv, 3);
        return;
      }
      static_cast<W*>(tocontent)[prefix + q] = __ldg(static_cast<const W*>(content) + at);
      if (tocarry) tocarry[prefix + q] = at;
    }
  });
}

// ------------------------------------------------------------------ carrylen
__global__ void carrylen_kernel(unsigned long long* __restrict__ carrylen,
                                const int64_t* __restrict__ slicestarts,
                                const int64_t* __restrict__ slicestops, long long n) {
  __shared__ long long scan[kMapBlock / 32 + 1];
  long long s = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s += slicestops[i] - slicestarts[i];
  long long total;
  auto add = [](long long a, long long b) { return a + b; };
  block_exclusive_scan<kMapBlock>(s, add, 0ll, scan, &total);
  if (threadIdx.x == 0) atomicAdd(carrylen, (unsigned long long)total);
}

// ------------------------------------------------------------------ descend
// errors: 0 jagged slice inner length differs from array inner length
template <class C>
__global__ void __launch_bounds__(kTileBlock)
    jagged_descend_kernel(int64_t* __restrict__ tooffsets,
                          const int64_t* __restrict__ slicestarts,
                          const int64_t* __restrict__ slicestops, long long n,
                          const C* __restrict__ fromstarts, const C* __restrict__ fromstops,
                          ScanTiles st, uint64_t inv, uint64_t* err) {
  __shared__ TileSmem sm;
  const long long tile = tile_claim(sm, st);
  const long long l0 = tile * kTileLists;
  long long cnt[kTileLPT];
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const long long i = l0 + threadIdx.x * kTileLPT + r;
    long long c = 0;
    if (i < n) {
      const long long slicecount = slicestops[i] - slicestarts[i];
      c = (long long)(fromstops[i] - fromstarts[i]);
      if (slicecount != c) raise_error(err, inv, 0);
    }
    cnt[r] = c;
  }
  const long long prefix = tile_scan(sm, st, tile, cnt, inv, err);
  const long long base = slicestarts[0];
  for (int li = threadIdx.x; li < kTileLists; li += kTileBlock) {
    const long long i = l0 + li;
    if (i < n) tooffsets[i + 1] = base + prefix + sm.loc[li + 1];
  }
  if (tile == 0 && threadIdx.x == 0) tooffsets[0] = base;
}

// ------------------------------------------------------------------ expand
// errors: 0 stops[i] < starts[i]; 1 cannot fit jagged slice into nested list
template <class C>
__global__ void jagged_expand_kernel(int64_t* __restrict__ multistarts,
                                     int64_t* __restrict__ multistops,
                                     const int64_t* __restrict__ singleoffsets,
                                     int64_t* __restrict__ tocarry,
                                     const C* __restrict__ fromstarts,
                                     const C* __restrict__ fromstops, long long jaggedsize,
                                     long long length, uint64_t inv, uint64_t* err) {
  const long long total = jaggedsize * length;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long i = q / jaggedsize, j = q - i * jaggedsize;
    const C start = fromstarts[i], stop = fromstops[i];
    if (stop < start) { raise_error(err, inv, 0); continue; }
    if ((long long)(stop - start) != jaggedsize) { raise_error(err, inv, 1); continue; }
    multistarts[q] = singleoffsets[j];
    multistops[q] = singleoffsets[j + 1];
    tocarry[q] = (long long)start + j;
  }
  // lists whose slice is empty still validate their bounds
  if (jaggedsize == 0) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < length;
         i += (long long)gridDim.x * blockDim.x) {
      const C start = fromstarts[i], stop = fromstops[i];
      if (stop < start) raise_error(err, inv, 0);
      else if ((long long)(stop - start) != 0) raise_error(err, inv, 1);
    }
  }
}

// ------------------------------------------------------------------ numvalid
// errors: 0 jagged slice's stops[i] < starts[i]; 1 jagged slice's offsets
// extend beyond its content
__global__ void __launch_bounds__(kTileBlock)
    jagged_numvalid_kernel(unsigned long long* __restrict__ numvalid,
                           const int64_t* __restrict__ slicestarts,
                           const int64_t* __restrict__ slicestops, long long n,
                           const int64_t* __restrict__ missing, long long missinglength,
                           uint64_t inv, uint64_t* err) {
  __shared__ long long loc[kTileLists + 1];
  __shared__ long long s_slice[kTileLists];
  __shared__ long long scan[kTileBlock / 32 + 1];
  const long long l0 = blockIdx.x * (long long)kTileLists;
  long long cnt[kTileLPT];
  long long s = 0;
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const int li = threadIdx.x * kTileLPT + r;
    const long long i = l0 + li;
    long long c = 0;
    if (i < n) {
      const long long ss = slicestarts[i], se = slicestops[i];
      if (ss != se) {
        if (se < ss) raise_error(err, inv, 0);
        else if (se > missinglength) raise_error(err, inv, 1);
        else c = se - ss;
      }
      s_slice[li] = ss;
    }
    cnt[r] = c;
    s += c;
  }
  long long total;
  auto add = [](long long a, long long b) { return a + b; };
  long long run = block_exclusive_scan<kTileBlock>(s, add, 0ll, scan, &total);
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    loc[threadIdx.x * kTileLPT + r] = run;
    run += cnt[r];
  }
  if (threadIdx.x == 0) loc[kTileLists] = total;
  __syncthreads();
  long long valid = 0;
  for (long long q = threadIdx.x; q < total; q += kTileBlock) {
    int lo = 0, hi = kTileLists;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (loc[mid] <= q) lo = mid;
      else hi = mid;
    }
    valid += missing[s_slice[lo] + (q - loc[lo])] >= 0 ? 1 : 0;
  }
  long long vt;
  block_exclusive_scan<kTileBlock>(valid, add, 0ll, scan, &vt);
  if (threadIdx.x == 0 && vt) atomicAdd(numvalid, (unsigned long long)vt);
}

// ------------------------------------------------------------------ shrink
// Compacts the slice positions j whose missing[j] >= 0 (tile-ordered), and
// writes the small (kept) and large (all) offsets.  Two look-backs: one over
// kept counts, one over slice lengths.
__global__ void __launch_bounds__(kTileBlock)
    jagged_shrink_kernel(int64_t* __restrict__ tocarry, int64_t* __restrict__ tosmalloffsets,
                         int64_t* __restrict__ tolargeoffsets,
                         const int64_t* __restrict__ slicestarts,
                         const int64_t* __restrict__ slicestops, long long n,
                         const int64_t* __restrict__ missing, ScanTiles st_small,
                         ScanTiles st_large, uint64_t inv, uint64_t* err) {
  __shared__ TileSmem sm;
  __shared__ long long s_slice[kTileLists];
  __shared__ long long s_small[kTileLists];
  __shared__ long long scan2[kTileBlock / 32 + 1];
  __shared__ long long large_prefix;
  const long long tile = tile_claim(sm, st_small);
  const long long l0 = tile * kTileLists;
  long long cnt[kTileLPT];
  long long large = 0;
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const int li = threadIdx.x * kTileLPT + r;
    const long long i = l0 + li;
    long long c = 0;
    if (i < n) {
      const long long ss = slicestarts[i], se = slicestops[i];
      if (ss != se && se > ss) c = se - ss;
      large += se - ss;
      s_slice[li] = ss;
    }
    s_small[li] = 0;
    cnt[r] = c;
  }
  // local offsets over slice elements (to enumerate them) -- no look-back
  long long s = 0;
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) s += cnt[r];
  long long total;
  auto add = [](long long a, long long b) { return a + b; };
  long long run = block_exclusive_scan<kTileBlock>(s, add, 0ll, sm.scan, &total);
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    sm.loc[threadIdx.x * kTileLPT + r] = run;
    run += cnt[r];
  }
  if (threadIdx.x == 0) sm.loc[kTileLists] = total;
  __syncthreads();
  // pass 1: kept count per list
  for (long long q = threadIdx.x; q < total; q += kTileBlock) {
    const int r = tile_find(sm, q);
    if (missing[s_slice[r] + (q - sm.loc[r])] >= 0)
      atomicAdd(reinterpret_cast<unsigned long long*>(&s_small[r]), 1ull);
  }
  __syncthreads();
  long long small_cnt[kTileLPT];
  long long small_sum = 0;
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    small_cnt[r] = s_small[threadIdx.x * kTileLPT + r];
    small_sum += small_cnt[r];
  }
  long long small_total;
  long long small_run = block_exclusive_scan<kTileBlock>(small_sum, add, 0ll, scan2, &small_total);
  long long large_total;
  long long large_run = block_exclusive_scan<kTileBlock>(large, add, 0ll, scan2, &large_total);
  if (threadIdx.x < 32) {
    long long ps = lookback_exclusive(st_small, tile, small_total, inv, err, GB_MSG_TIMEOUT);
    long long pl = lookback_exclusive(st_large, tile, large_total, inv, err, GB_MSG_TIMEOUT);
    if (threadIdx.x == 0) {
      sm.prefix = ps;
      large_prefix = pl;
    }
  }
  __syncthreads();
  const long long base = n > 0 ? slicestarts[0] : 0;
  const long long sp = sm.prefix, lp = large_prefix;
  // offsets: each thread writes its own lists' inclusive values
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const long long i = l0 + threadIdx.x * kTileLPT + r;
    small_run += small_cnt[r];
    if (i < n) {
      const long long ss = slicestarts[i], se = slicestops[i];
      large_run += se - ss;
      tosmalloffsets[i + 1] = base + sp + small_run;
      tolargeoffsets[i + 1] = base + lp + large_run;
    }
  }
  if (tile == 0 && threadIdx.x == 0) {
    tosmalloffsets[0] = base;
    tolargeoffsets[0] = base;
  }
  // pass 2: compacted positions by a chunked block scan over kept flags
  long long kept_before = 0;
  for (long long q0 = 0; q0 < total; q0 += kTileBlock) {
    const long long q = q0 + threadIdx.x;
    long long j = 0, keep = 0;
    if (q < total) {
      const int r = tile_find(sm, q);
      j = s_slice[r] + (q - sm.loc[r]);
      keep = missing[j] >= 0 ? 1 : 0;
    }
    long long chunk_total;
    long long pos = block_exclusive_scan<kTileBlock>(keep, add, 0ll, sm.scan, &chunk_total);
    if (keep) tocarry[sp + kept_before + pos] = j;
    kept_before += chunk_total;
  }
}

// ------------------------------------------------------------------ RegularArray expand
__global__ void regular_jagged_expand_kernel(int64_t* __restrict__ multistarts,
                                             int64_t* __restrict__ multistops,
                                             const int64_t* __restrict__ singleoffsets,
                                             long long regularsize, long long regularlength) {
  const long long total = regularsize * regularlength;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long j = q % regularsize;
    multistarts[q] = singleoffsets[j];
    multistops[q] = singleoffsets[j + 1];
  }
}

// ------------------------------------------------------------------ localindex
template <class C>
__global__ void __launch_bounds__(kTileBlock)
    localindex_kernel(int64_t* __restrict__ toindex, const C* __restrict__ offsets, long long n) {
  __shared__ long long loc[kTileLists + 1];
  const long long l0 = blockIdx.x * (long long)kTileLists;
  const long long l1 = l0 + kTileLists < n ? l0 + kTileLists : n;
  for (long long li = threadIdx.x; li <= l1 - l0; li += kTileBlock) loc[li] = (long long)offsets[l0 + li];
  __syncthreads();
  const int nl = (int)(l1 - l0);
  const long long e0 = loc[0], e1 = loc[nl];
  for (long long j = e0 + threadIdx.x; j < e1; j += kTileBlock) {
    int lo = 0, hi = nl;  // last r with loc[r] <= j
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (loc[mid] <= j) lo = mid;
      else hi = mid;
    }
    toindex[j] = j - loc[lo];
  }
}

}  // namespace

// ================================================================== entry points
#define GB_JAGGED_APPLY(NAME, C)                                                               \
  GB_EXPORT int NAME(int64_t* tooffsets, int64_t* tocarry, const int64_t* slicestarts,         \
                     const int64_t* slicestops, int64_t sliceouterlen, const int64_t* sliceindex, \
                     int64_t sliceinnerlen, const C* fromstarts, const C* fromstops,          \
                     int64_t contentlen, uint64_t invocation_index, uint64_t* err_code,       \
                     void* stream) {                                                          \
    cudaStream_t s = (cudaStream_t)stream;                                                    \
    if (sliceouterlen <= 0)                                                                   \
      return (int)cudaMemsetAsync(tooffsets, 0, sizeof(int64_t), s);                          \
    const long long nt = tile_count(sliceouterlen);                                           \
    ScanTiles st;                                                                             \
    void* base = nullptr;                                                                     \
    cudaError_t e = scan_tiles_alloc(&st, &base, nt, s);                                      \
    if (e != cudaSuccess) return (int)e;                                                      \
    jagged_apply_kernel<C><<<(unsigned)nt, kTileBlock, 0, s>>>(                               \
        tooffsets, tocarry, slicestarts, slicestops, sliceouterlen, sliceindex, sliceinnerlen, \
        fromstarts, fromstops, contentlen, st, invocation_index, err_code);                   \
    e = cudaGetLastError();                                                                   \
    cudaError_t f = scratch_free(base, s);                                                    \
    return (int)(e != cudaSuccess ? e : f);                                                   \
  }
GB_JAGGED_APPLY(awkward_ListArray32_getitem_jagged_apply_64, int32_t)
GB_JAGGED_APPLY(awkward_ListArrayU32_getitem_jagged_apply_64, uint32_t)
GB_JAGGED_APPLY(awkward_ListArray64_getitem_jagged_apply_64, int64_t)

// array[index] in one pass: the list-tile apply above with the content
// gathered at each carry, so the carry is neither written nor read back
// (tocarry may be null).  The index lists are index[index_offsets[i] ..
// index_offsets[i+1]) and the lists content[offsets[i] .. offsets[i+1]); the
// errors are the apply's (invocation index 0).
GB_EXPORT int awkward_gb300_jagged_index_select(int64_t* tooffsets, void* tocontent,
                                                int64_t* tocarry, const int64_t* index_offsets,
                                                const int64_t* index, int64_t indexlen,
                                                const int64_t* offsets, const void* content,
                                                int64_t itemsize, int64_t contentlen,
                                                int64_t nlists, uint64_t* err_code,
                                                void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (itemsize != 1 && itemsize != 2 && itemsize != 4 && itemsize != 8)
    return (int)cudaErrorInvalidValue;
  if (nlists <= 0) return (int)cudaMemsetAsync(tooffsets, 0, sizeof(int64_t), s);
  const long long nt = tile_count(nlists);
  ScanTiles st;
  void* base = nullptr;
  cudaError_t e = scan_tiles_alloc(&st, &base, nt, s);
  if (e != cudaSuccess) return (int)e;
#define GB_INDEX_SELECT(W)                                                                     \
  jagged_apply_kernel<int64_t, W><<<(unsigned)nt, kTileBlock, 0, s>>>(                         \
      tooffsets, tocarry, index_offsets, index_offsets + 1, nlists, index, indexlen, offsets,  \
      offsets + 1, contentlen, st, 0, err_code, tocontent, content)
  switch (itemsize) {
    case 1: GB_INDEX_SELECT(uint8_t); break;
    case 2: GB_INDEX_SELECT(uint16_t); break;
    case 4: GB_INDEX_SELECT(uint32_t); break;
    default: GB_INDEX_SELECT(uint64_t);
  }
#undef GB_INDEX_SELECT
  e = cudaGetLastError();
  cudaError_t f = scratch_free(base, s);
  return (int)(e != cudaSuccess ? e : f);
}

GB_EXPORT int awkward_ListArray_getitem_jagged_carrylen_64(int64_t* carrylen,
                                                          const int64_t* slicestarts,
                                                          const int64_t* slicestops,
                                                          int64_t sliceouterlen,
                                                          uint64_t invocation_index,
                                                          uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(carrylen, 0, sizeof(int64_t), s);
  if (e != cudaSuccess || sliceouterlen <= 0) return (int)e;
  carrylen_kernel<<<map_grid(sliceouterlen), kMapBlock, 0, s>>>(
      reinterpret_cast<unsigned long long*>(carrylen), slicestarts, slicestops, sliceouterlen);
  return (int)cudaGetLastError();
}

#define GB_JAGGED_DESCEND(NAME, C)                                                             \
  GB_EXPORT int NAME(int64_t* tooffsets, const int64_t* slicestarts, const int64_t* slicestops, \
                     int64_t sliceouterlen, const C* fromstarts, const C* fromstops,          \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {           \
    cudaStream_t s = (cudaStream_t)stream;                                                    \
    if (sliceouterlen <= 0) return (int)cudaMemsetAsync(tooffsets, 0, sizeof(int64_t), s);    \
    const long long nt = tile_count(sliceouterlen);                                           \
    ScanTiles st;                                                                             \
    void* base = nullptr;                                                                     \
    cudaError_t e = scan_tiles_alloc(&st, &base, nt, s);                                      \
    if (e != cudaSuccess) return (int)e;                                                      \
    jagged_descend_kernel<C><<<(unsigned)nt, kTileBlock, 0, s>>>(                             \
        tooffsets, slicestarts, slicestops, sliceouterlen, fromstarts, fromstops, st,         \
        invocation_index, err_code);                                                          \
    e = cudaGetLastError();                                                                   \
    cudaError_t f = scratch_free(base, s);                                                    \
    return (int)(e != cudaSuccess ? e : f);                                                   \
  }
GB_JAGGED_DESCEND(awkward_ListArray32_getitem_jagged_descend_64, int32_t)
GB_JAGGED_DESCEND(awkward_ListArrayU32_getitem_jagged_descend_64, uint32_t)
GB_JAGGED_DESCEND(awkward_ListArray64_getitem_jagged_descend_64, int64_t)

#define GB_JAGGED_EXPAND(NAME, C)                                                              \
  GB_EXPORT int NAME(int64_t* multistarts, int64_t* multistops, const int64_t* singleoffsets,   \
                     int64_t* tocarry, const C* fromstarts, const C* fromstops,               \
                     int64_t jaggedsize, int64_t length, uint64_t invocation_index,           \
                     uint64_t* err_code, void* stream) {                                      \
    if (length <= 0) return 0;                                                                \
    long long work = jaggedsize > 0 ? jaggedsize * length : length;                          \
    jagged_expand_kernel<C><<<map_grid(work), kMapBlock, 0, (cudaStream_t)stream>>>(          \
        multistarts, multistops, singleoffsets, tocarry, fromstarts, fromstops, jaggedsize,   \
        length, invocation_index, err_code);                                                  \
    return (int)cudaGetLastError();                                                           \
  }
GB_JAGGED_EXPAND(awkward_ListArray32_getitem_jagged_expand_64, int32_t)
GB_JAGGED_EXPAND(awkward_ListArrayU32_getitem_jagged_expand_64, uint32_t)
GB_JAGGED_EXPAND(awkward_ListArray64_getitem_jagged_expand_64, int64_t)

GB_EXPORT int awkward_ListArray_getitem_jagged_numvalid_64(
    int64_t* numvalid, const int64_t* slicestarts, const int64_t* slicestops, int64_t length,
    const int64_t* missing, int64_t missinglength, uint64_t invocation_index, uint64_t* err_code,
    void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(numvalid, 0, sizeof(int64_t), s);
  if (e != cudaSuccess || length <= 0) return (int)e;
  jagged_numvalid_kernel<<<(unsigned)tile_count(length), kTileBlock, 0, s>>>(
      reinterpret_cast<unsigned long long*>(numvalid), slicestarts, slicestops, length, missing,
      missinglength, invocation_index, err_code);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_ListArray_getitem_jagged_shrink_64(
    int64_t* tocarry, int64_t* tosmalloffsets, int64_t* tolargeoffsets,
    const int64_t* slicestarts, const int64_t* slicestops, int64_t length,
    const int64_t* missing, uint64_t invocation_index, uint64_t* err_code, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (length <= 0) {
    cudaError_t e = cudaMemsetAsync(tosmalloffsets, 0, sizeof(int64_t), s);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaMemsetAsync(tolargeoffsets, 0, sizeof(int64_t), s);
  }
  const long long nt = tile_count(length);
  ScanTiles a, b;
  void *ba = nullptr, *bb = nullptr;
  cudaError_t e = scan_tiles_alloc(&a, &ba, nt, s);
  if (e != cudaSuccess) return (int)e;
  e = scan_tiles_alloc(&b, &bb, nt, s);
  if (e != cudaSuccess) {
    scratch_free(ba, s);
    return (int)e;
  }
  jagged_shrink_kernel<<<(unsigned)nt, kTileBlock, 0, s>>>(tocarry, tosmalloffsets,
                                                           tolargeoffsets, slicestarts,
                                                           slicestops, length, missing, a, b,
                                                           invocation_index, err_code);
  e = cudaGetLastError();
  cudaError_t f1 = scratch_free(ba, s), f2 = scratch_free(bb, s);
  return (int)(e != cudaSuccess ? e : (f1 != cudaSuccess ? f1 : f2));
}

GB_EXPORT int awkward_RegularArray_getitem_jagged_expand_64(int64_t* multistarts,
                                                           int64_t* multistops,
                                                           const int64_t* singleoffsets,
                                                           int64_t regularsize,
                                                           int64_t regularlength,
                                                           uint64_t invocation_index,
                                                           uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  const long long total = regularsize * regularlength;
  if (total <= 0) return 0;
  regular_jagged_expand_kernel<<<map_grid(total), kMapBlock, 0, (cudaStream_t)stream>>>(
      multistarts, multistops, singleoffsets, regularsize, regularlength);
  return (int)cudaGetLastError();
}

#define GB_LOCALINDEX(NAME, C)                                                                  \
  GB_EXPORT int NAME(int64_t* toindex, const C* offsets, int64_t length,                        \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {             \
    (void)invocation_index;                                                                     \
    (void)err_code;                                                                             \
    if (length <= 0) return 0;                                                                  \
    localindex_kernel<C><<<(unsigned)tile_count(length), kTileBlock, 0, (cudaStream_t)stream>>>( \
        toindex, offsets, length);                                                              \
    return (int)cudaGetLastError();                                                             \
  }
GB_LOCALINDEX(awkward_ListArray32_localindex_64, int32_t)
GB_LOCALINDEX(awkward_ListArrayU32_localindex_64, uint32_t)
GB_LOCALINDEX(awkward_ListArray64_localindex_64, int64_t)

// ================================================================== no-alloc variant
// A copy of awkward_ListArray64_getitem_jagged_apply_64 for callers that may
// not allocate device memory at call time.  Such callers are, for example,
// awkward code embedded in a process whose device memory is owned by another
// framework's pooling allocator (XLA-style preallocation of most of the GPU,
// an RMM pool): there cudaMalloc either fails for lack of memory or bypasses
// the pool's accounting, and the embedded code holds no handle to the pool.
//
// The only scratch the kernel needs is the look-back tile states (one
// 64-bit ticket counter plus one 64-bit word per tile of 1024 lists).  Here
// they live in a file-scope device array of fixed size, so every GPU that
// loads the library holds kNoAllocTileWords * 8 bytes (512 KiB + 8 B) until
// the process exits.  The array is shared by all calls:
//   * sliceouterlen is limited to kNoAllocMaxLists = 65536 * 1024 lists;
//     larger calls return cudaErrorInvalidValue without launching anything;
//   * each call zeroes the words it uses (cudaMemsetAsync on its stream)
//     before the kernel, because the array keeps the previous call's states;
//   * two calls whose work overlaps on the GPU (different streams, or
//     different host threads on one device) race on the array and give wrong
//     offsets: issue them on one stream or order them with events.
// The array's host-side name is only a stand-in symbol, not a device
// address, so the device address is looked up with cudaGetSymbolAddress the
// first time the entry point runs in a context (with that context's device
// current) and cached per (device, CUDA context): a context made later on the
// same device, for instance after cudaDeviceReset, gets its own lookup.  The
// first call in a context should therefore come before any stream capture
// on it.  The entry point calls no cudaMalloc, cudaFree or other allocating
// routine.
namespace {

constexpr long long kNoAllocMaxTiles = 1ll << 16;
constexpr long long kNoAllocMaxLists = kNoAllocMaxTiles * kTileLists;
constexpr long long kNoAllocTileWords = kNoAllocMaxTiles + 1;  // + the ticket counter

static __device__ __align__(256) unsigned long long g_noalloc_tiles[kNoAllocTileWords];

struct NoAllocEntry {
  int dev;
  void* ctx;
  unsigned long long* addr;
};
constexpr int kNoAllocCache = 64;
std::mutex g_noalloc_mutex;
NoAllocEntry g_noalloc_cache[kNoAllocCache];
int g_noalloc_used = 0;

// The current CUDA context (the driver's cuCtxGetCurrent, found in the driver
// library the runtime has already loaded), or null if it cannot be asked.
void* current_context() {
  using Fn = int (*)(void**);
  static Fn fn = [] {
    void* h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_NOLOAD);
    if (!h) h = dlopen("libcuda.so.1", RTLD_NOW);
    return h ? reinterpret_cast<Fn>(dlsym(h, "cuCtxGetCurrent")) : nullptr;
  }();
  void* ctx = nullptr;
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}

// Device address of g_noalloc_tiles in the current context (looked up once
// per device and context).
cudaError_t noalloc_tiles_address(unsigned long long** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  void* ctx = current_context();
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (ctx)
    for (int i = 0; i < g_noalloc_used; i++)
      if (g_noalloc_cache[i].dev == dev && g_noalloc_cache[i].ctx == ctx) {
        *out = g_noalloc_cache[i].addr;
        return cudaSuccess;
      }
  // (the lookup also makes the device's runtime context current when no
  // context was current yet)
  void* ptr = nullptr;
  e = cudaGetSymbolAddress(&ptr, g_noalloc_tiles);
  if (e != cudaSuccess) return e;
  if (!ptr) return cudaErrorInvalidSymbol;
  if (!ctx) ctx = current_context();
  if (ctx && g_noalloc_used < kNoAllocCache)
    g_noalloc_cache[g_noalloc_used++] = {dev, ctx, static_cast<unsigned long long*>(ptr)};
  *out = static_cast<unsigned long long*>(ptr);
  return cudaSuccess;
}

}  // namespace

GB_EXPORT int awkward_ListArray64_getitem_jagged_apply_64_noalloc(
    int64_t* tooffsets, int64_t* tocarry, const int64_t* slicestarts, const int64_t* slicestops,
    int64_t sliceouterlen, const int64_t* sliceindex, int64_t sliceinnerlen,
    const int64_t* fromstarts, const int64_t* fromstops, int64_t contentlen,
    uint64_t invocation_index, uint64_t* err_code, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (sliceouterlen > kNoAllocMaxLists) return (int)cudaErrorInvalidValue;
  unsigned long long* tiles = nullptr;
  cudaError_t e = noalloc_tiles_address(&tiles);
  if (e != cudaSuccess) return (int)e;
  if (sliceouterlen <= 0) return (int)cudaMemsetAsync(tooffsets, 0, sizeof(int64_t), s);
  const long long nt = tile_count(sliceouterlen);
  e = cudaMemsetAsync(tiles, 0, (size_t)(nt + 1) * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return (int)e;
  ScanTiles st;
  st.ticket = tiles;
  st.status = tiles + 1;
  jagged_apply_kernel<int64_t><<<(unsigned)nt, kTileBlock, 0, s>>>(
      tooffsets, tocarry, slicestarts, slicestops, sliceouterlen, sliceindex, sliceinnerlen,
      fromstarts, fromstops, contentlen, st, invocation_index, err_code);
  return (int)cudaGetLastError();
}
