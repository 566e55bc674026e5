// nonlocal.cu -- reductions above the innermost axis (non-local) and through
// option types: the bookkeeping kernels awkward runs between two segmented
// reducer launches.
//
//   ListOffsetArray   reduce_nonlocal_maxcount_offsetscopy_64   (.cpp:7-21)
//                     reduce_nonlocal_preparenext_64            (.cpp:7-57)
//                     reduce_nonlocal_outstartsstops_64         (.cpp:10-44)
//                     reduce_nonlocal_nextshifts_64             (.cpp:7-43)
//                     reduce_local_nextparents_64 (32/U32/64)   (.cpp:14-27)
//                     local_preparenext_64                      (.cpp:11-26)
//   RegularArray      reduce_local_nextparents_64               (.cpp:14-26)
//                     reduce_nonlocal_preparenext_64            (.cpp:7-36)
//   IndexedArray      reduce_next_64 (32/U32/64)                (.cpp:7-30)
//                     reduce_next_fix_offsets_64                (.cpp:7-17)
//                     reduce_next_nonlocal_nextshifts[_fromshifts]_64
//                     local_preparenext_64                      (.cpp:7-31)
//   ByteMaskedArray   reduce_next_64                            (.cpp:7-32)
//                     reduce_next_nonlocal_nextshifts[_fromshifts]_64
//   Content           getitem_next_missing_jagged_getmaskstartstop (.cpp:7-28)
//   MaskedArray       getitem_next_jagged_project (32/U32/64)   (.cpp:7-25)
//
// The non-local "preparenext" regroups the elements of every outer bin column
// by column: next bin b*maxcount + col lists column `col` of each row of bin b
// that reaches it, rows in order.  That is a stable sort of the elements by
// the key b*maxcount + col (they arrive in row-major order), done here with
// the library's LSD radix sort; the next offsets are the lower bounds of every
// key in the sorted keys.  "nextshifts" needs, for element (row, col), the
// rows of its bin before `row` that end at or before column `col`: that is
// (row - first row of the bin) minus the element's rank among its key's
// elements, which the same sort gives as (sorted position - lower bound).
//
// The option-type kernels are stream compactions (valid entries get
// consecutive outputs): one pass over tiles of 4096 entries with warp ballots
// and a decoupled look-back for the tile's prefix.
//
// Offsets are taken to be non-decreasing, as awkward builds them; with other
// offsets the kernels stay inside the buffers they are given but their output
// is not defined.
#include "list_tile.cuh"
#include "radix_sort.cuh"

using namespace gb;

namespace {

constexpr int kBlock = 256;

long long grid_cap() { return (long long)device_sm_count() * 16; }
unsigned grid_for(long long work, long long per_block) {
  long long g = (work + per_block - 1) / per_block;
  const long long cap = grid_cap();
  if (g < 1) g = 1;
  return (unsigned)(g < cap ? g : cap);
}

// Read `n` int64 device words (each from its own address) back to the host.
cudaError_t read_words(const long long* const* srcs, long long* dst, int n, cudaStream_t s) {
  for (int i = 0; i < n; i++) {
    cudaError_t e = cudaMemcpyAsync(dst + i, srcs[i], sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
  }
  return cudaStreamSynchronize(s);
}

// ------------------------------------------------ maxcount and offsets copy
__global__ void __launch_bounds__(kBlock)
    maxcount_offsetscopy_kernel(long long* maxcount, long long* offsetscopy,
                                const long long* __restrict__ offsets, long long length) {
  __shared__ long long s_max[kBlock / 32];
  long long best = 0;
  for (long long i = blockIdx.x * (long long)kBlock + threadIdx.x; i < length;
       i += (long long)gridDim.x * kBlock) {
    const long long hi = offsets[i + 1];
    const long long c = hi - offsets[i];
    if (c > best) best = c;
    offsetscopy[i + 1] = hi;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) offsetscopy[0] = offsets[0];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const long long o = __shfl_xor_sync(0xffffffffu, best, d);
    best = o > best ? o : best;
  }
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kBlock / 32; w++) best = s_max[w] > best ? s_max[w] : best;
    if (best > 0) atomicMax(maxcount, best);
  }
}

// ------------------------------------------- non-local regrouping: the keys
__device__ __forceinline__ long long upper_bound_ll(const long long* a, long long lo, long long hi,
                                                   long long x) {
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// For every element (row, col) of the rows [R0, R1) -- slot = its offset
// minus E0 -- key = bin(row)*maxcount + col (nbins = outlength*maxcount for
// columns at or past maxcount, which sort last and are dropped), value = the
// element's offset.  With `rib`, also the row's position inside its bin.
__global__ void __launch_bounds__(kTileBlock)
    nonlocal_keys_kernel(const long long* __restrict__ offsets,
                         const long long* __restrict__ outer_offsets, long long outlength,
                         long long maxcount, long long R0, long long R1, long long E0, long long n,
                         unsigned long long* __restrict__ keys, long long* __restrict__ vals,
                         long long* __restrict__ rib) {
  __shared__ TileSmem sm;
  __shared__ long long s_bin[kTileLists];
  __shared__ long long s_rib[kTileLists];
  const long long nrows = R1 - R0;
  const unsigned long long nbins = (unsigned long long)(outlength * maxcount);
  for (long long l0 = (long long)blockIdx.x * kTileLists; l0 < nrows;
       l0 += (long long)gridDim.x * kTileLists) {
    const long long total =
        stage_lists(sm, l0, nrows, [&](long long l) { return offsets[R0 + l + 1] - offsets[R0 + l]; });
    for (int r = threadIdx.x; r < kTileLists; r += kTileBlock) {
      const long long row = R0 + l0 + r;
      if (row < R1) {
        // the bin of a row: last b with outer_offsets[b] <= row (empty bins skipped)
        const long long b = upper_bound_ll(outer_offsets, 0, outlength + 1, row) - 1;
        s_bin[r] = b;
        s_rib[r] = row - outer_offsets[b];
      }
    }
    __syncthreads();
    tile_for_each_slot(sm, total, [&](long long q, int r) {
      const long long row = R0 + l0 + r;
      const long long col = q - sm.loc[r];
      const long long e = offsets[row] + col;
      const long long slot = e - E0;
      if (slot < 0 || slot >= n) return;
      keys[slot] = col < maxcount ? (unsigned long long)(s_bin[r] * maxcount + col) : nbins;
      vals[slot] = e;
      if (rib != nullptr) rib[slot] = s_rib[r];
    });
    __syncthreads();
  }
}

// distincts[j] = j when next bin j is not empty, else -1 (j < distinctslen);
// *maxnextparents = the last non-empty next bin, or -1.
__global__ void __launch_bounds__(kBlock)
    distincts_kernel(long long* __restrict__ distincts, long long distinctslen,
                     const long long* __restrict__ lb, long long nbins,
                     const unsigned long long* __restrict__ skeys, long long* maxnextparents) {
  for (long long j = blockIdx.x * (long long)kBlock + threadIdx.x; j < distinctslen;
       j += (long long)gridDim.x * kBlock)
    distincts[j] = (j < nbins && lb[j + 1] > lb[j]) ? j : -1;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const long long m = nbins > 0 ? lb[nbins] : 0;
    *maxnextparents = m > 0 ? (long long)skeys[m - 1] : -1;
  }
}

// nextcarry[p] = the sorted values of the kept elements (p < min(kept, nextlen)).
__global__ void __launch_bounds__(kBlock)
    gather_kept_kernel(long long* __restrict__ nextcarry, long long nextlen,
                       const unsigned long long* __restrict__ skeys,
                       const long long* __restrict__ svals, long long n, unsigned long long nbins) {
  const long long m = n < nextlen ? n : nextlen;
  for (long long p = blockIdx.x * (long long)kBlock + threadIdx.x; p < m;
       p += (long long)gridDim.x * kBlock)
    if (skeys[p] < nbins) nextcarry[p] = svals[p];
}

// missing[e] = (row - first row of its bin) - (rank of e among its key's elements).
__global__ void __launch_bounds__(kBlock)
    missing_kernel(long long* __restrict__ missing, const unsigned long long* __restrict__ skeys,
                   const long long* __restrict__ svals, const long long* __restrict__ lb,
                   const long long* __restrict__ rib, long long n, unsigned long long nbins,
                   long long E0) {
  for (long long p = blockIdx.x * (long long)kBlock + threadIdx.x; p < n;
       p += (long long)gridDim.x * kBlock) {
    const unsigned long long k = skeys[p];
    if (k >= nbins) continue;
    const long long e = svals[p];
    missing[e] = rib[e - E0] - (p - lb[k]);
  }
}

__global__ void __launch_bounds__(kBlock)
    nextshifts_gather_kernel(long long* __restrict__ nextshifts, const long long* __restrict__ missing,
                             const long long* __restrict__ nextcarry, long long nextlen,
                             long long lo, long long hi) {
  for (long long j = blockIdx.x * (long long)kBlock + threadIdx.x; j < nextlen;
       j += (long long)gridDim.x * kBlock) {
    const long long e = nextcarry[j];
    if (e >= lo && e < hi) nextshifts[j] = missing[e];
  }
}

// hist[c] += rows of [r0, r1) with count c (0 <= c < maxcount); warp-aggregated.
__global__ void __launch_bounds__(kBlock)
    count_hist_kernel(long long* __restrict__ hist, const long long* __restrict__ offsets, long long r0,
                      long long r1, long long maxcount) {
  const long long span = r1 - r0;
  const long long stride = (long long)gridDim.x * kBlock;
  for (long long base = blockIdx.x * (long long)kBlock; base < span; base += stride) {
    const long long i = base + threadIdx.x;
    long long c = -1;
    if (i < span) c = offsets[r0 + i + 1] - offsets[r0 + i];
    const bool use = c >= 0 && c < maxcount;
    const unsigned long long key = use ? (unsigned long long)c : ~0ull;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const unsigned lower = peers & ((1u << (threadIdx.x & 31)) - 1u);
    if (use && lower == 0) atomicAdd(reinterpret_cast<unsigned long long*>(hist + c),
                                     (unsigned long long)__popc(peers));
  }
}

// ------------------------------------------------------------ outstartsstops
__global__ void __launch_bounds__(kBlock)
    outstartsstops_init_kernel(long long* outstarts, long long* outstops, long long nsub,
                               long long maxcount) {
  for (long long k = blockIdx.x * (long long)kBlock + threadIdx.x; k < nsub;
       k += (long long)gridDim.x * kBlock) {
    outstarts[k] = k * maxcount;
    outstops[k] = k * maxcount;
  }
}
__global__ void __launch_bounds__(kBlock)
    outstops_kernel(long long* outstops, const long long* __restrict__ distincts, long long len,
                    long long maxcount, long long outlength) {
  for (long long i = blockIdx.x * (long long)kBlock + threadIdx.x; i < len;
       i += (long long)gridDim.x * kBlock) {
    if (distincts[i] == -1) continue;
    const long long k = maxcount > 0 ? i / maxcount : 0;
    if (k < outlength) atomicMax(outstops + k, i + 1);
  }
}
__global__ void __launch_bounds__(kBlock) zero2_kernel(long long* a, long long* b, long long n) {
  for (long long k = blockIdx.x * (long long)kBlock + threadIdx.x; k < n;
       k += (long long)gridDim.x * kBlock)
    a[k] = b[k] = 0;
}

// ------------------------------------------------------ local next parents
template <class C>
__global__ void __launch_bounds__(kTileBlock)
    local_nextparents_kernel(C* __restrict__ nextparents, const C* __restrict__ offsets,
                             long long length, long long limit) {
  __shared__ TileSmem sm;
  const long long base = (long long)offsets[0];
  for (long long l0 = (long long)blockIdx.x * kTileLists; l0 < length;
       l0 += (long long)gridDim.x * kTileLists) {
    const long long total = stage_lists(
        sm, l0, length, [&](long long l) { return (long long)offsets[l + 1] - (long long)offsets[l]; });
    tile_for_each_slot(sm, total, [&](long long q, int r) {
      const long long i = l0 + r;
      const long long j = (long long)offsets[i] - base + (q - sm.loc[r]);
      if (j >= 0 && j < limit) nextparents[j] = (C)i;
    });
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kBlock)
    regular_nextparents_kernel(long long* __restrict__ nextparents, long long size, long long n) {
  for (long long k = blockIdx.x * (long long)kBlock + threadIdx.x; k < n;
       k += (long long)gridDim.x * kBlock)
    nextparents[k] = k / size;
}

// ------------------------------------------- RegularArray non-local regroup
// Output slot (offsets[b] - offsets[0])*size + j*rows_b + (i - offsets[b])
// holds i*size + j for every row i of bin b and column j.
__global__ void __launch_bounds__(kTileBlock)
    regular_preparenext_kernel(long long* __restrict__ nextcarry, const long long* __restrict__ offsets,
                               long long size, long long outlength, long long limit) {
  __shared__ TileSmem sm;
  const long long o0 = offsets[0];
  for (long long l0 = (long long)blockIdx.x * kTileLists; l0 < outlength;
       l0 += (long long)gridDim.x * kTileLists) {
    const long long total = stage_lists(
        sm, l0, outlength, [&](long long b) { return (offsets[b + 1] - offsets[b]) * size; });
    tile_for_each_slot(sm, total, [&](long long q, int r) {
      const long long b = l0 + r;
      const long long rs = offsets[b], rows = offsets[b + 1] - rs;
      const long long local = q - sm.loc[r];
      const long long j = local / rows, i = rs + (local - j * rows);
      const long long slot = (rs - o0) * size + local;
      if (slot >= 0 && slot < limit) nextcarry[slot] = i * size + j;
    });
    __syncthreads();
  }
}
__global__ void __launch_bounds__(kBlock)
    regular_nextoffsets_kernel(long long* __restrict__ nextoffsets, const long long* __restrict__ offsets,
                               long long size, long long nbins) {
  const long long o0 = offsets[0];
  for (long long e = blockIdx.x * (long long)kBlock + threadIdx.x; e < nbins;
       e += (long long)gridDim.x * kBlock) {
    const long long b = e / size, j = e - b * size;
    const long long rs = offsets[b], rows = offsets[b + 1] - rs;
    nextoffsets[e + 1] = (rs - o0) * size + (j + 1) * rows;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) nextoffsets[0] = 0;
}

// --------------------------------------------- IndexedArray local prepare
__global__ void __launch_bounds__(kTileBlock)
    indexed_local_preparenext_kernel(long long* __restrict__ tocarry,
                                     const long long* __restrict__ offsets,
                                     const long long* __restrict__ nextoffsets, long long outlength) {
  __shared__ TileSmem sm;
  for (long long l0 = (long long)blockIdx.x * kTileLists; l0 < outlength;
       l0 += (long long)gridDim.x * kTileLists) {
    const long long total =
        stage_lists(sm, l0, outlength, [&](long long b) { return offsets[b + 1] - offsets[b]; });
    tile_for_each_slot(sm, total, [&](long long q, int r) {
      const long long b = l0 + r;
      const long long local = q - sm.loc[r];
      const long long k = nextoffsets[b] + local;
      tocarry[offsets[b] + local] = k < nextoffsets[b + 1] ? k : -1;
    });
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kBlock)
    fix_offsets_kernel(long long* __restrict__ outoffsets, const long long* __restrict__ starts,
                       long long n, long long last) {
  for (long long i = blockIdx.x * (long long)kBlock + threadIdx.x; i <= n;
       i += (long long)gridDim.x * kBlock)
    outoffsets[i] = i < n ? starts[i] : last;
}

// ------------------------------------------------------------- compaction
constexpr int kCSteps = 16;                     // steps of 32 entries per warp
constexpr int kCWarps = kBlock / 32;
constexpr int kCWarpSpan = kCSteps * 32;        // 512 consecutive entries per warp
constexpr int kCTile = kCWarps * kCWarpSpan;    // 4096 entries per tile

// kMaskStartStop: Content_getitem_next_missing_jagged_getmaskstartstop;
// kProject: MaskedArray_getitem_next_jagged_project.
enum CompactMode { kReduceNext = 0, kNextShifts = 1, kMaskStartStop = 2, kProject = 3 };

template <class T, bool MASKED, int MODE, bool FROMSHIFTS>
struct CompactArgs {
  const T* index;          // IndexedArray: entry valid when index >= 0
  const int8_t* mask;      // ByteMaskedArray: valid when (mask != 0) == validwhen
  bool validwhen;
  const long long* offsets;  // reduce_next: bins
  long long outlength;
  long long* nextcarry;
  long long* nextoffsets;
  long long* outindex;
  long long* nextshifts;
  const long long* shifts;
  const long long* offsets_in;  // kMaskStartStop
  long long* mask_out;
  const long long* starts_in;   // kProject
  const long long* stops_in;
  long long* starts_out;        // kMaskStartStop, kProject
  long long* stops_out;
  long long e0, e1;  // entries [e0, e1)
};

template <class T, bool MASKED, int MODE, bool FROMSHIFTS>
__device__ __forceinline__ bool entry_valid(const CompactArgs<T, MASKED, MODE, FROMSHIFTS>& a,
                                            long long e) {
  if constexpr (MASKED) return (a.mask[e] != 0) == a.validwhen;
  else return (long long)a.index[e] >= 0;
}

template <class T, bool MASKED, int MODE, bool FROMSHIFTS>
__global__ void __launch_bounds__(kBlock)
    compact_kernel(CompactArgs<T, MASKED, MODE, FROMSHIFTS> a, ScanTiles st, uint64_t inv,
                   uint64_t* err) {
  __shared__ unsigned s_mask[kCWarps][kCSteps];
  __shared__ long long s_wbase[kCWarps + 1];
  __shared__ long long s_tile, s_prefix;
  if (threadIdx.x == 0) s_tile = (long long)atomicAdd(st.ticket, 1ull);
  __syncthreads();
  const long long tile = s_tile;
  const long long t0 = a.e0 + tile * kCTile;
  const long long t1 = t0 + kCTile < a.e1 ? t0 + kCTile : a.e1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long wb = t0 + (long long)warp * kCWarpSpan;
  unsigned m[kCSteps];
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < kCSteps; j++) {
    const long long e = wb + j * 32 + lane;
    const bool v = e < t1 && entry_valid(a, e);
    m[j] = __ballot_sync(0xffffffffu, v);
    cnt += __popc(m[j]);
    if (lane == 0) s_mask[warp][j] = m[j];
  }
  if (lane == 0) s_wbase[warp] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long run = 0;
    for (int w = 0; w < kCWarps; w++) {
      const long long c = s_wbase[w];
      s_wbase[w] = run;
      run += c;
    }
    s_wbase[kCWarps] = run;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const long long p = lookback_exclusive(st, tile, s_wbase[kCWarps], inv, err, GB_MSG_TIMEOUT);
    if (threadIdx.x == 0) s_prefix = p;
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  long long run = s_prefix + s_wbase[warp];
#pragma unroll
  for (int j = 0; j < kCSteps; j++) {
    const long long e = wb + j * 32 + lane;
    if (e < t1) {
      const bool v = (m[j] >> lane) & 1u;
      const long long k = run + __popc(m[j] & lt);  // valid entries before e
      if constexpr (MODE == kReduceNext) {
        if (v) {
          a.nextcarry[k] = MASKED ? e : (long long)a.index[e];
          a.outindex[e] = k;
        } else {
          a.outindex[e] = -1;
        }
      } else if constexpr (MODE == kNextShifts) {
        if (v) a.nextshifts[k] = (FROMSHIFTS ? a.shifts[e] : 0ll) + (e - k);
      } else if constexpr (MODE == kMaskStartStop) {
        a.starts_out[e] = a.offsets_in[k];
        a.mask_out[e] = v ? e : -1;
        a.stops_out[e] = a.offsets_in[k + (v ? 1 : 0)];
      } else {
        if (v) {
          a.starts_out[k] = a.starts_in[e];
          a.stops_out[k] = a.stops_in[e];
        }
      }
    }
    run += __popc(m[j]);
  }
  if constexpr (MODE == kReduceNext) {
    // next offsets of the bins that end inside this tile: (t0, t1], and
    // [t0, t1] for the first tile (bins ending where the entries begin)
    __shared__ long long s_blo, s_bhi;
    const long long* ends = a.offsets + 1;
    if (threadIdx.x == 0) {
      long long lo = 0, hi = a.outlength;
      const long long lim = tile == 0 ? t0 - 1 : t0;  // first bin with end > lim
      while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (ends[mid] <= lim) lo = mid + 1;
        else hi = mid;
      }
      s_blo = lo;
      hi = a.outlength;
      while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (ends[mid] <= t1) lo = mid + 1;
        else hi = mid;
      }
      s_bhi = lo;
      if (tile == 0) a.nextoffsets[0] = 0;
    }
    __syncthreads();
    for (long long b = s_blo + threadIdx.x; b < s_bhi; b += kBlock) {
      long long L = ends[b] - t0;  // entries of this tile before the bin's end
      if (L < 0) L = 0;
      long long c;
      const int w = (int)(L / kCWarpSpan);
      if (w >= kCWarps) {
        c = s_wbase[kCWarps];
      } else {
        const int rem = (int)(L - (long long)w * kCWarpSpan);
        const int jj = rem >> 5, l = rem & 31;
        c = s_wbase[w];
        for (int j = 0; j < jj; j++) c += __popc(s_mask[w][j]);
        c += __popc(s_mask[w][jj] & ((1u << l) - 1u));
      }
      a.nextoffsets[b + 1] = s_prefix + c;
    }
  }
}

template <class T, bool MASKED, int MODE, bool FROMSHIFTS>
cudaError_t launch_compact(CompactArgs<T, MASKED, MODE, FROMSHIFTS> a, uint64_t inv, uint64_t* err,
                           cudaStream_t s) {
  long long ntiles = (a.e1 - a.e0 + kCTile - 1) / kCTile;
  if (MODE == kReduceNext) {
    if (ntiles < 1) ntiles = 1;  // the bins still get their (zero) offsets
  } else if (ntiles < 1) {
    return cudaSuccess;
  }
  ScanTiles st;
  void* base = nullptr;
  cudaError_t e = scan_tiles_alloc(&st, &base, ntiles, s);
  if (e != cudaSuccess) return e;
  compact_kernel<T, MASKED, MODE, FROMSHIFTS><<<(unsigned)ntiles, kBlock, 0, s>>>(a, st, inv, err);
  e = cudaGetLastError();
  cudaError_t f = scratch_free(base, s);
  return e != cudaSuccess ? e : f;
}

// reduce_next over bins: entries [offsets[0], offsets[outlength]).
template <class T, bool MASKED>
cudaError_t launch_reduce_next(long long* nextcarry, long long* nextoffsets, long long* outindex,
                               const T* index, const int8_t* mask, bool validwhen,
                               const long long* offsets, long long outlength, uint64_t inv,
                               uint64_t* err, cudaStream_t s) {
  if (nextoffsets == nullptr) return cudaSuccess;
  CompactArgs<T, MASKED, kReduceNext, false> a{};
  a.index = index;
  a.mask = mask;
  a.validwhen = validwhen;
  a.offsets = offsets;
  a.outlength = outlength < 0 ? 0 : outlength;
  a.nextcarry = nextcarry;
  a.nextoffsets = nextoffsets;
  a.outindex = outindex;
  if (a.outlength > 0) {
    const long long* srcs[2] = {offsets, offsets + a.outlength};
    long long w[2];
    cudaError_t e = read_words(srcs, w, 2, s);
    if (e != cudaSuccess) return e;
    a.e0 = w[0];
    a.e1 = w[1] > w[0] ? w[1] : w[0];
  }
  return launch_compact(a, inv, err, s);
}

template <class T, bool MASKED, bool FROMSHIFTS>
cudaError_t launch_nextshifts(long long* nextshifts, const T* index, const int8_t* mask,
                              bool validwhen, long long length, const long long* shifts,
                              uint64_t inv, uint64_t* err, cudaStream_t s) {
  CompactArgs<T, MASKED, kNextShifts, FROMSHIFTS> a{};
  a.index = index;
  a.mask = mask;
  a.validwhen = validwhen;
  a.nextshifts = nextshifts;
  a.shifts = shifts;
  a.e0 = 0;
  a.e1 = length < 0 ? 0 : length;
  return launch_compact(a, inv, err, s);
}

// ------------------------------------------------- non-local regrouping host
struct Regroup {
  long long R0 = 0, R1 = 0, E0 = 0, E1 = 0, n = 0;
  unsigned long long nbins = 0;
  void* scratch = nullptr;
  unsigned long long* skeys = nullptr;
  long long* svals = nullptr;
  long long* rib = nullptr;  // row position inside its bin, by slot
};

// Keys, values (and row positions) of the elements of the bins, sorted.
cudaError_t regroup(Regroup& g, const long long* offsets, long long length,
                    const long long* outer_offsets, long long outlength, long long maxcount,
                    bool with_rib, uint64_t inv, uint64_t* err, cudaStream_t s) {
  {
    const long long* srcs[2] = {outer_offsets, outer_offsets + outlength};
    long long w[2];
    cudaError_t e = read_words(srcs, w, 2, s);
    if (e != cudaSuccess) return e;
    // rows outside [0, length] have no offsets to read
    const long long lim = length > 0 ? length : 0;
    g.R0 = w[0] < 0 ? 0 : w[0] > lim ? lim : w[0];
    g.R1 = w[1] < g.R0 ? g.R0 : w[1] > lim ? lim : w[1];
  }
  {
    const long long* srcs[2] = {offsets + g.R0, offsets + g.R1};
    long long w[2];
    cudaError_t e = read_words(srcs, w, 2, s);
    if (e != cudaSuccess) return e;
    g.E0 = w[0];
    g.E1 = w[1] > w[0] ? w[1] : w[0];
  }
  g.n = g.E1 - g.E0;
  g.nbins = (unsigned long long)(outlength * maxcount);
  if (g.n <= 0) return cudaSuccess;
  const size_t n = (size_t)g.n;
  cudaError_t e = scratch_alloc(&g.scratch, sizeof(long long) * n * (with_rib ? 5 : 4), s);
  if (e != cudaSuccess) return e;
  unsigned long long* keys = static_cast<unsigned long long*>(g.scratch);
  long long* vals = reinterpret_cast<long long*>(keys + n);
  g.skeys = reinterpret_cast<unsigned long long*>(vals + n);
  g.svals = reinterpret_cast<long long*>(g.skeys + n);
  g.rib = with_rib ? g.svals + n : nullptr;
  // slots no row covers (possible only with decreasing offsets) sort last
  e = cudaMemsetAsync(keys, 0xff, sizeof(long long) * n, s);
  if (e != cudaSuccess) return e;
  const long long nrows = g.R1 - g.R0;
  if (nrows > 0) {
    const long long tiles = (nrows + kTileLists - 1) / kTileLists;
    const long long cap = grid_cap();
    nonlocal_keys_kernel<<<(unsigned)(tiles < cap ? tiles : cap), kTileBlock, 0, s>>>(
        offsets, outer_offsets, outlength, maxcount, g.R0, g.R1, g.E0, g.n, keys, vals, g.rib);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  // keys < 2^bits except the uncovered-slot fill, which only ever ranks last
  return radix_sort_pairs(keys, vals, g.skeys, g.svals, g.n, bit_length(g.nbins), inv, err, s);
}

}  // namespace

// ===================================================================== entries

GB_EXPORT int awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64(
    int64_t* maxcount, int64_t* offsetscopy, const int64_t* offsets, int64_t length,
    uint64_t invocation_index, uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  cudaStream_t s = (cudaStream_t)stream;
  if (maxcount != nullptr) {
    cudaError_t e = cudaMemsetAsync(maxcount, 0, sizeof(int64_t), s);
    if (e != cudaSuccess) return (int)e;
  }
  if (offsets == nullptr || offsetscopy == nullptr || maxcount == nullptr) return (int)cudaSuccess;
  const long long n = length < 0 ? 0 : length;
  maxcount_offsetscopy_kernel<<<grid_for(n, kBlock), kBlock, 0, s>>>(
      (long long*)maxcount, (long long*)offsetscopy, (const long long*)offsets, n);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_ListOffsetArray_reduce_nonlocal_preparenext_64(
    int64_t* nextcarry, int64_t* nextoffsets, int64_t nextlen, int64_t* maxnextparents,
    int64_t* distincts, int64_t distinctslen, int64_t* offsetscopy, const int64_t* offsets,
    int64_t length, const int64_t* outer_offsets, int64_t outlength, int64_t maxcount,
    uint64_t invocation_index, uint64_t* err_code, void* stream) {
  (void)offsetscopy;
  cudaStream_t s = (cudaStream_t)stream;
  const long long nb = (outlength > 0 && maxcount > 0) ? (long long)outlength * maxcount : 0;
  Regroup g;
  cudaError_t e = cudaSuccess;
  if (nb > 0)
    e = regroup(g, (const long long*)offsets, length, (const long long*)outer_offsets, outlength,
                maxcount, false, invocation_index, err_code, s);
  void* lbmem = nullptr;
  long long* lb = nullptr;
  if (e == cudaSuccess) e = scratch_alloc(&lbmem, sizeof(long long) * (size_t)(nb + 1), s);
  if (e == cudaSuccess) {
    lb = static_cast<long long*>(lbmem);
    if (g.n > 0) e = fill_lower_bounds(g.skeys, g.n, lb, nb + 1, s);
    else e = cudaMemsetAsync(lb, 0, sizeof(long long) * (size_t)(nb + 1), s);
  }
  if (e == cudaSuccess && nextoffsets != nullptr)
    e = cudaMemcpyAsync(nextoffsets, lb, sizeof(long long) * (size_t)(nb + 1),
                        cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) {
    const long long dl = distinctslen > 0 ? distinctslen : 0;
    distincts_kernel<<<grid_for(dl, kBlock), kBlock, 0, s>>>((long long*)distincts, dl, lb, nb,
                                                           g.skeys, (long long*)maxnextparents);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && g.n > 0 && nextlen > 0) {
    gather_kept_kernel<<<grid_for(g.n, kBlock), kBlock, 0, s>>>((long long*)nextcarry, nextlen,
                                                              g.skeys, g.svals, g.n, g.nbins);
    e = cudaGetLastError();
  }
  if (lbmem != nullptr) {
    cudaError_t f = scratch_free(lbmem, s);
    if (e == cudaSuccess) e = f;
  }
  if (g.scratch != nullptr) {
    cudaError_t f = scratch_free(g.scratch, s);
    if (e == cudaSuccess) e = f;
  }
  return (int)e;
}

GB_EXPORT int awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64(
    int64_t* outstarts, int64_t* outstops, const int64_t* distincts, int64_t lendistincts,
    int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  cudaStream_t s = (cudaStream_t)stream;
  if (outlength <= 0) return (int)cudaSuccess;
  if (lendistincts <= 0) {
    zero2_kernel<<<grid_for(outlength, kBlock), kBlock, 0, s>>>((long long*)outstarts,
                                                              (long long*)outstops, outlength);
    return (int)cudaGetLastError();
  }
  const long long M = lendistincts / outlength;
  // sublists start at multiples of maxcount (all entries form one when it is 0)
  long long nsub = M > 0 ? (lendistincts + M - 1) / M : 1;
  if (nsub > outlength) nsub = outlength;
  outstartsstops_init_kernel<<<grid_for(nsub, kBlock), kBlock, 0, s>>>(
      (long long*)outstarts, (long long*)outstops, nsub, M);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  outstops_kernel<<<grid_for(lendistincts, kBlock), kBlock, 0, s>>>(
      (long long*)outstops, (const long long*)distincts, lendistincts, M, nsub);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64(
    int64_t* nummissing, int64_t* missing, int64_t* nextshifts, const int64_t* offsets,
    int64_t length, const int64_t* starts, const int64_t* outer_offsets, int64_t outlength,
    int64_t maxcount, int64_t nextlen, const int64_t* nextcarry, uint64_t invocation_index,
    uint64_t* err_code, void* stream) {
  (void)starts;
  cudaStream_t s = (cudaStream_t)stream;
  if (outlength <= 0) return (int)cudaSuccess;  // nothing written, nothing to gather
  const long long M = maxcount > 0 ? maxcount : 0;
  const long long nb = outlength * M;
  Regroup g;
  cudaError_t e = cudaSuccess;
  void* lbmem = nullptr;
  if (nb > 0) {
    e = regroup(g, (const long long*)offsets, length, (const long long*)outer_offsets, outlength,
                M, true, invocation_index, err_code, s);
    if (e == cudaSuccess && g.n > 0) {
      e = scratch_alloc(&lbmem, sizeof(long long) * (size_t)(nb + 1), s);
      if (e == cudaSuccess) e = fill_lower_bounds(g.skeys, g.n, (long long*)lbmem, nb + 1, s);
      if (e == cudaSuccess) {
        missing_kernel<<<grid_for(g.n, kBlock), kBlock, 0, s>>>(
            (long long*)missing, g.skeys, g.svals, (const long long*)lbmem, g.rib, g.n, g.nbins,
            g.E0);
        e = cudaGetLastError();
      }
    }
  } else {
    // no columns: still the element range for the gather below
    const long long* srcs[2] = {(const long long*)outer_offsets,
                                (const long long*)outer_offsets + outlength};
    long long w[2];
    e = read_words(srcs, w, 2, s);
    if (e == cudaSuccess) {
      const long long lim = length > 0 ? length : 0;
      const long long r0 = w[0] < 0 ? 0 : w[0] > lim ? lim : w[0];
      const long long r1 = w[1] < r0 ? r0 : w[1] > lim ? lim : w[1];
      const long long* srcs2[2] = {(const long long*)offsets + r0, (const long long*)offsets + r1};
      long long v[2];
      e = read_words(srcs2, v, 2, s);
      g.E0 = v[0];
      g.E1 = v[1] > v[0] ? v[1] : v[0];
    }
  }
  if (e == cudaSuccess && nextlen > 0) {
    nextshifts_gather_kernel<<<grid_for(nextlen, kBlock), kBlock, 0, s>>>(
        (long long*)nextshifts, (const long long*)missing, (const long long*)nextcarry, nextlen,
        g.E0, g.E1);
    e = cudaGetLastError();
  }
  // nummissing ends as the last bin's counts: rows with count <= c, c < maxcount
  if (e == cudaSuccess && M > 0 && nummissing != nullptr) {
    const long long* srcs[2] = {(const long long*)outer_offsets + outlength - 1,
                                (const long long*)outer_offsets + outlength};
    long long w[2];
    e = read_words(srcs, w, 2, s);
    void* hmem = nullptr;
    if (e == cudaSuccess) e = scratch_alloc(&hmem, sizeof(long long) * (size_t)(2 * (M + 1)), s);
    if (e == cudaSuccess) {
      long long* hist = static_cast<long long*>(hmem);
      long long* ex = hist + (M + 1);
      e = cudaMemsetAsync(hist, 0, sizeof(long long) * (size_t)(M + 1), s);
      if (e == cudaSuccess && w[1] > w[0]) {
        count_hist_kernel<<<grid_for(w[1] - w[0], kBlock), kBlock, 0, s>>>(
            hist, (const long long*)offsets, w[0], w[1], M);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = exclusive_scan_i64(hist, ex, M + 1, nullptr, invocation_index, err_code, s);
      // rows with count <= c = rows with count < c + 1
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(nummissing, ex + 1, sizeof(long long) * (size_t)M,
                            cudaMemcpyDeviceToDevice, s);
      cudaError_t f = scratch_free(hmem, s);
      if (e == cudaSuccess) e = f;
    }
  }
  if (lbmem != nullptr) {
    cudaError_t f = scratch_free(lbmem, s);
    if (e == cudaSuccess) e = f;
  }
  if (g.scratch != nullptr) {
    cudaError_t f = scratch_free(g.scratch, s);
    if (e == cudaSuccess) e = f;
  }
  return (int)e;
}

#define GB_LOCAL_NEXTPARENTS(NAME, C)                                                           \
  GB_EXPORT int NAME(C* nextparents, const C* offsets, int64_t length,                         \
                     int64_t nextparents_length, uint64_t invocation_index, uint64_t* err_code, \
                     void* stream) {                                                            \
    (void)invocation_index;                                                                     \
    (void)err_code;                                                                             \
    if (length <= 0) return (int)cudaSuccess;                                                   \
    const long long tiles = (length + kTileLists - 1) / kTileLists;                             \
    const long long cap = grid_cap();                                                           \
    local_nextparents_kernel<C><<<(unsigned)(tiles < cap ? tiles : cap), kTileBlock, 0,        \
                                  (cudaStream_t)stream>>>(nextparents, offsets, length,         \
                                                          nextparents_length);                  \
    return (int)cudaGetLastError();                                                             \
  }
GB_LOCAL_NEXTPARENTS(awkward_ListOffsetArray32_reduce_local_nextparents_64, int32_t)
GB_LOCAL_NEXTPARENTS(awkward_ListOffsetArrayU32_reduce_local_nextparents_64, uint32_t)
GB_LOCAL_NEXTPARENTS(awkward_ListOffsetArray64_reduce_local_nextparents_64, int64_t)

namespace {
__global__ void __launch_bounds__(kBlock)
    index_keys_kernel(unsigned long long* __restrict__ keys, long long* __restrict__ vals,
                      const long long* __restrict__ from, long long n, unsigned long long* range) {
  // range[0] = min, range[1] = max of the order keys (value ^ sign bit)
  unsigned long long lo = ~0ull, hi = 0;
  for (long long i = blockIdx.x * (long long)kBlock + threadIdx.x; i < n;
       i += (long long)gridDim.x * kBlock) {
    const unsigned long long k = (unsigned long long)from[i] ^ 0x8000000000000000ull;
    keys[i] = k;
    vals[i] = i;
    lo = k < lo ? k : lo;
    hi = k > hi ? k : hi;
  }
  atomicMin(range, lo);
  atomicMax(range + 1, hi);
}
__global__ void __launch_bounds__(kBlock)
    rebase_keys_kernel(unsigned long long* keys, long long n, const unsigned long long* range) {
  const unsigned long long lo = range[0];
  for (long long i = blockIdx.x * (long long)kBlock + threadIdx.x; i < n;
       i += (long long)gridDim.x * kBlock)
    keys[i] -= lo;
}
}  // namespace

GB_EXPORT int awkward_ListOffsetArray_local_preparenext_64(int64_t* tocarry,
                                                           const int64_t* fromindex,
                                                           int64_t length,
                                                           uint64_t invocation_index,
                                                           uint64_t* err_code, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (length <= 0) return (int)cudaSuccess;
  const size_t n = (size_t)length;
  void* mem = nullptr;
  cudaError_t e = scratch_alloc(&mem, sizeof(long long) * (3 * n + 2), s);
  if (e != cudaSuccess) return (int)e;
  unsigned long long* range = static_cast<unsigned long long*>(mem);
  unsigned long long* keys = range + 2;
  long long* vals = reinterpret_cast<long long*>(keys + n);
  unsigned long long* skeys = reinterpret_cast<unsigned long long*>(vals + n);
  const unsigned long long init[2] = {~0ull, 0ull};
  e = cudaMemcpyAsync(range, init, sizeof(init), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    index_keys_kernel<<<grid_for(length, kBlock), kBlock, 0, s>>>(keys, vals,
                                                                (const long long*)fromindex,
                                                                length, range);
    e = cudaGetLastError();
  }
  unsigned long long hr[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(hr, range, sizeof(hr), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) {
    rebase_keys_kernel<<<grid_for(length, kBlock), kBlock, 0, s>>>(keys, length, range);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = radix_sort_pairs(keys, vals, skeys, (long long*)tocarry, length, bit_length(hr[1] - hr[0]),
                         invocation_index, err_code, s);
  cudaError_t f = scratch_free(mem, s);
  return (int)(e != cudaSuccess ? e : f);
}

GB_EXPORT int awkward_RegularArray_reduce_local_nextparents_64(int64_t* nextparents, int64_t size,
                                                               int64_t length,
                                                               uint64_t invocation_index,
                                                               uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  if (size <= 0 || length <= 0) return (int)cudaSuccess;
  const long long n = (long long)size * length;
  regular_nextparents_kernel<<<grid_for(n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
      (long long*)nextparents, size, n);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_RegularArray_reduce_nonlocal_preparenext_64(
    int64_t* nextcarry, int64_t* nextoffsets, const int64_t* offsets, int64_t size, int64_t length,
    int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  cudaStream_t s = (cudaStream_t)stream;
  if (nextoffsets == nullptr) return (int)cudaSuccess;
  const long long nb = (outlength > 0 && size > 0) ? (long long)outlength * size : 0;
  regular_nextoffsets_kernel<<<grid_for(nb, kBlock), kBlock, 0, s>>>(
      (long long*)nextoffsets, (const long long*)offsets, size > 0 ? size : 1, nb);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nb == 0) return (int)e;
  const long long tiles = (outlength + kTileLists - 1) / kTileLists;
  const long long cap = grid_cap();
  regular_preparenext_kernel<<<(unsigned)(tiles < cap ? tiles : cap), kTileBlock, 0, s>>>(
      (long long*)nextcarry, (const long long*)offsets, size, outlength,
      length > 0 ? (long long)length * size : 0);
  return (int)cudaGetLastError();
}

#define GB_INDEXED_REDUCE_NEXT(NAME, T)                                                        \
  GB_EXPORT int NAME(int64_t* nextcarry, int64_t* nextoffsets, int64_t* outindex,             \
                     const T* index, const int64_t* offsets, int64_t outlength,               \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {           \
    return (int)launch_reduce_next<T, false>(                                                  \
        (long long*)nextcarry, (long long*)nextoffsets, (long long*)outindex, index, nullptr,  \
        false, (const long long*)offsets, outlength, invocation_index, err_code,               \
        (cudaStream_t)stream);                                                                 \
  }
GB_INDEXED_REDUCE_NEXT(awkward_IndexedArray32_reduce_next_64, int32_t)
GB_INDEXED_REDUCE_NEXT(awkward_IndexedArrayU32_reduce_next_64, uint32_t)
GB_INDEXED_REDUCE_NEXT(awkward_IndexedArray64_reduce_next_64, int64_t)

GB_EXPORT int awkward_ByteMaskedArray_reduce_next_64(int64_t* nextcarry, int64_t* nextoffsets,
                                                     int64_t* outindex, const int8_t* mask,
                                                     const int64_t* offsets, int64_t outlength,
                                                     bool validwhen, uint64_t invocation_index,
                                                     uint64_t* err_code, void* stream) {
  return (int)launch_reduce_next<int8_t, true>(
      (long long*)nextcarry, (long long*)nextoffsets, (long long*)outindex, nullptr, mask,
      validwhen, (const long long*)offsets, outlength, invocation_index, err_code,
      (cudaStream_t)stream);
}

GB_EXPORT int awkward_IndexedArray_reduce_next_fix_offsets_64(int64_t* outoffsets,
                                                              const int64_t* starts,
                                                              int64_t startslength,
                                                              int64_t outindexlength,
                                                              uint64_t invocation_index,
                                                              uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  const long long n = startslength > 0 ? startslength : 0;
  fix_offsets_kernel<<<grid_for(n + 1, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
      (long long*)outoffsets, (const long long*)starts, n, outindexlength);
  return (int)cudaGetLastError();
}

#define GB_INDEXED_NEXTSHIFTS(NAME, T)                                                          \
  GB_EXPORT int NAME(int64_t* nextshifts, const T* index, int64_t length,                       \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {            \
    return (int)launch_nextshifts<T, false, false>((long long*)nextshifts, index, nullptr,      \
                                                   false, length, nullptr, invocation_index,    \
                                                   err_code, (cudaStream_t)stream);             \
  }
#define GB_INDEXED_NEXTSHIFTS_FROM(NAME, T)                                                     \
  GB_EXPORT int NAME(int64_t* nextshifts, const T* index, int64_t length,                       \
                     const int64_t* shifts, uint64_t invocation_index, uint64_t* err_code,      \
                     void* stream) {                                                            \
    return (int)launch_nextshifts<T, false, true>((long long*)nextshifts, index, nullptr,       \
                                                  false, length, (const long long*)shifts,      \
                                                  invocation_index, err_code,                   \
                                                  (cudaStream_t)stream);                        \
  }
GB_INDEXED_NEXTSHIFTS(awkward_IndexedArray32_reduce_next_nonlocal_nextshifts_64, int32_t)
GB_INDEXED_NEXTSHIFTS(awkward_IndexedArrayU32_reduce_next_nonlocal_nextshifts_64, uint32_t)
GB_INDEXED_NEXTSHIFTS(awkward_IndexedArray64_reduce_next_nonlocal_nextshifts_64, int64_t)
GB_INDEXED_NEXTSHIFTS_FROM(awkward_IndexedArray32_reduce_next_nonlocal_nextshifts_fromshifts_64, int32_t)
GB_INDEXED_NEXTSHIFTS_FROM(awkward_IndexedArrayU32_reduce_next_nonlocal_nextshifts_fromshifts_64, uint32_t)
GB_INDEXED_NEXTSHIFTS_FROM(awkward_IndexedArray64_reduce_next_nonlocal_nextshifts_fromshifts_64, int64_t)

GB_EXPORT int awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64(
    int64_t* nextshifts, const int8_t* mask, int64_t length, bool valid_when,
    uint64_t invocation_index, uint64_t* err_code, void* stream) {
  return (int)launch_nextshifts<int8_t, true, false>((long long*)nextshifts, nullptr, mask,
                                                     valid_when, length, nullptr,
                                                     invocation_index, err_code,
                                                     (cudaStream_t)stream);
}
GB_EXPORT int awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64(
    int64_t* nextshifts, const int8_t* mask, int64_t length, bool valid_when,
    const int64_t* shifts, uint64_t invocation_index, uint64_t* err_code, void* stream) {
  return (int)launch_nextshifts<int8_t, true, true>((long long*)nextshifts, nullptr, mask,
                                                    valid_when, length, (const long long*)shifts,
                                                    invocation_index, err_code,
                                                    (cudaStream_t)stream);
}

GB_EXPORT int awkward_IndexedArray_local_preparenext_64(int64_t* tocarry, const int64_t* starts,
                                                        const int64_t* offsets,
                                                        const int64_t* nextoffsets,
                                                        int64_t outlength,
                                                        uint64_t invocation_index,
                                                        uint64_t* err_code, void* stream) {
  (void)starts;
  (void)invocation_index;
  (void)err_code;
  if (outlength <= 0) return (int)cudaSuccess;
  const long long tiles = (outlength + kTileLists - 1) / kTileLists;
  const long long cap = grid_cap();
  indexed_local_preparenext_kernel<<<(unsigned)(tiles < cap ? tiles : cap), kTileBlock, 0,
                                     (cudaStream_t)stream>>>(
      (long long*)tocarry, (const long long*)offsets, (const long long*)nextoffsets, outlength);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_Content_getitem_next_missing_jagged_getmaskstartstop(
    int64_t* index_in, int64_t* offsets_in, int64_t* mask_out, int64_t* starts_out,
    int64_t* stops_out, int64_t length, uint64_t invocation_index, uint64_t* err_code,
    void* stream) {
  CompactArgs<int64_t, false, kMaskStartStop, false> a{};
  a.index = index_in;
  a.offsets_in = (const long long*)offsets_in;
  a.mask_out = (long long*)mask_out;
  a.starts_out = (long long*)starts_out;
  a.stops_out = (long long*)stops_out;
  a.e0 = 0;
  a.e1 = length < 0 ? 0 : length;
  return (int)launch_compact(a, invocation_index, err_code, (cudaStream_t)stream);
}

#define GB_JAGGED_PROJECT(NAME, T)                                                              \
  GB_EXPORT int NAME(T* index, int64_t* starts_in, int64_t* stops_in, int64_t* starts_out,     \
                     int64_t* stops_out, int64_t length, uint64_t invocation_index,             \
                     uint64_t* err_code, void* stream) {                                        \
    CompactArgs<T, false, kProject, false> a{};                                                 \
    a.index = index;                                                                            \
    a.starts_in = (const long long*)starts_in;                                                  \
    a.stops_in = (const long long*)stops_in;                                                    \
    a.starts_out = (long long*)starts_out;                                                      \
    a.stops_out = (long long*)stops_out;                                                        \
    a.e0 = 0;                                                                                   \
    a.e1 = length < 0 ? 0 : length;                                                             \
    return (int)launch_compact(a, invocation_index, err_code, (cudaStream_t)stream);            \
  }
GB_JAGGED_PROJECT(awkward_MaskedArray32_getitem_next_jagged_project, int32_t)
GB_JAGGED_PROJECT(awkward_MaskedArrayU32_getitem_next_jagged_project, uint32_t)
GB_JAGGED_PROJECT(awkward_MaskedArray64_getitem_next_jagged_project, int64_t)
