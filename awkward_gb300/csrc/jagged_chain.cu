// jagged_chain.cu -- the two steps of jagged getitem that awkward performs with
// cupy array operations rather than kernels of its kernel specification:
//
//   jagged boolean mask -> jagged local index (src/awkward/_slicing.py:476-530:
//     localindex of the mask, boolean compaction of it, counts and their
//     cumsum for the new offsets);
//   content carry (NumpyArray._carry, src/awkward/contents/numpyarray.py:367-373:
//     content[carry], a gather).
//
// mask_to_index: one CTA per tile of kTileLists lists.  Thread-per-list counts
// of true entries are scanned across tiles (decoupled look-back) into the new
// offsets.  A tile of at most kMaskBits elements is first staged as a bitmap
// in shared memory (16-byte loads); the counts are popcounts of it, each
// thread lists its lists' true positions in rank order in shared memory, and
// the tile's positions are copied out coalesced (a tile with more than
// kMaskPos true entries writes them from the lists' threads directly).  A
// larger tile counts from global memory and then each warp walks a contiguous
// share of its elements 32 at a time, ranking the true entries with a ballot
// prefix and writing the local index (position within its list) of each at
// its rank.
#include "list_tile.cuh"
#include "mask_select.cuh"

using namespace gb;

namespace {

struct MaskTile {
  long long loc[kTileLists + 1];  // list offsets relative to the tile's first element
  long long base;
  int count;
};

// A tile whose mask bytes (plus the first byte's offset in its 16-byte line)
// fit kMaskBits is staged as a bitmap in shared memory; the positions of its
// true entries (when at most kMaskPos) are gathered there in rank order and
// copied out coalesced, or else written straight to global memory.
constexpr int kMaskPos = 8192;
struct MaskStage {
  unsigned bits[kMaskBits / 32];   // bit p: byte (tile's first byte - shift + p) is nonzero
  unsigned short pos[kMaskPos];    // position within its list of each true entry, by rank
};

__global__ void __launch_bounds__(kTileBlock, 6)
    mask_to_index_kernel(int64_t* __restrict__ tooffsets, int64_t* __restrict__ toindex,
                         const uint8_t* __restrict__ mask, const int64_t* __restrict__ offsets,
                         long long nlists, long long ntiles, ScanTiles st, uint64_t* err) {
  __shared__ TileSmem sm;
  __shared__ MaskTile t;
  __shared__ MaskStage ms;
  const long long tile = tile_claim(sm, st);
  const long long l0 = tile * kTileLists;
  const long long rem = nlists - l0;
  const int count = (int)(rem < kTileLists ? rem : kTileLists);
  const long long base = __ldg(offsets + l0);
  for (int i = threadIdx.x; i <= kTileLists; i += kTileBlock) {
    const int k = i < count ? i : count;
    t.loc[i] = __ldg(offsets + l0 + k) - base;
  }
  if (threadIdx.x == 0) {
    t.base = base;
    t.count = count;
  }
  __syncthreads();
  const long long total = t.loc[count];
  const uint8_t* p0 = mask + base;
  const int sh = (int)(reinterpret_cast<uintptr_t>(p0) & 15);
  const bool staged = total + sh <= kMaskBits;
  long long c[kTileLPT];
  if (staged) {
    // bitmap of the tile's bytes: 32 bytes per word, two aligned 16-byte loads
    // for words inside [p0, p0 + total), byte loads for the partial ends
    const int nbits = (int)total + sh;
    const uint8_t* a0 = p0 - sh;
    for (int w = threadIdx.x; w < (nbits + 31) >> 5; w += kTileBlock) {
      const int lo = 32 * w, hi = lo + 32;
      unsigned word = 0;
      if (lo >= sh && hi <= nbits) {
        const uint4 v0 = __ldg(reinterpret_cast<const uint4*>(a0 + lo));
        const uint4 v1 = __ldg(reinterpret_cast<const uint4*>(a0 + lo + 16));
        word = nonzero_bits16(v0) | nonzero_bits16(v1) << 16;
      } else {
        const int b0 = lo > sh ? lo : sh, b1 = hi < nbits ? hi : nbits;
        for (int b = b0; b < b1; b++) word |= (unsigned)(a0[b] != 0) << (b - lo);
      }
      ms.bits[w] = word;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kTileLPT; r++) {
      const int li = threadIdx.x * kTileLPT + r;
      c[r] = li < count ? bitmap_count(ms.bits, (int)t.loc[li] + sh, (int)t.loc[li + 1] + sh) : 0;
    }
  } else {
#pragma unroll
    for (int r = 0; r < kTileLPT; r++) {
      const int li = threadIdx.x * kTileLPT + r;
      long long n = 0;
      if (li < count)
        for (long long j = base + t.loc[li]; j < base + t.loc[li + 1]; j++) n += mask[j] != 0;
      c[r] = n;
    }
  }
  const long long prefix = tile_scan(sm, st, tile, c, 0, err);
  for (int li = threadIdx.x; li < kTileLists; li += kTileBlock)
    if (li < count) tooffsets[l0 + li] = prefix + sm.loc[li];
  if (tile == ntiles - 1 && threadIdx.x == 0) tooffsets[nlists] = prefix + sm.total;
  if (staged) {
    // each thread lists its lists' true entries in rank order, then the tile's
    // positions are copied out with consecutive threads on consecutive ranks
    const int ntrue = (int)sm.total;
    const bool gather = ntrue <= kMaskPos;
#pragma unroll
    for (int r = 0; r < kTileLPT; r++) {
      const int li = threadIdx.x * kTileLPT + r;
      if (li >= count || c[r] == 0) continue;
      const int a = (int)t.loc[li] + sh, b = (int)t.loc[li + 1] + sh;
      int o = (int)sm.loc[li];
      for (int w = a >> 5; w <= (b - 1) >> 5; w++) {
        unsigned word = ms.bits[w];
        if (w == a >> 5) word &= ~((1u << (a & 31)) - 1u);
        if (w == b >> 5) word &= (1u << (b & 31)) - 1u;
        while (word) {
          const int bit = __ffs(word) - 1;
          word &= word - 1;
          const int v = 32 * w + bit - a;
          if (gather) ms.pos[o] = (unsigned short)v;
          else toindex[prefix + o] = v;
          o++;
        }
      }
    }
    if (!gather) return;
    __syncthreads();
    for (int i = threadIdx.x; i < ntrue; i += kTileBlock) toindex[prefix + i] = ms.pos[i];
    return;
  }
  // element pass of a tile with long lists
  constexpr int kWarps = kTileBlock / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long qa = total * warp / kWarps, qb = total * (warp + 1) / kWarps;
  if (qa >= qb) return;
  int lo = 0, hi = count;  // list holding element qa: last r with loc[r] <= qa
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (t.loc[mid] <= qa) lo = mid;
    else hi = mid;
  }
  int r = lo;
  // true entries of list r before qa
  long long before = 0;
  for (long long q = t.loc[r] + lane; q < qa; q += 32) before += mask[base + q] != 0;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) before += __shfl_xor_sync(0xffffffffu, before, d);
  long long run = prefix + sm.loc[r] + before;  // rank of the next true entry
  for (long long g = qa; g < qb; g += 32) {
    while (t.loc[r + 1] <= g) r++;
    const long long q = g + lane;
    const bool in = q < qb;
    const bool m = in && mask[base + q] != 0;
    const unsigned b = __ballot_sync(0xffffffffu, m);
    if (m) {
      int rl = r;
      while (t.loc[rl + 1] <= q) rl++;
      toindex[run + __popc(b & ((1u << lane) - 1u))] = q - t.loc[rl];
    }
    run += __popc(b);
  }
}

// Four elements per thread and step, loads before stores (4 gathers in flight).
template <class W>
__global__ void take_kernel(W* __restrict__ out, const W* __restrict__ content,
                            const int64_t* __restrict__ carry, long long n, long long contentlen,
                            uint64_t inv, uint64_t* err) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
    long long c[4];
    W v[4];
    bool ok[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const long long i = i0 + k * stride;
      c[k] = i < n ? __ldg(carry + i) : 0;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      ok[k] = c[k] >= 0 && c[k] < contentlen;
      v[k] = ok[k] ? __ldg(content + c[k]) : W(0);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const long long i = i0 + k * stride;
      if (i >= n) continue;
      if (ok[k]) out[i] = v[k];
      else raise_error(err, inv, 0);
    }
  }
}

// array[mask] in one pass (mask_select_tile, one CTA per tile of kTileLists
// lists); the local index and the carry of the three-step chain are never
// materialised.
template <class W>
__global__ void __launch_bounds__(kTileBlock, 8)
    mask_select_kernel(int64_t* __restrict__ tooffsets, W* __restrict__ tocontent,
                       int64_t* __restrict__ tocarry, const uint8_t* __restrict__ mask,
                       const int64_t* __restrict__ offsets, const W* __restrict__ content,
                       long long nlists, ScanTiles st, uint64_t* err) {
  __shared__ MaskSelectSmem sm;
  const long long tile = tile_claim(sm.tile, st);
  mask_select_tile<W>(sm, tile, nlists, offsets, mask, content, tooffsets, tocontent, tocarry,
                      nullptr, st, err);
}

}  // namespace

// The new offsets (nlists + 1 entries) and, for each true entry of the mask
// in order, its position within its list.  toindex must hold as many entries
// as the mask has true values in the offsets' span (at most offsets[nlists] -
// offsets[0]).
GB_EXPORT int awkward_gb300_jagged_mask_to_index(int64_t* tooffsets, int64_t* toindex,
                                                 const uint8_t* mask, const int64_t* offsets,
                                                 int64_t nlists, uint64_t* err_code,
                                                 void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (nlists <= 0) return (int)cudaMemsetAsync(tooffsets, 0, sizeof(int64_t), s);
  const long long nt = tile_count(nlists);
  ScanTiles st;
  void* scratch = nullptr;
  cudaError_t e = scan_tiles_alloc(&st, &scratch, nt, s);
  if (e != cudaSuccess) return (int)e;
  mask_to_index_kernel<<<(unsigned)nt, kTileBlock, 0, s>>>(tooffsets, toindex, mask, offsets,
                                                           nlists, nt, st, err_code);
  e = cudaGetLastError();
  cudaError_t f = scratch_free(scratch, s);
  return (int)(e != cudaSuccess ? e : f);
}

// out[i] = content[carry[i]] for element widths of 1, 2, 4 and 8 bytes; a carry
// outside [0, contentlen) raises code 0 ("index out of range").
GB_EXPORT int awkward_gb300_take(void* out, const void* content, int64_t itemsize,
                                 const int64_t* carry, int64_t n, int64_t contentlen,
                                 uint64_t invocation_index, uint64_t* err_code, void* stream) {
  if (n <= 0) return 0;
  long long g = (n + 255) / 256;
  const long long cap = (long long)device_sm_count() * 32;
  const unsigned grid = (unsigned)(g < cap ? g : cap);
  cudaStream_t s = (cudaStream_t)stream;
  switch (itemsize) {
    case 1:
      take_kernel<uint8_t><<<grid, 256, 0, s>>>((uint8_t*)out, (const uint8_t*)content, carry, n,
                                                contentlen, invocation_index, err_code);
      break;
    case 2:
      take_kernel<uint16_t><<<grid, 256, 0, s>>>((uint16_t*)out, (const uint16_t*)content, carry,
                                                 n, contentlen, invocation_index, err_code);
      break;
    case 4:
      take_kernel<uint32_t><<<grid, 256, 0, s>>>((uint32_t*)out, (const uint32_t*)content, carry,
                                                 n, contentlen, invocation_index, err_code);
      break;
    case 8:
      take_kernel<uint64_t><<<grid, 256, 0, s>>>((uint64_t*)out, (const uint64_t*)content, carry,
                                                 n, contentlen, invocation_index, err_code);
      break;
    default:
      return (int)cudaErrorInvalidValue;
  }
  return (int)cudaGetLastError();
}

// array[mask] for a ListOffsetArray over content of 1, 2, 4 or 8-byte items
// in one pass: the new offsets (nlists + 1), the selected content and, when
// tocarry is not NULL, each selected element's position in the content (the
// carry the three-step chain would produce).  tocontent / tocarry hold as many
// entries as the mask has true values in the offsets' span.
GB_EXPORT int awkward_gb300_jagged_mask_select(int64_t* tooffsets, void* tocontent,
                                               int64_t* tocarry, const uint8_t* mask,
                                               const int64_t* offsets, const void* content,
                                               int64_t itemsize, int64_t nlists,
                                               uint64_t* err_code, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (itemsize != 1 && itemsize != 2 && itemsize != 4 && itemsize != 8)
    return (int)cudaErrorInvalidValue;
  if (nlists <= 0) return (int)cudaMemsetAsync(tooffsets, 0, sizeof(int64_t), s);
  const long long nt = tile_count(nlists);
  ScanTiles st;
  void* scratch = nullptr;
  cudaError_t e = scan_tiles_alloc(&st, &scratch, nt, s);
  if (e != cudaSuccess) return (int)e;
  const unsigned grid = (unsigned)nt;
  switch (itemsize) {
    case 1:
      mask_select_kernel<uint8_t><<<grid, kTileBlock, 0, s>>>(
          tooffsets, (uint8_t*)tocontent, tocarry, mask, offsets, (const uint8_t*)content,
          nlists, st, err_code);
      break;
    case 2:
      mask_select_kernel<uint16_t><<<grid, kTileBlock, 0, s>>>(
          tooffsets, (uint16_t*)tocontent, tocarry, mask, offsets, (const uint16_t*)content,
          nlists, st, err_code);
      break;
    case 4:
      mask_select_kernel<uint32_t><<<grid, kTileBlock, 0, s>>>(
          tooffsets, (uint32_t*)tocontent, tocarry, mask, offsets, (const uint32_t*)content,
          nlists, st, err_code);
      break;
    default:
      mask_select_kernel<uint64_t><<<grid, kTileBlock, 0, s>>>(
          tooffsets, (uint64_t*)tocontent, tocarry, mask, offsets, (const uint64_t*)content,
          nlists, st, err_code);
  }
  e = cudaGetLastError();
  cudaError_t f = scratch_free(scratch, s);
  return (int)(e != cudaSuccess ? e : f);
}
