// mask_select.cuh -- array[mask] for one tile of kTileLists lists, shared by
// the per-array entry point (awkward_gb300_jagged_mask_select) and the batched
// one (batch_select_kernel); and the mask bitmap helpers it shares with
// mask_to_index.
//
// The tile's list ends are loaded once.  When its mask bytes (plus the first
// byte's offset in its 16-byte line) fit kMaskBits, they are staged as a
// bitmap in shared memory (two aligned 16-byte loads per 32 bytes, byte loads
// at the ragged ends) and the per-list counts of true entries are popcounts
// of it; a larger tile counts with thread-per-list byte loops.  The counts are
// scanned across tiles (decoupled look-back) into the new offsets.  Then each
// warp walks a contiguous share of the tile's elements: a staged tile one
// bitmap word (32 elements) per group -- a lane's flag is its bit of the word,
// its rank the set bits below it, in 32-bit tile-local arithmetic -- a larger
// one 32 mask bytes per group ranked by a ballot; four groups' content loads
// are issued before they are ranked and stored.  Each selected element (and,
// when asked, its carry: its position in the content) is written at its rank.
#pragma once

#include "list_tile.cuh"

namespace gb {

constexpr int kMaskBits = 16384;  // largest staged tile, in mask bytes

// 4 mask bytes -> 4 bits (byte k nonzero -> bit k).  Bit 7 of each byte of
// ((w & 0x7f..) + 0x7f..) | w is set iff the byte is nonzero (no carries
// between bytes); the multiply gathers the four bit-7s into bits 21..24.
__device__ __forceinline__ unsigned nonzero_nibble(unsigned w) {
  const unsigned hi = ((((w & 0x7f7f7f7fu) + 0x7f7f7f7fu) | w) & 0x80808080u) >> 7;
  return (hi * 0x00204081u) >> 21 & 0xfu;
}
__device__ __forceinline__ unsigned nonzero_bits16(uint4 v) {
  return nonzero_nibble(v.x) | nonzero_nibble(v.y) << 4 | nonzero_nibble(v.z) << 8 |
         nonzero_nibble(v.w) << 12;
}

// Set bits of bits[] in the bit range [a, b).
__device__ __forceinline__ int bitmap_count(const unsigned* bits, int a, int b) {
  if (a >= b) return 0;
  int w = a >> 5;
  const int we = b >> 5;
  if (w == we) return __popc(bits[w] & ((1u << (b & 31)) - 1u) & ~((1u << (a & 31)) - 1u));
  int n = __popc(bits[w] >> (a & 31));
  for (w++; w < we; w++) n += __popc(bits[w]);
  if (b & 31) n += __popc(bits[we] & ((1u << (b & 31)) - 1u));
  return n;
}

struct MaskSelectSmem {
  TileSmem tile;
  long long loc[kTileLists + 1];  // list ends relative to the tile's first element
  unsigned bits[kMaskBits / 32];  // the tile's mask as a bitmap (when it fits)
};

// array[mask] for tile `tile` of the lists offsets[0 .. nlists]: writes the
// new offsets tooffsets[tile's lists] (and tooffsets[nlists] from the last
// tile), the selected content, the carry when tocarry is not null and each
// list's length when tocount is not null.  All threads of the CTA call it.
template <class W>
__device__ __forceinline__ void mask_select_tile(MaskSelectSmem& s, long long tile,
                                                 long long nlists,
                                                 const int64_t* __restrict__ offsets,
                                                 const uint8_t* __restrict__ mask,
                                                 const W* __restrict__ content,
                                                 int64_t* __restrict__ tooffsets,
                                                 W* __restrict__ tocontent,
                                                 int64_t* __restrict__ tocarry,
                                                 int64_t* __restrict__ tocount, ScanTiles st,
                                                 uint64_t* err) {
  const long long l0 = tile * kTileLists;
  const long long rem = nlists - l0;
  const int count = (int)(rem < kTileLists ? rem : kTileLists);
  const long long base = __ldg(offsets + l0);
  for (int i = threadIdx.x; i <= kTileLists; i += kTileBlock) {
    const int k = i < count ? i : count;
    s.loc[i] = __ldg(offsets + l0 + k) - base;
  }
  __syncthreads();
  const long long total = s.loc[count];
  const uint8_t* p0 = mask + base;
  const int sh = (int)(reinterpret_cast<uintptr_t>(p0) & 15);
  const bool staged = total + sh <= kMaskBits;
  long long c[kTileLPT];
  if (staged) {
    // the tile's mask bytes as a bitmap (two aligned 16-byte loads per word,
    // byte loads at the partial ends); counts are popcounts of it
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
      s.bits[w] = word;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kTileLPT; r++) {
      const int li = threadIdx.x * kTileLPT + r;
      c[r] = li < count ? bitmap_count(s.bits, (int)s.loc[li] + sh, (int)s.loc[li + 1] + sh) : 0;
      if (tocount && li < count) tocount[l0 + li] = s.loc[li + 1] - s.loc[li];
    }
  } else {
#pragma unroll
    for (int r = 0; r < kTileLPT; r++) {
      const int li = threadIdx.x * kTileLPT + r;
      long long n = 0;
      if (li < count) {
        for (long long j = base + s.loc[li]; j < base + s.loc[li + 1]; j++) n += __ldg(mask + j) != 0;
        if (tocount) tocount[l0 + li] = s.loc[li + 1] - s.loc[li];
      }
      c[r] = n;
    }
  }
  const long long prefix = tile_scan(s.tile, st, tile, c, 0, err);
  for (int li = threadIdx.x; li < count; li += kTileBlock) tooffsets[l0 + li] = prefix + s.tile.loc[li];
  if (l0 + count == nlists && threadIdx.x == 0) tooffsets[nlists] = prefix + s.tile.total;
  constexpr int kWarps = kTileBlock / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long qa = total * warp / kWarps, qb = total * (warp + 1) / kWarps;
  if (qa >= qb) return;
  int lo = 0, hi = count;  // the list holding element qa
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (s.loc[mid] <= qa) lo = mid;
    else hi = mid;
  }
  long long before;  // true entries of that list before qa
  if (staged) {
    before = bitmap_count(s.bits, (int)s.loc[lo] + sh, (int)qa + sh);
  } else {
    before = 0;
    for (long long q = s.loc[lo] + lane; q < qa; q += 32) before += __ldg(mask + base + q) != 0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) before += __shfl_xor_sync(0xffffffffu, before, d);
  }
  long long run = prefix + s.tile.loc[lo] + before;
  // kWalkUnroll groups of 32 elements per step: their content loads are all
  // issued before the groups are ranked, so a warp keeps several loads in
  // flight instead of one per group
  constexpr int kWalkUnroll = 4;
  const unsigned below = (1u << lane) - 1u;
  if (staged) {
    // the warp's bit positions [b0, b1) of the staged bitmap, one bitmap word
    // (32 elements) per group: a lane's flag is its bit of the word and its
    // rank the set bits below it, in 32-bit tile-local arithmetic
    const int b0 = (int)qa + sh, b1 = (int)qb + sh;
    const int w0 = b0 >> 5, wl = (b1 - 1) >> 5;
    const unsigned first = ~0u << (b0 & 31);
    const unsigned last = (b1 & 31) ? (1u << (b1 & 31)) - 1u : ~0u;
    const W* cbase = content + base;
    W* obase = tocontent + run;
    int64_t* kbase = tocarry ? tocarry + run : nullptr;
    int r = 0;
    for (int w = w0; w <= wl; w += kWalkUnroll) {
      unsigned bits[kWalkUnroll];
      W v[kWalkUnroll];
#pragma unroll
      for (int u = 0; u < kWalkUnroll; u++) {
        const int ww = w + u;
        unsigned b = ww <= wl ? s.bits[ww] : 0u;
        if (ww == w0) b &= first;
        if (ww == wl) b &= last;
        bits[u] = b;
        v[u] = (b >> lane) & 1u ? __ldg(cbase + (32 * ww + lane - sh)) : W(0);
      }
#pragma unroll
      for (int u = 0; u < kWalkUnroll; u++) {
        if ((bits[u] >> lane) & 1u) {
          const int at = r + __popc(bits[u] & below);
          obase[at] = v[u];
          if (kbase) kbase[at] = base + (32 * (w + u) + lane - sh);
        }
        r += __popc(bits[u]);
      }
    }
    return;
  }
  for (long long g = qa; g < qb; g += 32 * kWalkUnroll) {
    bool m[kWalkUnroll];
    W v[kWalkUnroll];
#pragma unroll
    for (int u = 0; u < kWalkUnroll; u++) {
      const long long q = g + 32 * u + lane;
      m[u] = false;
      if (q < qb) m[u] = __ldg(mask + base + q) != 0;
      v[u] = m[u] ? __ldg(content + base + q) : W(0);
    }
#pragma unroll
    for (int u = 0; u < kWalkUnroll; u++) {
      const unsigned b = __ballot_sync(0xffffffffu, m[u]);
      if (m[u]) {
        const long long at = run + __popc(b & below);
        tocontent[at] = v[u];
        if (tocarry) tocarry[at] = base + g + 32 * u + lane;
      }
      run += __popc(b);
    }
  }
}

}  // namespace gb
