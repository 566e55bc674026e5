// seg_reduce.cuh -- segmented reduction over ListOffsetArray offsets.
//
// Replaces the per-bin loops of awkward-cpp's reducers
// (awkward-cpp/src/cpu-kernels/awkward_reduce_*.cpp) for the cupy backend.
//
// Balance.  The reduction is a merge of two sorted streams, the list ends
// offsets[i+1] and the element indices; the merged sequence has
// D = nlists + E items.  Every warp of a persistent grid takes an equal
// diagonal range of it (balanced for any length distribution: empty lists,
// Poisson, heavy tails, one giant list), found with a warp-wide 32-ary
// merge-path search in global memory: lists I0..I1-1 end inside the warp's
// range, list I1 is open at its end (the "tail"), and list I0 may have begun
// in an earlier range (the "head").
//
// Reduction.  The warp walks its lists 32 at a time, one list per lane: a
// list of at most 32 elements is reduced by its lane straight from global
// memory (read-only path; 64 resident warps per SM keep enough loads in
// flight, and the warp's loads cover one contiguous stretch of content); a
// longer list is reduced by the whole warp, strided over 32 lanes (coalesced)
// and combined with a butterfly.  Each input byte is read from HBM once and
// results are stored coalesced.
//
// Arithmetic.  Every reducer's combine is commutative and associative
// (extremum reducers carry the element index and break ties towards the
// lowest index), so the cooperative reductions give the CPU's results:
// bit-exact for integers, counts, max/min and argmax/argmin (including the
// NaN and signed-zero rules).  Float64 data never touch the float64 pipe per
// element (see reduce_ops.cuh): comparisons use integer keys, sums an exact
// fixed-point accumulator.
//
// Lists that cross warp ranges leave one head and one tail record per warp;
// a one-block fix-up kernel combines them with a segmented scan in range
// order.  No warp ever waits on another.
#pragma once

#include <type_traits>

#include "gb_common.cuh"

namespace gb {

// Storage type of a content element (bool is read as a byte).
template <class T>
using store_t = typename std::conditional<std::is_same<T, bool>::value, uint8_t, T>::type;

template <class Acc>
struct SegVal {
  Acc acc;
  uint32_t flag;  // a segment (list) starts inside this range
  uint32_t pad;
};

// Partial results of the lists that cross the ends of one warp's range.
template <class Acc>
struct RangeRecord {
  long long head_list;  // list that began before this range and ends in it, or -1
  long long tail_list;  // list open at the end of this range (nlists: none)
  Acc head_acc;
  Acc tail_acc;
  int tail_fresh;  // tail list has no elements before this range
  int pad;
};

constexpr int kSegBlock = 256;        // threads per CTA (8 warps)
constexpr int kSegMinBlocks = 5;      // resident CTAs per SM (40 warps of loads in flight)
constexpr int kShortList = 32;        // longest list reduced by one lane
constexpr int kMediumList = 256;      // longest list reduced by a group of 8 lanes
constexpr int kMinRangeItems = 512;   // smallest merge range given to a warp
constexpr long long kAbsorb = 4096;   // longest list reduced whole by the range where it ends
constexpr int kPrefetchLines = 16;    // 128-byte lines after each round prefetched towards L2
constexpr int kPrefetchSkip = 0;      // lines skipped before the prefetched ones

// Merge-path split of diagonal d in global memory by a half warp (16 lanes,
// `mask` selects them).  Returns the number of list ends among the first d
// merged items: the first k in [max(0, d-E), min(d, nlists)] with
// k + offsets[k+1] - e0 >= d.  The first probe brackets a proportional guess
// (exact for evenly spread lengths), then 16-ary narrowing.
__device__ __forceinline__ long long mp_search_half(const int64_t* __restrict__ offsets,
                                                    long long nlists, long long e0, long long E,
                                                    long long d, unsigned mask) {
  const int hl = threadIdx.x & 15;
  long long lo = d - E > 0 ? d - E : 0;
  long long hi = d < nlists ? d : nlists;  // answer in [lo, hi]
  auto pred = [&](long long k) { return (k + (__ldg(offsets + k + 1) - e0)) < d; };
  if (hi - lo > 16) {
    // proportional guess g (float32: only a starting point, the probes that
    // follow are exact); probe g + (hl - 8) * w
    const long long D = nlists + E;
    long long g = D > 0 ? (long long)((float)d * ((float)nlists / (float)D)) : lo;
    const long long w = ((hi - lo) >> 12) + 1;
    long long k = g + (long long)(hl - 8) * w;
    k = k < lo ? lo : (k > hi - 1 ? hi - 1 : k);
    const unsigned m = __ballot_sync(mask, pred(k)) >> (threadIdx.x & 16);
    const long long k0 = __shfl_sync(mask, k, 0, 16), k15 = __shfl_sync(mask, k, 15, 16);
    const int cnt = __popc(m & 0xffffu);
    // window valid when the split lies between the first and last probe
    if (cnt > 0 && cnt < 16 && (m & 1u)) {
      const long long kp = __shfl_sync(mask, k, cnt - 1, 16), kn = __shfl_sync(mask, k, cnt, 16);
      lo = kp + 1;
      hi = kn;
    } else if (cnt == 0) {
      hi = k0;
    } else if (cnt == 16) {
      lo = k15 + 1;
    }
  }
  while (hi - lo > 16) {
    const long long step = (hi - lo) / 16;
    const long long k = lo + (long long)hl * step;
    const unsigned m = __ballot_sync(mask, pred(k)) >> (threadIdx.x & 16);
    const int cnt = __popc(m & 0xffffu);
    const long long nlo = cnt > 0 ? lo + (long long)(cnt - 1) * step + 1 : lo;
    const long long nhi = cnt < 16 ? lo + (long long)cnt * step : hi;
    lo = nlo;
    hi = nhi;
  }
  const long long k = lo + hl;
  const unsigned m = __ballot_sync(mask, (k < hi) && pred(k)) >> (threadIdx.x & 16);
  return lo + __popc(m & 0xffffu);
}

template <class Op>
__device__ __forceinline__ typename Op::Acc warp_allreduce(const Op& op, typename Op::Acc a) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    constexpr int W = sizeof(typename Op::Acc) / 4;
    union U { typename Op::Acc v; uint32_t w[W]; } u;
    u.v = a;
#pragma unroll
    for (int i = 0; i < W; i++) u.w[i] = __shfl_xor_sync(0xffffffffu, u.w[i], d);
    a = op.combine(a, u.v);
  }
  return a;
}

// Reduction of one run of a list by a group of G lanes (defined, with its
// per-reducer overloads, in reduce_ops.cuh).
template <int G, class Op>
__device__ typename Op::Acc run_coop(const Op& op, const store_t<typename Op::In>* x, long long s,
                                     long long e, long long st, long long li);

// The lanes' lists li = base + lane of one round of a warp range (st, en:
// the list's offsets; `act`: li <= last_list), read from global memory:
// lists of at most kShortList elements by their lane, longer ones by groups
// of 8 lanes or the whole warp.  Lists that end in the range are emitted; the
// partials of the giant list crossing the range start (head) or open at its
// end (I1, tail) go to `rec`; a list of at most kAbsorb elements open at the
// end is left to the range where it ends.
template <class Op, class Emit>
__device__ __forceinline__ void seg_direct_lists(const Op& op,
                                                 const store_t<typename Op::In>* __restrict__ x,
                                                 long long base, bool act, long long st,
                                                 long long en, long long I1, long long J0,
                                                 long long J1, Emit& emit,
                                                 RangeRecord<typename Op::Acc>& rec) {
  const int lane = threadIdx.x & 31;
  const long long li = base + lane;
  long long s0 = 0, e = 0;
  bool skip = false;
  if (act) {
    const bool small = en - st <= kAbsorb;  // reduced whole by the range where it ends
    s0 = (st < J0 && !small) ? J0 : st;
    e = li == I1 ? J1 : en;
    skip = li == I1 && small;  // the range where it ends takes all of it
    if (e < s0) e = s0;
  }
  typename Op::Acc acc = op.identity();
  if (act && !skip && e - s0 <= kShortList) acc = run_short(op, x + s0, (int)(e - s0), s0, st, li);
  const bool longer = act && !skip && e - s0 > kShortList;
  // medium lists: four at a time, 8 lanes each (four load chains in flight)
  unsigned med = __ballot_sync(0xffffffffu, longer && e - s0 <= kMediumList);
  unsigned coop = __ballot_sync(0xffffffffu, longer) & ~med;
  while (med) {
    int src = -1;  // the list of this lane's group
#pragma unroll
    for (int g = 0; g < 4; g++) {
      const int cand = med ? __ffs(med) - 1 : -1;
      if (cand >= 0) med &= med - 1;
      if ((lane >> 3) == g) src = cand;
    }
    const int from = src < 0 ? 0 : src;
    long long s2 = __shfl_sync(0xffffffffu, s0, from);
    long long e2 = __shfl_sync(0xffffffffu, e, from);
    const long long st2 = __shfl_sync(0xffffffffu, st, from);
    if (src < 0) e2 = s2;  // an idle group reduces nothing
    const typename Op::Acc a2 = run_coop<8>(op, x, s2, e2, st2, base + from);
    // the owner lane takes its list's result from the first lane of its group
    int owner_group = -1;
#pragma unroll
    for (int g = 0; g < 4; g++)
      if (__shfl_sync(0xffffffffu, src, g * 8) == lane) owner_group = g;
    const typename Op::Acc mine = shfl_idx(a2, owner_group < 0 ? 0 : owner_group * 8);
    if (owner_group >= 0) acc = mine;
  }
  while (coop) {  // longer lists: the whole warp, strided (coalesced)
    const int src = __ffs(coop) - 1;
    coop &= coop - 1;
    const long long s2 = __shfl_sync(0xffffffffu, s0, src);
    const long long e2 = __shfl_sync(0xffffffffu, e, src);
    const long long st2 = __shfl_sync(0xffffffffu, st, src);
    const long long l2 = base + src;
    const typename Op::Acc a2 = run_coop<32>(op, x, s2, e2, st2, l2);
    if (lane == src) acc = a2;
  }
  if (act && !skip) {
    if (li == I1) {
      rec.tail_acc = acc;  // a giant list continues in the next range
    } else if (s0 > st) {
      rec.head_acc = acc;  // the end of a giant list that began earlier
    } else {
      emit(li, acc);
    }
  }
}

// The records of a warp range (lane 0): the giant list crossing its start
// and the one open at its end.
template <class Op>
__device__ __forceinline__ void seg_range_records(const Op& op,
                                                  const int64_t* __restrict__ offsets,
                                                  long long nlists, long long I0, long long I1,
                                                  long long J0,
                                                  RangeRecord<typename Op::Acc>& rec) {
  const long long st0 = __ldg(offsets + I0);
  const bool head = I0 < I1 && st0 < J0 && __ldg(offsets + I0 + 1) - st0 > kAbsorb;
  rec.head_list = head ? I0 : -1;
  const bool tail = I1 < nlists && __ldg(offsets + I1 + 1) - __ldg(offsets + I1) > kAbsorb;
  rec.tail_list = tail ? I1 : -1;
  rec.tail_fresh = (tail && __ldg(offsets + I1) >= J0) ? 1 : 0;
  if (!tail) rec.tail_acc = op.identity();
}

// The reducers with a direct finisher for a whole list of at most
// kShortList elements (lane_final, defined with them in reduce_ops.cuh).
template <class Op>
struct LaneFinal : std::false_type {};

// Reduce the lists of merge-path diagonal range [d0, d1) of one array (whole
// warp), writing each list that ends in the range to out[list]; the partials
// of the giant lists crossing the range ends go to `rec`.
//
// The warp walks the range 32 lists per round, one lane per list.  The lanes'
// list ends are one coalesced 8-byte load per round (starts come from the lane
// below).  A round whose lists all end inside the range with at most
// kShortList elements each -- nearly every round of short-list data -- is
// finished by the lanes alone: each computes its list's output with the
// reducer's short-run arithmetic (lane_final where the reducer has one, else
// finalize(run_short)) and stores it.  Other rounds (a list longer than
// kShortList, the giant list crossing the range start, the list open at its
// end) take seg_direct_lists.  Both give the same bits for a list, so the
// per-array kernel and the batched one (which both call this) agree bit for bit.
template <class Op>
__device__ __forceinline__ void seg_reduce_range(const Op& op,
                                                 const store_t<typename Op::In>* __restrict__ x,
                                                 const int64_t* __restrict__ offsets,
                                                 long long nlists, long long e0, long long E,
                                                 long long d0, long long d1,
                                                 typename Op::Out* __restrict__ out,
                                                 RangeRecord<typename Op::Acc>& rec) {
  const int lane = threadIdx.x & 31;
  auto emit = [&](long long li, const typename Op::Acc& a) { out[li] = op.finalize(a, li); };
  // both ends at once: lanes 0-15 search d0, lanes 16-31 search d1
  const bool upper = lane >= 16;
  const long long split = mp_search_half(offsets, nlists, e0, E, upper ? d1 : d0,
                                         upper ? 0xffff0000u : 0x0000ffffu);
  const long long I0 = __shfl_sync(0xffffffffu, split, 0);
  const long long I1 = __shfl_sync(0xffffffffu, split, 16);
  const long long J0 = e0 + (d0 - I0), J1 = e0 + (d1 - I1);
  const long long last_list = I1 < nlists ? I1 : I1 - 1;  // I1 itself is the tail, if any
  long long carry = __ldg(offsets + I0);  // start of the round's first list
  for (long long base = I0; base <= last_list; base += 32) {
    const long long li = base + lane;
    const bool act = li <= last_list;
    const long long en = __ldg(offsets + (act ? li : last_list) + 1);
    long long st = __shfl_up_sync(0xffffffffu, en, 1);
    if (lane == 0) st = carry;
    carry = __shfl_sync(0xffffffffu, en, 31);
    if (kPrefetchLines > 0 && base + 32 <= last_list && lane < kPrefetchLines) {
      // the content after this round (the next round's, contiguous) towards
      // L2: one 128-byte line per lane, kPrefetchSkip lines ahead, never past
      // the array's last element
      const long long ahead = (long long)(lane + kPrefetchSkip) * 128 / (long long)sizeof(*x);
      if (carry + ahead < e0 + E)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(x + carry + ahead));
    }
    const long long n = en - st;
    // every list of the round whole, short and ending in the range (I1 is
    // the list open at the range end)
    const bool plain = li != I1 && (unsigned long long)n <= (unsigned long long)kShortList;
    if (__all_sync(0xffffffffu, !act || plain)) {
      const int m = act ? (int)n : 0;
      typename Op::Out r;
      bool fast = true;
      if constexpr (LaneFinal<Op>::value) r = lane_final(op, x + st, m, st, fast);
      else r = op.finalize(run_short(op, x + st, m, st, st, li), li);
      if (!__all_sync(0xffffffffu, fast) && !fast)
        r = op.finalize(run_short(op, x + st, m, st, st, li), li);
      if (act) out[li] = r;
    } else {
      seg_direct_lists(op, x, base, act, st, en, I1, J0, J1, emit, rec);
    }
  }
  if (lane == 0) seg_range_records(op, offsets, nlists, I0, I1, J0, rec);
}

// Number of warp ranges an array of nlists lists and E elements is split
// into when W warps are available (the batched path uses the same split, so
// both give bit-identical results).
__host__ __device__ __forceinline__ int seg_ranges_min(long long nlists, long long E, int W,
                                                       long long min_items) {
  const long long D = nlists + E;
  const long long wanted = (D + min_items - 1) / min_items;
  return (int)(wanted < W ? wanted : W);
}
__host__ __device__ __forceinline__ int seg_ranges(long long nlists, long long E, int W) {
  return seg_ranges_min(nlists, E, W, kMinRangeItems);
}

// The per-array kernel: a persistent grid of warps, each reducing one
// merge-path range (seg_reduce_range).
template <class Op>
__global__ void __launch_bounds__(kSegBlock, kSegMinBlocks)
    seg_reduce_kernel(Op op, const store_t<typename Op::In>* __restrict__ x,
                      const int64_t* __restrict__ offsets, long long nlists,
                      typename Op::Out* __restrict__ out, RangeRecord<typename Op::Acc>* records,
                      int W, uint64_t inv, uint64_t* err) {
  (void)inv;
  (void)err;
  const int w = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const long long e0 = __ldg(offsets);
  const long long eN = __ldg(offsets + nlists);
  const long long E = eN > e0 ? eN - e0 : 0;
  const long long D = nlists + E;
  const int Weff = seg_ranges(nlists, E, W);
  if (w >= Weff) return;
  const long long d0 = D * w / Weff, d1 = D * (w + 1) / Weff;
  seg_reduce_range(op, x, offsets, nlists, e0, E, d0, d1, out, records[w]);
}

// Giant lists (more than kAbsorb elements) that cross warp ranges: one warp
// per 32 records; for each record holding the end of such a list, the warp
// walks back over the preceding records 32 at a time, combining the tail
// partials of the same list up to the range where it began.
template <class Op>
__global__ void __launch_bounds__(256)
    seg_reduce_fixup_kernel(Op op, const int64_t* __restrict__ offsets, long long nlists,
                            typename Op::Out* __restrict__ out,
                            const RangeRecord<typename Op::Acc>* __restrict__ records, int W) {
  using Acc = typename Op::Acc;
  const int lane = threadIdx.x & 31;
  const long long e0 = __ldg(offsets), eN = __ldg(offsets + nlists);
  const long long E = eN > e0 ? eN - e0 : 0;
  const int Weff = seg_ranges(nlists, E, W);
  const int c0 = (int)(((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5) * 32);
  if (c0 >= Weff) return;
  const int c = c0 + lane;
  const long long hl = c < Weff ? records[c].head_list : -1;
  unsigned todo = __ballot_sync(0xffffffffu, hl >= 0);
  while (todo) {
    const int src = __ffs(todo) - 1;
    todo &= todo - 1;
    const int cc = c0 + src;
    const long long L = __shfl_sync(0xffffffffu, hl, src);
    Acc acc = op.identity();
    for (int base = cc - 1; base >= 0; base -= 32) {
      const int r = base - lane;  // lane 0 is the nearest preceding range
      const bool valid = r >= 0 && records[r].tail_list == L;
      const bool fresh = valid && records[r].tail_fresh;  // the range where L began
      const unsigned inval = __ballot_sync(0xffffffffu, !valid);
      const unsigned fr = __ballot_sync(0xffffffffu, fresh);
      const int stop_inv = inval ? __ffs(inval) - 1 : 32;
      const int stop_fr = fr ? __ffs(fr) - 1 : 32;
      const int lim = stop_inv < stop_fr + 1 ? stop_inv : stop_fr + 1;  // lanes < lim contribute
      if (lane < lim) acc = op.combine(acc, records[r].tail_acc);
      if (inval || fr) break;
    }
    acc = warp_allreduce(op, acc);
    if (lane == 0) out[L] = op.finalize(op.combine(acc, records[cc].head_acc), L);
  }
}

}  // namespace gb
