// seg_reduce.cuh -- merge-path segmented reduction over ListOffsetArray offsets.
//
// Replaces the per-bin loops of awkward-cpp's reducers
// (awkward-cpp/src/cpu-kernels/awkward_reduce_*.cpp) for the cupy backend.
//
// Work decomposition.  The reduction is a merge of two sorted streams: the
// list ends A[i] = offsets[i+1] (i < nlists) and the element indices
// j in [offsets[0], offsets[nlists]).  Consuming an element accumulates it
// into the current list; consuming a list end emits that list's result.  The
// merged sequence has D = nlists + E items.  A persistent grid of G CTAs
// splits D into G equal diagonal ranges (perfect balance for any length
// distribution: empty lists, Poisson, heavy tails, one giant list), each
// CTA locating its two ends with a warp-wide 32-ary merge-path search in
// global memory.
//
// Inside a CTA the two streams are read strictly sequentially into two
// shared-memory rings (offsets ring and element ring), each kept filled to
// one chunk ahead of the cursor.  Refills are 1-D TMA bulk copies
// (cp.async.bulk, 16-byte aligned interior; ragged edges by plain loads)
// issued for chunk c+1 before chunk c is reduced, so HBM traffic is one pass
// over offsets and content with no re-reads.  Each chunk is IPC = BLOCK*IPT
// merge items; every thread walks IPT consecutive items (found by a binary
// search in shared memory), accumulates its lists with the reducer policy,
// writes the lists that end inside its range, and a block-wide segmented
// scan stitches lists that cross threads.  Lists that cross CTAs leave one
// head and one tail record per CTA; a one-block fix-up kernel combines them
// with a segmented scan in CTA order.  No CTA ever waits on another.
//
// Combination order is always earlier-then-later, so order-sensitive
// reducers (max/min/argmax/argmin tie and NaN rules) are bit-exact with the
// sequential CPU loops; floating-point sums differ from the CPU only by
// rounding (a tree instead of a left-to-right sum).
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

template <class Acc>
struct CtaRecord {
  long long head_list;  // list that started before this CTA and ends in it, or -1
  long long tail_list;  // list open at the end of this CTA (nlists: none)
  Acc head_acc;
  Acc tail_acc;
  int tail_fresh;  // tail list has no elements before this CTA
  int pad;
};

template <int BLOCK, int IPT, class Store>
struct SegReduceLayout {
  static constexpr int IPC = BLOCK * IPT;
  static constexpr int RE = 2 * IPC;        // element ring entries (power of two)
  static constexpr int RL = 2 * IPC + 16;   // offsets ring entries (even)
  static constexpr size_t off_ring = 0;
  static constexpr size_t elem_ring = (size_t)RL * 8;
  static constexpr size_t elem_bytes = ((size_t)RE * sizeof(Store) + 15) / 16 * 16;
  static constexpr size_t misc = elem_ring + elem_bytes;  // barrier + small shared state
  static constexpr size_t bytes = misc + 256;
  static_assert((RE & (RE - 1)) == 0, "element ring must be a power of two");
  static_assert(((size_t)RE * sizeof(Store)) % 16 == 0, "ring must be a 16-byte multiple");
};

// Fill ring slots for global indices [g0, g1) of `src` (one thread).  Returns
// the bytes issued as TMA bulk copies (to be announced on the mbarrier
// before the copies are issued: call with issue=false first).
template <class T, int R>
__device__ __forceinline__ uint32_t ring_fill(T* ring, const T* src, long long g0, long long g1,
                                              uint64_t* bar, bool use_tma, bool issue) {
  constexpr int A = 16 / (int)sizeof(T);  // elements per 16 bytes
  uint32_t bytes = 0;
  long long a = g0;
  while (a < g1) {
    long long wrap = (a / R + 1) * (long long)R;
    long long b = g1 < wrap ? g1 : wrap;
    long long a16 = use_tma ? (a + A - 1) / A * A : b;
    long long b16 = use_tma ? b / A * A : b;
    if (a16 < b16) {
      uint32_t n = (uint32_t)((b16 - a16) * (long long)sizeof(T));
      if (issue) bulk_g2s(ring + (a16 % R), src + a16, n, bar);
      bytes += n;
    } else {
      a16 = b;
      b16 = b;
    }
    if (issue) {
      for (long long g = a; g < (a16 < b ? a16 : b); g++) ring[g % R] = src[g];
      for (long long g = (b16 > a ? b16 : a); g < b; g++) ring[g % R] = src[g];
    }
    a = b;
  }
  return bytes;
}

// Cooperative plain-load fill (used when a base pointer is not 16-byte aligned).
template <int BLOCK, class T, int R>
__device__ __forceinline__ void ring_fill_coop(T* ring, const T* src, long long g0, long long g1) {
  for (long long g = g0 + threadIdx.x; g < g1; g += BLOCK) ring[g % R] = src[g];
}

// Merge-path split of diagonal d in global memory (one warp).  Returns the
// number of list ends consumed among the first d merged items.
__device__ __forceinline__ long long mp_search_global(const int64_t* __restrict__ offsets,
                                                      long long nlists, long long e0,
                                                      long long E, long long d) {
  const int lane = threadIdx.x & 31;
  long long lo = d - E > 0 ? d - E : 0;
  long long hi = d < nlists ? d : nlists;  // answer in [lo, hi]
  while (hi - lo > 32) {
    long long step = (hi - lo) / 32;
    long long k = lo + (long long)lane * step;
    bool p = (k + (offsets[k + 1] - e0)) < d;
    unsigned m = __ballot_sync(0xffffffffu, p);
    int cnt = __popc(m);
    long long k_prev = lo + (long long)(cnt - 1) * step;
    long long k_next = lo + (long long)cnt * step;
    long long nlo = cnt > 0 ? k_prev + 1 : lo;
    long long nhi = cnt < 32 ? k_next : hi;
    lo = nlo;
    hi = nhi;
  }
  long long k = lo + lane;
  bool p = (k < hi) && ((k + (offsets[k + 1] - e0)) < d);
  unsigned m = __ballot_sync(0xffffffffu, p);
  return lo + __popc(m);
}

template <class Op, int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK)
    seg_reduce_kernel(Op op, const store_t<typename Op::In>* __restrict__ x,
                      const int64_t* __restrict__ offsets, long long nlists,
                      typename Op::Out* __restrict__ out, CtaRecord<typename Op::Acc>* records,
                      int G, int use_tma, uint64_t inv, uint64_t* err) {
  using Acc = typename Op::Acc;
  using Store = store_t<typename Op::In>;
  using L = SegReduceLayout<BLOCK, IPT, Store>;
  using V = SegVal<Acc>;
  constexpr int IPC = L::IPC, RE = L::RE, RL = L::RL;
  constexpr int NW = BLOCK / 32;

  extern __shared__ __align__(128) unsigned char smem[];
  int64_t* oring = reinterpret_cast<int64_t*>(smem + L::off_ring);
  Store* xring = reinterpret_cast<Store*>(smem + L::elem_ring);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::misc);
  long long* sh = reinterpret_cast<long long*>(smem + L::misc + 16);  // 6 words
  __shared__ V scan_smem[NW + 1];
  __shared__ V cta_carry;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long e0 = offsets[0];
  const long long eN = offsets[nlists];
  const long long E = eN > e0 ? eN - e0 : 0;
  const long long D = nlists + E;
  const int Geff = (int)((D + IPC - 1) / IPC < G ? (D + IPC - 1) / IPC : G);
  const int b = blockIdx.x;
  if (b >= Geff) return;
  const long long d_begin = D * b / Geff, d_end = D * (b + 1) / Geff;

  if (warp < 2) {
    long long d = warp == 0 ? d_begin : d_end;
    long long i = mp_search_global(offsets, nlists, e0, E, d);
    if (lane == 0) {
      sh[warp * 2] = i;
      sh[warp * 2 + 1] = e0 + (d - i);
    }
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
    records[b].head_list = -1;
  }
  __syncthreads();
  const long long I0 = sh[0], J0 = sh[1], I1 = sh[2], J1 = sh[3];

  // initial windows: offsets [I0, min(I0+IPC, I1)], elements [J0, min(J0+IPC, J1))
  long long ohi = (I0 + IPC < I1 ? I0 + IPC : I1) + 1;  // exclusive fill end of offsets
  long long ehi = J0 + IPC < J1 ? J0 + IPC : J1;        // exclusive fill end of elements
  uint32_t phase = 0;
  if (use_tma) {
    if (tid == 0) {
      uint32_t nb = ring_fill<int64_t, RL>(oring, offsets, I0, ohi, bar, true, false) +
                    ring_fill<Store, RE>(xring, x, J0, ehi, bar, true, false);
      mbar_arrive_expect_tx(bar, nb);
      ring_fill<int64_t, RL>(oring, offsets, I0, ohi, bar, true, true);
      ring_fill<Store, RE>(xring, x, J0, ehi, bar, true, true);
    }
  } else {
    ring_fill_coop<BLOCK, int64_t, RL>(oring, offsets, I0, ohi);
    ring_fill_coop<BLOCK, Store, RE>(xring, x, J0, ehi);
  }

  const bool head_pending0 = offsets[I0] < J0;  // list I0 has elements in earlier CTAs
  if (tid == 0) {
    cta_carry.acc = op.identity();
    cta_carry.flag = 0;
    sh[4] = head_pending0 ? 1 : 0;
  }
  long long ci = I0, cj = J0, cd = d_begin;
  bool timed_out = false;

  while (cd < d_end) {
    const int len = (int)(d_end - cd < IPC ? d_end - cd : IPC);
    if (use_tma) {
      if (!mbar_wait(bar, phase, 1u << 22)) timed_out = true;
      phase ^= 1;
    }
    __syncthreads();
    const long long Lrem = I1 - ci;
    const int Lw = (int)(Lrem < IPC ? Lrem : IPC);
    const long long Erem = J1 - cj;
    const int Ew = (int)(Erem < IPC ? Erem : IPC);
    const int obase = (int)(ci % RL);
    const int xbase = (int)(cj % RE);
    auto A = [&](int k) -> long long {  // end of list ci+k
      int s = obase + 1 + k;
      if (s >= RL) s -= RL;
      return oring[s];
    };
    auto S = [&](int k) -> long long {  // start of list ci+k
      int s = obase + k;
      if (s >= RL) s -= RL;
      return oring[s];
    };
    // merge-path split of local diagonal dl within the resident windows
    auto split = [&](int dl) -> int {
      int lo = dl - Ew > 0 ? dl - Ew : 0;
      int hi = dl < Lw ? dl : Lw;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((long long)mid + (A(mid) - cj) < dl) lo = mid + 1;
        else hi = mid;
      }
      return lo;
    };
    if (tid == 0) {
      int kend = split(len);
      sh[5] = kend;
    }
    const int dt = tid * IPT;
    int k = dt < len ? split(dt) : 0;
    int m = dt - k;
    __syncthreads();
    const int kend = (int)sh[5];
    const long long ci_next = ci + kend, cj_next = cj + (len - kend);

    // prefetch the next chunk's windows into the slots freed by consumed data
    const long long ohi_next = (ci_next + IPC < I1 ? ci_next + IPC : I1) + 1;
    const long long ehi_next = cj_next + IPC < J1 ? cj_next + IPC : J1;
    if (use_tma) {
      if (tid == 0) {
        fence_proxy_async_smem();
        uint32_t nb = ring_fill<int64_t, RL>(oring, offsets, ohi, ohi_next, bar, true, false) +
                      ring_fill<Store, RE>(xring, x, ehi, ehi_next, bar, true, false);
        mbar_arrive_expect_tx(bar, nb);
        ring_fill<int64_t, RL>(oring, offsets, ohi, ohi_next, bar, true, true);
        ring_fill<Store, RE>(xring, x, ehi, ehi_next, bar, true, true);
      }
    } else {
      ring_fill_coop<BLOCK, int64_t, RL>(oring, offsets, ohi, ohi_next);
      ring_fill_coop<BLOCK, Store, RE>(xring, x, ehi, ehi_next);
    }

    // walk IPT merge items
    Acc acc = op.identity();
    Acc head_acc = op.identity();
    bool has_end = false;
    long long head_list = -1;
    const int nitems = dt < len ? (len - dt < IPT ? len - dt : IPT) : 0;
    for (int s = 0; s < nitems; s++) {
      bool take_end = (k < Lw) && (m >= Ew || A(k) <= cj + m);
      if (take_end) {
        const long long list = ci + k;
        if (!has_end) {
          has_end = true;
          head_list = list;
          head_acc = acc;
        } else {
          out[list] = op.finalize(acc, list);
        }
        acc = op.identity();
        k++;
      } else {
        if (m >= Ew) break;  // inconsistent offsets: never read past the window
        const long long j = cj + m;
        const Store v = xring[(xbase + m) & (RE - 1)];
        bool first = false;
        if (Op::kNeedsFirst) first = (S(k) == j);
        acc = op.combine(acc, op.lift(v, j, first, ci + k));
        m++;
      }
    }

    // block segmented scan of the thread tails
    auto seg = [&](const V& a, const V& bb) -> V {
      V r;
      r.flag = a.flag | bb.flag;
      r.acc = bb.flag ? bb.acc : op.combine(a.acc, bb.acc);
      r.pad = 0;
      return r;
    };
    V ident;
    ident.acc = op.identity();
    ident.flag = 0;
    ident.pad = 0;
    V mine;
    mine.acc = acc;
    mine.flag = has_end ? 1u : 0u;
    mine.pad = 0;
    V total;
    V excl = block_exclusive_scan<BLOCK>(mine, seg, ident, scan_smem, &total);
    const V carry = cta_carry;
    V cin = seg(carry, excl);
    if (has_end) {
      Acc whole = op.combine(cin.acc, head_acc);
      if (head_list == I0 && sh[4]) {
        // list I0 began in an earlier CTA: leave it to the fix-up
        records[b].head_list = I0;
        records[b].head_acc = whole;
      } else {
        out[head_list] = op.finalize(whole, head_list);
      }
    }
    __syncthreads();
    if (tid == 0) {
      cta_carry = seg(carry, total);
      if (total.flag) sh[4] = 0;
    }
    ci = ci_next;
    cj = cj_next;
    cd += len;
    ohi = ohi_next;
    ehi = ehi_next;
    __syncthreads();
  }
  if (tid == 0) {
    records[b].tail_list = I1;
    records[b].tail_acc = cta_carry.acc;
    records[b].tail_fresh = (I1 < nlists) ? (offsets[I1] >= J0 ? 1 : 0) : 1;
  }
  if (timed_out) raise_error(err, inv, GB_MSG_TIMEOUT);
}

// One block: resolve lists that cross CTA boundaries, in CTA order.
template <class Op, int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    seg_reduce_fixup_kernel(Op op, const int64_t* __restrict__ offsets, long long nlists,
                            typename Op::Out* __restrict__ out,
                            const CtaRecord<typename Op::Acc>* __restrict__ records, int G,
                            int ipc) {
  using Acc = typename Op::Acc;
  using V = SegVal<Acc>;
  constexpr int NW = BLOCK / 32;
  __shared__ V scan_smem[NW + 1];
  __shared__ V running;
  const long long e0 = offsets[0];
  const long long eN = offsets[nlists];
  const long long E = eN > e0 ? eN - e0 : 0;
  const long long D = nlists + E;
  const int Geff = (int)((D + ipc - 1) / ipc < G ? (D + ipc - 1) / ipc : G);
  auto seg = [&](const V& a, const V& bb) -> V {
    V r;
    r.flag = a.flag | bb.flag;
    r.acc = bb.flag ? bb.acc : op.combine(a.acc, bb.acc);
    r.pad = 0;
    return r;
  };
  V ident;
  ident.acc = op.identity();
  ident.flag = 0;
  ident.pad = 0;
  if (threadIdx.x == 0) running = ident;
  __syncthreads();
  for (int base = 0; base < Geff; base += BLOCK) {
    const int c = base + threadIdx.x;
    V mine = ident;
    long long tl = -1;
    if (c < Geff) {
      tl = records[c].tail_list;
      mine.acc = records[c].tail_acc;
      mine.flag = (c == 0 || records[c].tail_fresh || records[c - 1].tail_list != tl) ? 1u : 0u;
    }
    V total;
    V excl = block_exclusive_scan<BLOCK>(mine, seg, ident, scan_smem, &total);
    V before = seg(running, excl);  // scan through CTA c-1
    if (c < Geff && c > 0) {
      long long hl = records[c].head_list;
      if (hl >= 0 && hl < nlists) {
        Acc whole = op.combine(before.acc, records[c].head_acc);
        out[hl] = op.finalize(whole, hl);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) running = seg(running, total);
    __syncthreads();
  }
}

}  // namespace gb
