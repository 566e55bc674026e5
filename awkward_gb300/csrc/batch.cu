// batch.cu -- many jagged arrays of uneven sizes in one launch per operation.
//
// A batch plan holds, for A float64 ListOffsetArrays with a jagged boolean
// mask each, the device tables of a work queue and the outputs of
//   sum, max, argmax (axis=-1)   the segmented reducers of seg_reduce.cuh;
//   count (axis=-1)              offsets differences;
//   array[mask]                  new offsets and selected content.
// Reducers: every array is split into exactly the warp ranges the per-array
// launch would use (seg_ranges with the same warp count), so the batched
// results are bit-identical to the per-array ones; the (array, range) items
// form one queue that the warps of a persistent grid drain with an atomic
// counter, in an order chosen on the host from the items' sizes.  Giant-list
// records are combined per array by one fix-up launch (a record's `pad` holds
// its array, so walks never cross arrays).  Select + count: list tiles of all
// arrays form one ticketed sequence; each array's tiles scan with their own
// decoupled look-back chain.
//
// Launches per run: 3 x (reducer + fix-up) + select, after 2 memsets; no host
// synchronisation and no allocation, so a run can be captured in a CUDA graph.
#include <algorithm>
#include <numeric>
#include <vector>

#include "list_tile.cuh"
#include "mask_select.cuh"
#include "reduce_ops.cuh"

using namespace gb;

namespace {

constexpr int kOps = 3;  // sum, max, argmax

struct BatchArray {
  const double* x;
  const int64_t* offsets;
  const uint8_t* mask;
  long long nlists;
  long long E;
  int ranges[kOps];
  int item0[kOps];
  long long tile0;
  double* out_sum;
  double* out_max;
  int64_t* out_argmax;
  int64_t* out_count;
  int64_t* sel_offsets;
  double* sel_content;
};

using SumOpD = FixedSumOp<double>;
using MaxOpD = ExtremumOp<double, true>;
using ArgOpD = ArgExtremumOp<double, true>;

template <int K>
struct OpOf;
template <>
struct OpOf<0> {
  using type = SumOpD;
};
template <>
struct OpOf<1> {
  using type = MaxOpD;
};
template <>
struct OpOf<2> {
  using type = ArgOpD;
};

template <int K>
__device__ __forceinline__ typename OpOf<K>::type::Out* out_of(const BatchArray& a) {
  if constexpr (K == 0) return a.out_sum;
  else if constexpr (K == 1) return a.out_max;
  else return a.out_argmax;
}

template <int K, int BLOCK>
__global__ void __launch_bounds__(BLOCK, kSegMinBlocks * kSegBlock / BLOCK)
    batch_reduce_kernel(typename OpOf<K>::type op, const BatchArray* __restrict__ arrays,
                        const int2* __restrict__ items, const int* __restrict__ order, int nitems,
                        RangeRecord<typename OpOf<K>::type::Acc>* records, unsigned* counter) {
  using Op = typename OpOf<K>::type;
  const int lane = threadIdx.x & 31;
  while (true) {
    int k = 0;
    if (lane == 0) k = (int)atomicAdd(counter, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= nitems) break;
    const int id = order[k];
    const int2 it = items[id];
    const BatchArray& A = arrays[it.x];
    const long long e0 = __ldg(A.offsets);
    const long long D = A.nlists + A.E;
    const int Weff = A.ranges[K];
    const long long d0 = D * it.y / Weff, d1 = D * (it.y + 1) / Weff;
    typename Op::Out* out = out_of<K>(A);
    seg_reduce_range(op, A.x, A.offsets, A.nlists, e0, A.E, d0, d1, out, records[id]);
    if (lane == 0) records[id].pad = it.x;
  }
}

// One warp per 32 records: for a record holding the end of a giant list, walk
// back over the preceding records of the same array (ranges in order).
template <int K>
__global__ void __launch_bounds__(256)
    batch_fixup_kernel(typename OpOf<K>::type op, const BatchArray* __restrict__ arrays,
                       const RangeRecord<typename OpOf<K>::type::Acc>* __restrict__ records,
                       int nitems) {
  using Op = typename OpOf<K>::type;
  using Acc = typename Op::Acc;
  const int lane = threadIdx.x & 31;
  const int c0 = (int)(((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5) * 32);
  if (c0 >= nitems) return;
  const int c = c0 + lane;
  const long long hl = c < nitems ? records[c].head_list : -1;
  unsigned todo = __ballot_sync(0xffffffffu, hl >= 0);
  while (todo) {
    const int src = __ffs(todo) - 1;
    todo &= todo - 1;
    const int cc = c0 + src;
    const long long L = __shfl_sync(0xffffffffu, hl, src);
    const int arr = records[cc].pad;
    Acc acc = op.identity();
    for (int base = cc - 1; base >= 0; base -= 32) {
      const int r = base - lane;
      const bool valid = r >= 0 && records[r].pad == arr && records[r].tail_list == L;
      const bool fresh = valid && records[r].tail_fresh;
      const unsigned inval = __ballot_sync(0xffffffffu, !valid);
      const unsigned fr = __ballot_sync(0xffffffffu, fresh);
      const int stop_inv = inval ? __ffs(inval) - 1 : 32;
      const int stop_fr = fr ? __ffs(fr) - 1 : 32;
      const int lim = stop_inv < stop_fr + 1 ? stop_inv : stop_fr + 1;
      if (lane < lim) acc = op.combine(acc, records[r].tail_acc);
      if (inval || fr) break;
    }
    acc = warp_allreduce(op, acc);
    if (lane == 0) out_of<K>(arrays[arr])[L] = op.finalize(op.combine(acc, records[cc].head_acc), L);
  }
}

// array[mask] and count for every list tile of every array (mask_select_tile;
// tiles are claimed from one ticket over all arrays' tiles in order).
__global__ void __launch_bounds__(kTileBlock, 8)
    batch_select_kernel(const BatchArray* __restrict__ arrays, int narrays,
                        const long long* __restrict__ tile_base, unsigned long long* ticket,
                        unsigned long long* status, uint64_t* err) {
  __shared__ MaskSelectSmem sm;
  __shared__ int s_arr;
  if (threadIdx.x == 0) {
    const long long g = (long long)atomicAdd(ticket, 1ull);
    int lo = 0, hi = narrays;  // last array with tile_base <= g
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (tile_base[mid] <= g) lo = mid;
      else hi = mid;
    }
    sm.tile.tile = g - tile_base[lo];
    s_arr = lo;
  }
  __syncthreads();
  const long long tile = sm.tile.tile;
  const BatchArray& A = arrays[s_arr];
  ScanTiles st;
  st.ticket = ticket;
  st.status = status + A.tile0;
  mask_select_tile<double>(sm, tile, A.nlists, A.offsets, A.mask, A.x, A.sel_offsets,
                           A.sel_content, nullptr, A.out_count, st, err);
}

struct Plan {
  int narrays = 0;
  int block = kSegBlock;  // threads per CTA of the reducer launches
  int nitems[kOps] = {};
  int blocks[kOps] = {};
  long long ntiles = 0;
  BatchArray* d_arrays = nullptr;
  int2* d_items[kOps] = {};
  int* d_order[kOps] = {};
  void* d_records[kOps] = {};
  unsigned* d_counters = nullptr;          // one per reducer
  unsigned long long* d_scan = nullptr;    // select ticket + tile states
  long long* d_tile_base = nullptr;
  uint64_t* err = nullptr;
};

template <int K, int BLOCK>
int occupancy_blocks() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_reduce_kernel<K, BLOCK>, BLOCK, 0) !=
          cudaSuccess ||
      n < 1)
    n = 1;
  return n;
}

template <int K>
int occupancy_blocks(int block) {
  return block == 128 ? occupancy_blocks<K, 128>() : occupancy_blocks<K, 256>();
}

void free_plan(Plan* p) {
  cudaFree(p->d_arrays);
  for (int k = 0; k < kOps; k++) {
    cudaFree(p->d_items[k]);
    cudaFree(p->d_order[k]);
    cudaFree(p->d_records[k]);
  }
  cudaFree(p->d_counters);
  cudaFree(p->d_scan);
  cudaFree(p->d_tile_base);
  delete p;
}

template <class T>
cudaError_t upload(T** dst, const std::vector<T>& v) {
  cudaError_t e = cudaMalloc((void**)dst, sizeof(T) * (v.empty() ? 1 : v.size()));
  if (e != cudaSuccess || v.empty()) return e;
  return cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
}

}  // namespace

// Build a plan (set-up time: allocates and uploads its tables; synchronous).
// Host arrays of length narrays: nlists, nelements (offsets[n] - offsets[0]),
// maxlen (each array's longest list, -1 if unknown; may be null), and the
// device pointers of every array's content, offsets, mask and
// outputs.  The tuning knobs (the autotuner's search space):
//   order_mode     0: items in array order; 1: largest ranges first;
//   occupancy_div  persistent CTAs per SM = reducer occupancy / occupancy_div;
//   range_min      items per reduction range of arrays whose lists all have
//                  at most kAbsorb elements (any split gives their bits;
//                  at least kMinRangeItems);
//   block          threads per CTA of the reducer launches (128 or 256).
// err_code: device word for bounded-wait failures of the select scan.
GB_EXPORT int awkward_gb300_batch_plan_create(
    void** plan, int64_t narrays, const int64_t* nlists, const int64_t* nelements,
    const int64_t* maxlen,
    const double* const* x, const int64_t* const* offsets, const uint8_t* const* mask,
    double* const* out_sum, double* const* out_max, int64_t* const* out_argmax,
    int64_t* const* out_count, int64_t* const* sel_offsets, double* const* sel_content,
    int64_t order_mode, int64_t occupancy_div, int64_t range_min, int64_t block,
    uint64_t* err_code) {
  *plan = nullptr;
  if (narrays <= 0 || occupancy_div < 1 || range_min < kMinRangeItems ||
      (block != 128 && block != 256))
    return (int)cudaErrorInvalidValue;
  Plan* p = new Plan();
  p->narrays = (int)narrays;
  p->block = (int)block;
  p->err = err_code;
  const int sms = device_sm_count();
  const int W[kOps] = {sms * SegReduceConfig<SumOpD>::blocks_per_sm() * (kSegBlock / 32),
                       sms * SegReduceConfig<MaxOpD>::blocks_per_sm() * (kSegBlock / 32),
                       sms * SegReduceConfig<ArgOpD>::blocks_per_sm() * (kSegBlock / 32)};
  const int occ[kOps] = {occupancy_blocks<0>(p->block), occupancy_blocks<1>(p->block),
                         occupancy_blocks<2>(p->block)};
  std::vector<BatchArray> arrays(narrays);
  std::vector<std::vector<int2>> items(kOps);
  std::vector<long long> tile_base(narrays + 1, 0);
  for (int a = 0; a < narrays; a++) {
    BatchArray& A = arrays[a];
    A.x = x[a];
    A.offsets = offsets[a];
    A.mask = mask[a];
    A.nlists = nlists[a];
    A.E = nelements[a] > 0 ? nelements[a] : 0;
    // Lists of at most kAbsorb elements are reduced whole by the range where
    // they end, so any split gives their bits: such arrays take ranges of at
    // least range_min items (fewer range searches per element).  An
    // array with a longer list keeps its per-array split, whose partials the
    // fix-up combines in the same order.
    const bool any_split = maxlen != nullptr && maxlen[a] >= 0 && maxlen[a] <= kAbsorb;
    for (int k = 0; k < kOps; k++) {
      A.ranges[k] = nlists[a] <= 0 ? 0
                    : any_split ? seg_ranges_min(nlists[a], A.E, W[k], range_min)
                                : seg_ranges(nlists[a], A.E, W[k]);
      A.item0[k] = (int)items[k].size();
      for (int w = 0; w < A.ranges[k]; w++) items[k].push_back(make_int2(a, w));
    }
    A.tile0 = tile_base[a];
    tile_base[a + 1] = tile_base[a] + (nlists[a] > 0 ? tile_count(nlists[a]) : 0);
    A.out_sum = out_sum[a];
    A.out_max = out_max[a];
    A.out_argmax = out_argmax[a];
    A.out_count = out_count[a];
    A.sel_offsets = sel_offsets[a];
    A.sel_content = sel_content[a];
  }
  p->ntiles = tile_base[narrays];
  cudaError_t e = upload(&p->d_arrays, arrays);
  for (int k = 0; k < kOps && e == cudaSuccess; k++) {
    p->nitems[k] = (int)items[k].size();
    std::vector<int> order(items[k].size());
    std::iota(order.begin(), order.end(), 0);
    if (order_mode == 1) {
      std::stable_sort(order.begin(), order.end(), [&](int i, int j) {
        const BatchArray& a = arrays[items[k][i].x];
        const BatchArray& b = arrays[items[k][j].x];
        return (a.nlists + a.E) / a.ranges[k] > (b.nlists + b.E) / b.ranges[k];
      });
    }
    e = upload(&p->d_items[k], items[k]);
    if (e == cudaSuccess) e = upload(&p->d_order[k], order);
    size_t rec_bytes = k == 0 ? sizeof(RangeRecord<SumOpD::Acc>)
                              : (k == 1 ? sizeof(RangeRecord<MaxOpD::Acc>)
                                        : sizeof(RangeRecord<ArgOpD::Acc>));
    if (e == cudaSuccess)
      e = cudaMalloc(&p->d_records[k], rec_bytes * (items[k].empty() ? 1 : items[k].size()));
    long long b = (long long)sms * std::max(1, occ[k] / (int)occupancy_div);
    p->blocks[k] = (int)b;
  }
  if (e == cudaSuccess) e = cudaMalloc(&p->d_counters, sizeof(unsigned) * kOps);
  if (e == cudaSuccess)
    e = cudaMalloc(&p->d_scan, sizeof(unsigned long long) * (size_t)(p->ntiles + 1));
  if (e == cudaSuccess) e = upload(&p->d_tile_base, tile_base);
  if (e != cudaSuccess) {
    free_plan(p);
    return (int)e;
  }
  *plan = p;
  return 0;
}

// Run every operation of the plan on `stream` (launches only: capturable).
GB_EXPORT int awkward_gb300_batch_plan_run(void* plan, void* stream) {
  Plan* p = static_cast<Plan*>(plan);
  if (!p) return (int)cudaErrorInvalidValue;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(p->d_counters, 0, sizeof(unsigned) * kOps, s);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(p->d_scan, 0, sizeof(unsigned long long) * (size_t)(p->ntiles + 1), s);
  if (e != cudaSuccess) return (int)e;
  SumOpD op0{};
  MaxOpD op1{};
  op1.ident = -INFINITY;
  ArgOpD op2{};
  if (p->nitems[0] > 0) {
    auto* rec0 = static_cast<RangeRecord<SumOpD::Acc>*>(p->d_records[0]);
    if (p->block == 128)
      batch_reduce_kernel<0, 128><<<p->blocks[0], 128, 0, s>>>(
          op0, p->d_arrays, p->d_items[0], p->d_order[0], p->nitems[0], rec0,
          p->d_counters + 0);
    else
      batch_reduce_kernel<0, 256><<<p->blocks[0], 256, 0, s>>>(
          op0, p->d_arrays, p->d_items[0], p->d_order[0], p->nitems[0], rec0,
          p->d_counters + 0);
    batch_fixup_kernel<0><<<(p->nitems[0] + 255) / 256, 256, 0, s>>>(
        op0, p->d_arrays, static_cast<RangeRecord<SumOpD::Acc>*>(p->d_records[0]), p->nitems[0]);
  }
  if (p->nitems[1] > 0) {
    auto* rec1 = static_cast<RangeRecord<MaxOpD::Acc>*>(p->d_records[1]);
    if (p->block == 128)
      batch_reduce_kernel<1, 128><<<p->blocks[1], 128, 0, s>>>(
          op1, p->d_arrays, p->d_items[1], p->d_order[1], p->nitems[1], rec1,
          p->d_counters + 1);
    else
      batch_reduce_kernel<1, 256><<<p->blocks[1], 256, 0, s>>>(
          op1, p->d_arrays, p->d_items[1], p->d_order[1], p->nitems[1], rec1,
          p->d_counters + 1);
    batch_fixup_kernel<1><<<(p->nitems[1] + 255) / 256, 256, 0, s>>>(
        op1, p->d_arrays, static_cast<RangeRecord<MaxOpD::Acc>*>(p->d_records[1]), p->nitems[1]);
  }
  if (p->nitems[2] > 0) {
    auto* rec2 = static_cast<RangeRecord<ArgOpD::Acc>*>(p->d_records[2]);
    if (p->block == 128)
      batch_reduce_kernel<2, 128><<<p->blocks[2], 128, 0, s>>>(
          op2, p->d_arrays, p->d_items[2], p->d_order[2], p->nitems[2], rec2,
          p->d_counters + 2);
    else
      batch_reduce_kernel<2, 256><<<p->blocks[2], 256, 0, s>>>(
          op2, p->d_arrays, p->d_items[2], p->d_order[2], p->nitems[2], rec2,
          p->d_counters + 2);
    batch_fixup_kernel<2><<<(p->nitems[2] + 255) / 256, 256, 0, s>>>(
        op2, p->d_arrays, static_cast<RangeRecord<ArgOpD::Acc>*>(p->d_records[2]), p->nitems[2]);
  }
  if (p->ntiles > 0) {
    batch_select_kernel<<<(unsigned)p->ntiles, kTileBlock, 0, s>>>(
        p->d_arrays, p->narrays, p->d_tile_base, p->d_scan, p->d_scan + 1, p->err);
  }
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_gb300_batch_plan_destroy(void* plan) {
  if (plan) free_plan(static_cast<Plan*>(plan));
  return 0;
}
