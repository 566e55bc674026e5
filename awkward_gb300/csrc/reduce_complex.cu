// reduce_complex.cu -- the complex reducers (interleaved re, im pairs).
//
//   awkward_reduce_sum_complex        awkward_reduce_sum_complex.cpp:7-24
//   awkward_reduce_prod_complex       awkward_reduce_prod_complex.cpp:9-31
//   awkward_reduce_max/min_complex    awkward_reduce_max_complex.cpp:7-33 (min alike)
//   awkward_reduce_argmax/argmin_complex  awkward_reduce_argmax_complex.cpp:7-33
//   awkward_reduce_countnonzero_complex / _sum_bool_complex / _prod_bool_complex
//
// All but prod run on the segmented reducer (seg_reduce.cuh) with a complex
// element type.  The extrema follow the CPU loop exactly: the first element
// seeds, a later one replaces the best when x > bx || (x == bx && y > by).
// With NaN that relation is not a total order, but its sequential result is
// still an associative reduction: if the list's first element has a NaN real
// part, nothing replaces it ("sink"); otherwise elements with a NaN real part
// never take part, the level X = largest real part wins, the level's first
// element ("entry") wins if its imaginary part is NaN, and otherwise the first
// element of the largest non-NaN imaginary part at that level wins.  The sum
// is exact per component in fixed point (FxAcc), rounded once.  The product is
// computed per list in the CPU's order with unfused multiplies and adds, so it
// rounds exactly like the CPU loop.
#include "reduce_ops.cuh"

namespace gb {

template <class T>
struct Cx {
  T re, im;
};

// Element loads of the generic reducer paths (found by argument-dependent
// lookup when they are instantiated for Cx).
__device__ __forceinline__ Cx<double> __ldg(const Cx<double>* p) {
  return Cx<double>{::__ldg(&p->re), ::__ldg(&p->im)};
}
__device__ __forceinline__ Cx<float> __ldg(const Cx<float>* p) {
  return Cx<float>{::__ldg(&p->re), ::__ldg(&p->im)};
}

constexpr uint32_t kCxHas = 1, kCxSink = 2, kCxEntryNan = 4, kCxHasY = 8;

template <class T, bool MAX, bool ARG>
struct CxExtremumOp {
  using In = Cx<T>;
  using Out = typename std::conditional<ARG, int64_t, Cx<T>>::type;
  struct Acc {
    T level;     // real part of the winning level
    T ere, eim;  // the level's first element (or the sink)
    T bre, by;   // the level's first element of the best non-NaN imaginary part
    long long eidx, bidx;
    uint32_t flags, pad;
  };
  static constexpr bool kNeedsFirst = true;
  T ident;
  __device__ static bool better(T a, T b) { return MAX ? a > b : a < b; }
  __device__ Acc identity() const {
    Acc a{};
    a.eidx = a.bidx = -1;
    return a;
  }
  __device__ Acc lift(Cx<T> v, long long j, bool first, long long) const {
    Acc a = identity();
    if (v.re != v.re) {
      if (first) {
        a.ere = v.re;
        a.eim = v.im;
        a.eidx = j;
        a.flags = kCxHas | kCxSink;
      }
      return a;
    }
    a.level = v.re;
    a.ere = v.re;
    a.eim = v.im;
    a.eidx = j;
    a.flags = kCxHas;
    if (v.im != v.im) {
      a.flags |= kCxEntryNan;
    } else {
      a.bre = v.re;
      a.by = v.im;
      a.bidx = j;
      a.flags |= kCxHasY;
    }
    return a;
  }
  __device__ Acc combine(Acc a, Acc b) const {
    if (a.flags & kCxSink) return a;
    if (b.flags & kCxSink) return b;
    if (!(a.flags & kCxHas)) return b;
    if (!(b.flags & kCxHas)) return a;
    if (better(a.level, b.level)) return a;
    if (better(b.level, a.level)) return b;
    // the same level: the earlier entry, the best imaginary part of both
    const bool a_first = a.eidx < b.eidx;
    Acc r = a_first ? a : b;
    const Acc& o = a_first ? b : a;
    if ((o.flags & kCxHasY) &&
        (!(r.flags & kCxHasY) || better(o.by, r.by) || (o.by == r.by && o.bidx < r.bidx))) {
      r.bre = o.bre;
      r.by = o.by;
      r.bidx = o.bidx;
      r.flags |= kCxHasY;
    }
    return r;
  }
  __device__ Acc step(Acc a, Cx<T> v, long long j, bool first, long long li) const {
    return combine(a, lift(v, j, first, li));
  }
  __device__ Out finalize(Acc a, long long) const {
    const bool entry = (a.flags & (kCxSink | kCxEntryNan)) != 0;
    if constexpr (ARG) {
      if (!(a.flags & kCxHas)) return -1;
      return entry ? a.eidx : a.bidx;
    } else {
      if (!(a.flags & kCxHas)) return Cx<T>{ident, T(0)};
      return entry ? Cx<T>{a.ere, a.eim} : Cx<T>{a.bre, a.by};
    }
  }
};

template <class T>
struct CxSumOp {
  using In = Cx<T>;
  using Out = Cx<T>;
  struct Acc {
    FxAcc re, im;
  };
  static constexpr bool kNeedsFirst = false;
  __device__ static FxAcc add(FxAcc a, T v) {
    if constexpr (std::is_same<T, double>::value) return fx_add_f64(a, v);
    else return fx_add_f32(a, v);
  }
  __device__ Acc identity() const { return Acc{FxAcc{0, 1, 0}, FxAcc{0, 1, 0}}; }
  __device__ Acc lift(Cx<T> v, long long, bool, long long) const {
    return Acc{add(FxAcc{0, 1, 0}, v.re), add(FxAcc{0, 1, 0}, v.im)};
  }
  __device__ Acc combine(Acc a, Acc b) const {
    return Acc{fx_combine(a.re, b.re), fx_combine(a.im, b.im)};
  }
  __device__ Acc step(Acc a, Cx<T> v, long long, bool, long long) const {
    return Acc{add(a.re, v.re), add(a.im, v.im)};
  }
  __device__ Out finalize(Acc a, long long) const {
    return Cx<T>{static_cast<T>(fx_finalize(a.re)), static_cast<T>(fx_finalize(a.im))};
  }
};

// MODE 0: count of nonzero elements; 1: any nonzero; 2: every element nonzero.
template <class T, int MODE>
struct CxNonzeroOp {
  using In = Cx<T>;
  using Out = typename std::conditional<MODE == 0, int64_t, bool>::type;
  using Acc = long long;  // nonzero (MODE 0, 1) or zero (MODE 2) elements
  static constexpr bool kNeedsFirst = false;
  __device__ static long long hit(Cx<T> v) {
    const bool nz = v.re != T(0) || v.im != T(0);
    return MODE == 2 ? !nz : nz;
  }
  __device__ Acc identity() const { return 0; }
  __device__ Acc lift(Cx<T> v, long long, bool, long long) const { return hit(v); }
  __device__ Acc combine(Acc a, Acc b) const { return a + b; }
  __device__ Acc step(Acc a, Cx<T> v, long long, bool, long long) const { return a + hit(v); }
  __device__ Out finalize(Acc a, long long) const {
    if constexpr (MODE == 0) return a;
    else if constexpr (MODE == 1) return a > 0;
    else return a == 0;
  }
};

}  // namespace gb

using namespace gb;

namespace {

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// One list per thread, the CPU's loop: (a, b) *= (c, d) in list order.
template <class T>
__global__ void __launch_bounds__(256)
    prod_complex_kernel(T* __restrict__ out, const T* __restrict__ x,
                        const int64_t* __restrict__ offsets, long long n) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n;
       l += (long long)gridDim.x * blockDim.x) {
    T a = T(1), b = T(0);
    for (long long i = offsets[l]; i < offsets[l + 1]; i++) {
      const T c = x[2 * i], d = x[2 * i + 1];
      const T na = sub_rn(mul_rn(a, c), mul_rn(b, d));
      const T nb = add_rn(mul_rn(a, d), mul_rn(b, c));
      a = na;
      b = nb;
    }
    out[2 * l] = a;
    out[2 * l + 1] = b;
  }
}

template <class T>
int launch_prod_complex(T* toptr, const T* fromptr, const int64_t* offsets, int64_t outlength,
                        cudaStream_t s) {
  if (outlength <= 0) return (int)cudaSuccess;
  long long g = (outlength + 255) / 256;
  const long long cap = (long long)device_sm_count() * 16;
  prod_complex_kernel<T><<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(toptr, fromptr, offsets,
                                                                    outlength);
  return (int)cudaGetLastError();
}

}  // namespace

#define GB_CX_SUM(NAME, T)                                                                    \
  GB_EXPORT int NAME(T* toptr, const T* fromptr, const int64_t* offsets, int64_t outlength,   \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {           \
    return (int)launch_seg_reduce(CxSumOp<T>{}, reinterpret_cast<const Cx<T>*>(fromptr),      \
                                  offsets, outlength, reinterpret_cast<Cx<T>*>(toptr),        \
                                  invocation_index, err_code, (cudaStream_t)stream);          \
  }
GB_CX_SUM(awkward_reduce_sum_complex64_complex64_64, float)
GB_CX_SUM(awkward_reduce_sum_complex128_complex128_64, double)

#define GB_CX_PROD(NAME, T)                                                                   \
  GB_EXPORT int NAME(T* toptr, const T* fromptr, const int64_t* offsets, int64_t outlength,   \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {           \
    (void)invocation_index;                                                                   \
    (void)err_code;                                                                           \
    return launch_prod_complex<T>(toptr, fromptr, offsets, outlength, (cudaStream_t)stream);  \
  }
GB_CX_PROD(awkward_reduce_prod_complex64_complex64_64, float)
GB_CX_PROD(awkward_reduce_prod_complex128_complex128_64, double)

#define GB_CX_EXT(NAME, T, MAX)                                                               \
  GB_EXPORT int NAME(T* toptr, const T* fromptr, const int64_t* offsets, int64_t outlength,   \
                     T identity, uint64_t invocation_index, uint64_t* err_code,               \
                     void* stream) {                                                          \
    CxExtremumOp<T, MAX, false> op;                                                           \
    op.ident = identity;                                                                      \
    return (int)launch_seg_reduce(op, reinterpret_cast<const Cx<T>*>(fromptr), offsets,      \
                                  outlength, reinterpret_cast<Cx<T>*>(toptr),                 \
                                  invocation_index, err_code, (cudaStream_t)stream);          \
  }
GB_CX_EXT(awkward_reduce_max_complex64_complex64_64, float, true)
GB_CX_EXT(awkward_reduce_max_complex128_complex128_64, double, true)
GB_CX_EXT(awkward_reduce_min_complex64_complex64_64, float, false)
GB_CX_EXT(awkward_reduce_min_complex128_complex128_64, double, false)

#define GB_CX_ARG(NAME, T, MAX)                                                               \
  GB_EXPORT int NAME(int64_t* toptr, const T* fromptr, const int64_t* offsets,                \
                     int64_t outlength, uint64_t invocation_index, uint64_t* err_code,        \
                     void* stream) {                                                          \
    CxExtremumOp<T, MAX, true> op;                                                            \
    op.ident = T(0);                                                                          \
    return (int)launch_seg_reduce(op, reinterpret_cast<const Cx<T>*>(fromptr), offsets,      \
                                  outlength, toptr, invocation_index, err_code,               \
                                  (cudaStream_t)stream);                                      \
  }
GB_CX_ARG(awkward_reduce_argmax_complex64_64, float, true)
GB_CX_ARG(awkward_reduce_argmax_complex128_64, double, true)
GB_CX_ARG(awkward_reduce_argmin_complex64_64, float, false)
GB_CX_ARG(awkward_reduce_argmin_complex128_64, double, false)

#define GB_CX_NZ(NAME, OUT, T, MODE)                                                          \
  GB_EXPORT int NAME(OUT* toptr, const T* fromptr, const int64_t* offsets, int64_t outlength, \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {           \
    return (int)launch_seg_reduce(CxNonzeroOp<T, MODE>{},                                     \
                                  reinterpret_cast<const Cx<T>*>(fromptr), offsets,           \
                                  outlength, toptr, invocation_index, err_code,               \
                                  (cudaStream_t)stream);                                      \
  }
GB_CX_NZ(awkward_reduce_countnonzero_complex64_64, int64_t, float, 0)
GB_CX_NZ(awkward_reduce_countnonzero_complex128_64, int64_t, double, 0)
GB_CX_NZ(awkward_reduce_sum_bool_complex64_64, bool, float, 1)
GB_CX_NZ(awkward_reduce_sum_bool_complex128_64, bool, double, 1)
GB_CX_NZ(awkward_reduce_prod_bool_complex64_64, bool, float, 2)
GB_CX_NZ(awkward_reduce_prod_bool_complex128_64, bool, double, 2)
