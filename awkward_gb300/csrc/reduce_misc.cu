// Entry points of awkward_reduce_countnonzero (kernel-specification.yml:4460),
// awkward_reduce_sumofsquares (:5196), awkward_reduce_sumofpowers (:5273),
// awkward_reduce_centered_sumofsquares (:5361), awkward_reduce_count_64
// (:4447), awkward_NumpyArray_reduce_adjust_starts_64 (:2550) and
// awkward_NumpyArray_reduce_mask_ByteMaskedArray_64 (:2585).
#include "reduce_ops.cuh"

using namespace gb;

#define GB_CNZ(NAME, IN)                                                                      \
  GB_EXPORT int NAME(int64_t* toptr, const IN* fromptr, const int64_t* offsets,               \
                     int64_t outlength, uint64_t invocation_index, uint64_t* err_code,        \
                     void* stream) {                                                          \
    return (int)launch_seg_reduce(CountNonzeroOp<IN>{},                                       \
                                  reinterpret_cast<const store_t<IN>*>(fromptr), offsets,     \
                                  outlength, toptr, invocation_index, err_code,               \
                                  (cudaStream_t)stream);                                      \
  }
#define GB_FOR_ALL_IN(M, PREFIX)                                                         \
  M(PREFIX##bool_64, bool) M(PREFIX##int8_64, int8_t) M(PREFIX##uint8_64, uint8_t)       \
  M(PREFIX##int16_64, int16_t) M(PREFIX##uint16_64, uint16_t)                            \
  M(PREFIX##int32_64, int32_t) M(PREFIX##uint32_64, uint32_t)                            \
  M(PREFIX##int64_64, int64_t) M(PREFIX##uint64_64, uint64_t)                            \
  M(PREFIX##float32_64, float) M(PREFIX##float64_64, double)
GB_FOR_ALL_IN(GB_CNZ, awkward_reduce_countnonzero_)

#define GB_SUMSQ(NAME, IN)                                                                      \
  GB_EXPORT int NAME(double* toptr, const IN* fromptr, const int64_t* offsets, int64_t outlength, \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {             \
    return (int)launch_seg_reduce(SumSqOp<IN>{}, reinterpret_cast<const store_t<IN>*>(fromptr), \
                                  offsets, outlength, toptr, invocation_index, err_code,        \
                                  (cudaStream_t)stream);                                        \
  }
#define GB_SUMPOW(NAME, IN)                                                                     \
  GB_EXPORT int NAME(double* toptr, const IN* fromptr, const int64_t* offsets, int64_t outlength, \
                     int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream) {  \
    SumPowOp<IN> op;                                                                            \
    op.n = n;                                                                                   \
    return (int)launch_seg_reduce(op, reinterpret_cast<const store_t<IN>*>(fromptr), offsets,   \
                                  outlength, toptr, invocation_index, err_code,                 \
                                  (cudaStream_t)stream);                                        \
  }
#define GB_CSUMSQ(NAME, IN)                                                                     \
  GB_EXPORT int NAME(double* toptr, const IN* fromptr, const int64_t* offsets, int64_t outlength, \
                     const double* means, uint64_t invocation_index, uint64_t* err_code,        \
                     void* stream) {                                                            \
    CenteredSumSqOp<IN> op;                                                                     \
    op.means = means;                                                                           \
    return (int)launch_seg_reduce(op, reinterpret_cast<const store_t<IN>*>(fromptr), offsets,   \
                                  outlength, toptr, invocation_index, err_code,                 \
                                  (cudaStream_t)stream);                                        \
  }
#define GB_FOR_F64_OUT(M, PREFIX)                                                          \
  M(PREFIX##float64_int8_64, int8_t) M(PREFIX##float64_uint8_64, uint8_t)                  \
  M(PREFIX##float64_int16_64, int16_t) M(PREFIX##float64_uint16_64, uint16_t)              \
  M(PREFIX##float64_int32_64, int32_t) M(PREFIX##float64_uint32_64, uint32_t)              \
  M(PREFIX##float64_int64_64, int64_t) M(PREFIX##float64_uint64_64, uint64_t)              \
  M(PREFIX##float64_bool_64, bool) M(PREFIX##float64_float32_64, float)                    \
  M(PREFIX##float64_float64_64, double)
GB_FOR_F64_OUT(GB_SUMSQ, awkward_reduce_sumofsquares_)
GB_FOR_F64_OUT(GB_SUMPOW, awkward_reduce_sumofpowers_)
GB_FOR_F64_OUT(GB_CSUMSQ, awkward_reduce_centered_sumofsquares_)

// ---------------------------------------------------------------- per-list maps
namespace {
constexpr int kMapBlock = 256;

inline int map_grid(long long n) {
  long long g = (n + kMapBlock - 1) / kMapBlock;
  long long cap = (long long)device_sm_count() * 16;
  return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

// awkward_reduce_count_64.cpp:7-15
__global__ void count_kernel(int64_t* __restrict__ toptr, const int64_t* __restrict__ offsets,
                             long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    toptr[i] = offsets[i + 1] - offsets[i];
}

// awkward_NumpyArray_reduce_adjust_starts_64.cpp:7-25
__global__ void adjust_starts_kernel(int64_t* __restrict__ toptr, long long n,
                                     const int64_t* __restrict__ starts) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    int64_t i = toptr[k];
    if (i >= 0) toptr[k] = i - starts[k];
  }
}

// awkward_NumpyArray_reduce_mask_ByteMaskedArray_64.cpp:7-20
__global__ void reduce_mask_kernel(int8_t* __restrict__ toptr,
                                   const int64_t* __restrict__ offsets, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    toptr[i] = (offsets[i + 1] - offsets[i] > 0) ? 0 : 1;
}
}  // namespace

GB_EXPORT int awkward_reduce_count_64(int64_t* toptr, const int64_t* offsets, int64_t outlength,
                                      uint64_t invocation_index, uint64_t* err_code,
                                      void* stream) {
  (void)invocation_index;
  (void)err_code;
  if (outlength <= 0) return 0;
  count_kernel<<<map_grid(outlength), kMapBlock, 0, (cudaStream_t)stream>>>(toptr, offsets,
                                                                            outlength);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_NumpyArray_reduce_adjust_starts_64(int64_t* toptr, int64_t outlength,
                                                         const int64_t* offsets,
                                                         const int64_t* starts,
                                                         uint64_t invocation_index,
                                                         uint64_t* err_code, void* stream) {
  (void)offsets;
  (void)invocation_index;
  (void)err_code;
  if (outlength <= 0) return 0;
  adjust_starts_kernel<<<map_grid(outlength), kMapBlock, 0, (cudaStream_t)stream>>>(
      toptr, outlength, starts);
  return (int)cudaGetLastError();
}

GB_EXPORT int awkward_NumpyArray_reduce_mask_ByteMaskedArray_64(int8_t* toptr,
                                                                const int64_t* offsets,
                                                                int64_t outlength,
                                                                uint64_t invocation_index,
                                                                uint64_t* err_code, void* stream) {
  (void)invocation_index;
  (void)err_code;
  if (outlength <= 0) return 0;
  reduce_mask_kernel<<<map_grid(outlength), kMapBlock, 0, (cudaStream_t)stream>>>(
      toptr, offsets, outlength);
  return (int)cudaGetLastError();
}
