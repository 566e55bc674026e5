// Entry points of awkward_reduce_max (kernel-specification.yml:4562) and
// awkward_reduce_min (:4678).
#include "reduce_ops.cuh"

using namespace gb;

#define GB_EXT(NAME, T, MAX)                                                                   \
  GB_EXPORT int NAME(T* toptr, const T* fromptr, const int64_t* offsets, int64_t outlength,    \
                     T identity, uint64_t invocation_index, uint64_t* err_code, void* stream) { \
    ExtremumOp<T, MAX> op;                                                                     \
    op.ident = identity;                                                                       \
    return (int)launch_seg_reduce(op, fromptr, offsets, outlength, toptr, invocation_index,    \
                                  err_code, (cudaStream_t)stream);                             \
  }
#define GB_FOR_NUMERIC_SAME(M, PREFIX, ARG)                                                  \
  M(PREFIX##int8_int8_64, int8_t, ARG) M(PREFIX##uint8_uint8_64, uint8_t, ARG)               \
  M(PREFIX##int16_int16_64, int16_t, ARG) M(PREFIX##uint16_uint16_64, uint16_t, ARG)         \
  M(PREFIX##int32_int32_64, int32_t, ARG) M(PREFIX##uint32_uint32_64, uint32_t, ARG)         \
  M(PREFIX##int64_int64_64, int64_t, ARG) M(PREFIX##uint64_uint64_64, uint64_t, ARG)         \
  M(PREFIX##float32_float32_64, float, ARG) M(PREFIX##float64_float64_64, double, ARG)

GB_FOR_NUMERIC_SAME(GB_EXT, awkward_reduce_max_, true)
GB_FOR_NUMERIC_SAME(GB_EXT, awkward_reduce_min_, false)
