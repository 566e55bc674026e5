// Entry points of awkward_reduce_argmax (kernel-specification.yml:4225) and
// awkward_reduce_argmin (:4336).  `starts` is unused, as in the CPU kernels.
#include "reduce_ops.cuh"

using namespace gb;

#define GB_ARG(NAME, T, MAX)                                                                  \
  GB_EXPORT int NAME(int64_t* toptr, const T* fromptr, const int64_t* offsets,                \
                     const int64_t* starts, int64_t outlength, uint64_t invocation_index,     \
                     uint64_t* err_code, void* stream) {                                      \
    (void)starts;                                                                             \
    return (int)launch_seg_reduce(ArgExtremumOp<T, MAX>{}, fromptr, offsets, outlength, toptr, \
                                  invocation_index, err_code, (cudaStream_t)stream);          \
  }
#define GB_FOR_NUMERIC_IN(M, PREFIX, ARG)                                              \
  M(PREFIX##int8_64, int8_t, ARG) M(PREFIX##uint8_64, uint8_t, ARG)                    \
  M(PREFIX##int16_64, int16_t, ARG) M(PREFIX##uint16_64, uint16_t, ARG)                \
  M(PREFIX##int32_64, int32_t, ARG) M(PREFIX##uint32_64, uint32_t, ARG)                \
  M(PREFIX##int64_64, int64_t, ARG) M(PREFIX##uint64_64, uint64_t, ARG)                \
  M(PREFIX##float32_64, float, ARG) M(PREFIX##float64_64, double, ARG)

GB_FOR_NUMERIC_IN(GB_ARG, awkward_reduce_argmax_, true)
GB_FOR_NUMERIC_IN(GB_ARG, awkward_reduce_argmin_, false)
