// Entry points of awkward_reduce_prod (kernel-specification.yml:4794),
// awkward_reduce_prod_bool (:4931) and awkward_reduce_sum_bool (:5477).
#include "reduce_ops.cuh"

using namespace gb;

#define GB_PROD(NAME, OUT, IN)                                                                  \
  GB_EXPORT int NAME(OUT* toptr, const IN* fromptr, const int64_t* offsets, int64_t outlength,  \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {             \
    return (int)launch_seg_reduce(ProdOp<OUT, IN>{}, fromptr, offsets, outlength, toptr,        \
                                  invocation_index, err_code, (cudaStream_t)stream);            \
  }
#define GB_ANYALL(NAME, IN, ALL)                                                                 \
  GB_EXPORT int NAME(bool* toptr, const IN* fromptr, const int64_t* offsets, int64_t outlength, \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {             \
    return (int)launch_seg_reduce(AnyAllOp<IN, ALL>{},                                          \
                                  reinterpret_cast<const store_t<IN>*>(fromptr), offsets,       \
                                  outlength, toptr, invocation_index, err_code,                 \
                                  (cudaStream_t)stream);                                        \
  }
#define GB_FOR_ALL_IN(M, PREFIX, ARG)                                                       \
  M(PREFIX##bool_64, bool, ARG) M(PREFIX##int8_64, int8_t, ARG)                             \
  M(PREFIX##uint8_64, uint8_t, ARG) M(PREFIX##int16_64, int16_t, ARG)                       \
  M(PREFIX##uint16_64, uint16_t, ARG) M(PREFIX##int32_64, int32_t, ARG)                     \
  M(PREFIX##uint32_64, uint32_t, ARG) M(PREFIX##int64_64, int64_t, ARG)                     \
  M(PREFIX##uint64_64, uint64_t, ARG) M(PREFIX##float32_64, float, ARG)                     \
  M(PREFIX##float64_64, double, ARG)

GB_PROD(awkward_reduce_prod_int64_int8_64, int64_t, int8_t)
GB_PROD(awkward_reduce_prod_uint64_uint8_64, uint64_t, uint8_t)
GB_PROD(awkward_reduce_prod_int64_int16_64, int64_t, int16_t)
GB_PROD(awkward_reduce_prod_uint64_uint16_64, uint64_t, uint16_t)
GB_PROD(awkward_reduce_prod_int64_int32_64, int64_t, int32_t)
GB_PROD(awkward_reduce_prod_uint64_uint32_64, uint64_t, uint32_t)
GB_PROD(awkward_reduce_prod_int64_int64_64, int64_t, int64_t)
GB_PROD(awkward_reduce_prod_uint64_uint64_64, uint64_t, uint64_t)
GB_PROD(awkward_reduce_prod_float32_float32_64, float, float)
GB_PROD(awkward_reduce_prod_float64_float64_64, double, double)
GB_PROD(awkward_reduce_prod_int32_int8_64, int32_t, int8_t)
GB_PROD(awkward_reduce_prod_uint32_uint8_64, uint32_t, uint8_t)
GB_PROD(awkward_reduce_prod_int32_int16_64, int32_t, int16_t)
GB_PROD(awkward_reduce_prod_uint32_uint16_64, uint32_t, uint16_t)
GB_PROD(awkward_reduce_prod_int32_int32_64, int32_t, int32_t)
GB_PROD(awkward_reduce_prod_uint32_uint32_64, uint32_t, uint32_t)
GB_FOR_ALL_IN(GB_ANYALL, awkward_reduce_prod_bool_, true)
GB_FOR_ALL_IN(GB_ANYALL, awkward_reduce_sum_bool_, false)
