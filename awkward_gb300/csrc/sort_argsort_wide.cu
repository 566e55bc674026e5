// sort_argsort_wide.cu -- awkward_argsort for uint32, the 64-bit integers and
// floating point (segmented sort kernels: sort_impl.cuh).
#include "sort_impl.cuh"

GB_ARGSORT_ALL(uint32, uint32_t)
GB_ARGSORT_ALL(int64, int64_t)
GB_ARGSORT_ALL(uint64, uint64_t)
GB_ARGSORT_ALL(float32, float)
GB_ARGSORT_ALL(float64, double)
