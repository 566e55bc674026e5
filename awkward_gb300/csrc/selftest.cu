// selftest.cu -- a look-back that is made to run out, for the failure-report
// tests.  One warp claims tile 1 of a fresh scan (tile states zeroed, so tile
// 0 never publishes) and runs the same decoupled look-back as the scan
// kernels with a short spin limit: the wait gives up, the warp raises
// GB_MSG_TIMEOUT through awkward's error protocol (atomicMin on err_code) and
// the kernel returns.  No GPU fault, trap or hang is involved.
#include "gb_common.cuh"

using namespace gb;

namespace {

__global__ void selftest_lookback_kernel(ScanTiles st, uint32_t spin_limit, uint64_t inv,
                                         uint64_t* err) {
  lookback_exclusive(st, 1, 1, inv, err, GB_MSG_TIMEOUT, spin_limit);
}

}  // namespace

GB_EXPORT int awkward_gb300_selftest_lookback_timeout(uint32_t spin_limit,
                                                      uint64_t invocation_index,
                                                      uint64_t* err_code, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (spin_limit < 1) spin_limit = 1;
  if (spin_limit > kSpinLimit) spin_limit = kSpinLimit;
  ScanTiles st;
  void* base = nullptr;
  cudaError_t e = scan_tiles_alloc(&st, &base, 2, s);
  if (e != cudaSuccess) return (int)e;
  selftest_lookback_kernel<<<1, 32, 0, s>>>(st, spin_limit, invocation_index, err_code);
  e = cudaGetLastError();
  cudaError_t f = scratch_free(base, s);
  return (int)(e != cudaSuccess ? e : f);
}
