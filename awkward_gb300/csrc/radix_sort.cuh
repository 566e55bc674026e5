// radix_sort.cuh -- device-wide building blocks shared by the non-local
// reduction kernels: a stable LSD radix sort of (key, value) pairs, an
// exclusive scan of int64 values and a "lower bound of every key" fill.
#pragma once

#include "gb_common.cuh"

namespace gb {

// Stable sort of n (key, value) pairs by the low `bits` bits of the keys
// (every key must be < 2^bits; 0 <= bits <= 64).  Reads keys_in / vals_in
// (left unchanged) and leaves the sorted pairs in keys_out / vals_out.
// Passes of 8 bits: per-tile digit counts, one scan of the counts, then a
// scatter that ranks equal digits in element order (which keeps it stable).
cudaError_t radix_sort_pairs(const unsigned long long* keys_in, const long long* vals_in,
                             unsigned long long* keys_out, long long* vals_out, long long n,
                             int bits, uint64_t inv, uint64_t* err, cudaStream_t s);

// out[i] = in[0] + ... + in[i-1] for i < n (single pass, decoupled
// look-back); `out` may alias `in`.  *total (a device word, may be null)
// receives the sum of all n values.  A look-back that gives up raises
// GB_MSG_TIMEOUT on (inv, err) -- the same for the sort, which scans with it.
cudaError_t exclusive_scan_i64(const long long* in, long long* out, long long n,
                               long long* total, uint64_t inv, uint64_t* err, cudaStream_t s);

// out[j] = number of sorted keys < j, for j in [0, count).
cudaError_t fill_lower_bounds(const unsigned long long* sorted_keys, long long n, long long* out,
                              long long count, cudaStream_t s);

// Number of bits needed to write v (0 for v == 0).
inline int bit_length(unsigned long long v) {
  int b = 0;
  while (v) {
    b++;
    v >>= 1;
  }
  return b;
}

}  // namespace gb
