// sv_sort.cuh -- stable LSD radix sort of (u32 key, u32 value) pairs and the
// run-based sort used for particle binning.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sv {

// Temporary storage needed by radix_sort_pairs for n elements (bytes).
size_t radix_sort_temp_bytes(uint64_t n);

// Stable sort of keys_in/vals_in (n pairs) on the low `key_bits` bits.
// vals_in may be nullptr: the values are then the element indices, so
// vals_out is the stable sorting permutation.  Results land in keys_out/vals_out.  `temp` must hold
// radix_sort_temp_bytes(n) bytes.  keys_in/vals_in are left intact.
cudaError_t radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                             uint32_t *vals_out, uint64_t n, int key_bits, void *temp, cudaStream_t stream);

// Exclusive scan of n u32 values (in place allowed).  temp must hold
// scan_temp_bytes(n) bytes.
size_t scan_temp_bytes(uint64_t n);

// Number of kernel launches the two calls above make for a given size.
int scan_launches(uint64_t n);
int radix_sort_launches(uint64_t n, int key_bits);
cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n, void *temp, cudaStream_t stream);

}  // namespace sv
