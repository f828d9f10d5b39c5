// Device-wide primitives: decoupled look-back exclusive scan and onesweep LSD radix sort.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace qses {

// Exclusive scan of n uint2 values (in place allowed).  *d_total (device) receives the sum.
size_t scan_u2_tmp_bytes(unsigned n);
cudaError_t scan_u2(const uint2 *in, uint2 *out, unsigned n, uint2 *d_total, void *tmp, int *d_err,
                    cudaStream_t s, int *launches);

// Stable LSD radix sort of (key, value) pairs on the low `bits` bits of the keys.
// Ping-pongs between (keys, vals) and (keys_alt, vals_alt); *in_alt tells which pair holds
// the result.  With identity = true the input values are the positions 0..n-1 and `vals`
// is only used as storage.  keys_in (optional): the input keys, left unchanged; `keys` is
// then only storage.
size_t radix_sort_tmp_bytes(unsigned n, int bits);
template <typename K>
cudaError_t radix_sort(K *keys, K *keys_alt, unsigned *vals, unsigned *vals_alt, unsigned n, int bits,
                       bool identity, void *tmp, int *d_err, cudaStream_t s, int *launches, int *in_alt,
                       const K *keys_in = nullptr);

inline int bits_for(unsigned long long max_value) {
    int b = 0;
    while (b < 64 && (max_value >> b) != 0) b++;
    return b;
}

}  // namespace qses
