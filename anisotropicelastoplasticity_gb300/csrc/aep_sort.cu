// aep_sort.cu -- per-step particle ordering: a stable LSD radix sort of
// (cell key, particle slot) pairs, restricted to the key bits in use.
// Stability keeps particles that stay in their cell in their previous relative
// order, so the permutation is close to the identity from step to step and
// the permuted reads of the particle arrays stay nearly coalesced.
#include <cub/device/device_radix_sort.cuh>

#include "aep_kernels.h"

namespace aep {

size_t sort_temp_bytes(int n, int key_bits) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (const int32_t*)nullptr, (int32_t*)nullptr, n, 0, key_bits);
    return bytes;
}

cudaError_t sort_pairs(void* temp, size_t temp_bytes, const uint32_t* keys_in, uint32_t* keys_out,
                       const int32_t* vals_in, int32_t* vals_out, int n, int key_bits, cudaStream_t s) {
    return cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys_in, keys_out, vals_in, vals_out, n, 0, key_bits, s);
}

}  // namespace aep
