// aep_sort.cu -- per-step particle ordering by (cell key, particle slot).
//
// Full sort: a stable LSD radix sort (CUB) of the key bits in use.  Stability
// keeps particles that stay in their cell in their previous relative order, so
// the permutation is close to the identity from step to step and the permuted
// reads of the particle arrays stay nearly coalesced.
//
// Incremental sort: from one step to the next only the particles that crossed a
// cell boundary change key (about 1% at the workloads' time steps).  With `prev`
// any ascending key array of the same length (the last sorted keys), the slots
// whose new key equals prev[j] form an ascending subsequence.  So: partition the
// slots into movers (key != prev) and stayers, keeping slot order (CUB
// DevicePartition); sort the few movers by (key, slot) (a brute-force rank for
// small counts, the radix sort otherwise); merge the two ascending lists, stayers
// before movers on equal keys.  The result is an ascending key order; it is a
// deterministic function of the keys, so steps repeat bit for bit.
#include <cub/device/device_partition.cuh>
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

namespace {

struct MoverOp {
    const uint32_t* keys;
    const uint32_t* prev;
    __device__ __forceinline__ bool operator()(const int32_t& j) const { return keys[j] != prev[j]; }
};

constexpr int kRankThreads = 256;

// rank of mover i among all movers by (key, partition index), one warp per mover;
// partition order is slot order, so ties keep slot order
__global__ void __launch_bounds__(kRankThreads) k_rank_movers(const uint32_t* __restrict__ keys,
                                                              const int32_t* __restrict__ part, int m,
                                                              uint32_t* __restrict__ mkeys, int32_t* __restrict__ mslot) {
    const int i = (int)(((long)blockIdx.x * kRankThreads + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= m) return;
    const int ji = part[i];
    const uint32_t ki = keys[ji];
    int rank = 0;
    for (int k = lane; k < m; k += 32) {
        const uint32_t kk = keys[part[k]];
        rank += (kk < ki) | ((kk == ki) & (k < i));
    }
    rank = __reduce_add_sync(0xffffffffu, rank);
    if (lane == 0) {
        mkeys[rank] = ki;
        mslot[rank] = ji;
    }
}

__global__ void k_gather_movers(const uint32_t* __restrict__ keys, const int32_t* __restrict__ part, int m,
                                uint32_t* __restrict__ mk, int32_t* __restrict__ mj) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < m) {
        const int j = part[r];
        mk[r] = keys[j];
        mj[r] = j;
    }
}

// merge of the stayers (partition tail, reversed: stayer q is part[n-1-q]) and the
// sorted movers; stayers go before movers with an equal key
__global__ void k_merge_movers(const uint32_t* __restrict__ keys, const int32_t* __restrict__ part, int n, int m,
                               const uint32_t* __restrict__ mkeys, const int32_t* __restrict__ mslot,
                               uint32_t* __restrict__ keys_out, int32_t* __restrict__ perm_out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ns = n - m;
    if (t < ns) {
        const int j = part[n - 1 - t];
        const uint32_t k = keys[j];
        int lo = 0, hi = m;  // movers with key < k
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (mkeys[mid] < k) lo = mid + 1;
            else hi = mid;
        }
        keys_out[t + lo] = k;
        perm_out[t + lo] = j;
    } else if (t < n) {
        const int r = t - ns;
        const uint32_t k = mkeys[r];
        int lo = 0, hi = ns;  // stayers with key <= k
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (keys[part[n - 1 - mid]] <= k) lo = mid + 1;
            else hi = mid;
        }
        keys_out[r + lo] = k;
        perm_out[r + lo] = mslot[r];
    }
}

}  // namespace

size_t partition_temp_bytes(int n) {
    size_t bytes = 0;
    cub::DevicePartition::If(nullptr, bytes, (const int32_t*)nullptr, (int32_t*)nullptr, (int32_t*)nullptr, n,
                             MoverOp{nullptr, nullptr});
    return bytes;
}

cudaError_t partition_movers(void* temp, size_t temp_bytes, const uint32_t* keys, const uint32_t* prev,
                             const int32_t* iota, int32_t* part, int32_t* num_movers, int n, cudaStream_t s) {
    return cub::DevicePartition::If(temp, temp_bytes, iota, part, num_movers, n, MoverOp{keys, prev}, s);
}

cudaError_t sort_movers(void* temp, size_t temp_bytes, const uint32_t* keys, const int32_t* part, int m,
                        uint32_t* mk_tmp, int32_t* mj_tmp, uint32_t* mkeys, int32_t* mslot, int key_bits,
                        cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    if (m <= kBruteMovers) {
        const long threads = 32l * m;
        k_rank_movers<<<(unsigned)((threads + kRankThreads - 1) / kRankThreads), kRankThreads, 0, s>>>(keys, part, m,
                                                                                                     mkeys, mslot);
        return cudaGetLastError();
    }
    k_gather_movers<<<(m + 255) / 256, 256, 0, s>>>(keys, part, m, mk_tmp, mj_tmp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // stable radix sort: ties keep partition (= slot) order
    return cub::DeviceRadixSort::SortPairs(temp, temp_bytes, mk_tmp, mkeys, mj_tmp, mslot, m, 0, key_bits, s);
}

cudaError_t merge_movers(const uint32_t* keys, const int32_t* part, int n, int m, const uint32_t* mkeys,
                         const int32_t* mslot, uint32_t* keys_out, int32_t* perm_out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_merge_movers<<<(n + 255) / 256, 256, 0, s>>>(keys, part, n, m, mkeys, mslot, keys_out, perm_out);
    return cudaGetLastError();
}

}  // namespace aep
