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
// partition order is slot order, so ties keep slot order.  m is read on the device.
__global__ void __launch_bounds__(kRankThreads) k_rank_movers(const uint32_t* __restrict__ keys,
                                                              const int32_t* __restrict__ part,
                                                              const int32_t* __restrict__ nmov, int cap,
                                                              uint32_t* __restrict__ mkeys, int32_t* __restrict__ mslot) {
    const int m = *nmov;
    if (m > cap) return;  // not this branch (the decision kernel never sends it here)
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

// movers into `cap` sort slots; slots past m get the largest key of the sorted
// bits (`pad`) and, coming last, stay after any mover with that key (stable sort)
__global__ void k_gather_movers(const uint32_t* __restrict__ keys, const int32_t* __restrict__ part,
                                const int32_t* __restrict__ nmov, int cap, uint32_t pad, uint32_t* __restrict__ mk,
                                int32_t* __restrict__ mj) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= cap) return;
    if (r < *nmov) {
        const int j = part[r];
        mk[r] = keys[j];
        mj[r] = j;
    } else {
        mk[r] = pad;
        mj[r] = -1;
    }
}

// merge of the stayers (partition tail, reversed: stayer q is part[n-1-q]) and the
// sorted movers; stayers go before movers with an equal key
__global__ void k_merge_movers(const uint32_t* __restrict__ keys, const int32_t* __restrict__ part, int n, int cap,
                               const int32_t* __restrict__ nmov, const uint32_t* __restrict__ mkeys,
                               const int32_t* __restrict__ mslot, uint32_t* __restrict__ keys_out,
                               int32_t* __restrict__ perm_out) {
    const int m = *nmov;
    if (m > cap || m > n) return;  // not this branch
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

// the branch of the ordering graph: 0 rank (m <= kBruteMovers), 1 radix sort of the
// movers (m <= cap), 2 full sort
__global__ void k_order_decide(const int32_t* __restrict__ nmov, int cap, cudaGraphConditionalHandle h,
                               DevStats* st) {
    const int m = *nmov;
    // the mover arrays hold `cap` entries: more movers take the full sort
    const unsigned branch = m > cap ? 2u : (m <= kBruteMovers ? 0u : 1u);
    cudaGraphSetConditional(h, branch);
    st->movers = branch == 2u ? -1ll : (long long)m;
}

struct OrderGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

#define OG_CK(x)                                 \
    do {                                         \
        cudaError_t e_ = (x);                    \
        if (e_ != cudaSuccess) {                 \
            cudaGraph_t open_ = nullptr;         \
            cudaStreamEndCapture(cs, &open_);    \
            cudaGetLastError();                  \
            cudaGraphDestroy(g);                 \
            return e_;                           \
        }                                        \
    } while (0)

}  // namespace

size_t partition_temp_bytes(int n) {
    size_t bytes = 0;
    cub::DevicePartition::If(nullptr, bytes, (const int32_t*)nullptr, (int32_t*)nullptr, (int32_t*)nullptr, n,
                             MoverOp{nullptr, nullptr});
    return bytes;
}

// Capture the incremental ordering into a graph: partition (CUB), the branch
// decision on the device, and a three-way switch (rank + merge | radix sort of
// the movers + merge | full radix sort).  No host synchronisation per step.
cudaError_t order_graph_build(void** out, cudaStream_t cs, const OrderBuffers& b) {
    *out = nullptr;
    cudaGraph_t g = nullptr, dummy = nullptr;  // dummy receives the graph a capture ended into
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h;
    OG_CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
    OG_CK(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    size_t part_bytes = b.part_bytes, sort_bytes = b.sort_bytes;  // CUB takes them by reference
    OG_CK(cub::DevicePartition::If(b.part_tmp, part_bytes, b.iota, b.part, b.nmov, b.n,
                                   MoverOp{b.keys, b.keys_sorted}, cs));
    k_order_decide<<<1, 1, 0, cs>>>(b.nmov, b.cap, h, b.st);
    OG_CK(cudaGetLastError());
    cudaStreamCaptureStatus status;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    OG_CK(cudaStreamGetCaptureInfo(cs, &status, nullptr, nullptr, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeSwitch;
    cp.conditional.size = 3;
    cudaGraphNode_t cnode;
    OG_CK(cudaGraphAddNode(&cnode, g, deps, nullptr, ndeps, &cp));
    OG_CK(cudaStreamEndCapture(cs, &dummy));
    dummy = nullptr;
    cudaGraph_t* body = cp.conditional.phGraph_out;
    const int n = b.n;
    // case 0: brute-force rank of at most kBruteMovers movers, merge
    OG_CK(cudaStreamBeginCaptureToGraph(cs, body[0], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    k_rank_movers<<<(unsigned)((32l * kBruteMovers + kRankThreads - 1) / kRankThreads), kRankThreads, 0, cs>>>(
        b.keys, b.part, b.nmov, b.cap, b.mkeys, b.mslot);
    k_merge_movers<<<(n + 255) / 256, 256, 0, cs>>>(b.keys, b.part, n, b.cap, b.nmov, b.mkeys, b.mslot,
                                                     b.keys_sorted, b.perm);
    OG_CK(cudaGetLastError());
    OG_CK(cudaStreamEndCapture(cs, &dummy));
    dummy = nullptr;
    // case 1: radix sort of the movers in `cap` padded slots (stable: ties keep slot order), merge
    OG_CK(cudaStreamBeginCaptureToGraph(cs, body[1], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const uint32_t pad = b.key_bits >= 32 ? 0xFFFFFFFFu : ((1u << b.key_bits) - 1u);
    k_gather_movers<<<(b.cap + 255) / 256, 256, 0, cs>>>(b.keys, b.part, b.nmov, b.cap, pad, b.mk_tmp, b.mj_tmp);
    OG_CK(cudaGetLastError());
    OG_CK(cub::DeviceRadixSort::SortPairs(b.sort_tmp, sort_bytes, b.mk_tmp, b.mkeys, b.mj_tmp, b.mslot, b.cap, 0,
                                          b.key_bits, cs));
    k_merge_movers<<<(n + 255) / 256, 256, 0, cs>>>(b.keys, b.part, n, b.cap, b.nmov, b.mkeys, b.mslot,
                                                     b.keys_sorted, b.perm);
    OG_CK(cudaGetLastError());
    OG_CK(cudaStreamEndCapture(cs, &dummy));
    dummy = nullptr;
    // case 2: full radix sort
    OG_CK(cudaStreamBeginCaptureToGraph(cs, body[2], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    sort_bytes = b.sort_bytes;
    OG_CK(cub::DeviceRadixSort::SortPairs(b.sort_tmp, sort_bytes, b.keys, b.keys_sorted, b.iota, b.perm, n, 0,
                                          b.key_bits, cs));
    OG_CK(cudaStreamEndCapture(cs, &dummy));
    dummy = nullptr;
    OrderGraph* og = new OrderGraph();
    og->graph = g;
    e = cudaGraphInstantiate(&og->exec, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        delete og;
        return e;
    }
    *out = og;
    return cudaSuccess;
}

cudaError_t order_graph_launch(void* og, cudaStream_t s) {
    return cudaGraphLaunch(static_cast<OrderGraph*>(og)->exec, s);
}

void order_graph_destroy(void* og) {
    if (!og) return;
    OrderGraph* o = static_cast<OrderGraph*>(og);
    if (o->exec) cudaGraphExecDestroy(o->exec);
    if (o->graph) cudaGraphDestroy(o->graph);
    delete o;
}

}  // namespace aep
