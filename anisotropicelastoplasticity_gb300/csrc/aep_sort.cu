// aep_sort.cu -- per-step particle ordering by (cell key, particle slot).
//
// Full sort: a stable LSD radix sort of the key bits in use (below).  Stability
// keeps particles that stay in their cell in their previous relative order, so
// the permutation is close to the identity from step to step and the permuted
// reads of the particle arrays stay nearly coalesced.
//
// Incremental ordering: from one step to the next only the particles that
// crossed a cell boundary change key (well under 1% at the workloads' time
// steps).  With `prev` any ascending key array of the same length (the last
// sorted keys), the slots whose new key equals prev[j] ("stayers") form an
// ascending subsequence; the others are "movers".  The result is the merge of
// the stayers (slot order) with the movers sorted by (key, slot), stayers first
// on equal keys:
//   position of stayer j  = (stayers before slot j) + (movers with key < key_j)
//   position of mover r   = (movers before it by (key, slot))
//                           + (stayers with key <= its key)
// where "stayers with key <= k" = upper_bound(prev, k) - (movers whose prev key
// is <= k), since a stayer's key is its prev key.  Kernels:
//   k_flag_movers   mover bitmask, per-block mover counts and the mover list
//                   (appended in any order: placement depends only on (key,
//                   slot)); the last block to finish scans the block counts,
//                   places up to kSmallMovers movers itself and picks the branch
//   k_place_movers  the same placement for up to kBruteMovers movers, one warp each
//   k_place_stayers each stayer's position from the block offsets and bitmask,
//                   and the movers' entries
// captured in a CUDA graph whose switch node runs (stayers | movers + stayers |
// full sort).  The ordering is a deterministic function of the keys, so steps
// repeat bit for bit, and no host synchronisation is needed.
#include <algorithm>

#include "aep_kernels.h"

namespace aep {

// ===================================================================================
// Stable LSD radix sort of (uint32 key, int32 value) pairs on the low key_bits bits.
// The bits are cut into P = ceil(key_bits / 8) digits of R = ceil(key_bits / P) <= 8
// bits.  Each pass is three kernels over tiles of kRsTile pairs:
//   k_rs_hist     per tile, the count of every digit value -> hist[digit][tile]
//   k_rs_scan     per digit (one block each): exclusive scan of its row over the
//                 tiles in place, and the digit's total
//   k_rs_scatter  per tile: the digits' bases (exclusive scan of the totals) plus
//                 the row offsets give each digit's first output slot for the tile;
//                 the tile is read in rounds of one pair per thread in input order,
//                 and a pair's rank among the tile's equal digits comes from
//                 __match_any_sync inside its warp, the counts of the warps before
//                 it in the round and the running count of earlier rounds, so equal
//                 digits keep their input order (the sort is stable).
// Passes alternate between the output arrays and a scratch copy, arranged so that
// the last pass writes the output.  Traffic per pass: keys and values read twice
// and written once.
constexpr int kRsThreads = 256;
constexpr int kRsRounds = 16;
constexpr int kRsTile = kRsThreads * kRsRounds;  // 4096 pairs per tile
constexpr int kRsBins = 256;
constexpr int kRsWarps = kRsThreads / 32;

struct RsPlan {
    int passes, radix, tiles;
};

RsPlan rs_plan(int n, int key_bits) {
    RsPlan p;
    key_bits = std::max(1, std::min(32, key_bits));
    p.passes = (key_bits + 7) / 8;
    p.radix = (key_bits + p.passes - 1) / p.passes;
    p.tiles = std::max(1, (n + kRsTile - 1) / kRsTile);
    return p;
}

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t* __restrict__ keys, int n, int shift,
                                                        uint32_t mask, int tiles, int32_t* __restrict__ hist) {
    __shared__ int32_t cnt[kRsBins];
    for (int i = threadIdx.x; i < kRsBins; i += kRsThreads) cnt[i] = 0;
    __syncthreads();
    const long base = (long)blockIdx.x * kRsTile;
    for (int r = 0; r < kRsRounds; ++r) {
        const long i = base + (long)r * kRsThreads + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & mask], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d <= (int)mask; d += kRsThreads) hist[(long)d * tiles + blockIdx.x] = cnt[d];
}

// block-wide exclusive scan of one value per thread; returns the block total
__device__ __forceinline__ int32_t rs_block_scan(int32_t v, int32_t& total, int32_t* warp_tot) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    int32_t off = 0;
    total = 0;
    for (int k = 0; k < kRsWarps; ++k) {
        const int32_t t = warp_tot[k];
        if (k < w) off += t;
        total += t;
    }
    __syncthreads();
    return off + x - v;
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scan(int32_t* __restrict__ hist, int tiles,
                                                        int32_t* __restrict__ totals) {
    __shared__ int32_t warp_tot[kRsWarps];
    int32_t* row = hist + (long)blockIdx.x * tiles;
    int32_t carry = 0;
    for (int t0 = 0; t0 < tiles; t0 += kRsThreads) {  // block-uniform trip count
        const int t = t0 + threadIdx.x;
        const int32_t v = t < tiles ? row[t] : 0;
        int32_t total;
        const int32_t ex = rs_block_scan(v, total, warp_tot);
        if (t < tiles) row[t] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t* __restrict__ keys_in,
                                                           const int32_t* __restrict__ vals_in, int n, int shift,
                                                           uint32_t mask, int tiles,
                                                           const int32_t* __restrict__ hist,
                                                           const int32_t* __restrict__ totals,
                                                           uint32_t* __restrict__ keys_out,
                                                           int32_t* __restrict__ vals_out) {
    __shared__ int32_t start[kRsBins];              // first output slot of each digit for this tile
    __shared__ int32_t wcnt[kRsWarps][kRsBins];     // this round's count per warp and digit
    __shared__ int32_t warp_tot[kRsWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nd = (int)mask + 1;
    {  // digit bases: exclusive scan of the totals (nd <= 256 = one per thread)
        const int d = threadIdx.x;
        int32_t total;
        const int32_t ex = rs_block_scan(d < nd ? totals[d] : 0, total, warp_tot);
        if (d < nd) start[d] = ex + hist[(long)d * tiles + blockIdx.x];
    }
    for (int i = threadIdx.x; i < kRsWarps * kRsBins; i += kRsThreads) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    const long base = (long)blockIdx.x * kRsTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kRsRounds; ++r) {
        const long i = base + (long)r * kRsThreads + threadIdx.x;
        const bool live = i < n;
        const uint32_t k = live ? keys_in[i] : 0u;
        const int32_t v = live ? vals_in[i] : 0;
        const int d = live ? (int)((k >> shift) & mask) : kRsBins;  // past the end: its own group
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank_w = __popc(peers & lt);
        const bool leader = rank_w == 0;
        if (leader && live) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (live) {
            int32_t pos = start[d] + rank_w;
            for (int ww = 0; ww < w; ++ww) pos += wcnt[ww][d];
            keys_out[pos] = k;
            vals_out[pos] = v;
        }
        __syncthreads();
        if (leader && live) {
            atomicAdd(&start[d], wcnt[w][d]);
            wcnt[w][d] = 0;
        }
        __syncthreads();
    }
}

size_t sort_temp_bytes(int n, int key_bits) {
    const RsPlan p = rs_plan(n, key_bits);
    const size_t hist = sizeof(int32_t) * ((size_t)kRsBins * p.tiles + kRsBins);
    const size_t pairs = (sizeof(uint32_t) + sizeof(int32_t)) * (size_t)std::max(n, 1);
    return ((hist + 255) & ~(size_t)255) + pairs;
}

cudaError_t sort_pairs(void* temp, size_t temp_bytes, const uint32_t* keys_in, uint32_t* keys_out,
                       const int32_t* vals_in, int32_t* vals_out, int n, int key_bits, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (temp_bytes < sort_temp_bytes(n, key_bits)) return cudaErrorInvalidValue;
    const RsPlan p = rs_plan(n, key_bits);
    int32_t* hist = static_cast<int32_t*>(temp);
    int32_t* totals = hist + (size_t)kRsBins * p.tiles;
    const size_t hist_bytes = (sizeof(int32_t) * ((size_t)kRsBins * p.tiles + kRsBins) + 255) & ~(size_t)255;
    uint32_t* tk = reinterpret_cast<uint32_t*>(static_cast<char*>(temp) + hist_bytes);
    int32_t* tv = reinterpret_cast<int32_t*>(tk + n);
    const uint32_t mask = (1u << p.radix) - 1u;
    const uint32_t* ik = keys_in;
    const int32_t* iv = vals_in;
    for (int pass = 0; pass < p.passes; ++pass) {
        // the last pass writes the output: passes alternate back from it
        const bool to_out = ((p.passes - 1 - pass) & 1) == 0;
        uint32_t* ok = to_out ? keys_out : tk;
        int32_t* ov = to_out ? vals_out : tv;
        const int shift = pass * p.radix;
        k_rs_hist<<<p.tiles, kRsThreads, 0, s>>>(ik, n, shift, mask, p.tiles, hist);
        k_rs_scan<<<(int)mask + 1, kRsThreads, 0, s>>>(hist, p.tiles, totals);
        k_rs_scatter<<<p.tiles, kRsThreads, 0, s>>>(ik, iv, n, shift, mask, p.tiles, hist, totals, ok, ov);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        ik = ok;
        iv = ov;
    }
    return cudaSuccess;
}

namespace {

constexpr int kFlagThreads = 1024;  // slots per block of the flag and stayer kernels
constexpr int kRankThreads = 256;
constexpr int kSmallMovers = 32;    // movers placed by the last flag block (one warp each)
constexpr int kMoverBlocks = 256;   // k_place_movers: 2,048 warps, a mover each (more: in turn)

// first index i of the ascending a[0, n) with a[i] > k, found by one warp with
// 32-way probes (about four dependent loads for a million entries)
__device__ __forceinline__ int warp_upper_bound(const uint32_t* __restrict__ a, int n, uint32_t k, int lane) {
    int lo = 0, hi = n;  // a[lo - 1] <= k (or lo = 0); the answer is in [lo, hi]
    while (hi - lo > 32) {
        const int step = (hi - lo + 31) >> 5;
        const int idx = lo + lane * step;
        const unsigned above = __ballot_sync(0xffffffffu, idx >= hi || a[idx] > k);
        if (above == 0u) {
            lo += 31 * step + 1;
        } else {
            const int f = __ffs(above) - 1;
            if (f == 0) return lo;
            hi = min(hi, lo + f * step);
            lo += (f - 1) * step + 1;
        }
    }
    const int idx = lo + lane;
    return lo + __popc(__ballot_sync(0xffffffffu, idx < hi && a[idx] <= k));
}

// placement of mover i (one warp): its (key, slot) rank among the m movers and
// the number of stayers with a key <= its key
__device__ __forceinline__ void place_mover(int i, int m, const uint32_t* __restrict__ prev, int n,
                                            const uint32_t* __restrict__ mk, const int32_t* __restrict__ mj,
                                            uint32_t* __restrict__ mkeys, int32_t* __restrict__ mslot,
                                            int32_t* __restrict__ mpos, int lane) {
    // the list was written by other blocks of the flag kernel: read it from L2
    const uint32_t ki = __ldcg(&mk[i]);
    const int ji = __ldcg(&mj[i]);
    int rank = 0, prev_le = 0;
    for (int k = lane; k < m; k += 32) {
        const uint32_t kk = __ldcg(&mk[k]);
        const int jk = __ldcg(&mj[k]);
        rank += (kk < ki) | ((kk == ki) & (jk < ji));
        prev_le += prev[jk] <= ki;
    }
    rank = __reduce_add_sync(0xffffffffu, rank);
    prev_le = __reduce_add_sync(0xffffffffu, prev_le);
    const int ub = warp_upper_bound(prev, n, ki, lane);
    if (lane == 0) {
        mkeys[rank] = ki;
        mslot[rank] = ji;
        mpos[rank] = rank + ub - prev_le;
    }
}

// counters: [0] movers, [1] finished flag blocks
__global__ void __launch_bounds__(kFlagThreads, 2) k_flag_movers(const uint32_t* __restrict__ keys,
                                                              const uint32_t* __restrict__ prev, int n, int cap,
                                                              uint32_t* __restrict__ mask, int32_t* __restrict__ blk,
                                                              uint32_t* __restrict__ mk, int32_t* __restrict__ mj,
                                                              uint32_t* __restrict__ mkeys, int32_t* __restrict__ mslot,
                                                              int32_t* __restrict__ mpos,
                                                              int32_t* __restrict__ counters,
                                                              cudaGraphConditionalHandle h, DevStats* st) {
    __shared__ bool last;
    __shared__ int warp_sum[kFlagThreads / 32];
    const int j = blockIdx.x * kFlagThreads + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool mover = false;
    if (j < n) {
        const uint32_t k = keys[j];
        mover = k != prev[j];
        if (mover) {
            const int idx = atomicAdd(&counters[0], 1);
            if (idx < cap) {
                mk[idx] = k;
                mj[idx] = j;
            }
        }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, mover);
    if (lane == 0 && j < n) mask[j >> 5] = bal;
    const int cnt = __syncthreads_count(mover);
    if (threadIdx.x == 0) {
        blk[blockIdx.x] = cnt;
        __threadfence();
        last = atomicAdd(&counters[1], 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // last block: exclusive scan of the block counts in place
    __threadfence();
    const int nb = gridDim.x;
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += kFlagThreads) {
        const int b = b0 + threadIdx.x;
        const int v = b < nb ? __ldcg(&blk[b]) : 0;  // written by other blocks: read from L2
        int x = v;  // inclusive warp scan
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sum[threadIdx.x >> 5] = x;
        __syncthreads();
        int woff = 0;
        for (int w = 0; w < (int)(threadIdx.x >> 5); ++w) woff += warp_sum[w];
        int total = 0;
        for (int w = 0; w < kFlagThreads / 32; ++w) total += warp_sum[w];
        if (b < nb) blk[b] = carry + woff + x - v;  // this thread alone read blk[b] (as v)
        carry += total;
        __syncthreads();
    }
    const int m = carry;  // the movers
    const unsigned branch = (m > cap || m > kBruteMovers) ? 2u : (m > kSmallMovers ? 1u : 0u);
    if (branch == 0u) {  // place the few movers here; all flag blocks are done with prev
        __threadfence();
        for (int i = threadIdx.x >> 5; i < m; i += kFlagThreads / 32)
            place_mover(i, m, prev, n, mk, mj, mkeys, mslot, mpos, lane);
    }
    if (threadIdx.x == 0) {
        cudaGraphSetConditional(h, branch);
        st->movers = branch == 2u ? -1ll : (long long)m;
        counters[0] = m;
        counters[1] = 0;
    }
}

// placement of up to kBruteMovers movers, one warp each (grid-stride over the movers)
__global__ void __launch_bounds__(kRankThreads) k_place_movers(const uint32_t* __restrict__ prev, int n, int cap,
                                                               const uint32_t* __restrict__ mk,
                                                               const int32_t* __restrict__ mj,
                                                               const int32_t* __restrict__ counters,
                                                               uint32_t* __restrict__ mkeys, int32_t* __restrict__ mslot,
                                                               int32_t* __restrict__ mpos) {
    const int m = counters[0];
    if (m > cap || m > kBruteMovers) return;  // the full-sort branch (never launched with these)
    const int warps = (int)(((long)gridDim.x * kRankThreads) >> 5);
    for (int i = (int)(((long)blockIdx.x * kRankThreads + threadIdx.x) >> 5); i < m; i += warps)  // warp-uniform
        place_mover(i, m, prev, n, mk, mj, mkeys, mslot, mpos, threadIdx.x & 31);
}

// stayer j: (stayers before j) + (movers with key < key_j); threads t < m also
// write the movers' entries
__global__ void __launch_bounds__(kFlagThreads) k_place_stayers(const uint32_t* __restrict__ keys, int n, int cap,
                                                                const uint32_t* __restrict__ mask,
                                                                const int32_t* __restrict__ blk,
                                                                const uint32_t* __restrict__ mkeys,
                                                                const int32_t* __restrict__ mslot,
                                                                const int32_t* __restrict__ mpos,
                                                                const int32_t* __restrict__ counters,
                                                                uint32_t* __restrict__ keys_out,
                                                                int32_t* __restrict__ perm_out) {
    __shared__ int warp_movers[kFlagThreads / 32];
    const int j = blockIdx.x * kFlagThreads + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m = counters[0];
    if (m > cap || m > kBruteMovers) return;  // the full-sort branch (never launched with these); block-uniform
    const unsigned bal = j - lane < n ? mask[j >> 5] : 0u;
    if (lane == 0) warp_movers[warp] = __popc(bal);
    __syncthreads();
    if (j < m) {
        const int p = mpos[j];
        keys_out[p] = mkeys[j];
        perm_out[p] = mslot[j];
    }
    if (j >= n || ((bal >> lane) & 1u)) return;
    int before = blk[blockIdx.x] + __popc(bal & ((1u << lane) - 1u));
    for (int w = 0; w < warp; ++w) before += warp_movers[w];
    const uint32_t k = keys[j];
    int lo = 0, hi = m;  // movers with key < k
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (mkeys[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    const int pos = j - before + lo;
    keys_out[pos] = k;
    perm_out[pos] = j;
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

size_t order_scratch_words(int n) {
    const size_t nb = ((size_t)n + kFlagThreads - 1) / kFlagThreads;
    // mask (n/32 + 1), block offsets (nb), counters (2)
    return (size_t)n / 32 + 1 + nb + 2;
}

cudaError_t order_graph_build(void** out, cudaStream_t cs, const OrderBuffers& b) {
    *out = nullptr;
    cudaGraph_t g = nullptr, ended = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    const int n = b.n;
    const int nb = (n + kFlagThreads - 1) / kFlagThreads;
    uint32_t* mask = b.scratch;
    int32_t* blk = reinterpret_cast<int32_t*>(mask + n / 32 + 1);
    int32_t* counters = blk + nb;
    // counters[1] is reset by the last flag block; zero both once here
    OG_CK(cudaMemsetAsync(counters, 0, 2 * sizeof(int32_t), cs));
    OG_CK(cudaStreamSynchronize(cs));
    cudaGraphConditionalHandle h;
    OG_CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
    OG_CK(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    OG_CK(cudaMemsetAsync(counters, 0, sizeof(int32_t), cs));
    k_flag_movers<<<nb, kFlagThreads, 0, cs>>>(b.keys, b.keys_sorted, n, b.cap, mask, blk, b.mk, b.mj, b.mkeys,
                                               b.mslot, b.mpos, counters, h, b.st);
    OG_CK(cudaGetLastError());
    cudaStreamCaptureStatus status;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    OG_CK(cudaStreamGetCaptureInfo(cs, &status, nullptr, nullptr, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeSwitch;
    cp.conditional.size = 3;  // 0: stayers, 1: movers + stayers, 2: full sort
    cudaGraphNode_t cnode;
    OG_CK(cudaGraphAddNode(&cnode, g, deps, nullptr, ndeps, &cp));
    OG_CK(cudaStreamEndCapture(cs, &ended));
    cudaGraph_t* body = cp.conditional.phGraph_out;
    for (int c = 0; c < 2; ++c) {
        OG_CK(cudaStreamBeginCaptureToGraph(cs, body[c], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        if (c == 1)
            k_place_movers<<<kMoverBlocks, kRankThreads, 0, cs>>>(b.keys_sorted, n, b.cap, b.mk, b.mj, counters,
                                                                  b.mkeys, b.mslot, b.mpos);
        k_place_stayers<<<nb, kFlagThreads, 0, cs>>>(b.keys, n, b.cap, mask, blk, b.mkeys, b.mslot, b.mpos, counters,
                                                     b.keys_sorted, b.perm);
        OG_CK(cudaGetLastError());
        OG_CK(cudaStreamEndCapture(cs, &ended));
    }
    OG_CK(cudaStreamBeginCaptureToGraph(cs, body[2], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    OG_CK(sort_pairs(b.sort_tmp, b.sort_bytes, b.keys, b.keys_sorted, b.iota, b.perm, n, b.key_bits, cs));
    OG_CK(cudaStreamEndCapture(cs, &ended));
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
