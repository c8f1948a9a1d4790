// aep_mlp.cu -- training and batched inference of the learned return map
// (see aep_mlp.cuh).  Everything runs on the device with hand-written kernels:
//   k_mlp_train_tile : forward + backward of 64 training rows per block on the tensor
//                      cores (mma.sync bf16, f32 accumulation); each block writes its
//                      weight and bias gradients to its own row of a partial array
//   k_mlp_reduce     : sums the partial rows in block order (training is
//                      deterministic: the same records give the same parameters)
//   k_mlp_adam       : Adam on the f32 master parameters, refreshes the bf16 copies
//   k_mlp_infer      : batched forward pass (32 rows per warp), as used inside G2P
// Training records (harvested from the exact return mapping where it changed the
// state, 8 floats each):
//   [ln s0, ln s1, ln s2 (trial, sorted descending), q, material, d0, d1, d2]
// with d = ln s_projected - ln s_trial in the same order.  The loss is the mean
// squared error of the network output against d in the scaling of mlp_features.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/aep.h"
#include "aep_mlp.cuh"

using namespace aep;

namespace {

// packed f32 parameter vector: W^T blocks then biases
constexpr int kOffW1 = 0;
constexpr int kOffW2 = kOffW1 + 64 * 16;
constexpr int kOffW3 = kOffW2 + 64 * 64;
constexpr int kOffW4 = kOffW3 + 64 * 64;
constexpr int kOffB1 = kOffW4 + 8 * 64;
constexpr int kOffB2 = kOffB1 + 64;
constexpr int kOffB3 = kOffB2 + 64;
constexpr int kOffB4 = kOffB3 + 64;
constexpr int kNumParams = kOffB4 + 8;  // 9928
constexpr int kNumWeights = kOffB1;     // 9728 bf16 copies
static_assert(kNumParams == AEP_MLP_NUM_PARAMS, "parameter count");

constexpr int kTrainRows = 64;
constexpr int kPartBlocks = 256;  // blocks of one gradient pass (16,384 rows)
constexpr int kTrainThreads = 256;
constexpr int kTrainWarps = kTrainThreads / 32;

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// generic 16x8 tile: c += sum_{k < K} A(m0+i, k) B(k, n0+j); element (i,k) of A at
// A[i*ars + k*acs] for i < am (zero otherwise), element (k,j) of B at B[k*brs + j*bcs]
// for k < kmax (zero otherwise).  Used by training, where operands are transposed.
template <int K>
__device__ __forceinline__ void tile_mma(float c[4], const bf16* A, int ars, int acs, int am, const bf16* B, int brs,
                                         int bcs, int kmax, int m0, int n0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const bf16 z = __float2bfloat16(0.0f);
    auto la = [&](int i, int k) { return (i < am && k < kmax) ? A[i * ars + k * acs] : z; };
    auto lb = [&](int k, int j) { return k < kmax ? B[k * brs + j * bcs] : z; };
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += 16) {
        const int r0 = m0 + g, r1 = m0 + g + 8, ka = k0 + 2 * t;
        uint32_t a0 = pack2(la(r0, ka), la(r0, ka + 1)), a1 = pack2(la(r1, ka), la(r1, ka + 1));
        uint32_t a2 = pack2(la(r0, ka + 8), la(r0, ka + 9)), a3 = pack2(la(r1, ka + 8), la(r1, ka + 9));
        uint32_t b0 = pack2(lb(ka, n0 + g), lb(ka + 1, n0 + g)), b1 = pack2(lb(ka + 8, n0 + g), lb(ka + 9, n0 + g));
        mma_bf16(c, a0, a1, a2, a3, b0, b1);
    }
}

// 114,480 bytes: two blocks fit on an SM
struct TrainSmem {
    bf16 W1[64 * 16], W2[64 * 64], W3[64 * 64], W4[8 * 64];  // W^T, dense rows (the layout of the bf16 copy)
    float b[200];
    bf16 X[kTrainRows * 16];
    bf16 H[3][kTrainRows * 64];   // post-activations
    float Z[3][kTrainRows * 64];  // pre-activations
    float T[kTrainRows * 4];
    bf16 dY[kTrainRows * 8];
    bf16 dZ[2][kTrainRows * 64];  // ping-pong
    float wloss[kTrainWarps];
};

__device__ __forceinline__ float dsilu(float z) {
    const float s = __frcp_rn(1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// Forward and backward of one block of rows.  The block's gradient (f32, packed)
// goes to its own row of `part` and its loss to part_loss[block]; k_mlp_reduce
// sums the rows in block order, so training repeats bit for bit.
__global__ void __launch_bounds__(kTrainThreads, 2) k_mlp_train_tile(const float* __restrict__ params,
                                                                     const bf16* __restrict__ wb,
                                                                     const float* __restrict__ rec, int n, int row0,
                                                                     int row_end, int rows_total,
                                                                     float* __restrict__ part,
                                                                     float* __restrict__ part_loss) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int base = row0 + blockIdx.x * kTrainRows;
    float* const grad = part + (long)blockIdx.x * kNumParams;
    // the bf16 copy of the weights (refreshed by every Adam step) has the layout of
    // W1..W4 here: one 16-byte copy per 8 weights; the rows of W1^T repeat their 7
    // weights in columns 7..13, against the lo halves of the features (mlp_features)
    static_assert(kNumWeights % 8 == 0 && kOffW2 == 128 * 8, "weight copy in 16-byte pieces");
    for (int r = tid; r < 64; r += kTrainThreads) {
        const uint4 a = reinterpret_cast<const uint4*>(wb)[2 * r], b = reinterpret_cast<const uint4*>(wb)[2 * r + 1];
        const uint32_t u[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        const bf16* w = reinterpret_cast<const bf16*>(u);
        bf16 d[16];
#pragma unroll
        for (int k = 0; k < kMlpFeat; ++k) d[k] = d[kMlpFeat + k] = w[k];
        d[14] = d[15] = __float2bfloat16(0.0f);
        reinterpret_cast<uint4*>(S.W1 + 16 * r)[0] = reinterpret_cast<const uint4*>(d)[0];
        reinterpret_cast<uint4*>(S.W1 + 16 * r)[1] = reinterpret_cast<const uint4*>(d)[1];
    }
    for (int i = 128 + tid; i < kNumWeights / 8; i += kTrainThreads)
        reinterpret_cast<uint4*>(S.W1)[i] = reinterpret_cast<const uint4*>(wb)[i];
    for (int i = tid; i < 200; i += kTrainThreads) S.b[i] = params[kOffB1 + i];
    for (int r = tid; r < kTrainRows; r += kTrainThreads) {
        const long gi = (long)(base + r) % n;  // wrap around the record set
        const float* q = rec + 8 * gi;
        const bool live = base + r < row_end;
        float ln[3] = {q[0], q[1], q[2]};
        const float sc = mlp_features(ln, q[3], (int)q[4], S.X + r * 16);
        for (int k = 0; k < 3; ++k) S.T[r * 4 + k] = live ? q[5 + k] * sc : 0.0f;
        S.T[r * 4 + 3] = live ? 1.0f : 0.0f;  // row weight
    }
    __syncthreads();
    // ---- forward
    const bf16* Hin[4] = {S.X, S.H[0], S.H[1], S.H[2]};
    const bf16* Wl[3] = {S.W1, S.W2, S.W3};
    const int Kin[3] = {16, 64, 64};
    for (int l = 0; l < 3; ++l) {
        for (int tt = warp; tt < 32; tt += kTrainWarps) {  // 4 m-tiles x 8 n-tiles
            const int m0 = (tt >> 3) * 16, n0 = (tt & 7) * 8;
            float c[4] = {0, 0, 0, 0};
            if (l == 0) tile_mma<16>(c, Hin[0], 16, 1, kTrainRows, Wl[0], 1, 16, 16, m0, n0, lane);
            else tile_mma<64>(c, Hin[l], 64, 1, kTrainRows, Wl[l], 1, 64, 64, m0, n0, lane);
            const int g = lane >> 2, t = lane & 3;
            for (int e = 0; e < 4; ++e) {
                const int r = m0 + g + (e >> 1) * 8, col = n0 + 2 * t + (e & 1);
                const float z = c[e] + S.b[64 * l + col];
                S.Z[l][r * 64 + col] = z;
                S.H[l][r * 64 + col] = __float2bfloat16(silu(z));
            }
        }
        __syncthreads();
        (void)Kin;
    }
    if (warp >= 4) {
        if (lane == 0) S.wloss[warp] = 0.0f;
    } else {  // output layer: 4 m-tiles x 1 n-tile, one per warp
        const int m0 = warp * 16;
        float c[4] = {0, 0, 0, 0};
        tile_mma<64>(c, S.H[2], 64, 1, kTrainRows, S.W4, 1, 64, 64, m0, 0, lane);
        const int g = lane >> 2, t = lane & 3;
        float lsum = 0.0f;
        for (int e = 0; e < 4; ++e) {
            const int r = m0 + g + (e >> 1) * 8, col = 2 * t + (e & 1);
            const float y = c[e] + S.b[192 + col];
            float d = 0.0f;
            if (col < 3) {
                const float diff = y - S.T[r * 4 + col];
                d = S.T[r * 4 + 3] * diff;
                lsum += d * diff;
            }
            // d loss / d y for loss = sum w (y - t)^2 / (3 rows_total)
            S.dY[r * 8 + col] = __float2bfloat16(2.0f * d / (3.0f * rows_total));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        if (lane == 0) S.wloss[warp] = lsum;
    }
    __syncthreads();
    // ---- backward
    // dW4t[j][k] = sum_r dY[r][j] H3[r][k]; db4[j] = sum_r dY[r][j]
    for (int tt = warp; tt < 8; tt += kTrainWarps) {
        const int n0 = tt * 8;
        float c[4] = {0, 0, 0, 0};
        tile_mma<64>(c, S.dY, 1, 8, 8, S.H[2], 64, 1, kTrainRows, 0, n0, lane);
        const int g = lane >> 2, t = lane & 3;
        for (int e = 0; e < 4; ++e) {
            const int j = g + (e >> 1) * 8, k = n0 + 2 * t + (e & 1);
            if (j < 8) grad[kOffW4 + j * 64 + k] = c[e];
        }
    }
    if (tid < 8) {
        float s = 0.0f;
        for (int r = 0; r < kTrainRows; ++r) s += __bfloat162float(S.dY[r * 8 + tid]);
        grad[kOffB4 + tid] = s;
    }
    // dZ3 = (dY W4^T) * silu'(Z3):  dH3[r][k] = sum_j dY[r][j] W4t[j][k]
    for (int tt = warp; tt < 32; tt += kTrainWarps) {
        const int m0 = (tt >> 3) * 16, n0 = (tt & 7) * 8;
        float c[4] = {0, 0, 0, 0};
        tile_mma<16>(c, S.dY, 8, 1, kTrainRows, S.W4, 64, 1, 8, m0, n0, lane);
        const int g = lane >> 2, t = lane & 3;
        for (int e = 0; e < 4; ++e) {
            const int r = m0 + g + (e >> 1) * 8, k = n0 + 2 * t + (e & 1);
            S.dZ[0][r * 64 + k] = __float2bfloat16(c[e] * dsilu(S.Z[2][r * 64 + k]));
        }
    }
    __syncthreads();
    // layers 3, 2, 1: dW_l^T[n][k] = sum_r dZ_l[r][n] H_{l-1}[r][k];  dZ_{l-1} = (dZ_l W_l^T) * silu'
    const bf16* Wt[3] = {S.W1, S.W2, S.W3};
    const int offW[3] = {kOffW1, kOffW2, kOffW3};
    const int offB[3] = {kOffB1, kOffB2, kOffB3};
    int cur = 0;
    for (int l = 2; l >= 0; --l) {
        const bf16* dZ = S.dZ[cur];
        const bf16* Hp = l == 0 ? S.X : S.H[l - 1];
        const int kin = l == 0 ? 16 : 64;
        const int ntiles = (64 / 16) * (kin / 8);
        for (int tt = warp; tt < ntiles; tt += kTrainWarps) {
            const int m0 = (tt / (kin / 8)) * 16, n0 = (tt % (kin / 8)) * 8;
            float c[4] = {0, 0, 0, 0};
            tile_mma<kTrainRows>(c, dZ, 1, 64, 64, Hp, kin, 1, kTrainRows, m0, n0, lane);
            const int g = lane >> 2, t = lane & 3;
            for (int e = 0; e < 4; ++e) {
                const int nn = m0 + g + (e >> 1) * 8, k = n0 + 2 * t + (e & 1);
                grad[offW[l] + nn * kin + k] = c[e];
            }
        }
        if (tid < 64) {
            float s = 0.0f;
            for (int r = 0; r < kTrainRows; ++r) s += __bfloat162float(dZ[r * 64 + tid]);
            grad[offB[l] + tid] = s;
        }
        if (l > 0) {
            bf16* dZn = S.dZ[1 - cur];
            for (int tt = warp; tt < 32; tt += kTrainWarps) {
                const int m0 = (tt >> 3) * 16, n0 = (tt & 7) * 8;
                float c[4] = {0, 0, 0, 0};
                // dH_{l-1}[r][k] = sum_n dZ_l[r][n] W_l^T[n][k]
                tile_mma<64>(c, dZ, 64, 1, kTrainRows, Wt[l], 64, 1, 64, m0, n0, lane);
                const int g = lane >> 2, t = lane & 3;
                for (int e = 0; e < 4; ++e) {
                    const int r = m0 + g + (e >> 1) * 8, k = n0 + 2 * t + (e & 1);
                    dZn[r * 64 + k] = __float2bfloat16(c[e] * dsilu(S.Z[l - 1][r * 64 + k]));
                }
            }
        }
        __syncthreads();
        if (l == 0) {  // W1's gradient: the hi and lo columns of a feature share its weight
            for (int i = tid; i < 64 * kMlpFeat; i += kTrainThreads) {
                float* gw = grad + kOffW1 + (i / kMlpFeat) * 16 + i % kMlpFeat;
                gw[0] += gw[kMlpFeat];
                gw[kMlpFeat] = 0.0f;
            }
        }
        cur = 1 - cur;
    }
    if (tid == 0) {
        float l = 0.0f;
        for (int w = 0; w < kTrainWarps; ++w) l += S.wloss[w];
        part_loss[blockIdx.x] = l / (3.0f * rows_total);
    }
}

// grad[i] (+)= sum over the blocks of part[b][i]; loss likewise.  A block of 256
// threads takes 32 parameters: thread (q, i) sums the blocks q*c .. q*c + c - 1 of
// parameter i in order (c = ceil(blocks / 8)), and the eight partial sums are added
// in q order, so the result is the same on every run.
constexpr int kReduceParams = 32;
constexpr int kReduceSplit = 8;
__global__ void __launch_bounds__(kReduceParams * kReduceSplit) k_mlp_reduce(const float* __restrict__ part,
                                                                            const float* __restrict__ part_loss,
                                                                            int blocks, float* __restrict__ grad,
                                                                            float* __restrict__ loss, int accumulate) {
    __shared__ float ps[kReduceSplit][kReduceParams + 1];
    const int ii = threadIdx.x % kReduceParams, q = threadIdx.x / kReduceParams;
    const int i = blockIdx.x * kReduceParams + ii;
    const int c = (blocks + kReduceSplit - 1) / kReduceSplit;
    const int b0 = q * c, b1 = min(blocks, b0 + c);
    float s = 0.0f;
    if (i < kNumParams)
        for (int b = b0; b < b1; ++b) s += part[(long)b * kNumParams + i];
    ps[q][ii] = s;
    __syncthreads();
    if (q == 0 && i < kNumParams) {
        float t = accumulate ? grad[i] : 0.0f;
#pragma unroll
        for (int k = 0; k < kReduceSplit; ++k) t += ps[k][ii];
        grad[i] = t;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float l = accumulate ? *loss : 0.0f;
        for (int b = 0; b < blocks; ++b) l += part_loss[b];
        *loss = l;
    }
}

// Adam (Kingma & Ba 2015) on the f32 master parameters; zeroes the gradient and
// refreshes the bf16 weight copies
__global__ void k_mlp_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                           bf16* __restrict__ wb, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNumParams) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    g[i] = 0.0f;
    if (i < kNumWeights) wb[i] = __float2bfloat16(pi);
}

__global__ void k_mlp_refresh_bf16(const float* __restrict__ p, bf16* __restrict__ wb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kNumWeights) wb[i] = __float2bfloat16(p[i]);
}

// batched inference, 32 rows per warp; kStep: with the SiLU of the step's kernels
template <bool kStep>
__global__ void __launch_bounds__(128) k_mlp_infer(MlpParams P, const float* __restrict__ rec, int n,
                                                   float* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const MlpSmem W = mlp_smem_carve(smem_raw);
    mlp_load_smem(P, W, threadIdx.x, blockDim.x);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wbase = smem_raw + kMlpSmemBytes + warp * kMlpWarpBytes;
    bf16* X = reinterpret_cast<bf16*>(wbase);
    float* Y = reinterpret_cast<float*>(X + kMlpWarpX);
    const long r = ((long)blockIdx.x * 4 + warp) * 32 + lane;
    float sc = 1.0f;
    if (r < n) {
        const float* q = rec + 8 * r;
        float ln[3] = {q[0], q[1], q[2]};
        sc = mlp_features(ln, q[3], (int)q[4], X + lane * kStrideIn);
    } else {
        float ln[3] = {0, 0, 0};
        mlp_features(ln, 0.0f, 0, X + lane * kStrideIn);
    }
    mlp_forward_warp<kStep>(W, X, Y, lane);
    if (r < n)
        for (int k = 0; k < 3; ++k) out[3 * r + k] = Y[lane * kMlpOut + k] / sc;
}

}  // namespace

struct aep_mlp {
    float* p = nullptr;   // f32 master parameters
    float* g = nullptr;   // gradient
    float* m = nullptr;   // Adam moments
    float* v = nullptr;
    bf16* wb = nullptr;   // bf16 weights (W^T blocks)
    float* loss = nullptr;
    float* part = nullptr;       // per-block gradients of one pass [kPartBlocks][kNumParams]
    float* part_loss = nullptr;  // per-block losses
    int64_t t = 0;        // Adam step
    std::string err;
};

namespace aep {
// device view for the learned G2P path (defined here, used by aep_capi.cu)
MlpParams mlp_device_params(const aep_mlp* m) {
    MlpParams P;
    P.w1t = m->wb + kOffW1;
    P.w2t = m->wb + kOffW2;
    P.w3t = m->wb + kOffW3;
    P.w4t = m->wb + kOffW4;
    P.b1 = m->p + kOffB1;
    P.b2 = m->p + kOffB2;
    P.b3 = m->p + kOffB3;
    P.b4 = m->p + kOffB4;
    return P;
}
}  // namespace aep

#define MCK(call)                                                               \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) {                                                \
            if (mlp) mlp->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return e_ == cudaErrorMemoryAllocation ? AEP_OUT_OF_MEMORY : AEP_CUDA_ERROR; \
        }                                                                       \
    } while (0)

extern "C" {

aep_status aep_mlp_create(uint64_t seed, aep_mlp** out) {
    if (!out) return AEP_INVALID_ARG;
    aep_mlp* mlp = new aep_mlp();
    *out = nullptr;
    MCK(cudaMalloc(&mlp->p, sizeof(float) * kNumParams));
    MCK(cudaMalloc(&mlp->g, sizeof(float) * kNumParams));
    MCK(cudaMalloc(&mlp->m, sizeof(float) * kNumParams));
    MCK(cudaMalloc(&mlp->v, sizeof(float) * kNumParams));
    MCK(cudaMalloc(&mlp->wb, sizeof(bf16) * kNumWeights));
    MCK(cudaMalloc(&mlp->loss, sizeof(float)));
    MCK(cudaMalloc(&mlp->part, sizeof(float) * kNumParams * kPartBlocks));
    MCK(cudaMalloc(&mlp->part_loss, sizeof(float) * kPartBlocks));
    // He-normal weights (SiLU), zero biases, seeded
    std::vector<float> h(kNumParams, 0.0f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int nout, int kin_used, int kin) {
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / kin_used));
        for (int o = 0; o < nout; ++o)
            for (int k = 0; k < kin; ++k) h[off + o * kin + k] = k < kin_used ? nd(rng) : 0.0f;
    };
    fill(kOffW1, 64, 6, 16);
    fill(kOffW2, 64, 64, 64);
    fill(kOffW3, 64, 64, 64);
    fill(kOffW4, 8, 64, 64);
    for (int o = 3; o < 8; ++o)
        for (int k = 0; k < 64; ++k) h[kOffW4 + o * 64 + k] = 0.0f;
    for (int k = 0; k < 3 * 64; ++k) h[kOffW4 + k] *= 0.1f;  // small initial output
    MCK(cudaMemcpy(mlp->p, h.data(), sizeof(float) * kNumParams, cudaMemcpyHostToDevice));
    MCK(cudaMemset(mlp->g, 0, sizeof(float) * kNumParams));
    MCK(cudaMemset(mlp->m, 0, sizeof(float) * kNumParams));
    MCK(cudaMemset(mlp->v, 0, sizeof(float) * kNumParams));
    k_mlp_refresh_bf16<<<(kNumWeights + 255) / 256, 256>>>(mlp->p, mlp->wb);
    MCK(cudaGetLastError());
    MCK(cudaDeviceSynchronize());
    *out = mlp;
    return AEP_OK;
}

aep_status aep_mlp_destroy(aep_mlp* mlp) {
    if (!mlp) return AEP_INVALID_ARG;
    cudaFree(mlp->p);
    cudaFree(mlp->g);
    cudaFree(mlp->m);
    cudaFree(mlp->v);
    cudaFree(mlp->wb);
    cudaFree(mlp->loss);
    cudaFree(mlp->part);
    cudaFree(mlp->part_loss);
    delete mlp;
    return AEP_OK;
}

aep_status aep_mlp_get_params(aep_mlp* mlp, float* host, int64_t count) {
    if (!mlp || !host || count != kNumParams) return AEP_INVALID_ARG;
    MCK(cudaMemcpy(host, mlp->p, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost));
    return AEP_OK;
}

aep_status aep_mlp_set_params(aep_mlp* mlp, const float* host, int64_t count) {
    if (!mlp || !host || count != kNumParams) return AEP_INVALID_ARG;
    MCK(cudaMemcpy(mlp->p, host, sizeof(float) * kNumParams, cudaMemcpyHostToDevice));
    k_mlp_refresh_bf16<<<(kNumWeights + 255) / 256, 256>>>(mlp->p, mlp->wb);
    MCK(cudaGetLastError());
    MCK(cudaDeviceSynchronize());
    return AEP_OK;
}

// gradient and loss of `rows` records from row0 (cyclic) into mlp->g / mlp->loss:
// passes of at most kPartBlocks blocks, each reduced in block order
static aep_status grad_pass(aep_mlp* mlp, const float* rec, int64_t n, int64_t row0, int rows, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        MCK(cudaFuncSetAttribute(k_mlp_train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem)));
        attr = true;
    }
    const int blocks = (rows + kTrainRows - 1) / kTrainRows;
    for (int b0 = 0; b0 < blocks; b0 += kPartBlocks) {
        const int nb = std::min(kPartBlocks, blocks - b0);
        k_mlp_train_tile<<<nb, kTrainThreads, sizeof(TrainSmem), s>>>(mlp->p, mlp->wb, rec, (int)n,
                                                                      (int)(row0 + (int64_t)b0 * kTrainRows),
                                                                      (int)(row0 + rows), rows, mlp->part,
                                                                      mlp->part_loss);
        MCK(cudaGetLastError());
        k_mlp_reduce<<<(kNumParams + kReduceParams - 1) / kReduceParams, kReduceParams * kReduceSplit, 0, s>>>(
            mlp->part, mlp->part_loss, nb, mlp->g, mlp->loss, b0 > 0 ? 1 : 0);
        MCK(cudaGetLastError());
    }
    return AEP_OK;
}

aep_status aep_mlp_gradient(aep_mlp* mlp, const float* d_records, int64_t n, float* host_grad, double* loss) {
    if (!mlp || !d_records || n <= 0 || n > (1 << 24) || !host_grad) return AEP_INVALID_ARG;
    aep_status st = grad_pass(mlp, d_records, n, 0, (int)n, nullptr);
    if (st) return st;
    MCK(cudaDeviceSynchronize());
    MCK(cudaMemcpy(host_grad, mlp->g, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost));
    float l = 0.f;
    MCK(cudaMemcpy(&l, mlp->loss, sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) *loss = l;
    MCK(cudaMemset(mlp->g, 0, sizeof(float) * kNumParams));
    return AEP_OK;
}

aep_status aep_mlp_train(aep_mlp* mlp, const float* d_records, int64_t n, int64_t steps, int32_t batch, double lr,
                         double lr_final, double* final_loss, void* cuda_stream) {
    if (!mlp || !d_records || n <= 0 || steps <= 0 || batch <= 0 || batch > (1 << 20) || !(lr > 0))
        return AEP_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    int64_t row0 = 0;
    double last = 0.0;
    for (int64_t it = 0; it < steps; ++it) {
        // cosine decay from lr to lr_final
        const double frac = steps > 1 ? (double)it / (double)(steps - 1) : 1.0;
        const double lri = lr_final + 0.5 * (lr - lr_final) * (1.0 + std::cos(3.14159265358979323846 * frac));
        const bool report = it == steps - 1;
        aep_status st = grad_pass(mlp, d_records, n, row0 % n, batch, s);
        if (st) return st;
        ++mlp->t;
        const float c1 = 1.0f - (float)std::pow(b1, (double)mlp->t), c2 = 1.0f - (float)std::pow(b2, (double)mlp->t);
        k_mlp_adam<<<(kNumParams + 255) / 256, 256, 0, s>>>(mlp->p, mlp->g, mlp->m, mlp->v, mlp->wb, (float)lri, b1,
                                                            b2, eps, c1, c2);
        MCK(cudaGetLastError());
        row0 += batch;
        if (report) {
            float l = 0.f;
            MCK(cudaMemcpyAsync(&l, mlp->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
            MCK(cudaStreamSynchronize(s));
            last = l;
        }
    }
    if (final_loss) *final_loss = last;
    return AEP_OK;
}

static aep_status mlp_forward(aep_mlp* mlp, const float* d_records, int64_t n, float* d_out, void* cuda_stream,
                              bool step_form) {
    if (!mlp || !d_records || !d_out || n <= 0 || n > (int64_t)INT32_MAX / 2) return AEP_INVALID_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    const int smem = kMlpSmemBytes + 4 * kMlpWarpBytes;
    const auto kernel = step_form ? k_mlp_infer<true> : k_mlp_infer<false>;
    MCK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    kernel<<<(int)((n + 127) / 128), 128, smem, s>>>(mlp_device_params(mlp), d_records, (int)n, d_out);
    MCK(cudaGetLastError());
    return AEP_OK;
}

aep_status aep_mlp_forward(aep_mlp* mlp, const float* d_records, int64_t n, float* d_out, void* cuda_stream) {
    return mlp_forward(mlp, d_records, n, d_out, cuda_stream, false);
}

aep_status aep_mlp_forward_step_form(aep_mlp* mlp, const float* d_records, int64_t n, float* d_out,
                                     void* cuda_stream) {
    return mlp_forward(mlp, d_records, n, d_out, cuda_stream, true);
}

const char* aep_mlp_last_error(aep_mlp* mlp) { return mlp ? mlp->err.c_str() : "null mlp"; }

}  // extern "C"
