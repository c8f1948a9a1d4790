// aep_mlp.cuh -- the learned return map: a 7 -> 64 -> 64 -> 64 -> 3 MLP with SiLU,
// BF16 weights on the tensor cores (mma.sync m16n8k16, FP32 accumulation).
//
// Input features (one row per particle): the trial log singular values of F_E^tr
// sorted descending (3; normalised for sand, scaled by kLnScale for snow, see
// mlp_features), the sand plastic amount q (1), and the material one-hot (snow,
// sand, cloth) (3); padded to 16 columns.  Cloth elements use the same network
// on (r13, r23, r33 - 1) of their QR factor, normalised, with the ratio of the
// friction cap to the trial shear force in column 3.  Output: the correction
// (ln s_projected - ln s_trial) in the same order and the same scaling (3 of 8).
// The return mappings it stands in for (HybridSolver.cpp:626-674) are invariant
// under permutations of the singular values, so sorting canonicalises the input.
//
// Matrix fragments (PTX ISA, mma.m16n8k16 with .bf16 A/B and .f32 C/D), g = lane>>2,
// t = lane&3: A row-major 16x16: {a0a1} = (g, 2t..2t+1), {a2a3} = (g+8, 2t..),
// {a4a5} = (g, 2t+8..), {a6a7} = (g+8, 2t+8..); B 16x8: {b0b1} = (k 2t..2t+1, n g),
// {b2b3} = (k 2t+8.., n g); C 16x8: c0,c1 = (g, 2t..2t+1), c2,c3 = (g+8, 2t..).
// Shared-memory rows are padded (16 -> 24 and 64 -> 72 halves) so that the eight
// groups of a fragment load fall on distinct banks.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace aep {

constexpr int kMlpIn = 16;     // padded input width (6 used)
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 8;     // padded output width (3 used)
constexpr int kStrideIn = 24;  // bf16 per row of a 16-wide operand in shared memory
constexpr int kStrideH = 72;   // bf16 per row of a 64-wide operand in shared memory
constexpr float kLnScale = 50.0f;  // features and outputs are ln-strains times this

// device parameter block (global memory)
struct MlpParams {
    const __nv_bfloat16* w1t;  // [64][16]  W1^T (n-major, k contiguous)
    const __nv_bfloat16* w2t;  // [64][64]
    const __nv_bfloat16* w3t;  // [64][64]
    const __nv_bfloat16* w4t;  // [8][64]
    const float* b1;           // [64]
    const float* b2;           // [64]
    const float* b3;           // [64]
    const float* b4;           // [8]
};

// shared-memory copy of the weights with padded rows (bytes)
constexpr int kMlpSmemW1 = 64 * kStrideIn;
constexpr int kMlpSmemW2 = 64 * kStrideH;
constexpr int kMlpSmemW4 = 8 * kStrideH;
constexpr int kMlpSmemWeightsBf16 = kMlpSmemW1 + 2 * kMlpSmemW2 + kMlpSmemW4;  // halves
constexpr int kMlpSmemBias = 64 * 3 + 8;                                        // floats

struct MlpSmem {
    __nv_bfloat16* w1t;
    __nv_bfloat16* w2t;
    __nv_bfloat16* w3t;
    __nv_bfloat16* w4t;
    float* b1;
    float* b2;
    float* b3;
    float* b4;
};

__device__ __forceinline__ MlpSmem mlp_smem_carve(void* base) {
    MlpSmem s;
    __nv_bfloat16* h = reinterpret_cast<__nv_bfloat16*>(base);
    s.w1t = h;
    s.w2t = s.w1t + kMlpSmemW1;
    s.w3t = s.w2t + kMlpSmemW2;
    s.w4t = s.w3t + kMlpSmemW2;
    float* f = reinterpret_cast<float*>(s.w4t + kMlpSmemW4);
    s.b1 = f;
    s.b2 = f + 64;
    s.b3 = f + 128;
    s.b4 = f + 192;
    return s;
}
constexpr int kMlpSmemBytes = kMlpSmemWeightsBf16 * 2 + kMlpSmemBias * 4;

// cooperative copy of the weights into padded shared rows (all threads of the block)
__device__ __forceinline__ void mlp_load_smem(const MlpParams& p, const MlpSmem& s, int tid, int nthreads) {
    for (int i = tid; i < 64 * 16; i += nthreads) s.w1t[(i / 16) * kStrideIn + (i % 16)] = p.w1t[i];
    for (int i = tid; i < 64 * 64; i += nthreads) {
        s.w2t[(i / 64) * kStrideH + (i % 64)] = p.w2t[i];
        s.w3t[(i / 64) * kStrideH + (i % 64)] = p.w3t[i];
    }
    for (int i = tid; i < 8 * 64; i += nthreads) s.w4t[(i / 64) * kStrideH + (i % 64)] = p.w4t[i];
    for (int i = tid; i < 64; i += nthreads) {
        s.b1[i] = p.b1[i];
        s.b2[i] = p.b2[i];
        s.b3[i] = p.b3[i];
    }
    for (int i = tid; i < 8; i += nthreads) s.b4[i] = p.b4[i];
}

__device__ __forceinline__ void mma_bf16(float c[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* p) {
    return *reinterpret_cast<const uint32_t*>(p);
}

// SiLU z * sigmoid(z) with the fast exponential and reciprocal (the activations
// are rounded to bfloat16 right after, 2^-8 relative, far above their error)
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }

// One dense layer for the 32 rows of a warp: out[32][N] = act(A[32][K] W + b).
// A: bf16 rows of stride sa; Wt: bf16 [N][K] rows of stride sw.  ACT: apply SiLU and
// store bf16 to `out` (stride so); otherwise store f32 to `outf` (stride sof).
template <int K, int N, bool ACT>
__device__ __forceinline__ void mlp_layer_warp(const __nv_bfloat16* A, int sa, const __nv_bfloat16* Wt, int sw,
                                               const float* bias, __nv_bfloat16* out, int so, float* outf, int sof,
                                               int lane) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
        float c[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
#pragma unroll
        for (int k0 = 0; k0 < K; k0 += 16) {
            const __nv_bfloat16* wb = Wt + (nt * 8 + g) * sw + k0 + 2 * t;
            const uint32_t b0 = ld_pair(wb), b1 = ld_pair(wb + 8);
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const __nv_bfloat16* ab = A + (mt * 16 + g) * sa + k0 + 2 * t;
                mma_bf16(c[mt], ld_pair(ab), ld_pair(ab + 8 * sa), ld_pair(ab + 8), ld_pair(ab + 8 * sa + 8), b0, b1);
            }
        }
        const int n0 = nt * 8 + 2 * t;
        const float bb0 = bias[n0], bb1 = bias[n0 + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int r0 = mt * 16 + g, r1 = r0 + 8;
            float v00 = c[mt][0] + bb0, v01 = c[mt][1] + bb1, v10 = c[mt][2] + bb0, v11 = c[mt][3] + bb1;
            if (ACT) {
                *reinterpret_cast<__nv_bfloat162*>(out + r0 * so + n0) = __floats2bfloat162_rn(silu(v00), silu(v01));
                *reinterpret_cast<__nv_bfloat162*>(out + r1 * so + n0) = __floats2bfloat162_rn(silu(v10), silu(v11));
            } else {
                outf[r0 * sof + n0] = v00;
                outf[r0 * sof + n0 + 1] = v01;
                outf[r1 * sof + n0] = v10;
                outf[r1 * sof + n0 + 1] = v11;
            }
        }
    }
}

// Per-warp scratch for one 32-row inference (halves / floats)
constexpr int kMlpWarpX = 32 * kStrideIn;   // bf16
constexpr int kMlpWarpH = 32 * kStrideH;    // bf16, two buffers
constexpr int kMlpWarpY = 32 * kMlpOut;     // f32
constexpr int kMlpWarpBytes = (kMlpWarpX + 2 * kMlpWarpH) * 2 + kMlpWarpY * 4;

// Forward pass of the 32 rows a warp holds in X (row r written by lane r); result
// rows in Y (row r read back by lane r).  All 32 lanes must call it.
__device__ __forceinline__ void mlp_forward_warp(const MlpSmem& W, __nv_bfloat16* X, __nv_bfloat16* H0,
                                                 __nv_bfloat16* H1, float* Y, int lane) {
    __syncwarp();
    mlp_layer_warp<kMlpIn, kMlpHidden, true>(X, kStrideIn, W.w1t, kStrideIn, W.b1, H0, kStrideH, nullptr, 0, lane);
    __syncwarp();
    mlp_layer_warp<kMlpHidden, kMlpHidden, true>(H0, kStrideH, W.w2t, kStrideH, W.b2, H1, kStrideH, nullptr, 0, lane);
    __syncwarp();
    mlp_layer_warp<kMlpHidden, kMlpHidden, true>(H1, kStrideH, W.w3t, kStrideH, W.b3, H0, kStrideH, nullptr, 0, lane);
    __syncwarp();
    mlp_layer_warp<kMlpHidden, kMlpOut, false>(H0, kStrideH, W.w4t, kStrideH, W.b4, nullptr, 0, Y, kMlpOut, lane);
    __syncwarp();
}

constexpr int kMlpCloth = 2;        // material code of cloth element records
constexpr float kQScale = 100.0f;   // sand plastic amount feature scale

// Feature row of one state and the scale of its output; returns the factor that
// maps a correction to the network's output.
// Sand (mat 1): the Drucker-Prager projection onto a cone is positively homogeneous
// in ln s, so the sorted trial log singular values are normalised by their norm r
// and the network predicts the correction divided by r; column 3 is the plastic
// amount q times kQScale (it sets the cone's opening through the hardening).
// Snow (mat 0): the clamp bounds are absolute, so ln s and the correction are
// scaled by kLnScale.
// Cloth (mat kMlpCloth): the input is u = (r13, r23, r33 - 1) / rho, rho = |(r13,
// r23, r33 - 1)|, of the QR factor of the element directions; column 3 (`q`) is the
// ratio of the friction cap to the trial shear force (HybridSolver.cpp:707-716),
// clamped to [0, 1]; the output is the change of (r13, r23, r33) divided by rho.
// Constant projections (the sand apex, cloth in tension) never reach the network.
__device__ __forceinline__ float mlp_features(const float ln_sorted[3], float q, int mat, __nv_bfloat16* row) {
    float sc = kLnScale;
    if (mat != 0) {
        const float r = sqrtf(ln_sorted[0] * ln_sorted[0] + ln_sorted[1] * ln_sorted[1] + ln_sorted[2] * ln_sorted[2]);
        sc = 1.0f / fmaxf(r, 1e-30f);
    }
    row[0] = __float2bfloat16(ln_sorted[0] * sc);
    row[1] = __float2bfloat16(ln_sorted[1] * sc);
    row[2] = __float2bfloat16(ln_sorted[2] * sc);
    row[3] = __float2bfloat16(mat == 1 ? q * kQScale : mat == kMlpCloth ? q : 0.0f);
    row[4] = __float2bfloat16(mat == 0 ? 1.0f : 0.0f);
    row[5] = __float2bfloat16(mat == 1 ? 1.0f : 0.0f);
    row[6] = __float2bfloat16(mat == kMlpCloth ? 1.0f : 0.0f);
#pragma unroll
    for (int k = 7; k < kMlpIn; ++k) row[k] = __float2bfloat16(0.0f);
    return sc;
}

// sort three values descending, remembering the permutation (perm[i] = source index)
__device__ __forceinline__ void sort3_desc(const float v[3], float s[3], int perm[3]) {
    int a = 0, b = 1, c = 2;
    if (v[b] > v[a]) { int t = a; a = b; b = t; }
    if (v[c] > v[b]) { int t = b; b = c; c = t; }
    if (v[b] > v[a]) { int t = a; a = b; b = t; }
    perm[0] = a; perm[1] = b; perm[2] = c;
    s[0] = v[a]; s[1] = v[b]; s[2] = v[c];
}

}  // namespace aep
