// aep_mlp.cuh -- the learned return map: a 7 -> 64 -> 64 -> 64 -> 3 MLP with SiLU,
// BF16 weights on the tensor cores (mma.sync m16n8k16, FP32 accumulation).
//
// Input features (one row per particle): the trial log singular values of F_E^tr
// sorted descending (3; normalised for sand, scaled by kLnScale for snow, see
// mlp_features), the sand plastic amount q (1), and the material one-hot (snow,
// sand, cloth) (3).  The first layer's A operand carries each FP32 feature as two
// bfloat16 values, hi = bf16(x) in column k and lo = bf16(x - hi) in column 7 + k,
// against the same weight in both columns (the shared-memory copy of W1^T repeats
// columns 0..6 in 7..13): the tensor cores then see the features to ~2^-17 instead
// of bfloat16's 2^-9, at no extra MMA (7 features use 14 of the 16 columns).
// Cloth elements use the same network on (r13, r23, r33 - 1) of their QR factor,
// normalised, with the ratio of the friction cap to the trial shear force in
// column 3.  Output: the correction
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

constexpr int kMlpIn = 16;     // padded input width (7 features as hi + lo: 14 used)
constexpr int kMlpFeat = 7;    // features
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

// cooperative copy of the weights into padded shared rows (all threads of the block),
// 16 bytes at a time: every block in global memory starts on a 16-byte boundary
// (offsets of 1024, 5120, 9216 halves and 9728.. floats into 256-byte aligned
// allocations), and the padded rows (48 and 144 bytes) keep 16-byte alignment
__device__ __forceinline__ void mlp_load_smem(const MlpParams& p, const MlpSmem& s, int tid, int nthreads) {
    const uint4* g1 = reinterpret_cast<const uint4*>(p.w1t);
    const uint4* g2 = reinterpret_cast<const uint4*>(p.w2t);
    const uint4* g3 = reinterpret_cast<const uint4*>(p.w3t);
    const uint4* g4 = reinterpret_cast<const uint4*>(p.w4t);
    for (int n = tid; n < 64; n += nthreads) {  // W1^T row n: [w0..w6, w0..w6, 0, 0]
        const uint4 a = g1[2 * n], b = g1[2 * n + 1];
        const uint32_t r[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        const __nv_bfloat16* w = reinterpret_cast<const __nv_bfloat16*>(r);
        __nv_bfloat16 d[16];
#pragma unroll
        for (int k = 0; k < kMlpFeat; ++k) d[k] = d[kMlpFeat + k] = w[k];
        d[14] = d[15] = __float2bfloat16(0.0f);
        *reinterpret_cast<uint4*>(s.w1t + n * kStrideIn) = *reinterpret_cast<const uint4*>(d);
        *reinterpret_cast<uint4*>(s.w1t + n * kStrideIn + 8) = *reinterpret_cast<const uint4*>(d + 8);
    }
    for (int i = tid; i < 64 * 8; i += nthreads) {
        *reinterpret_cast<uint4*>(s.w2t + (i >> 3) * kStrideH + (i & 7) * 8) = g2[i];
        *reinterpret_cast<uint4*>(s.w3t + (i >> 3) * kStrideH + (i & 7) * 8) = g3[i];
    }
    for (int i = tid; i < 8 * 8; i += nthreads)
        *reinterpret_cast<uint4*>(s.w4t + (i >> 3) * kStrideH + (i & 7) * 8) = g4[i];
    for (int i = tid; i < 16; i += nthreads) {
        reinterpret_cast<float4*>(s.b1)[i] = reinterpret_cast<const float4*>(p.b1)[i];
        reinterpret_cast<float4*>(s.b2)[i] = reinterpret_cast<const float4*>(p.b2)[i];
        reinterpret_cast<float4*>(s.b3)[i] = reinterpret_cast<const float4*>(p.b3)[i];
    }
    for (int i = tid; i < 2; i += nthreads) reinterpret_cast<float4*>(s.b4)[i] = reinterpret_cast<const float4*>(p.b4)[i];
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

// The step's SiLU: z sigmoid(z) = h + h tanh(h), h = z / 2, with the hardware tanh
// (one MUFU operation instead of an exponential and a reciprocal; relative error of
// tanh about 2^-11, so an activation is off by at most |z| 2^-12, below the
// bfloat16 rounding it then takes for |z| of order one).  The forward API and the
// training keep silu(); the step's predictions are checked against the projection's
// optimality conditions whatever the arithmetic that made them.
__device__ __forceinline__ float silu_step(float z) {
    const float h = 0.5f * z;
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
    return fmaf(h, t, h);
}

template <bool kStep>
__device__ __forceinline__ float silu_t(float z) {
    return kStep ? silu_step(z) : silu(z);
}

// Per-warp scratch for one 32-row inference (halves / floats): the input rows and
// the output rows; the hidden activations stay in registers (mlp_forward_warp)
constexpr int kMlpWarpX = 32 * kStrideIn;   // bf16
constexpr int kMlpWarpY = 32 * kMlpOut;     // f32
constexpr int kMlpWarpBytes = kMlpWarpX * 2 + kMlpWarpY * 4;

// four 8x8 bf16 matrices from shared memory (lane i gives the row address of
// matrix i/8, row i%8; register j of lane l holds matrix j's row l/4, columns
// 2(l%4), 2(l%4)+1)
__device__ __forceinline__ void ldmatrix_x4(const __nv_bfloat16* p, uint32_t& r0, uint32_t& r1, uint32_t& r2,
                                            uint32_t& r3) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// One hidden layer (64 -> 64, SiLU) of the warp's 32 rows with the activations in
// registers: a[mt][kt][.] is the m16n8k16 A fragment of rows mt*16.., columns
// kt*16.. of the input; the layer writes the same fragment of its output to o.
// The C fragment of output columns nt*8.. (rows g, g+8; columns 2t, 2t+1) is the A
// fragment's register pair {0,1} (nt even) or {2,3} (nt odd) of k tile nt/2, so the
// epilogue packs it in place.  B fragments come from the padded rows of W^T by
// ldmatrix (two k tiles of one n tile per instruction).
template <bool kStep>
__device__ __forceinline__ void mlp_hidden_layer_reg(const uint32_t (&a)[2][4][4], uint32_t (&o)[2][4][4],
                                                     const __nv_bfloat16* Wt, const float* bias, int lane) {
    const int t = lane & 3;
    // ldmatrix row address of this lane: matrix (lane>>3) = (k tile pair member lane>>4,
    // k half (lane>>3)&1), row lane&7 of the n tile
    const __nv_bfloat16* wrow = Wt + (lane & 7) * kStrideH + (lane >> 4) * 16 + ((lane >> 3) & 1) * 8;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float c[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
#pragma unroll
        for (int kp = 0; kp < 2; ++kp) {  // k tiles 2kp, 2kp+1
            uint32_t b00, b01, b10, b11;
            ldmatrix_x4(wrow + nt * 8 * kStrideH + kp * 32, b00, b01, b10, b11);
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                mma_bf16(c[mt], a[mt][2 * kp][0], a[mt][2 * kp][1], a[mt][2 * kp][2], a[mt][2 * kp][3], b00, b01);
                mma_bf16(c[mt], a[mt][2 * kp + 1][0], a[mt][2 * kp + 1][1], a[mt][2 * kp + 1][2],
                         a[mt][2 * kp + 1][3], b10, b11);
            }
        }
        const int n0 = nt * 8 + 2 * t;
        const float bb0 = bias[n0], bb1 = bias[n0 + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            o[mt][nt >> 1][(nt & 1) * 2] = pack_bf16x2(silu_t<kStep>(c[mt][0] + bb0), silu_t<kStep>(c[mt][1] + bb1));
            o[mt][nt >> 1][(nt & 1) * 2 + 1] =
                pack_bf16x2(silu_t<kStep>(c[mt][2] + bb0), silu_t<kStep>(c[mt][3] + bb1));
        }
    }
}

// Forward pass of the 32 rows a warp holds in X (row r written by lane r); result
// rows in Y (row r read back by lane r).  All 32 lanes must call it.  Each layer
// accumulates its 16-wide k tiles in order in FP32 and rounds its SiLU outputs to
// bfloat16 (the rounding points of the oracle's forward); the hidden activations
// stay in registers between layers.  kStep: the step's SiLU (silu_step).
template <bool kStep = false>
__device__ __forceinline__ void mlp_forward_warp(const MlpSmem& W, __nv_bfloat16* X, float* Y, int lane) {
    const int g = lane >> 2, t = lane & 3;
    __syncwarp();
    uint32_t h0[2][4][4], h1[2][4][4];
    {  // layer 1 (16 -> 64): A fragments from X, B fragments by pairs of 32-bit loads
        uint32_t x[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const __nv_bfloat16* ab = X + (mt * 16 + g) * kStrideIn + 2 * t;
            x[mt][0] = ld_pair(ab);
            x[mt][1] = ld_pair(ab + 8 * kStrideIn);
            x[mt][2] = ld_pair(ab + 8);
            x[mt][3] = ld_pair(ab + 8 * kStrideIn + 8);
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const __nv_bfloat16* wb = W.w1t + (nt * 8 + g) * kStrideIn + 2 * t;
            const uint32_t b0 = ld_pair(wb), b1 = ld_pair(wb + 8);
            const int n0 = nt * 8 + 2 * t;
            const float bb0 = W.b1[n0], bb1 = W.b1[n0 + 1];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                float c[4] = {0, 0, 0, 0};
                mma_bf16(c, x[mt][0], x[mt][1], x[mt][2], x[mt][3], b0, b1);
                h0[mt][nt >> 1][(nt & 1) * 2] = pack_bf16x2(silu_t<kStep>(c[0] + bb0), silu_t<kStep>(c[1] + bb1));
                h0[mt][nt >> 1][(nt & 1) * 2 + 1] = pack_bf16x2(silu_t<kStep>(c[2] + bb0), silu_t<kStep>(c[3] + bb1));
            }
        }
    }
    mlp_hidden_layer_reg<kStep>(h0, h1, W.w2t, W.b2, lane);
    mlp_hidden_layer_reg<kStep>(h1, h0, W.w3t, W.b3, lane);
    {  // output layer (64 -> 8), FP32 rows to Y
        float c[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const __nv_bfloat16* wb = W.w4t + g * kStrideH + kt * 16 + 2 * t;
            const uint32_t b0 = ld_pair(wb), b1 = ld_pair(wb + 8);
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) mma_bf16(c[mt], h0[mt][kt][0], h0[mt][kt][1], h0[mt][kt][2], h0[mt][kt][3], b0, b1);
        }
        const float bb0 = W.b4[2 * t], bb1 = W.b4[2 * t + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int r0 = mt * 16 + g, r1 = r0 + 8;
            Y[r0 * kMlpOut + 2 * t] = c[mt][0] + bb0;
            Y[r0 * kMlpOut + 2 * t + 1] = c[mt][1] + bb1;
            Y[r1 * kMlpOut + 2 * t] = c[mt][2] + bb0;
            Y[r1 * kMlpOut + 2 * t + 1] = c[mt][3] + bb1;
        }
    }
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
    const float x[kMlpFeat] = {ln_sorted[0] * sc, ln_sorted[1] * sc, ln_sorted[2] * sc,
                               mat == 1 ? q * kQScale : mat == kMlpCloth ? q : 0.0f, mat == 0 ? 1.0f : 0.0f,
                               mat == 1 ? 1.0f : 0.0f, mat == kMlpCloth ? 1.0f : 0.0f};
#pragma unroll
    for (int k = 0; k < kMlpFeat; ++k) {  // hi, lo: x to ~2^-17 as a sum of two bfloat16
        const __nv_bfloat16 hi = __float2bfloat16(x[k]);
        row[k] = hi;
        row[kMlpFeat + k] = __float2bfloat16(x[k] - __bfloat162float(hi));
    }
    row[14] = row[15] = __float2bfloat16(0.0f);
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
