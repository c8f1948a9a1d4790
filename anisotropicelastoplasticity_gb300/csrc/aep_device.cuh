// aep_device.cuh -- device-side building blocks of the sm_103a MPM step.
//
// Layout conventions used by every kernel:
//   * particles: structure of arrays in FP32, one array per component; 3x3
//     matrices are nine arrays, component (a,b) in array [3a+b] (row-major).
//   * grid: padded, blocked.  The reference node (i,j,k) (RegularGrid.cpp:
//     164-168) becomes padded node (i+4, j+4, k+4); padded nodes are grouped
//     in 4x4x4 blocks stored contiguously (64 nodes), blocks in x-fastest
//     order.  The padding lets every particle's 4x4x4 cubic stencil be
//     addressed without bounds checks; nodes outside the reference grid get
//     weight 0 exactly as HybridSolver.cpp:44-46 drops them.
//   * a particle's cell is floor((x - min)/h), its stencil base node is
//     cell - 1 and its stencil is base + {0..3}^3 (the nodes with nonzero
//     cubic weight among the 5^3 candidates of HybridSolver.cpp:38-47).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace aep {

constexpr int kMaxShapes = 8;
constexpr uint32_t kInvalidKey = 0xFFFFFFFFu;

enum : int { kSnow = 0, kSand = 1, kClothVertex = 2, kClothElement = 3 };
enum : int { kSdfPlane = 0, kSdfSphere = 1, kSdfWall2Ground = 2 };

struct DevShape {
    int type;
    float p[6];
};

// Per-launch constants (kernel parameter space).
struct KParams {
    float min[3], h[3], inv_h[3];
    int res[3];
    int nb[3];            // padded node blocks per axis
    float apic[3];        // (3 / hmin^2) * h_a: APIC D^-1 scaled to stencil offsets (HS:175-177)
    float mass_scale, inv_mass_scale;
    float mom_scale, inv_mom_scale;
    float snow_mu, snow_lambda, snow_xi, snow_lo, snow_hi;
    float snow_lnlo, snow_lnhi;  // ln of the clamp bounds, rounded once from FP64
    float sand_mu, sand_lambda, sand_h0, sand_h1, sand_h2, sand_h3, sand_k;  // k = (3l+2m)/(2m)
    float gravity[3];
    float friction;
    int friction_bug;
    float particle_damp;
    float mesh_damp;  // APIC damping of cloth vertices and elements, reference 1 (HS:926,932)
    int track_fp;
    int fp64_apex;        // redo sand return mappings near the Drucker-Prager apex in FP64
    int nshapes;
    DevShape shapes[kMaxShapes];
    float cell_volume;
    // adaptive time stepping (HybridSolver::solve): when set, the force pass and
    // grid update take dt_dev[0] and the G2P takes dt_dev[1] instead of their
    // dt arguments, and the normalisation / grid update reduce max |v|^2 into
    // vmax2[0] / vmax2[1] (float bits; non-negative floats order like integers)
    const float* dt_dev;
    unsigned int* vmax2;
};

__device__ __forceinline__ float step_dt(const KParams& P, float dt, int which) {
    return P.dt_dev ? P.dt_dev[which] : dt;
}

// warp max of a non-negative float, one atomic per warp (all lanes call it)
__device__ __forceinline__ void warp_max_atomic(unsigned int* dst, float v2) {
    unsigned int b = __float_as_uint(v2);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
    if ((threadIdx.x & 31) == 0 && b) atomicMax(dst, b);
}

// device state of the adaptive solve loop (HybridSolver.cpp:859-892)
struct SolveState {
    double cfl, inv_hmin;  // Dt = cfl / max(300, max|v| / hmin)
    double t, inner, Dt;   // simulated time, time inside the current frame, current Dt
    int initialized;       // the first Dt comes from the P2G velocities (:860)
    int frame, frame_flag; // frames completed; this step completed a frame
    int steps;
    float dt[2];           // Dt for the force pass / grid update, Dt for the G2P
    unsigned int vmax2[2]; // max |v|^2 after the normalisation / the grid update
};

// Particle state, structure of arrays.
struct PArrays {
    float* x[3];
    float* v[3];
    float* B[9];
    float* F[9];
    float* Fp[9];   // only when track_fp
    float* m;
    float* vol;
    float* plastic;  // sand: plasticAmount q; snow: J_P = det F_P
    uint8_t* mat;
    int32_t* id;     // caller's particle index
};

struct GArrays {
    unsigned long long* acc;  // 4 per node: mass, momentum/impulse x, y, z (fixed point)
    float4* vel;              // (v, m) after normalisation / after grid update
    float4* vbf;              // before-friction velocity (w unused)
    uint32_t* flag;           // per node block: touched this step
    int32_t* active;          // list of touched node blocks
    int32_t* nactive;         // its length
};

// LagrangianMesh state on the device (LagrangianMesh.h:37-73).  Vertices and
// elements live in the particle arrays with ids [vbase, vbase+nv) and
// [ebase, ebase+nf); their element directions [d1 d2 d3] are stored as the
// columns of the particle's F.
struct MeshArrays {
    int nv, nf, vbase, ebase;
    const int32_t* faces;          // 3 per element: vertex indices 0..nv-1
    const float* rest;             // 6 per element: inverseR of the rest in-plane R (i11, i12, i22)
                                   // and the third row of the rest direction matrix (HS:427)
    float* estress;                // 9 per element: -dt * (element normal stress), row-major
    unsigned long long* vforce;    // 3 per vertex: dt * in-plane force, fixed point
    int32_t* slot_of;              // per id: slot in this step's sorted order
    int32_t* curidx_of;            // per id: index in the current particle arrays
    float mu, lambda, shear, stiffness, friction, damp;
    int volume_weighting;          // multiply the in-plane vertex forces by the element volume
};

struct DevStats {
    unsigned long long out_of_domain;
    unsigned long long fallbacks;
    unsigned long long overflow;
    unsigned long long mass;       // int64 sums, exact
    unsigned long long mom[3];
    unsigned long long nodes;      // nodes with mass after P2G
    unsigned long long learned_ok;      // learned return maps accepted
    unsigned long long learned_rejected;  // learned outputs replaced by the exact mapping
    unsigned long long learned_exact;  // constant projections (sand apex, cloth tension) taken exactly
    long long movers;              // particles that changed key (incremental ordering), -1: full sort
    unsigned long long fp64_apex;  // sand return mappings near the apex redone in FP64 (fp64_apex option)
    unsigned int force_fp64;       // entries of the force pass's FP64 list (k_force_fp64)
    unsigned int mlp_rows;         // rows queued for the learned return map (k_mlp_finish)
    // length of the active node-block list (GArrays::nactive points here: zeroed with
    // the counters at each step), on its own cache line: every grid thread reads it
    // while the counters above take the blocks' atomics
    alignas(128) int32_t nactive;
};

// Rows of the learned return map that the G2P pass queues for k_mlp_finish
// (plastic snow and sand states whose projection is not a constant): field-major
// float arrays of `cap` rows, the fields below: the trial log singular values, the
// F update D and the right singular vectors V of F + D (the stretch form of the
// return mapping); F and the plastic scalar stay in the current state arrays.
struct MlpQueue {
    int32_t* j;   // slot in the new order
    int32_t* pj;  // slot in the current order
    float* f;     // [kQueueFields][cap]
    int cap;
};
constexpr int kQLn = 0, kQD = 3, kQV = 12;
constexpr int kQueueFields = 21;

// Training-pair harvest from the exact return mapping (plain G2P): records of 8
// floats [ln s trial sorted desc (3), q, material, ln s_new - ln s trial (3)].
struct Harvest {
    float* buf;
    unsigned long long* count;
    long long capacity;
    int stride;  // every stride-th particle slot
};

// ---------------------------------------------------------------------------------
// cubic B-spline weights on one axis for stencil offsets o = 0..3 (node cell-1+o):
// w[o] = N(f + 1 - o), dw[o] = N'(f + 1 - o) / h, with N, N' of interpolation.cpp:9-33.
__device__ __forceinline__ void bspline(float f, float inv_h, float w[4], float dw[4]) {
    float g = 1.0f - f;
    float f2 = f * f, g2 = g * g;
    w[0] = g2 * g * (1.0f / 6.0f);
    w[1] = 0.5f * f2 * f - f2 + (2.0f / 3.0f);
    w[2] = 0.5f * g2 * g - g2 + (2.0f / 3.0f);
    w[3] = f2 * f * (1.0f / 6.0f);
    dw[0] = -0.5f * g2 * inv_h;
    dw[1] = (1.5f * f2 - 2.0f * f) * inv_h;
    dw[2] = (2.0f * g - 1.5f * g2) * inv_h;
    dw[3] = 0.5f * f2 * inv_h;
}

// Particle location: reference cell (clamped into the grid), fraction in [0,1].
// Returns true if the particle had to be clamped (it left the grid).
__device__ __forceinline__ bool locate(const KParams& P, float px, float py, float pz, int cell[3],
                                       float f[3]) {
    float p[3] = {px, py, pz};
    bool clamped = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float u = (p[a] - P.min[a]) * P.inv_h[a];
        float c = floorf(u);
        int ci = (int)c;
        if (!(u >= 0.0f) || ci > P.res[a] - 1) {  // also catches NaN
            clamped = true;
            ci = !(u >= 0.0f) ? 0 : P.res[a] - 1;
        }
        float fr = u - (float)ci;
        fr = fminf(fmaxf(fr, 0.0f), 1.0f);
        cell[a] = ci;
        f[a] = fr;
    }
    return clamped;
}

// sort key: (padded base-node block, base position inside the block)
__device__ __forceinline__ uint32_t make_key(const KParams& P, const int cell[3]) {
    int bx = (cell[0] + 3) >> 2, by = (cell[1] + 3) >> 2, bz = (cell[2] + 3) >> 2;
    int wx = (cell[0] + 3) & 3, wy = (cell[1] + 3) & 3, wz = (cell[2] + 3) & 3;
    uint32_t blk = (uint32_t)((bz * P.nb[1] + by) * P.nb[0] + bx);
    return (blk << 6) | (uint32_t)((wz << 4) | (wy << 2) | wx);
}

// padded base node of a key
__device__ __forceinline__ void key_base(const KParams& P, uint32_t key, int base[3]) {
    uint32_t blk = key >> 6;
    int bx = (int)(blk % (uint32_t)P.nb[0]);
    uint32_t r = blk / (uint32_t)P.nb[0];
    int by = (int)(r % (uint32_t)P.nb[1]);
    int bz = (int)(r / (uint32_t)P.nb[1]);
    base[0] = 4 * bx + (int)(key & 3);
    base[1] = 4 * by + (int)((key >> 2) & 3);
    base[2] = 4 * bz + (int)((key >> 4) & 3);
}

// storage index of padded node (x, y, z)
__device__ __forceinline__ uint32_t node_index(const KParams& P, int x, int y, int z) {
    uint32_t blk = (uint32_t)(((z >> 2) * P.nb[1] + (y >> 2)) * P.nb[0] + (x >> 2));
    return (blk << 6) | (uint32_t)(((z & 3) << 4) | ((y & 3) << 2) | (x & 3));
}

// per-axis partial node indices: idx(ox,oy,oz) = X[ox] + Y[oy] + Z[oz]
__device__ __forceinline__ void stencil_offsets(const KParams& P, const int base[3], uint32_t X[4],
                                                uint32_t Y[4], uint32_t Z[4]) {
    uint32_t sy = (uint32_t)P.nb[0] * 64u, sz = (uint32_t)P.nb[0] * (uint32_t)P.nb[1] * 64u;
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        int x = base[0] + o, y = base[1] + o, z = base[2] + o;
        X[o] = (uint32_t)(x >> 2) * 64u + (uint32_t)(x & 3);
        Y[o] = (uint32_t)(y >> 2) * sy + (uint32_t)((y & 3) << 2);
        Z[o] = (uint32_t)(z >> 2) * sz + (uint32_t)((z & 3) << 4);
    }
}

// Grid tile of a block of sorted particles: the 2x2x2 node blocks (512 nodes)
// starting at the base-node block of the block's first particle.  Particles are
// ordered by base-node block, so almost every particle of the block has its
// whole 4x4x4 stencil inside; their gathers read shared memory instead of L1/L2.
constexpr int kTileNodes = 512;

__device__ __forceinline__ void tile_origin(const KParams& P, uint32_t key, int org[3]) {
    const uint32_t blk = key >> 6;
    org[0] = (int)(blk % (uint32_t)P.nb[0]);
    const uint32_t r = blk / (uint32_t)P.nb[0];
    org[1] = (int)(r % (uint32_t)P.nb[1]);
    org[2] = (int)(r / (uint32_t)P.nb[1]);
}

// Programmatic dependent launch within a step: a kernel launched with the
// programmatic-serialisation attribute may be scheduled while the kernel before it
// in the stream finishes.  pdl_entry() first lets the next kernel be launched once
// every block of this one has started (pdl_trigger), then waits until the previous
// kernel has completed and its memory is visible (griddepcontrol.wait), before
// this kernel reads or writes anything.  Both are no-ops for a kernel launched
// without the attribute.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_entry() {
    pdl_trigger();
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// asynchronous 4-byte copy global -> shared (cp.async; no registers held while in
// flight), its commit and the wait for all of this thread's copies
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// cooperative copy of the tile (all threads of the block); src2 / dst2 may be null
__device__ __forceinline__ void load_tile(const KParams& P, const int org[3], const float4* __restrict__ src,
                                          const float4* __restrict__ src2, float4* dst, float4* dst2) {
    for (int i = threadIdx.x; i < kTileNodes; i += blockDim.x) {
        const int t = i >> 6;
        const uint32_t gblk = (uint32_t)(((org[2] + (t >> 2)) * P.nb[1] + org[1] + ((t >> 1) & 1)) * P.nb[0] + org[0] +
                                         (t & 1));
        const uint32_t node = (gblk << 6) | (uint32_t)(i & 63);
        dst[i] = src[node];
        if (dst2) dst2[i] = src2[node];
    }
}

// stencil offsets inside the tile when the stencil's base block is the tile's
// origin (returns false otherwise); the same additive form as stencil_offsets
__device__ __forceinline__ bool tile_offsets(const int base[3], const int org[3], uint32_t X[4], uint32_t Y[4],
                                             uint32_t Z[4]) {
    if ((base[0] >> 2) != org[0] || (base[1] >> 2) != org[1] || (base[2] >> 2) != org[2]) return false;
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        const int x = base[0] + o - 4 * org[0], y = base[1] + o - 4 * org[1], z = base[2] + o - 4 * org[2];
        X[o] = (uint32_t)((x >> 2) * 64 + (x & 3));
        Y[o] = (uint32_t)((y >> 2) * 128 + ((y & 3) << 2));
        Z[o] = (uint32_t)((z >> 2) * 256 + ((z & 3) << 4));
    }
    return true;
}

// weights of one particle with the reference's out-of-grid node drop (HS:44-46)
__device__ __forceinline__ bool particle_weights(const KParams& P, const int cell[3], const float f[3],
                                                 float w[3][4], float dw[3][4]) {
    bool truncated = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        bspline(f[a], P.inv_h[a], w[a], dw[a]);
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            int node = cell[a] - 1 + o;
            if (node < 0 || node >= P.res[a]) {
                w[a][o] = 0.0f;
                dw[a][o] = 0.0f;
                truncated = true;
            }
        }
    }
    return truncated;
}

// ---------------------------------------------------------------------------------
// small row-major 3x3 helpers
template <typename T>
__device__ __forceinline__ void mat_mul(const T A[9], const T B[9], T C[9]) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) C[3 * a + b] = A[3 * a] * B[b] + A[3 * a + 1] * B[3 + b] + A[3 * a + 2] * B[6 + b];
}
// C = A * B^T
template <typename T>
__device__ __forceinline__ void mat_mul_bt(const T A[9], const T B[9], T C[9]) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
            C[3 * a + b] = A[3 * a] * B[3 * b] + A[3 * a + 1] * B[3 * b + 1] + A[3 * a + 2] * B[3 * b + 2];
}
template <typename T>
__device__ __forceinline__ T mat_det(const T A[9]) {
    return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
           A[2] * (A[3] * A[7] - A[4] * A[6]);
}
// cof(A) = det(A) A^-T
template <typename T>
__device__ __forceinline__ void mat_cofactor(const T A[9], T C[9]) {
    C[0] = A[4] * A[8] - A[5] * A[7];
    C[1] = A[5] * A[6] - A[3] * A[8];
    C[2] = A[3] * A[7] - A[4] * A[6];
    C[3] = A[2] * A[7] - A[1] * A[8];
    C[4] = A[0] * A[8] - A[2] * A[6];
    C[5] = A[1] * A[6] - A[0] * A[7];
    C[6] = A[1] * A[5] - A[2] * A[4];
    C[7] = A[2] * A[3] - A[0] * A[5];
    C[8] = A[0] * A[4] - A[1] * A[3];
}

__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }
__device__ __forceinline__ float sqrt_t(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_t(double x) { return sqrt(x); }
__device__ __forceinline__ float exp_t(float x) { return expf(x); }
__device__ __forceinline__ double exp_t(double x) { return exp(x); }
__device__ __forceinline__ float log_t(float x) { return logf(x); }
__device__ __forceinline__ double log_t(double x) { return log(x); }
__device__ __forceinline__ float sin_t(float x) { return sinf(x); }
__device__ __forceinline__ double sin_t(double x) { return sin(x); }
// division for the Jacobi rotation angle: the angle only has to be close (the
// rotation stays exactly orthogonal through c = rsqrt(1 + t^2), s = c t, and W = A V
// holds whatever angle is applied), so FP32 uses the 2-ulp fast division
__device__ __forceinline__ float rot_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double rot_div(double a, double b) { return a / b; }
__device__ __forceinline__ float abs_t(float x) { return fabsf(x); }
__device__ __forceinline__ double abs_t(double x) { return fabs(x); }
// square root for the Jacobi rotation angle (argument >= 1): the angle only has to
// be close, as for rot_div, so FP32 takes x rsqrt(x)
__device__ __forceinline__ float rot_sqrt(float x) { return x * rsqrtf(x); }
__device__ __forceinline__ double rot_sqrt(double x) { return sqrt(x); }

// 3x3 SVD by one-sided (Hestenes) Jacobi rotations on the columns of A:
// A V = U diag(s), s >= 0 (unsorted).  Every quantity the step needs from an
// SVD (U V^T, U f(s) V^T, V s^-1 U^T with f applied per singular value) is
// invariant under ordering, so no sort is done.  Returns false if a singular
// value is below `smin_rel` * the largest (caller falls back to FP64).
template <typename T>
__device__ __forceinline__ bool svd3(const T A[9], T U[9], T s[3], T V[9], int max_sweeps, T tol, T smin_rel) {
    T W[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) W[k] = A[k];
#pragma unroll
    for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0) ? T(1) : T(0);
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        bool rotated = false;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            T alpha = W[p] * W[p] + W[3 + p] * W[3 + p] + W[6 + p] * W[6 + p];
            T beta = W[q] * W[q] + W[3 + q] * W[3 + q] + W[6 + q] * W[6 + q];
            T gamma = W[p] * W[q] + W[3 + p] * W[3 + q] + W[6 + p] * W[6 + q];
            if (abs_t(gamma) > tol * sqrt_t(alpha * beta)) {
                rotated = true;
                T zeta = rot_div(beta - alpha, T(2) * gamma);
                T az = abs_t(zeta);
                T t = az > T(1e15) ? rot_div(T(0.5), zeta)
                                   : rot_div(zeta >= T(0) ? T(1) : T(-1), az + sqrt_t(T(1) + zeta * zeta));
                T c = rsqrt_t(T(1) + t * t), sn = c * t;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    T wp = W[3 * r + p], wq = W[3 * r + q];
                    W[3 * r + p] = c * wp - sn * wq;
                    W[3 * r + q] = sn * wp + c * wq;
                    T vp = V[3 * r + p], vq = V[3 * r + q];
                    V[3 * r + p] = c * vp - sn * vq;
                    V[3 * r + q] = sn * vp + c * vq;
                }
            }
        }
        if (!rotated) break;
    }
    T smax = T(0);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        s[b] = sqrt_t(W[b] * W[b] + W[3 + b] * W[3 + b] + W[6 + b] * W[6 + b]);
        smax = s[b] > smax ? s[b] : smax;
    }
    bool ok = true;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        if (!(s[b] > smin_rel * smax) || !(s[b] > T(0))) ok = false;
        T inv = s[b] > T(0) ? T(1) / s[b] : T(0);
#pragma unroll
        for (int r = 0; r < 3; ++r) U[3 * r + b] = W[3 * r + b] * inv;
    }
    return ok;
}

__device__ __forceinline__ float log1p_t(float x) { return log1pf(x); }
__device__ __forceinline__ double log1p_t(double x) { return log1p(x); }
__device__ __forceinline__ float expm1_t(float x) { return expm1f(x); }
__device__ __forceinline__ double expm1_t(double x) { return expm1(x); }

// One Jacobi rotation of a symmetric 3x3 matrix in the (p, q) plane, chosen to
// zero a_pq (the t = tan(phi) form: a_pp -= t a_pq, a_qq += t a_pq), with r the
// third index; V accumulates the rotations (columns p, q).  Skipped when a_pq
// is at most `thresh`.
template <typename T>
__device__ __forceinline__ bool jacobi_rot(T& app, T& aqq, T& apq, T& arp, T& arq, T V[9], int p, int q, T thresh) {
    if (!(abs_t(apq) > thresh)) return false;
    const T zeta = rot_div(aqq - app, T(2) * apq);
    const T az = abs_t(zeta);
    const T t = az > T(1e15) ? rot_div(T(0.5), zeta)
                             : rot_div(zeta >= T(0) ? T(1) : T(-1), az + rot_sqrt(T(1) + zeta * zeta));
    const T c = rsqrt_t(T(1) + t * t), s = c * t;
    app -= t * apq;
    aqq += t * apq;
    apq = T(0);
    const T rp = arp, rq = arq;
    arp = c * rp - s * rq;
    arq = s * rp + c * rq;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const T vp = V[3 * r + p], vq = V[3 * r + q];
        V[3 * r + p] = c * vp - s * vq;
        V[3 * r + q] = s * vp + c * vq;
    }
    return true;
}

// Eigen-decomposition S = V diag(lam) V^T of the symmetric matrix
// S = [[a00, a01, a02], [a01, a11, a12], [a02, a12, a22]] by cyclic Jacobi sweeps,
// until every off-diagonal entry is at most tol |S|_F (rotations keep |S|_F): the
// eigenvalues are then exact to ~tol |S|_F, all the step needs of them.
template <typename T>
__device__ __forceinline__ void sym_eig3(T a00, T a11, T a22, T a01, T a02, T a12, T lam[3], T V[9], int max_sweeps,
                                         T tol) {
#pragma unroll
    for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0) ? T(1) : T(0);
    const T thresh =
        tol * sqrt_t(a00 * a00 + a11 * a11 + a22 * a22 + T(2) * (a01 * a01 + a02 * a02 + a12 * a12));
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        bool r = jacobi_rot<T>(a00, a11, a01, a02, a12, V, 0, 1, thresh);
        r |= jacobi_rot<T>(a00, a22, a02, a01, a12, V, 0, 2, thresh);
        r |= jacobi_rot<T>(a11, a22, a12, a01, a02, V, 1, 2, thresh);
        if (!r) break;
    }
    lam[0] = a00;
    lam[1] = a11;
    lam[2] = a22;
}

// a + b = s + e exactly (Knuth's TwoSum; no multiplication, so nothing is fused)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// a0 b0 + a1 b1 + a2 b2 - c with the products split exactly (p + e = a b by fma)
// and the sum carried in twice the working precision, rounded once at the end:
// resolves F^T F - I to ~2^-48 where plain FP32 keeps ~2^-24 of the terms ~1.
__device__ __forceinline__ float dot3_minus_exact(float a0, float b0, float a1, float b1, float a2, float b2, float c) {
    const float p0 = __fmul_rn(a0, b0), p1 = __fmul_rn(a1, b1), p2 = __fmul_rn(a2, b2);
    const float e0 = fmaf(a0, b0, -p0), e1 = fmaf(a1, b1, -p1), e2 = fmaf(a2, b2, -p2);
    float s, t1, t2, t3;
    two_sum(p0, p1, s, t1);
    two_sum(s, p2, s, t2);
    two_sum(s, -c, s, t3);
    return __fadd_rn(s, __fadd_rn(__fadd_rn(__fadd_rn(e0, e1), e2), __fadd_rn(__fadd_rn(t1, t2), t3)));
}

// C - I = F_tr^T F_tr - I for F_tr = F + D (row-major 3x3), as its six entries
// (e00, e11, e22, e01, e02, e12): (F^T F - I) + F^T D + D^T F + D^T D.  The first
// term is where FP32 loses the state: F is near a rotation and its Gram matrix
// differs from I by a few units of 2^-24, so it is summed without loss (float)
// or in FP64 (double); the D terms are small and need no care.
__device__ __forceinline__ void trial_stretch(const float F[9], const float D[9], float e[6]) {
    const int I[6] = {0, 1, 2, 0, 0, 1}, J[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int i = I[k], j = J[k];
        const float g = dot3_minus_exact(F[i], F[j], F[3 + i], F[3 + j], F[6 + i], F[6 + j], i == j ? 1.0f : 0.0f);
        // F^T D + D^T F + D^T D = F^T D + D^T (F + D)
        float x = F[i] * D[j] + F[3 + i] * D[3 + j] + F[6 + i] * D[6 + j];
        x += D[i] * (F[j] + D[j]) + D[3 + i] * (F[3 + j] + D[3 + j]) + D[6 + i] * (F[6 + j] + D[6 + j]);
        e[k] = g + x;
    }
}
__device__ __forceinline__ void trial_stretch(const float F[9], const float D[9], double e[6]) {
    const int I[6] = {0, 1, 2, 0, 0, 1}, J[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int i = I[k], j = J[k];
        double x = -(i == j ? 1.0 : 0.0);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const double fi = F[3 * r + i] + (double)D[3 * r + i], fj = F[3 * r + j] + (double)D[3 * r + j];
            x = fma(fi, fj, x);
        }
        e[k] = x;
    }
}

// Complete U where a singular value vanished (FP64 path only).
__device__ inline void svd3_complete(double U[9], const double s[3]) {
    double smax = fmax(s[0], fmax(s[1], s[2]));
    double tiny = 1e-300 + 1e-14 * smax;
    int good[3], ng = 0, bad[3], nbd = 0;
    for (int b = 0; b < 3; ++b) {
        if (s[b] > tiny) good[ng++] = b;
        else bad[nbd++] = b;
    }
    for (int k = 0; k < nbd; ++k) {
        int b = bad[k];
        double u[3];
        if (ng == 2) {
            int c0 = good[0], c1 = good[1];
            u[0] = U[3 + c0] * U[6 + c1] - U[6 + c0] * U[3 + c1];
            u[1] = U[6 + c0] * U[c1] - U[c0] * U[6 + c1];
            u[2] = U[c0] * U[3 + c1] - U[3 + c0] * U[c1];
        } else {
            double best = -1;
            for (int e = 0; e < 3; ++e) {
                double t[3] = {e == 0 ? 1.0 : 0.0, e == 1 ? 1.0 : 0.0, e == 2 ? 1.0 : 0.0};
                for (int g = 0; g < ng; ++g) {
                    int c = good[g];
                    double d = t[0] * U[c] + t[1] * U[3 + c] + t[2] * U[6 + c];
                    for (int r = 0; r < 3; ++r) t[r] -= d * U[3 * r + c];
                }
                double nn = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
                if (nn > best) { best = nn; u[0] = t[0]; u[1] = t[1]; u[2] = t[2]; }
            }
        }
        double nn = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        for (int r = 0; r < 3; ++r) U[3 * r + b] = u[r] / nn;
        good[ng++] = b;
    }
}

// ---------------------------------------------------------------------------------
// Drucker-Prager projection in log-strain space (HybridSolver.cpp:632-674).
// ln: trial log singular values (in/out), q: plasticAmount (in/out).
// Returns 0 elastic, 1 apex (s = 1), 2 projected.
// the friction-angle hardening's exp and sin: FP32 takes the fast hardware forms
// (a few ulps; the cone coefficient they set enters the projection linearly)
__device__ __forceinline__ float dp_exp(float x) { return __expf(x); }
__device__ __forceinline__ double dp_exp(double x) { return exp(x); }
__device__ __forceinline__ float dp_sin(float x) { return __sinf(x); }
__device__ __forceinline__ double dp_sin(double x) { return sin(x); }

template <typename T>
__device__ __forceinline__ int dp_project(T ln[3], T& q, T h0, T h1, T h2, T h3, T k) {
    const T deg = T(3.14159265358979323846 / 180.0);
    T phi = (h0 + (h1 * q - h3) * dp_exp(-h2 * q)) * deg;
    T sphi = dp_sin(phi);
    T alpha = T(0.81649658092772603273) * T(2) * sphi / (T(3) - sphi);  // sqrt(2/3)
    T tr = ln[0] + ln[1] + ln[2];
    T dev[3] = {ln[0] - tr / T(3), ln[1] - tr / T(3), ln[2] - tr / T(3)};
    T nd = sqrt_t(dev[0] * dev[0] + dev[1] * dev[1] + dev[2] * dev[2]);
    T dg = nd + k * tr * alpha;
    if (dg <= T(0)) return 0;
    if (nd == T(0) || tr > T(0)) {
        q += sqrt_t(ln[0] * ln[0] + ln[1] * ln[1] + ln[2] * ln[2]);
        ln[0] = ln[1] = ln[2] = T(0);
        return 1;
    }
    T sc = dg / nd;
#pragma unroll
    for (int a = 0; a < 3; ++a) ln[a] -= sc * dev[a];
    q += dg;
    return 2;
}

// ---------------------------------------------------------------------------------
// level set union (LevelSet.cpp:8-42): phi = min over shapes, n of the minimiser
__device__ __forceinline__ void eval_levelset(const KParams& P, float x, float y, float z, float& phi,
                                              float n[3]) {
    phi = 3.0e38f;
    n[0] = 0.f; n[1] = 0.f; n[2] = 1.f;
    for (int i = 0; i < P.nshapes; ++i) {
        const DevShape& s = P.shapes[i];
        float ph, nx, ny, nz;
        if (s.type == kSdfPlane) {
            ph = s.p[0] * x + s.p[1] * y + s.p[2] * z - s.p[3];
            nx = s.p[0]; ny = s.p[1]; nz = s.p[2];
        } else if (s.type == kSdfSphere) {
            float dx = x - s.p[0], dy = y - s.p[1], dz = z - s.p[2];
            float r = sqrtf(dx * dx + dy * dy + dz * dz);
            ph = r - s.p[3];
            if (r > 0.f) { nx = dx / r; ny = dy / r; nz = dz / r; }
            else { nx = 0.f; ny = 0.f; nz = 1.f; }
        } else {
            float X = s.p[0], Y = s.p[1], G = s.p[2];
            ph = fminf(fminf(z - G, X - x), Y - y);
            float adz = fabsf(z - G), adx = fabsf(X - x), ady = fabsf(Y - y);
            if (adz <= adx && adz <= ady) { nx = 0.f; ny = 0.f; nz = 1.f; }
            else if (ady <= adx) { nx = 0.f; ny = -1.f; nz = 0.f; }
            else { nx = -1.f; ny = 0.f; nz = 0.f; }
        }
        if (ph < phi) { phi = ph; n[0] = nx; n[1] = ny; n[2] = nz; }
    }
}

// ---------------------------------------------------------------------------------
// classical Gram-Schmidt QR of D = [d1 d2 d3] (geometry.cpp:31-62); row-major 3x3.
__device__ __forceinline__ void gram_schmidt(const float D[9], float Q[9], float R[9]) {
    float d1[3] = {D[0], D[3], D[6]}, d2[3] = {D[1], D[4], D[7]}, d3[3] = {D[2], D[5], D[8]};
    const float r11 = sqrtf(d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]);
    float q1[3] = {d1[0] / r11, d1[1] / r11, d1[2] / r11};
    const float r12 = d2[0] * q1[0] + d2[1] * q1[1] + d2[2] * q1[2];
    float q2[3] = {d2[0] - r12 * q1[0], d2[1] - r12 * q1[1], d2[2] - r12 * q1[2]};
    const float r22 = sqrtf(q2[0] * q2[0] + q2[1] * q2[1] + q2[2] * q2[2]);
    q2[0] /= r22; q2[1] /= r22; q2[2] /= r22;
    const float r13 = d3[0] * q1[0] + d3[1] * q1[1] + d3[2] * q1[2];
    const float r23 = d3[0] * q2[0] + d3[1] * q2[1] + d3[2] * q2[2];
    float q3[3] = {d3[0] - r13 * q1[0] - r23 * q2[0], d3[1] - r13 * q1[1] - r23 * q2[1],
                   d3[2] - r13 * q1[2] - r23 * q2[2]};
    const float r33 = sqrtf(q3[0] * q3[0] + q3[1] * q3[1] + q3[2] * q3[2]);
    q3[0] /= r33; q3[1] /= r33; q3[2] /= r33;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        Q[3 * r + 0] = q1[r];
        Q[3 * r + 1] = q2[r];
        Q[3 * r + 2] = q3[r];
    }
    R[0] = r11; R[1] = r12; R[2] = r13;
    R[3] = 0.f; R[4] = r22; R[5] = r23;
    R[6] = 0.f; R[7] = 0.f; R[8] = r33;
}

// In-plane cloth forces of one element (LagrangianMesh.cpp:392-458): vertex forces
// f1, f2, f3 and invRest * P (the in-plane part of the element stress, HS:406-409).
// rest = (i11, i12, i22) of inverseR(rest in-plane R), geometry.cpp:67-73.
__device__ __forceinline__ void cloth_inplane(const float Q[9], const float R[9], const float rest[3], float mu,
                                              float lambda, float f[3][3], float ip[3]) {
    const float i11 = rest[0], i12 = rest[1], i22 = rest[2];
    const float t00 = i11 * R[0], t01 = i11 * R[1] + i12 * R[4], t11 = i22 * R[4];
    // polar rotation of the upper-triangular [[t00, t01], [0, t11]] (positive diagonal, det > 0)
    const float a = t00 + t11, c = -t01;
    const float rn = rsqrtf(a * a + c * c);
    const float cs = a * rn, sn = c * rn;
    const float J = t00 * t11;
    const float lj = lambda * (J - 1.0f);
    // P = 2 mu (Rt - rot) + lambda (J - 1) cof(Rt); cof(Rt) = [[t11, 0], [-t01, t00]]
    const float P00 = 2.0f * mu * (t00 - cs) + lj * t11;
    const float P01 = 2.0f * mu * (t01 + sn);
    const float P10 = 2.0f * mu * (-sn) - lj * t01;
    const float P11 = 2.0f * mu * (t11 - cs) + lj * t00;
    ip[0] = i11 * P00 + i12 * P10;  // (invRest P)(0,0)
    ip[1] = i11 * P01 + i12 * P11;  // (0,1)
    ip[2] = i22 * P11;              // (1,1)
    const float c2 = -(P00 * i11 + P01 * i12), c3a = -P01 * i22, c3b = -P11 * i22;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float q1 = Q[3 * r], q2 = Q[3 * r + 1];
        f[1][r] = c2 * q1;
        f[2][r] = c3a * q1 + c3b * q2;
        f[0][r] = -(f[1][r] + f[2][r]);
    }
}

// Normal/shear stress of one element (HybridSolver.cpp:389-441): V dF3 d3^T.
// w2 = third row of the rest direction matrix, (D_rest^T).col(2) at HS:427.
__device__ __forceinline__ void cloth_normal_stress(const float D[9], const float Q[9], const float R[9],
                                                    const float ip[3], const float w2[3], float shear, float stiffness,
                                                    float vol, float S[9]) {
    const float dr13 = shear * R[2], dr23 = shear * R[5];
    const float r33 = R[8];
    const float dr33 = r33 > 1.0f ? 0.0f : -stiffness * (1.0f - r33) * (1.0f - r33);
    // dR = [[ip0, ip1, dr13], [0, ip2, dr23], [0, 0, dr33]];  K = dR R^T
    const float dR[9] = {ip[0], ip[1], dr13, 0.f, ip[2], dr23, 0.f, 0.f, dr33};
    float K[9];
    mat_mul_bt(dR, R, K);
    // upper triangle of K mirrored: M(a,b) = K(min(a,b), max(a,b))
    const float M[9] = {K[0], K[1], K[2], K[1], K[4], K[5], K[2], K[5], K[8]};
    // y = R^-T w2  (forward substitution with R^T lower-triangular)
    const float y0 = w2[0] / R[0];
    const float y1 = (w2[1] - R[1] * y0) / R[4];
    const float y2 = (w2[2] - R[2] * y0 - R[5] * y1) / R[8];
    float z[3], dF3[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) z[a] = M[3 * a] * y0 + M[3 * a + 1] * y1 + M[3 * a + 2] * y2;
#pragma unroll
    for (int a = 0; a < 3; ++a) dF3[a] = Q[3 * a] * z[0] + Q[3 * a + 1] * z[1] + Q[3 * a + 2] * z[2];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) S[3 * a + b] = vol * dF3[a] * D[3 * b + 2];
}

// Cloth return mapping on the third column r = (r13, r23, r33) of the QR factor
// (HybridSolver.cpp:701-717): no tension (r33 <= 1, else r = e3) and a frictional
// cap of the shear by the normal force.
__device__ __forceinline__ void cloth_project(float r[3], float shear, float stiffness, float friction) {
    if (r[2] > 1.0f) {
        r[2] = 1.0f;
        r[0] = r[1] = 0.0f;
    } else {
        const float nf = stiffness * (r[2] - 1.0f) * (r[2] - 1.0f);
        const float sf = shear * sqrtf(r[0] * r[0] + r[1] * r[1]);
        if (sf > friction * nf) {
            const float sc = friction * nf / sf;
            r[0] *= sc;
            r[1] *= sc;
        }
    }
}

// Ratio of the friction cap to the trial shear force in cloth_project, in [0, 1]
// (1 when the shear is within the cap); the projected shear is the trial shear
// times this ratio.
__device__ __forceinline__ float cloth_cap_ratio(const float r[3], float shear, float stiffness, float friction) {
    const float nf = stiffness * (r[2] - 1.0f) * (r[2] - 1.0f);
    const float sf = shear * sqrtf(r[0] * r[0] + r[1] * r[1]);
    return sf > friction * nf ? friction * nf / sf : 1.0f;
}

// Cloth return mapping (HybridSolver.cpp:695-719): new d3 from the QR of [d1 d2 d3].
__device__ __forceinline__ void cloth_return_map(const float D[9], float shear, float stiffness, float friction,
                                                 float d3[3]) {
    float Q[9], R[9];
    gram_schmidt(D, Q, R);
    float r[3] = {R[2], R[5], R[8]};
    cloth_project(r, shear, stiffness, friction);
#pragma unroll
    for (int a = 0; a < 3; ++a) d3[a] = Q[3 * a] * r[0] + Q[3 * a + 1] * r[1] + Q[3 * a + 2] * r[2];
}

__device__ __forceinline__ unsigned long long to_fixed(float v, float scale) {
    return (unsigned long long)__float2ll_rn(v * scale);
}

}  // namespace aep
