// aep_kernels.cu -- the sm_103a kernels of one MPM step.
//
// Step dataflow (reference order HybridSolver.cpp:867-989, rotated so the
// P2G of :987 comes first):
//   sort (by padded base-node block, then base node)         -> perm
//   k_p2g        mass + APIC momentum scatter  (HS:113-240)
//   k_normalize  v_i = p_i / m_i               (HS:233-240)
//   k_force      gather grad v, SVD, stress, impulse scatter (HS:252-366, 457)
//   k_grid       v += impulse/m + dt g, level-set collision  (HS:725-737, 460-511)
//   k_g2p        G2P velocity, APIC, advection, F update, return mapping
//                (HS:739-825, 940-951, 553-577, 612-681)
//
// Scatter design (P2G and force): particles are ordered so that all particles
// with the same stencil base node are contiguous.  A warp streams through a
// chunk of ordered particles; lane l owns the stencil column (l&3, (l>>2)&3)
// and accumulates its nodes' contributions in FP32 registers in a fixed
// particle order.  When the base node changes, the lanes convert their sums to
// int64 fixed point and add them to the grid with 64-bit atomics.  Integer
// addition is associative, so the grid sums are order-independent and the step
// repeats bit-for-bit.  Same-node contributions of all particles that share a
// base node are merged in registers before any atomic (one atomic per node per
// run instead of one per particle).  The run structure of each batch of 32
// particles comes from comparing each lane's key with the previous lane's
// (__shfl_up_sync) and a __ballot_sync of the run heads: on ordered keys that
// is the grouping __match_any_sync would give, at the cost of one shuffle.
#include <algorithm>
#include <utility>

#include <cooperative_groups.h>

#include "aep_device.cuh"
#include "aep_kernels.h"
#include "aep_mlp.cuh"

namespace cg = cooperative_groups;

namespace aep {

// ===================================================================================
// keys of the current particle order (after an upload)
__global__ void k_keys(KParams P, PArrays cur, int n, uint32_t* keys, DevStats* st) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int cell[3];
    float f[3];
    bool clamped = locate(P, cur.x[0][j], cur.x[1][j], cur.x[2][j], cell, f);
    keys[j] = make_key(P, cell);
    if (clamped) atomicAdd(&st->out_of_domain, 1ull);
}

// ===================================================================================
// P2G: mass and APIC momentum (HybridSolver.cpp:113-231).
// momentum contribution of particle p to node o:  w m (v + D^-1 B (x_i - x_p)),
// D^-1 = 3/h^2 (:177), x_i - x_p = (o - 1 - f) h  =>  w (b + Mh o) with
// Mh[:,a] = m D^-1 h_a B[:,a] and b = m v - Mh (1 + f).
constexpr int kP2GThreads = 128;
// the P2G grid tile: 3 x 2 x 2 node blocks from the node block of the thread
// block's first particle (the particles are ordered by node block, x fastest: a
// block's 512 particles mostly sit in two x-adjacent node blocks, whose stencils
// the tile holds)
constexpr int kP2GTileBx = 3;
constexpr int kP2GTileNodes = kP2GTileBx * 2 * 2 * 64;
constexpr int kP2GMaxChunk = 128;  // particles per warp at most (the launch picks the chunk)
// Prep record of one particle, 9 float4 (36 words, 16-byte aligned):
//   q0 = (b, m)  q1 = Mh[0..3]  q2 = Mh[4..7]  q3 = (Mh[8], T lo, T hi, -)
//   q4 = wx  q5 = wy  q6 = wz  q7 = (base, key)
// A lane writes its own record with 128-bit stores; a stride of 36 words puts
// the 8 lanes of each store wavefront on distinct banks; the whole warp then
// reads one record at a time (broadcast).
constexpr int kP2GRec = 9;
constexpr int kP2GRegion = 32 * kP2GRec;  // float4 per warp region
__device__ __forceinline__ void mark_blocks(const KParams& P, const GArrays& G, uint32_t key) {
    uint32_t blk = key >> 6;
    int bx = (int)(blk % (uint32_t)P.nb[0]);
    uint32_t r = blk / (uint32_t)P.nb[0];
    int by = (int)(r % (uint32_t)P.nb[1]);
    int bz = (int)(r / (uint32_t)P.nb[1]);
#pragma unroll
    for (int d = 0; d < 8; ++d) {
        int x = bx + (d & 1), y = by + ((d >> 1) & 1), z = bz + (d >> 2);
        uint32_t nb = (uint32_t)((z * P.nb[1] + y) * P.nb[0] + x);
        if (atomicExch(&G.flag[nb], 1u) == 0u) {
            int slot = atomicAdd(G.nactive, 1);
            G.active[slot] = (int32_t)nb;
        }
    }
}

// One warp streams through a chunk of ordered particles (32 to 128: the particles
// spread evenly over the fewest waves of resident warps) run by run (a run: consecutive
// particles with the same base node): lane (l & 15) owns the stencil column
// (ox, oy) = (l & 3, (l >> 2) & 3), and the half h = l >> 4 takes the run's particles
// t + h, t + h + 2, ..., accumulating the column's 4 nodes x (mass, momentum) in
// FP32 registers.  At the end of a run (warp-uniform) the halves' sums are added,
// half h takes the z-layers 2h, 2h + 1, and the node sums are rounded to fixed
// point and added as integers: runs whose stencil lies in the block's grid tile
// (3 x 2 x 2 node blocks from the node block of its first particle, which holds the
// stencils of that node block's particles and of the next one's in x: ~91% of the
// runs on the sand + cloth scene, against ~68% for the 2 x 2 x 2 blocks of the
// middle particle) into a fixed-point copy of the tile in shared memory, which is
// added to the grid once per node at the end; other runs into the grid directly.
// Integer sums: the result does not depend on the order.
// Exact mass: rounding the node masses one by one loses the difference between
// a run's exact fixed-point particle mass T = sum_p T_p and the sum S of its
// rounded node masses; the run adds T - S to its stencil node (1,1,1), which
// always exists, so the grid mass is sum_p T_p exactly and is conserved bit for
// bit from step to step.  T - S is far below 2^31 (FP32 weight-sum error and
// roundings), so it is computed from the low 32 bits of T and of the node masses
// with one 32-bit warp reduction.
__global__ void __launch_bounds__(kP2GThreads) k_p2g(KParams P, PArrays cur, const uint32_t* __restrict__ keys,
                                                     const int32_t* __restrict__ perm, int n, int chunk, GArrays G,
                                                     int32_t* __restrict__ slot_of, int32_t* __restrict__ curidx_of) {
    pdl_trigger();  // the normalisation may launch once every block has started
    __shared__ float4 sm4[(kP2GThreads / 32) * kP2GRegion];
    __shared__ unsigned long long tacc[4 * kP2GTileNodes];  // [channel][tile node]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* const region = sm4 + warp * kP2GRegion;
    const int half = lane >> 4, ox = lane & 3, oy = (lane >> 2) & 3;
    const long blk0 = (long)blockIdx.x * (kP2GThreads / 32) * chunk;
    const long chunk0 = blk0 + (long)warp * chunk;
    const int cnt_total = (int)max(0L, min((long)chunk, (long)n - chunk0));  // warp-uniform
    // the tile's origin: the node block of the block's first particle
    int org[3];
    tile_origin(P, keys[min(blk0, (long)n - 1)], org);
    for (int i = threadIdx.x; i < 4 * kP2GTileNodes; i += kP2GThreads) tacc[i] = 0ull;
    __syncthreads();

    float am[4] = {0, 0, 0, 0}, ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0}, az[4] = {0, 0, 0, 0};
    uint32_t run_key = kInvalidKey;
    int rb[3] = {0, 0, 0};
    long long run_T = 0;
    auto flush = [&]() {  // warp-uniform
        if (run_key == kInvalidKey) return;
        // the two halves' sums added; half h then adds z-layers 2h, 2h + 1
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) {
            am[oz] += __shfl_xor_sync(0xffffffffu, am[oz], 16);
            ax[oz] += __shfl_xor_sync(0xffffffffu, ax[oz], 16);
            ay[oz] += __shfl_xor_sync(0xffffffffu, ay[oz], 16);
            az[oz] += __shfl_xor_sync(0xffffffffu, az[oz], 16);
        }
        run_T += __shfl_xor_sync(0xffffffffu, run_T, 16);
        float gm[2], gx[2], gy[2], gz[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            gm[k] = half ? am[2 + k] : am[k];
            gx[k] = half ? ax[2 + k] : ax[k];
            gy[k] = half ? ay[2 + k] : ay[k];
            gz[k] = half ? az[2 + k] : az[k];
        }
        long long mf[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) mf[k] = __float2ll_rn(gm[k] * P.mass_scale);
        const unsigned s_lo = __reduce_add_sync(0xffffffffu, (unsigned)mf[0] + (unsigned)mf[1]);
        if (lane == 5) mf[1] += (long long)(int)((unsigned)run_T - s_lo);  // (ox, oy, oz) = (1, 1, 1)
        const int x = rb[0] + ox, y = rb[1] + oy;
        const int rbx = (rb[0] >> 2) - org[0];
        if (rbx >= 0 && rbx < kP2GTileBx - 1 && (rb[1] >> 2) == org[1] && (rb[2] >> 2) == org[2]) {
            // the run's stencil (base .. base + 3) lies in the tile: node blocks
            // org.x + rbx, org.x + rbx + 1 in x, org.y, org.y + 1, org.z, org.z + 1
            const int tx = x - 4 * org[0], ty = y - 4 * org[1];
            const int txy = (tx >> 2) * 64 + (tx & 3) + (ty >> 2) * (64 * kP2GTileBx) + ((ty & 3) << 2);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (mf[k] != 0) {
                    const int tz = rb[2] + 2 * half + k - 4 * org[2];
                    unsigned long long* a = tacc + txy + (tz >> 2) * (128 * kP2GTileBx) + ((tz & 3) << 4);
                    atomicAdd(a, (unsigned long long)mf[k]);
                    atomicAdd(a + kP2GTileNodes, to_fixed(gx[k], P.mom_scale));
                    atomicAdd(a + 2 * kP2GTileNodes, to_fixed(gy[k], P.mom_scale));
                    atomicAdd(a + 3 * kP2GTileNodes, to_fixed(gz[k], P.mom_scale));
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (mf[k] != 0) {
                    unsigned long long* a = G.acc + 4ull * node_index(P, x, y, rb[2] + 2 * half + k);
                    atomicAdd(a + 0, (unsigned long long)mf[k]);
                    atomicAdd(a + 1, to_fixed(gx[k], P.mom_scale));
                    atomicAdd(a + 2, to_fixed(gy[k], P.mom_scale));
                    atomicAdd(a + 3, to_fixed(gz[k], P.mom_scale));
                }
            }
        }
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) am[oz] = ax[oz] = ay[oz] = az[oz] = 0.0f;
        run_T = 0;
    };

    for (int b0 = 0; b0 < cnt_total; b0 += 32) {
        const long j = chunk0 + b0 + lane;
        uint32_t my_key = kInvalidKey;
        const int pj_cur = b0 + lane < cnt_total ? perm[j] : 0;
        float xs_[16];  // the batch's particle state: x, m, v, B
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            xs_[a] = cur.x[a][pj_cur];
            xs_[4 + a] = cur.v[a][pj_cur];
        }
        xs_[3] = cur.m[pj_cur];
#pragma unroll
        for (int k = 0; k < 9; ++k) xs_[7 + k] = cur.B[k][pj_cur];
        if (b0 + lane < cnt_total) {
            const uint32_t key = keys[j];
            if (j == 0 || (keys[j - 1] >> 6) != (key >> 6)) mark_blocks(P, G, key);
            const int pj = pj_cur;
            if (slot_of) {  // a mesh is present: where each id sits in this step's order
                const int id = cur.id[pj];
                slot_of[id] = (int32_t)j;
                curidx_of[id] = pj;
            }
            float xp[3] = {xs_[0], xs_[1], xs_[2]};
            float m = xs_[3];
            int cell[3];
            float f[3], w[3][4], dw[3][4];
            locate(P, xp[0], xp[1], xp[2], cell, f);
            const bool trunc = particle_weights(P, cell, f, w, dw);
            // exact fixed-point mass; a stencil cut by the grid boundary keeps only
            // the weight inside the grid (HS:44-46), as the reference does
            float wsum = 1.0f;
            if (trunc)
                wsum = (w[0][0] + w[0][1] + w[0][2] + w[0][3]) * (w[1][0] + w[1][1] + w[1][2] + w[1][3]) *
                       (w[2][0] + w[2][1] + w[2][2] + w[2][3]);
            const long long T = __float2ll_rn(m * wsum * P.mass_scale);
            float Mh[9], b[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                float t = m * xs_[4 + a];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float mh = m * P.apic[c] * xs_[7 + 3 * a + c];
                    Mh[3 * a + c] = mh;
                    t -= mh * (1.0f + f[c]);
                }
                b[a] = t;
            }
            float4* r = region + lane * kP2GRec;
            r[0] = make_float4(b[0], b[1], b[2], m);
            r[1] = make_float4(Mh[0], Mh[1], Mh[2], Mh[3]);
            r[2] = make_float4(Mh[4], Mh[5], Mh[6], Mh[7]);
            r[3] = make_float4(Mh[8], __int_as_float((int)(unsigned)(T & 0xffffffffll)), __int_as_float((int)(T >> 32)),
                               0.0f);
            r[4] = make_float4(w[0][0], w[0][1], w[0][2], w[0][3]);
            r[5] = make_float4(w[1][0], w[1][1], w[1][2], w[1][3]);
            r[6] = make_float4(w[2][0], w[2][1], w[2][2], w[2][3]);
            r[7] = make_float4(__int_as_float(cell[0] + 3), __int_as_float(cell[1] + 3), __int_as_float(cell[2] + 3),
                               __uint_as_float(key));
            my_key = key;
        }
        // run heads: a particle whose key differs from the previous one's (any order)
        const uint32_t before = __shfl_up_sync(0xffffffffu, my_key, 1);
        const unsigned heads = __ballot_sync(0xffffffffu, my_key != (lane == 0 ? run_key : before));
        __syncwarp();
        const int cnt = min(32, cnt_total - b0);
        // run by run: half h takes the run's particles t + h, t + h + 2, ...
        for (int t = 0; t < cnt;) {
            if ((heads >> t) & 1u) {
                flush();
                const float4 q7 = region[t * kP2GRec + 7];
                run_key = __float_as_uint(q7.w);
                rb[0] = __float_as_int(q7.x); rb[1] = __float_as_int(q7.y); rb[2] = __float_as_int(q7.z);
            }
            const unsigned after = heads & ~((2u << t) - 1u);  // heads after t (none for t = 31)
            const int e = min(cnt, after ? __ffs(after) - 1 : 32);
            for (int i = t + half; i < e; i += 2) {
                const float4* r = region + i * kP2GRec;
                const float4 q0 = r[0], q1 = r[1], q2 = r[2], q3 = r[3], q6 = r[6];
                const float wxo = reinterpret_cast<const float*>(r + 4)[ox];
                const float wyo = reinterpret_cast<const float*>(r + 5)[oy];
                run_T += (long long)(((unsigned long long)(unsigned)__float_as_int(q3.z) << 32) |
                                     (unsigned long long)(unsigned)__float_as_int(q3.y));
                const float wxy = wxo * wyo;
                const float fx = (float)ox, fy = (float)oy;
                // Mh row-major: row a = (Mh[3a], Mh[3a+1], Mh[3a+2])
                float tx = q0.x + q1.x * fx + q1.y * fy;
                float ty = q0.y + q1.w * fx + q2.x * fy;
                float tz = q0.z + q2.z * fx + q2.w * fy;
                const float wz[4] = {q6.x, q6.y, q6.z, q6.w};
#pragma unroll
                for (int oz = 0; oz < 4; ++oz) {
                    const float w = wxy * wz[oz];
                    am[oz] = fmaf(w, q0.w, am[oz]);
                    ax[oz] = fmaf(w, tx, ax[oz]);
                    ay[oz] = fmaf(w, ty, ay[oz]);
                    az[oz] = fmaf(w, tz, az[oz]);
                    tx += q1.z;
                    ty += q2.y;
                    tz += q3.x;
                }
            }
            t = e;
        }
        __syncwarp();
    }
    flush();
    __syncthreads();
    // the tile into the grid, one atomic per nonzero node and channel
    for (int i = threadIdx.x; i < kP2GTileNodes; i += kP2GThreads) {
        const int t = i >> 6;  // tile block (bx, by, bz) = (t % 3, (t / 3) % 2, t / 6)
        const int bx = t % kP2GTileBx, by = (t / kP2GTileBx) & 1, bz = t / (2 * kP2GTileBx);
        if (org[0] + bx >= P.nb[0]) continue;  // past the padded grid: nothing was added there
        const uint32_t gblk = (uint32_t)(((org[2] + bz) * P.nb[1] + org[1] + by) * P.nb[0] + org[0] + bx);
        unsigned long long* a = G.acc + 4ull * ((gblk << 6) | (uint32_t)(i & 63));
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const unsigned long long v = tacc[c * kP2GTileNodes + i];
            if (v != 0ull) atomicAdd(a + c, v);
        }
    }
}

// ===================================================================================
// v_i = p_i / m_i on touched nodes (HybridSolver.cpp:233-240); clears the accumulators
// for the force impulse; exact int64 totals of mass and momentum (summed per block,
// one atomic per block and total).  Launched with 256 threads.
__global__ void __launch_bounds__(256) k_normalize(KParams P, GArrays G, DevStats* st) {
    pdl_entry();
    __shared__ long long red[5][8];
    const int nact = *G.nactive;
    const long total = (long)nact * 64;
    if ((long)blockIdx.x * blockDim.x >= total) return;  // no node for this block (block-uniform)
    long long sm_ = 0, sx = 0, sy = 0, sz = 0;
    unsigned long long cnt = 0;
    bool ovf = false;
    float vmax = 0.0f;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        uint32_t node = ((uint32_t)G.active[i >> 6] << 6) | (uint32_t)(i & 63);
        longlong2* a2 = reinterpret_cast<longlong2*>(G.acc + 4ull * node);
        longlong2 a = a2[0], b = a2[1];
        float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
        if (a.x > 0) {
            ++cnt;
            float m = __ll2float_rn(a.x) * P.inv_mass_scale;
            float inv = 1.0f / m;
            out = make_float4(__ll2float_rn(a.y) * P.inv_mom_scale * inv, __ll2float_rn(b.x) * P.inv_mom_scale * inv,
                              __ll2float_rn(b.y) * P.inv_mom_scale * inv, m);
            vmax = fmaxf(vmax, out.x * out.x + out.y * out.y + out.z * out.z);
        }
        const long long lim = 1ll << 61;
        ovf |= (a.x > lim) | (a.y > lim) | (a.y < -lim) | (b.x > lim) | (b.x < -lim) | (b.y > lim) | (b.y < -lim);
        G.vel[node] = out;
        a2[0] = make_longlong2(0, 0);
        a2[1] = make_longlong2(0, 0);
        sm_ += a.x; sx += a.y; sy += b.x; sz += b.y;
    }
    if (P.vmax2) warp_max_atomic(P.vmax2 + 0, vmax);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sm_ += __shfl_xor_sync(0xffffffffu, sm_, o);
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = (long long)cnt;
        red[1][w] = sm_;
        red[2][w] = sx;
        red[3][w] = sy;
        red[4][w] = sz;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        long long t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[threadIdx.x][k];
        unsigned long long* dst[5] = {&st->nodes, &st->mass, &st->mom[0], &st->mom[1], &st->mom[2]};
        if (t) atomicAdd(dst[threadIdx.x], (unsigned long long)t);
    }
    if (ovf) atomicOr(&st->overflow, 1ull);
}

// ===================================================================================
// per-particle stress of HybridSolver.cpp:277-352, times -dt (the impulse kernel)
template <typename T>
__device__ __forceinline__ void stress_from_svd(const KParams& P, int mat, const T Fh[9], const T F[9], const T U[9],
                                                const T s[3], const T V[9], T Jp, T vol, T out[9]) {
    T A[9];
    if (mat == kSnow) {
        T hard = exp_t(T(P.snow_xi) * (T(1) - Jp));
        T mu = T(P.snow_mu) * hard, lambda = T(P.snow_lambda) * hard;
        T R[9], C[9];
        mat_mul_bt(U, V, R);  // U V^T
        mat_cofactor(Fh, C);
        T J = mat_det(Fh);
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = T(2) * mu * (Fh[k] - R[k]) + lambda * (J - T(1)) * C[k];
    } else {
        T mu = T(P.sand_mu), lambda = T(P.sand_lambda);
        T ln[3] = {log_t(s[0]), log_t(s[1]), log_t(s[2])};
        T tr = ln[0] + ln[1] + ln[2];
        T d[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) d[a] = (T(2) * mu * ln[a] + lambda * tr) / s[a];
        T UD[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) UD[3 * r + c] = U[3 * r + c] * d[c];
        mat_mul_bt(UD, V, A);
    }
    T st[9];
    mat_mul_bt(A, F, st);  // * F_E^T
#pragma unroll
    for (int k = 0; k < 9; ++k) out[k] = vol * st[k];
}

constexpr int kFrcThreads = 128;
// Force prep record of one particle, 11 float4 (44 words):
//   q0..q2 = S[0..8] (-dt vol P F^T, row-major) + pad   q3 = wx  q4 = wy  q5 = wz
//   q6 = dwx  q7 = dwy  q8 = dwz  q9 = (base, key)  q10 unused
// 44-word stride: conflict-free 128-bit stores; the second half-warp's records are
// skewed by one float4 so both halves reading slot i hit different banks.
constexpr int kFrcRec = 11;
constexpr int kFrcWarpBuf = 32 * kFrcRec + 1;
__device__ __forceinline__ int frc_slot(int p) { return p * kFrcRec + (p >= 16 ? 1 : 0); }

// The FP32 stress impulse of one particle; a near-degenerate F-hat (a singular
// value under 2% of the largest) gives S = 0 here and the particle is listed for
// k_force_fp64, which redoes it in FP64 and scatters it on its own (keeping the
// FP64 code, and its registers, out of k_force).
// vel: the grid velocities (global) or the block's tile; X, Y, Z the stencil
// offsets into it; w, dw the particle's weights
// F_E, the plastic scalar and the volume of the particle come from the caller's
// shared-memory copies (sF[k][t], sq[t], svol[t]: copied while the grid tile loads)
__device__ void particle_stress_impulse(const KParams& P, const float4* vel, const uint32_t X[4], const uint32_t Y[4],
                                        const uint32_t Z[4], const PArrays& cur, int pj, int mat, const float* sF,
                                        int t, int tstride, float q_in, float vol, float dt_force, float S[9],
                                        const float w[3][4], const float dw[3][4], DevStats* st, int32_t* fp64_list,
                                        int fp64_cap) {
    // velocity gradient of the P2G velocity (the three SpMVs of HS:269-271),
    // contracted one axis at a time: Gm = sum v (grad w)^T with
    // grad w = (dwx wy wz, wx dwy wz, wx wy dwz)
    float Gm[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int oy = 0; oy < 4; ++oy) {
        float Bd[3] = {0, 0, 0}, Bw[3] = {0, 0, 0}, Bz[3] = {0, 0, 0};
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) {
            const uint32_t yz = Y[oy] + Z[oz];
            float Ad[3] = {0, 0, 0}, Aw[3] = {0, 0, 0};
#pragma unroll
            for (int ox = 0; ox < 4; ++ox) {
                const float4 v = vel[yz + X[ox]];
                const float a = w[0][ox], d = dw[0][ox];
                Ad[0] = fmaf(d, v.x, Ad[0]); Ad[1] = fmaf(d, v.y, Ad[1]); Ad[2] = fmaf(d, v.z, Ad[2]);
                Aw[0] = fmaf(a, v.x, Aw[0]); Aw[1] = fmaf(a, v.y, Aw[1]); Aw[2] = fmaf(a, v.z, Aw[2]);
            }
            const float cz = w[2][oz], dz = dw[2][oz];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                Bd[c] = fmaf(cz, Ad[c], Bd[c]);
                Bw[c] = fmaf(cz, Aw[c], Bw[c]);
                Bz[c] = fmaf(dz, Aw[c], Bz[c]);
            }
        }
        const float cy = w[1][oy], dy = dw[1][oy];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            Gm[3 * c + 0] = fmaf(cy, Bd[c], Gm[3 * c + 0]);
            Gm[3 * c + 1] = fmaf(dy, Bw[c], Gm[3 * c + 1]);
            Gm[3 * c + 2] = fmaf(cy, Bz[c], Gm[3 * c + 2]);
        }
    }
    float F[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) F[k] = sF[k * tstride + t];
    float GF[9], Fh[9];
    mat_mul(Gm, F, GF);
#pragma unroll
    for (int k = 0; k < 9; ++k) Fh[k] = F[k] + dt_force * GF[k];  // EDG + EDG_modifier * EDG (:306)
    float Jp = 1.0f;
    if (mat == kSnow) {
        if (P.track_fp) {
            float Fp[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) Fp[k] = cur.Fp[k][pj];
            Jp = mat_det(Fp);
        } else {
            Jp = q_in;
        }
    }
    float U[9], s[3], V[9];
    bool ok = svd3<float>(Fh, U, s, V, 8, 1e-7f, 2e-2f);
    float out[9];
    if (ok) {
        stress_from_svd<float>(P, mat, Fh, F, U, s, V, Jp, vol, out);
    } else {
        const unsigned k = atomicAdd(&st->force_fp64, 1u);
        if ((int)k < fp64_cap) fp64_list[k] = pj;
#pragma unroll
        for (int k2 = 0; k2 < 9; ++k2) out[k2] = 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) S[k] = -dt_force * out[k];
}

// FP64 stress impulses of the particles k_force listed, each scattered to its 64
// stencil nodes with its own fixed-point atomics (integer sums: the order does
// not matter).  Grid-stride over the list; usually empty.
__global__ void k_force_fp64(KParams P, PArrays cur, GArrays G, float dt_force, DevStats* st,
                             const int32_t* __restrict__ fp64_list, int fp64_cap) {
    pdl_entry();
    dt_force = step_dt(P, dt_force, 0);
    const int count = min((int)st->force_fp64, fp64_cap);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x) {
        const int pj = fp64_list[q];
        float f[3], w[3][4], dw[3][4];
        int cell[3];
        locate(P, cur.x[0][pj], cur.x[1][pj], cur.x[2][pj], cell, f);
        particle_weights(P, cell, f, w, dw);
        int base[3] = {cell[0] + 3, cell[1] + 3, cell[2] + 3};
        uint32_t X[4], Y[4], Z[4];
        stencil_offsets(P, base, X, Y, Z);
        float Gm[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // grad v (HS:269-271), as in particle_stress_impulse
        for (int oz = 0; oz < 4; ++oz)
            for (int oy = 0; oy < 4; ++oy)
                for (int ox = 0; ox < 4; ++ox) {
                    const float4 v = __ldg(&G.vel[Y[oy] + Z[oz] + X[ox]]);
                    const float g[3] = {dw[0][ox] * w[1][oy] * w[2][oz], w[0][ox] * dw[1][oy] * w[2][oz],
                                        w[0][ox] * w[1][oy] * dw[2][oz]};
                    const float vv[3] = {v.x, v.y, v.z};
                    for (int c = 0; c < 3; ++c)
                        for (int b = 0; b < 3; ++b) Gm[3 * c + b] = fmaf(vv[c], g[b], Gm[3 * c + b]);
                }
        float F[9], GF[9], Fh[9];
        for (int k = 0; k < 9; ++k) F[k] = cur.F[k][pj];
        mat_mul(Gm, F, GF);
        for (int k = 0; k < 9; ++k) Fh[k] = F[k] + dt_force * GF[k];
        const int mat = cur.mat[pj];
        float Jp = 1.0f;
        if (mat == kSnow) {
            if (P.track_fp) {
                float Fp[9];
                for (int k = 0; k < 9; ++k) Fp[k] = cur.Fp[k][pj];
                Jp = mat_det(Fp);
            } else {
                Jp = cur.plastic[pj];
            }
        }
        double Fd[9], Fhd[9], Ud[9], sd[3], Vd[9], od[9];
        for (int k = 0; k < 9; ++k) { Fd[k] = F[k]; Fhd[k] = Fh[k]; }
        svd3<double>(Fhd, Ud, sd, Vd, 40, 1e-15, 0.0);
        svd3_complete(Ud, sd);
        stress_from_svd<double>(P, mat, Fhd, Fd, Ud, sd, Vd, (double)Jp, (double)cur.vol[pj], od);
        float S[9];
        for (int k = 0; k < 9; ++k) S[k] = -dt_force * (float)od[k];
        for (int oz = 0; oz < 4; ++oz)
            for (int oy = 0; oy < 4; ++oy)
                for (int ox = 0; ox < 4; ++ox) {
                    const float g[3] = {dw[0][ox] * w[1][oy] * w[2][oz], w[0][ox] * dw[1][oy] * w[2][oz],
                                        w[0][ox] * w[1][oy] * dw[2][oz]};
                    if (g[0] == 0.0f && g[1] == 0.0f && g[2] == 0.0f) continue;
                    unsigned long long* a = G.acc + 4ull * node_index(P, base[0] + ox, base[1] + oy, base[2] + oz);
                    for (int c = 0; c < 3; ++c) {
                        const float fc = S[3 * c] * g[0] + S[3 * c + 1] * g[1] + S[3 * c + 2] * g[2];
                        atomicAdd(a + 1 + c, to_fixed(fc, P.mom_scale));
                    }
                }
        atomicAdd(&st->fallbacks, 1ull);
    }
}

// impulse scatter: f_i -= sum_p stress_p grad w_ip (HS:356-366), stored as dt * f_i
__global__ void __launch_bounds__(kFrcThreads, 6) k_force(KParams P, PArrays cur, const uint32_t* __restrict__ keys,
                                                       const int32_t* __restrict__ perm, int n, GArrays G,
                                                       float dt_force, DevStats* st, MeshArrays M,
                                                       int32_t* fp64_list, int fp64_cap) {
    pdl_entry();
    __shared__ float4 sm4[(kFrcThreads / 32) * kFrcWarpBuf];
    __shared__ float4 tile_v[kTileNodes];
    dt_force = step_dt(P, dt_force, 0);
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* const buf = sm4 + wid * kFrcWarpBuf;
    const long chunk0 = ((long)blockIdx.x * (kFrcThreads / 32) + wid) * 32;
    const long j = chunk0 + lane;
    int org[3];
    tile_origin(P, keys[(long)blockIdx.x * kFrcThreads], org);
    load_tile(P, org, G.vel, nullptr, tile_v, nullptr);
    // the particle's own loads and weights overlap the tile copy
    const bool live = j < n;
    const int pj = live ? perm[j] : 0;
    const int mat = live ? (int)cur.mat[pj] : 0;
    // a particle's F_E, plastic scalar and volume are copied to shared memory while
    // the tile loads (each thread reads back only its own entries)
    __shared__ float sF[9][kFrcThreads], sq[kFrcThreads], svol[kFrcThreads];
    if (live && mat <= kSand) {
#pragma unroll
        for (int k = 0; k < 9; ++k) cp_async4(&sF[k][threadIdx.x], &cur.F[k][pj]);
        cp_async4(&sq[threadIdx.x], &cur.plastic[pj]);
        cp_async4(&svol[threadIdx.x], &cur.vol[pj]);
        cp_async_commit();
    }
    int cell[3];
    float w[3][4], dw[3][4];
    uint32_t X[4], Y[4], Z[4];
    bool in_tile = false;
    {
        float f[3];
        locate(P, cur.x[0][pj], cur.x[1][pj], cur.x[2][pj], cell, f);
        particle_weights(P, cell, f, w, dw);
        const int base[3] = {cell[0] + 3, cell[1] + 3, cell[2] + 3};
        in_tile = tile_offsets(base, org, X, Y, Z);
        if (!in_tile) stencil_offsets(P, base, X, Y, Z);
    }
    __syncthreads();
    if (chunk0 >= n) return;
    uint32_t my_key = kInvalidKey;
    if (live) {
        float S[9];
        float av[3] = {0.f, 0.f, 0.f};  // w-weighted impulse (cloth vertices)
        if (mat <= kSand) {
            cp_async_wait_all();
            particle_stress_impulse(P, in_tile ? tile_v : G.vel, X, Y, Z, cur, pj, mat, &sF[0][0], threadIdx.x,
                                    kFrcThreads, sq[threadIdx.x], svol[threadIdx.x], dt_force, S, w, dw, st, fp64_list,
                                    fp64_cap);
        } else {
            const int id = cur.id[pj];
            if (mat == kClothVertex) {
                // rg.forces += vertexOmegas^T vertexInPlaneForces (HS:376-378)
                unsigned long long* vf = M.vforce + 3ull * (id - M.vbase);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    av[c] = __ll2float_rn((long long)vf[c]) * P.inv_mom_scale;
                    vf[c] = 0ull;
                }
#pragma unroll
                for (int k = 0; k < 9; ++k) S[k] = 0.f;
            } else {
                // element normal stress scattered with the element weight gradients (HS:444-454)
                const float* es = M.estress + 9ull * (id - M.ebase);
#pragma unroll
                for (int k = 0; k < 9; ++k) S[k] = es[k];
            }
        }
        float4* r = buf + frc_slot(lane);
        r[0] = make_float4(S[0], S[1], S[2], S[3]);
        r[1] = make_float4(S[4], S[5], S[6], S[7]);
        r[2] = make_float4(S[8], 0.f, 0.f, 0.f);
        r[3] = make_float4(w[0][0], w[0][1], w[0][2], w[0][3]);
        r[4] = make_float4(w[1][0], w[1][1], w[1][2], w[1][3]);
        r[5] = make_float4(w[2][0], w[2][1], w[2][2], w[2][3]);
        r[6] = make_float4(dw[0][0], dw[0][1], dw[0][2], dw[0][3]);
        r[7] = make_float4(dw[1][0], dw[1][1], dw[1][2], dw[1][3]);
        r[8] = make_float4(dw[2][0], dw[2][1], dw[2][2], dw[2][3]);
        my_key = keys[j];
        r[9] = make_float4(__int_as_float(cell[0] + 3), __int_as_float(cell[1] + 3), __int_as_float(cell[2] + 3),
                           __uint_as_float(my_key));
        r[10] = make_float4(av[0], av[1], av[2], mat == kClothVertex ? 1.0f : 0.0f);
    }
    __syncwarp();
    // stream the warp's particles run by run (a run: consecutive particles with the
    // same base node); half h takes the run's particles t + h, t + h + 2, ... and
    // both halves accumulate all 4 z-layers of the lane's stencil column (ox, oy);
    // at the end of the run (warp-uniform) the halves are added and half h adds
    // z-layers 2h, 2h + 1 to the grid
    const int h = lane >> 4, l = lane & 15, ox = l & 3, oy = l >> 2;
    const int cnt = (int)max(0l, min(32l, (long)n - chunk0));
    float fx[4] = {0, 0, 0, 0}, fy[4] = {0, 0, 0, 0}, fz[4] = {0, 0, 0, 0};
    // run heads: a particle whose key differs from the previous one's (any order)
    const uint32_t key_before = __shfl_up_sync(0xffffffffu, my_key, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || my_key != key_before);
    for (int t = 0; t < cnt;) {
        const unsigned after = heads & ~((2u << t) - 1u);  // heads after t (none for t = 31)
        const int e = min(cnt, after ? __ffs(after) - 1 : 32);
        const float4 q9 = (buf + frc_slot(t))[9];
        const int rb[3] = {__float_as_int(q9.x), __float_as_int(q9.y), __float_as_int(q9.z)};
        for (int i = t + h; i < e; i += 2) {
            const float4* r = buf + frc_slot(i);
            const float4 q0 = r[0], q1 = r[1], q2 = r[2], q5 = r[5], q8 = r[8];
            const float wxo = reinterpret_cast<const float*>(r + 3)[ox];
            const float wyo = reinterpret_cast<const float*>(r + 4)[oy];
            const float dxo = reinterpret_cast<const float*>(r + 6)[ox];
            const float dyo = reinterpret_cast<const float*>(r + 7)[oy];
            // grad w = (dwx wy wz, wx dwy wz, wx wy dwz); S g = wz (p1 S[:,0] + p2 S[:,1]) + dwz p3 S[:,2]
            // S row-major: S[3a+b] -> q0=(S0,S1,S2,S3) q1=(S4,S5,S6,S7) q2.x=S8
            const float p1 = dxo * wyo, p2 = wxo * dyo, p3 = wxo * wyo;
            const float ax_ = p1 * q0.x + p2 * q0.y, ay_ = p1 * q0.w + p2 * q1.x, az_ = p1 * q1.z + p2 * q1.w;
            const float cx = p3 * q0.z, cy = p3 * q1.y, cz = p3 * q2.x;
            const float wz4[4] = {q5.x, q5.y, q5.z, q5.w}, dz4[4] = {q8.x, q8.y, q8.z, q8.w};
#pragma unroll
            for (int oz = 0; oz < 4; ++oz) {
                fx[oz] = fmaf(wz4[oz], ax_, fmaf(dz4[oz], cx, fx[oz]));
                fy[oz] = fmaf(wz4[oz], ay_, fmaf(dz4[oz], cy, fy[oz]));
                fz[oz] = fmaf(wz4[oz], az_, fmaf(dz4[oz], cz, fz[oz]));
            }
            const float4 q10 = r[10];
            if (q10.w != 0.0f) {  // cloth vertex: + w f_v
                const float wx_ = p3 * q10.x, wy_ = p3 * q10.y, wz_ = p3 * q10.z;
#pragma unroll
                for (int oz = 0; oz < 4; ++oz) {
                    fx[oz] = fmaf(wz4[oz], wx_, fx[oz]);
                    fy[oz] = fmaf(wz4[oz], wy_, fy[oz]);
                    fz[oz] = fmaf(wz4[oz], wz_, fz[oz]);
                }
            }
        }
        // the run's sums: the two halves added, then z-layers 2h, 2h + 1 from half h
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) {
            fx[oz] += __shfl_xor_sync(0xffffffffu, fx[oz], 16);
            fy[oz] += __shfl_xor_sync(0xffffffffu, fy[oz], 16);
            fz[oz] += __shfl_xor_sync(0xffffffffu, fz[oz], 16);
        }
        const int x = rb[0] + ox, y = rb[1] + oy;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const float gx = h ? fx[2 + k] : fx[k], gy = h ? fy[2 + k] : fy[k], gz = h ? fz[2 + k] : fz[k];
            if (gx != 0.0f || gy != 0.0f || gz != 0.0f) {
                unsigned long long* a = G.acc + 4ull * node_index(P, x, y, rb[2] + 2 * h + k);
                atomicAdd(a + 1, to_fixed(gx, P.mom_scale));
                atomicAdd(a + 2, to_fixed(gy, P.mom_scale));
                atomicAdd(a + 3, to_fixed(gz, P.mom_scale));
            }
        }
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) fx[oz] = fy[oz] = fz[oz] = 0.0f;
        t = e;
    }
}

// ===================================================================================
// per-element cloth forces: in-plane vertex forces (LagrangianMesh.cpp:382-460)
// accumulated per vertex in fixed point, and the element normal/shear stress
// (HybridSolver.cpp:389-442) stored for the element's scatter in k_force.
__global__ void k_cloth_force(KParams P, PArrays cur, MeshArrays M, float dt_force) {
    pdl_entry();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M.nf) return;
    dt_force = step_dt(P, dt_force, 0);
    const int pc = M.curidx_of[M.ebase + e];
    float D[9], Q[9], R[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) D[k] = cur.F[k][pc];
    gram_schmidt(D, Q, R);
    const float* rest = M.rest + 6ull * e;
    const float rs[3] = {rest[0], rest[1], rest[2]}, w2[3] = {rest[3], rest[4], rest[5]};
    float f[3][3], ip[3];
    cloth_inplane(Q, R, rs, M.mu, M.lambda, f, ip);
    const float fw = dt_force * (M.volume_weighting ? cur.vol[pc] : 1.0f);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        unsigned long long* vf = M.vforce + 3ull * M.faces[3 * e + c];
#pragma unroll
        for (int r = 0; r < 3; ++r) atomicAdd(vf + r, to_fixed(fw * f[c][r], P.mom_scale));
    }
    float S[9];
    cloth_normal_stress(D, Q, R, ip, w2, M.shear, M.stiffness, cur.vol[pc], S);
    float* es = M.estress + 9ull * e;
#pragma unroll
    for (int k = 0; k < 9; ++k) es[k] = -dt_force * S[k];
}

// ===================================================================================
// grid velocity update + gravity (HS:725-737, 457) and level-set collision with
// friction (HS:460-511), fused; clears the accumulators and block flags.
__global__ void k_grid(KParams P, GArrays G, float dt_force, int write_force, double* force_out) {
    pdl_entry();
    const int nact = *G.nactive;
    const long total = (long)nact * 64;
    if ((long)blockIdx.x * blockDim.x >= total) return;  // no node for this block
    dt_force = step_dt(P, dt_force, 0);
    float vmax = 0.0f;  // max |v|^2 after the update, before collision (RegularGrid.cpp:188-200, HS:878)
    // the loop trip count differs between threads: the warp reduction runs after it
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const uint32_t blk = (uint32_t)G.active[i >> 6];
        const uint32_t node = (blk << 6) | (uint32_t)(i & 63);
        longlong2* a2 = reinterpret_cast<longlong2*>(G.acc + 4ull * node);
        longlong2 a = a2[0], b = a2[1];
        float4 v4 = G.vel[node];
        float4 bf = make_float4(0.f, 0.f, 0.f, 0.f);
        const float m = v4.w;
        if (m > 0.0f) {
            const float inv = P.inv_mom_scale / m;
            float vx = v4.x + __ll2float_rn(a.y) * inv + dt_force * P.gravity[0];
            float vy = v4.y + __ll2float_rn(b.x) * inv + dt_force * P.gravity[1];
            float vz = v4.z + __ll2float_rn(b.y) * inv + dt_force * P.gravity[2];
            vmax = fmaxf(vmax, vx * vx + vy * vy + vz * vz);
            bf = make_float4(vx, vy, vz, 0.f);
            // node position (unpadded coordinates)
            uint32_t bx = blk % (uint32_t)P.nb[0], r = blk / (uint32_t)P.nb[0];
            uint32_t by = r % (uint32_t)P.nb[1], bz = r / (uint32_t)P.nb[1];
            int ix = (int)(4 * bx + (i & 3)) - 4, iy = (int)(4 * by + ((i >> 2) & 3)) - 4,
                iz = (int)(4 * bz + ((i >> 4) & 3)) - 4;
            float px = P.min[0] + ix * P.h[0], py = P.min[1] + iy * P.h[1], pz = P.min[2] + iz * P.h[2];
            float phi, nn[3];
            eval_levelset(P, px, py, pz, phi, nn);
            if (phi <= 0.0f) {
                float vn = vx * nn[0] + vy * nn[1] + vz * nn[2];
                if (vn < 0.0f) {
                    float tx = vx - vn * nn[0], ty = vy - vn * nn[1], tz = vz - vn * nn[2];
                    bf = make_float4(tx, ty, tz, 0.f);
                    float nt = sqrtf(tx * tx + ty * ty + tz * tz);
                    if (nt < -P.friction * vn) {
                        vx = vy = vz = 0.0f;
                    } else if (P.friction_bug) {
                        vx = tx; vy = ty; vz = tz;
                    } else {
                        float sc = 1.0f + P.friction * vn / nt;
                        vx = tx * sc; vy = ty * sc; vz = tz * sc;
                    }
                }
            }
            v4 = make_float4(vx, vy, vz, m);
        }
        if (write_force) {  // f_i without gravity, for parity tests (reference dense order)
            int ix, iy, iz;
            uint32_t bx = blk % (uint32_t)P.nb[0], r = blk / (uint32_t)P.nb[0];
            uint32_t by = r % (uint32_t)P.nb[1], bz = r / (uint32_t)P.nb[1];
            ix = (int)(4 * bx + (i & 3)) - 4; iy = (int)(4 * by + ((i >> 2) & 3)) - 4; iz = (int)(4 * bz + ((i >> 4) & 3)) - 4;
            if (ix >= 0 && iy >= 0 && iz >= 0 && ix < P.res[0] && iy < P.res[1] && iz < P.res[2]) {
                long ng = (long)P.res[0] * P.res[1] * P.res[2];
                long idx = ((long)iz * P.res[1] + iy) * P.res[0] + ix;
                double s = (double)P.inv_mom_scale / (double)dt_force;
                force_out[idx] = (double)a.y * s;
                force_out[ng + idx] = (double)b.x * s;
                force_out[2 * ng + idx] = (double)b.y * s;
            }
            continue;  // force stage: leave velocities and accumulators untouched
        }
        G.vel[node] = v4;
        G.vbf[node] = bf;
        a2[0] = make_longlong2(0, 0);
        a2[1] = make_longlong2(0, 0);
        if ((i & 63) == 0) G.flag[blk] = 0u;
    }
    if (P.vmax2) warp_max_atomic(P.vmax2 + 1, vmax);
}

// Fixed cloth vertices (HybridSolver.cpp:513-550): for every node in the stencil
// of a fixed vertex (positive weight on all three axes, inside the grid), zero the
// velocity and the before-friction velocity of the 3x3x3 nodes around it.  The
// neighbours are addressed by the reference's linear index k*Rx*Ry + j*Rx + i
// and kept when 0 <= index < Rx*Ry*Rz, so i +- 1 wraps into the next row as in
// the reference.  One thread per (fixed vertex, stencil node, neighbour).
__global__ void k_fixed_vertices(KParams P, PArrays cur, GArrays G, MeshArrays M, const int32_t* __restrict__ fixed,
                                 int nfixed) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)nfixed * 64 * 27) return;
    const int fv = (int)(t / (64 * 27)), r = (int)(t % (64 * 27));
    const int o = r / 27, nb = r % 27;
    const int pj = M.curidx_of[M.vbase + fixed[fv]];
    int cell[3];
    float f[3], w[3][4], dw[3][4];
    locate(P, cur.x[0][pj], cur.x[1][pj], cur.x[2][pj], cell, f);
    particle_weights(P, cell, f, w, dw);
    const int ox = o & 3, oy = (o >> 2) & 3, oz = o >> 4;
    if (!(w[0][ox] > 0.0f && w[1][oy] > 0.0f && w[2][oz] > 0.0f)) return;
    const long rx = P.res[0], ry = P.res[1], ng = rx * ry * P.res[2];
    const long ri = cell[0] - 1 + ox, rj = cell[1] - 1 + oy, rk = cell[2] - 1 + oz;
    const long idx = (rk + nb / 9 - 1) * rx * ry + (rj + (nb / 3) % 3 - 1) * rx + (ri + nb % 3 - 1);
    if (idx < 0 || idx >= ng) return;
    const int ix = (int)(idx % rx), iy = (int)((idx / rx) % ry), iz = (int)(idx / (rx * ry));
    const uint32_t node = node_index(P, ix + 4, iy + 4, iz + 4);
    float4 v = G.vel[node];
    G.vel[node] = make_float4(0.f, 0.f, 0.f, v.w);
    G.vbf[node] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Interpolation weights of selected items (one row of the reference's sparse
// omegas / domegas_1..3 matrices, HybridSolver.cpp:18-97): one thread per (item,
// stencil node); node = reference linear index k*Rx*Ry + j*Rx + i, or -1 where
// the node is outside the grid or its weight is zero.  Entries are in ascending
// node order, as in the row of the reference's column-sorted matrix.
__global__ void k_query_weights(KParams P, PArrays cur, const int32_t* __restrict__ inv,
                                const int64_t* __restrict__ ids, int count, int64_t* nodes, double* w, double* g) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)count * 64) return;
    const int q = (int)(t >> 6), o = (int)(t & 63);
    const int pj = inv[ids[q]];
    int cell[3];
    float f[3], wa[3][4], da[3][4];
    locate(P, cur.x[0][pj], cur.x[1][pj], cur.x[2][pj], cell, f);
    particle_weights(P, cell, f, wa, da);
    const int ox = o & 3, oy = (o >> 2) & 3, oz = o >> 4;
    const float wx = wa[0][ox], wy = wa[1][oy], wz = wa[2][oz];
    if (wx > 0.0f && wy > 0.0f && wz > 0.0f) {
        const long i = cell[0] - 1 + ox, j = cell[1] - 1 + oy, k = cell[2] - 1 + oz;
        nodes[t] = (k * P.res[1] + j) * P.res[0] + i;
        w[t] = (double)(wx * wy * wz);
        g[3 * t + 0] = (double)(da[0][ox] * wy * wz);
        g[3 * t + 1] = (double)(wx * da[1][oy] * wz);
        g[3 * t + 2] = (double)(wx * wy * da[2][oz]);
    } else {
        nodes[t] = -1;
        w[t] = 0.0;
        g[3 * t + 0] = g[3 * t + 1] = g[3 * t + 2] = 0.0;
    }
}

// One thread: the Dt logic of HybridSolver::solve.  phase 0 (after the P2G
// normalisation): the first Dt of a solve comes from the P2G velocities (:860);
// the force pass and grid update use the current Dt (:873, :877).  phase 1 (after
// the grid update): Dt = CFL / max(300, max|v| / hmin) (:878) with the frame
// clamp (:880-892); the G2P of this step and the force pass of the next use it.
__global__ void k_solve_dt(SolveState* S, int phase) {
    if (phase == 0) {
        if (!S->initialized) {
            const double v = sqrt((double)__uint_as_float(S->vmax2[0]));
            S->Dt = S->cfl / fmax(3e2, v * S->inv_hmin);
            S->initialized = 1;
        }
        S->dt[0] = (float)S->Dt;
        S->vmax2[0] = 0u;
        S->vmax2[1] = 0u;
        S->frame_flag = 0;
        return;
    }
    const double v = sqrt((double)__uint_as_float(S->vmax2[1]));
    double Dt = S->cfl / fmax(3e2, v * S->inv_hmin);
    const double frame_dt = 1.0 / 60.0;
    if (S->inner + Dt >= frame_dt) {
        Dt = frame_dt - S->inner;
        S->t += frame_dt;
        S->inner = 0.0;
        S->frame_flag = 1;
        S->frame += 1;
    } else {
        S->inner += Dt;
    }
    S->Dt = Dt;
    S->dt[1] = (float)Dt;
    S->steps += 1;
}

// clear accumulators and flags of the touched blocks (after a partial step)
__global__ void k_grid_clear(GArrays G) {
    const int nact = *G.nactive;
    const long total = (long)nact * 64;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const uint32_t blk = (uint32_t)G.active[i >> 6];
        const uint32_t node = (blk << 6) | (uint32_t)(i & 63);
        longlong2* a2 = reinterpret_cast<longlong2*>(G.acc + 4ull * node);
        a2[0] = make_longlong2(0, 0);
        a2[1] = make_longlong2(0, 0);
        if ((i & 63) == 0) G.flag[blk] = 0u;
    }
}

// ===================================================================================
// return mapping for snow / sand (HybridSolver.cpp:612-677) from the SVD of F_tr.
// Returns the new singular values in s (in place); updates plastic.
template <typename T>
__device__ __forceinline__ void return_map(const KParams& P, int mat, T s[3], T& q) {
    if (mat == kSnow) {
#pragma unroll
        for (int a = 0; a < 3; ++a) s[a] = fmin(fmax(s[a], T(P.snow_lo)), T(P.snow_hi));
    } else {
        T ln[3] = {log_t(s[0]), log_t(s[1]), log_t(s[2])};
        int r = dp_project<T>(ln, q, T(P.sand_h0), T(P.sand_h1), T(P.sand_h2), T(P.sand_h3), T(P.sand_k));
        if (r == 1) { s[0] = s[1] = s[2] = T(1); }
        else if (r == 2) {
#pragma unroll
            for (int a = 0; a < 3; ++a) s[a] = exp_t(ln[a]);
        }
    }
}

// Return mapping (HybridSolver.cpp:612-677) in the stretch form, for a trial state
// F_tr = F + D (D = dt grad v^bf F) whose stretch C - I = F_tr^T F_tr - I = V diag(lam) V^T
// is below 1/2: ln s = log1p(lam) / 2, the projection in log space, and
//   F_E = U diag(s_new) V^T = F_tr V diag(s_new / s) V^T = F + [D + F_tr V diag(rho) V^T],
//   rho = expm1(ln s_new - ln s)        (U = F_tr V diag(1 / s)),
// i.e. the state plus a small correction, rounded once.  Computing s and then ln s,
// or U diag(s_new) V^T, loses the few units of 2^-24 that carry a small strain near
// s = 1 (the sand apex, s_new = 1, turns them into stress); this form keeps them.
// J_P (snow) is scaled by prod(s / s_new); sig = expm1(ln s - ln s_new) gives
// F_P <- F_P + V diag(sig) V^T F_P (HS:676).  T = double runs the whole mapping in
// FP64 from the same FP32 inputs.  Three parts: the trial state (ln s, V; false when
// the stretch is too large for this form), the projection (0 elastic, 1 sand apex,
// 2 snow clamp / sand cone), and F_E from the projected ln s.
template <typename T>
__device__ __forceinline__ bool stretch_trial(const float F[9], const float D[9], T ln[3], T V[9]) {
    T e[6];
    trial_stretch(F, D, e);
    const T n2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2] + T(2) * (e[3] * e[3] + e[4] * e[4] + e[5] * e[5]);
    if (!(n2 < T(0.25))) return false;
    T lam[3];
    sym_eig3<T>(e[0], e[1], e[2], e[3], e[4], e[5], lam, V, 10, sizeof(T) == 4 ? T(0x1p-24) : T(0x1p-52));
#pragma unroll
    for (int a = 0; a < 3; ++a) ln[a] = T(0.5) * log1p_t(lam[a]);
    return true;
}

template <typename T>
__device__ __forceinline__ int stretch_project(const KParams& P, int mat, const T ln[3], T lnn[3], T& q) {
#pragma unroll
    for (int a = 0; a < 3; ++a) lnn[a] = ln[a];
    if (mat == kSnow) {
        const T lo = sizeof(T) == 4 ? T(P.snow_lnlo) : log_t(T(P.snow_lo));
        const T hi = sizeof(T) == 4 ? T(P.snow_lnhi) : log_t(T(P.snow_hi));
        int kind = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const T c = fmin(fmax(ln[a], lo), hi);
            if (c != ln[a]) kind = 2;
            lnn[a] = c;
        }
        return kind;
    }
    return dp_project<T>(lnn, q, T(P.sand_h0), T(P.sand_h1), T(P.sand_h2), T(P.sand_h3), T(P.sand_k));
}

// F_E, the plastic scalar and sig from the trial and projected log singular values
template <typename T>
__device__ __forceinline__ void stretch_finish(int mat, const float F[9], const float D[9], const T V[9],
                                               const T ln[3], const T lnn[3], bool plastic, T q_new, float& q,
                                               float Fe[9], float sig[3]) {
    if (!plastic) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Fe[k] = F[k] + D[k];
        sig[0] = sig[1] = sig[2] = 0.0f;
        return;
    }
    T rho[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        rho[a] = expm1_t(lnn[a] - ln[a]);
        sig[a] = (float)expm1_t(ln[a] - lnn[a]);
    }
    // M = V diag(rho) V^T, then F_E = F + (D + (F + D) M)
    T M[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
            M[3 * a + b] = V[3 * a] * rho[0] * V[3 * b] + V[3 * a + 1] * rho[1] * V[3 * b + 1] +
                           V[3 * a + 2] * rho[2] * V[3 * b + 2];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T t0 = T(F[3 * a]) + T(D[3 * a]), t1 = T(F[3 * a + 1]) + T(D[3 * a + 1]),
                t2 = T(F[3 * a + 2]) + T(D[3 * a + 2]);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const T corr = T(D[3 * a + b]) + t0 * M[b] + t1 * M[3 + b] + t2 * M[6 + b];
            Fe[3 * a + b] = (float)(T(F[3 * a + b]) + corr);
        }
    }
    if (mat == kSnow) q = (float)(T(q) * exp_t((ln[0] - lnn[0]) + (ln[1] - lnn[1]) + (ln[2] - lnn[2])));
    else q = (float)q_new;
}

// The whole mapping; returns the projection's kind, or -1 when the stretch is too
// large for this form (the caller takes the SVD form); ln_tr / ln_new return the
// log singular values, Vo the right singular vectors.
template <typename T>
__device__ __forceinline__ int stretch_return_map(const KParams& P, int mat, const float F[9], const float D[9],
                                                  float& q, float Fe[9], float Vo[9], float sig[3], float ln_tr[3],
                                                  float ln_new[3]) {
    T ln[3], lnn[3], V[9];
    if (!stretch_trial<T>(F, D, ln, V)) return -1;
    T qq = q;
    const int kind = stretch_project<T>(P, mat, ln, lnn, qq);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ln_tr[a] = (float)ln[a];
        ln_new[a] = (float)lnn[a];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) Vo[k] = (float)V[k];
    stretch_finish<T>(mat, F, D, V, ln, lnn, kind != 0, qq, q, Fe, sig);
    return kind;
}

// Drucker-Prager cone coefficient k alpha(q) of the yield function
// |dev ln s| + k alpha tr ln s (HybridSolver.cpp:641-653)
__device__ __forceinline__ float dp_k_alpha(const KParams& P, float q) {
    const float phi = (P.sand_h0 + (P.sand_h1 * q - P.sand_h3) * dp_exp(-P.sand_h2 * q)) * (3.14159265358979f / 180.0f);
    const float sphi = dp_sin(phi);
    return P.sand_k * 0.81649658092772603f * 2.0f * sphi / (3.0f - sphi);
}

// Trial yield check of the learned path (HybridSolver.cpp:626-663), without the
// projection: 0 elastic, 1 sand apex (a constant projection), 2 plastic (the snow
// clamp or the sand cone, which the network predicts).
__device__ __forceinline__ int trial_kind(const KParams& P, int mat, const float ln[3], float q) {
    if (mat == kSnow) {
        const float lo = P.snow_lnlo, hi = P.snow_lnhi;
        return (ln[0] < lo || ln[0] > hi || ln[1] < lo || ln[1] > hi || ln[2] < lo || ln[2] > hi) ? 2 : 0;
    }
    const float tr = ln[0] + ln[1] + ln[2];
    const float d0 = ln[0] - tr / 3.0f, d1 = ln[1] - tr / 3.0f, d2 = ln[2] - tr / 3.0f;
    const float nd = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
    if (nd + dp_k_alpha(P, q) * tr <= 0.0f) return 0;
    return (nd == 0.0f || tr > 0.0f) ? 1 : 2;
}

// A sand trial state within reach of the apex of the Drucker-Prager cone: projected
// onto the apex, or |tr ln s| within 1e-3 of |ln s| of the switch between apex and
// cone (HybridSolver.cpp:652-663).  With the FP64 option these mappings run again in FP64.
__device__ __forceinline__ bool near_apex(int kind, const float ln[3]) {
    if (kind == 1) return true;
    const float tr = ln[0] + ln[1] + ln[2];
    return fabsf(tr) <= 1e-3f * sqrtf(ln[0] * ln[0] + ln[1] * ln[1] + ln[2] * ln[2]);
}

// Gather of v (G2P velocity + APIC) and v^bf (advection + velocity gradient) over
// the 4x4x4 stencil, contracted one axis at a time because the weights are tensor
// products: x first (A), then z (B), then y.
//   A0 = sum_x wx v      A1 = sum_x wx xi_x v   A2 = sum_x dwx vbf   A3 = sum_x wx vbf
//   vp = sum w v,  C = sum w v xi^T,  xs = sum w vbf,  Gb = sum vbf (grad w)^T
__device__ __forceinline__ void g2p_gather(const float4* vel, const float4* vbf, const float w[3][4],
                                           const float dw[3][4], const float xi[3][4], const uint32_t X[4],
                                           const uint32_t Y[4], const uint32_t Z[4], float vp[3], float C[9],
                                           float xs[3], float Gb[9]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) vp[k] = xs[k] = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) C[k] = Gb[k] = 0.f;
    float wxi[4];
#pragma unroll
    for (int o = 0; o < 4; ++o) wxi[o] = w[0][o] * xi[0][o];
#pragma unroll
    for (int oy = 0; oy < 4; ++oy) {
        float B0[3] = {0, 0, 0}, B1[3] = {0, 0, 0}, B2[3] = {0, 0, 0};
        float B3[3] = {0, 0, 0}, B4[3] = {0, 0, 0}, B5[3] = {0, 0, 0};
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) {
            const uint32_t yz = Y[oy] + Z[oz];
            float A0[3] = {0, 0, 0}, A1[3] = {0, 0, 0}, A2[3] = {0, 0, 0}, A3[3] = {0, 0, 0};
#pragma unroll
            for (int ox = 0; ox < 4; ++ox) {
                const float4 v = vel[yz + X[ox]];
                const float4 b = vbf[yz + X[ox]];
                const float a = w[0][ox], ax_ = wxi[ox], d = dw[0][ox];
                A0[0] = fmaf(a, v.x, A0[0]); A0[1] = fmaf(a, v.y, A0[1]); A0[2] = fmaf(a, v.z, A0[2]);
                A1[0] = fmaf(ax_, v.x, A1[0]); A1[1] = fmaf(ax_, v.y, A1[1]); A1[2] = fmaf(ax_, v.z, A1[2]);
                A2[0] = fmaf(d, b.x, A2[0]); A2[1] = fmaf(d, b.y, A2[1]); A2[2] = fmaf(d, b.z, A2[2]);
                A3[0] = fmaf(a, b.x, A3[0]); A3[1] = fmaf(a, b.y, A3[1]); A3[2] = fmaf(a, b.z, A3[2]);
            }
            const float cz = w[2][oz], czx = w[2][oz] * xi[2][oz], dz = dw[2][oz];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                B0[c] = fmaf(cz, A0[c], B0[c]);
                B1[c] = fmaf(cz, A1[c], B1[c]);
                B2[c] = fmaf(czx, A0[c], B2[c]);
                B3[c] = fmaf(cz, A2[c], B3[c]);
                B4[c] = fmaf(cz, A3[c], B4[c]);
                B5[c] = fmaf(dz, A3[c], B5[c]);
            }
        }
        const float cy = w[1][oy], cyx = w[1][oy] * xi[1][oy], dy = dw[1][oy];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            vp[c] = fmaf(cy, B0[c], vp[c]);
            C[3 * c + 0] = fmaf(cy, B1[c], C[3 * c + 0]);
            C[3 * c + 1] = fmaf(cyx, B0[c], C[3 * c + 1]);
            C[3 * c + 2] = fmaf(cy, B2[c], C[3 * c + 2]);
            xs[c] = fmaf(cy, B4[c], xs[c]);
            Gb[3 * c + 0] = fmaf(cy, B3[c], Gb[3 * c + 0]);
            Gb[3 * c + 1] = fmaf(dy, B4[c], Gb[3 * c + 1]);
            Gb[3 * c + 2] = fmaf(cy, B5[c], Gb[3 * c + 2]);
        }
    }
}

// APIC symmetric-part damping (HybridSolver.cpp:808-824): B = skew(C) + (1 - damp) sym(C)
__device__ __forceinline__ void apic_damp(const float C[9], float damp, float Bn[9]) {
    const float keep = 1.0f - damp;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float sym = 0.5f * (C[3 * a + b] + C[3 * b + a]);
            Bn[3 * a + b] = (C[3 * a + b] - sym) + keep * sym;
        }
}

// One training record of a plastic state: [ln s (trial, sorted descending), q,
// material, ln s_projected - ln s].  The sand projection is recomputed in log space
// on the sorted values, so that the target carries no exp/log rounding; states it
// sends to the apex (s = 1, a constant the network never predicts) are skipped, and
// so are sand states within kHarvestMinLn of s = 1, whose ln s carry the FP32
// rounding of s (2^-24 absolute) as more than 1e-3 of their size.
constexpr float kHarvestMinLn = 1e-4f;
__device__ __forceinline__ void harvest_record(const KParams& P, const Harvest& H, int mat, const float ln[3],
                                               const float ln_new[3], float q_old) {
    float srt[3], t[3];
    int pm[3];
    sort3_desc(ln, srt, pm);
    if (mat == kSand) {
        if (fmaxf(fabsf(srt[0]), fabsf(srt[2])) < kHarvestMinLn) return;
        t[0] = srt[0]; t[1] = srt[1]; t[2] = srt[2];
        float qq = q_old;
        if (dp_project<float>(t, qq, P.sand_h0, P.sand_h1, P.sand_h2, P.sand_h3, P.sand_k) != 2) return;
    } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) t[k] = ln_new[pm[k]];
    }
    const unsigned long long slot = atomicAdd(H.count, 1ull);
    if ((long long)slot >= H.capacity) return;
    float* r = H.buf + 8ull * slot;
    r[0] = srt[0]; r[1] = srt[1]; r[2] = srt[2];
    r[3] = q_old;
    r[4] = (float)mat;
#pragma unroll
    for (int k = 0; k < 3; ++k) r[5 + k] = t[k] - srt[k];
}

// G2P + APIC + advection + F update + return mapping, one thread per particle.
// kDefer (the learned return map): the trial state's yield check runs here; a
// plastic snow or sand state whose projection is not a constant is queued (trial
// ln s, D, V) for k_mlp_finish, which writes its F_E, F_P and plastic scalar;
// elastic states and the sand apex are mapped exactly here.
template <bool kDefer>
__global__ void __launch_bounds__(128, 4) k_g2p(KParams P, PArrays cur, PArrays nxt, const int32_t* __restrict__ perm,
                                             int n, GArrays G, float dt, uint32_t* __restrict__ keys_next,
                                             DevStats* st, Harvest H, const uint32_t* __restrict__ keys_sorted,
                                             MlpQueue Qu) {
    pdl_entry();
    __shared__ float4 tile_v[kTileNodes], tile_b[kTileNodes];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    int org[3];
    tile_origin(P, keys_sorted[blockIdx.x * blockDim.x], org);
    load_tile(P, org, G.vel, G.vbf, tile_v, tile_b);
    // the particle's own loads and weights overlap the tile copy; F_E and the
    // per-particle scalars, read after the gather, are copied to shared memory
    // asynchronously meanwhile (each thread reads back only its own entries).  The
    // learned form (kDefer), with its queue code, loads them directly: it is at its
    // register limit already.
    const bool live = j < n;
    const int pj = live ? perm[j] : 0;
    __shared__ float sF[9][128], sq[128], sm[128], svol[128];
    __shared__ int32_t sid[128];
    if (!kDefer) {
#pragma unroll
        for (int k = 0; k < 9; ++k) cp_async4(&sF[k][threadIdx.x], &cur.F[k][pj]);
        cp_async4(&sq[threadIdx.x], &cur.plastic[pj]);
        cp_async4(&sm[threadIdx.x], &cur.m[pj]);
        cp_async4(&svol[threadIdx.x], &cur.vol[pj]);
        cp_async4(&sid[threadIdx.x], &cur.id[pj]);
        cp_async_commit();
    }
    const int mat = live ? (int)cur.mat[pj] : (int)kClothElement;
    float xp[3] = {cur.x[0][pj], cur.x[1][pj], cur.x[2][pj]};
    int cell[3];
    float f[3], w[3][4], dw[3][4];
    locate(P, xp[0], xp[1], xp[2], cell, f);
    const bool truncated = particle_weights(P, cell, f, w, dw);
    int base[3] = {cell[0] + 3, cell[1] + 3, cell[2] + 3};
    uint32_t X[4], Y[4], Z[4];
    const bool in_tile = tile_offsets(base, org, X, Y, Z);
    if (!in_tile) stencil_offsets(P, base, X, Y, Z);
    __syncthreads();
    // elements follow their vertices (k_cloth_g2p)
    if (!live || mat == kClothElement) {
        cp_async_wait_all();  // no copy into this block's shared memory outlives the thread
        return;
    }
    dt = step_dt(P, dt, 1);
    float xi[3][4];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int o = 0; o < 4; ++o) xi[a][o] = ((float)(o - 1) - f[a]) * P.h[a];

    float vp[3], xs[3], C[9], Gb[9];
    g2p_gather(in_tile ? tile_v : G.vel, in_tile ? tile_b : G.vbf, w, dw, xi, X, Y, Z, vp, C, xs, Gb);
    // advection x = sum w (x_i + dt v^bf_i) (HS:944): exact linear reproduction for a
    // full stencil; a stencil cut by the grid boundary keeps its lost weight.
    float xn[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) xn[a] = xp[a] + dt * xs[a];
    if (truncated) {
        float s0[3], s1[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            s0[a] = w[a][0] + w[a][1] + w[a][2] + w[a][3];
            s1[a] = w[a][0] * xi[a][0] + w[a][1] * xi[a][1] + w[a][2] * xi[a][2] + w[a][3] * xi[a][3];
        }
        float sw = s0[0] * s0[1] * s0[2];
        float swx[3] = {s1[0] * s0[1] * s0[2], s0[0] * s1[1] * s0[2], s0[0] * s0[1] * s1[2]};
#pragma unroll
        for (int a = 0; a < 3; ++a) xn[a] += xp[a] * (sw - 1.0f) + swx[a];
    }
    // APIC damping (HS:916, 926)
    float Bn[9];
    apic_damp(C, mat == kClothVertex ? P.mesh_damp : P.particle_damp, Bn);
    if (mat == kClothVertex) {  // vertices carry no deformation gradient of their own
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            nxt.x[a][j] = xn[a];
            nxt.v[a][j] = vp[a];
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            nxt.B[k][j] = Bn[k];
            nxt.F[k][j] = cur.F[k][pj];
        }
        nxt.plastic[j] = cur.plastic[pj];
        nxt.mat[j] = (uint8_t)mat;
        nxt.m[j] = cur.m[pj];
        nxt.vol[j] = cur.vol[pj];
        nxt.id[j] = cur.id[pj];
        int vc[3];
        float vf[3];
        const bool vclamped = locate(P, xn[0], xn[1], xn[2], vc, vf);
        keys_next[j] = make_key(P, vc);
        if (vclamped) atomicAdd(&st->out_of_domain, 1ull);
        cp_async_wait_all();
        return;
    }
    // F update (HS:560-576): F_tr = F + D, D = dt grad v^bf F
    if (!kDefer) cp_async_wait_all();
    float F[9], GF[9], Ftr[9], D[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) F[k] = kDefer ? cur.F[k][pj] : sF[k][threadIdx.x];
    mat_mul(Gb, F, GF);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        D[k] = dt * GF[k];
        Ftr[k] = F[k] + D[k];
    }
    // return mapping (HS:612-677)
    float q = kDefer ? cur.plastic[pj] : sq[threadIdx.x];
    float U[9], s[3], V[9];
    float Fe[9], sn[3];
    float sprod = 1.0f;  // prod(s_trial / s_new) for J_P
    bool used_fp64 = false, deferred = false;
    double Ud[9], sd[3], Vd[9];
    // the stretch form (plain step): the state plus a correction; -1 for a trial
    // stretch beyond its range, which takes the SVD form below
    int skind = -1;
    float sig[3];
    if (!kDefer) {
        float lt[3], lnw[3];
        const float q_old = q;
        skind = stretch_return_map<float>(P, mat, F, D, q, Fe, V, sig, lt, lnw);
        if (skind >= 0 && P.fp64_apex && mat == kSand && near_apex(skind, lt)) {
            q = q_old;  // the same mapping again, in FP64
            skind = stretch_return_map<double>(P, mat, F, D, q, Fe, V, sig, lt, lnw);
            cg::coalesced_group g = cg::coalesced_threads();
            if (g.thread_rank() == 0) atomicAdd(&st->fp64_apex, (unsigned long long)g.size());
        }
        if (skind > 0 && H.buf && (j % H.stride) == 0) harvest_record(P, H, mat, lt, lnw, q_old);
    } else {
        // the learned return map: the trial state and its yield check here; a plastic
        // state with a projection the network predicts is queued for k_mlp_finish
        // (trial ln s, D, V), everything else is mapped exactly in place
        float ln[3];
        const bool in_range = stretch_trial<float>(F, D, ln, V);
        const int tk = in_range ? trial_kind(P, mat, ln, q) : -1;
        // the queue positions of the warp's plastic lanes: one atomic, issued here and
        // read after the exact mappings of its other lanes, which hide its round trip
        const unsigned qlanes = __activemask();
        const unsigned qmask = __ballot_sync(qlanes, tk == 2);
        const int qlane = threadIdx.x & 31, qleader = qmask ? __ffs(qmask) - 1 : __ffs(qlanes) - 1;
        unsigned qbase = 0;
        if (qmask && qlane == qleader) qbase = atomicAdd(&st->mlp_rows, (unsigned)__popc(qmask));
        if (in_range) {
            if (tk != 2) {
                float lnn[3], qq = q;
                const int kind = stretch_project<float>(P, mat, ln, lnn, qq);
                stretch_finish<float>(mat, F, D, V, ln, lnn, kind != 0, qq, q, Fe, sig);
                if (kind == 1) {
                    cg::coalesced_group g = cg::coalesced_threads();  // the apex: exact, counted
                    if (g.thread_rank() == 0) atomicAdd(&st->learned_exact, (unsigned long long)g.size());
                }
            }
            skind = 0;  // handled: no SVD form below
        } else {
            cg::coalesced_group g = cg::coalesced_threads();  // beyond the stretch form: exact SVD form
            if (g.thread_rank() == 0) atomicAdd(&st->learned_exact, (unsigned long long)g.size());
        }
        qbase = __shfl_sync(qlanes, qbase, qleader);
        if (tk == 2) {
            // the queue has a row per particle, so every position is below its capacity
            const int r = (int)(qbase + (unsigned)__popc(qmask & ((1u << qlane) - 1u)));
            deferred = true;
            if (r < Qu.cap) {
                const long cap = Qu.cap;
                float* f = Qu.f + r;
                Qu.j[r] = j;
                Qu.pj[r] = pj;
#pragma unroll
                for (int a = 0; a < 3; ++a) f[(kQLn + a) * cap] = ln[a];
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    f[(kQD + k) * cap] = D[k];
                    f[(kQV + k) * cap] = V[k];
                }
            }
        }
    }
    bool ok = skind >= 0 || svd3<float>(Ftr, U, s, V, 8, 1e-7f, 2e-2f);
    if (skind >= 0) {
    } else if (ok) {
        sn[0] = s[0]; sn[1] = s[1]; sn[2] = s[2];
        const float q_old = q;
        return_map<float>(P, mat, sn, q);
        if (H.buf && (j % H.stride) == 0 && (sn[0] != s[0] || sn[1] != s[1] || sn[2] != s[2])) {
            const float lt[3] = {logf(s[0]), logf(s[1]), logf(s[2])}, lnw[3] = {logf(sn[0]), logf(sn[1]), logf(sn[2])};
            harvest_record(P, H, mat, lt, lnw, q_old);  // plastic states only
        }
        if (!deferred) {
            sprod = (s[0] / sn[0]) * (s[1] / sn[1]) * (s[2] / sn[2]);
            float US[9];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) US[3 * r + c] = U[3 * r + c] * sn[c];
            mat_mul_bt(US, V, Fe);
        }
    } else {
        used_fp64 = true;
        double Fd[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Fd[k] = Ftr[k];
        svd3<double>(Fd, Ud, sd, Vd, 40, 1e-15, 0.0);
        svd3_complete(Ud, sd);
        double s0[3] = {sd[0], sd[1], sd[2]};
        double qd = q;
        return_map<double>(P, mat, sd, qd);
        q = (float)qd;
        sprod = (float)((s0[0] / sd[0]) * (s0[1] / sd[1]) * (s0[2] / sd[2]));
        double US[9], Fed[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) US[3 * r + c] = Ud[3 * r + c] * sd[c];
        mat_mul_bt(US, Vd, Fed);
#pragma unroll
        for (int k = 0; k < 9; ++k) Fe[k] = (float)Fed[k];
        atomicAdd(&st->fallbacks, 1ull);
    }
    if (deferred) {
    } else if (P.track_fp && skind >= 0) {
        // F_P = V S_new^-1 U^T F_tr F_P = V diag(s / s_new) V^T F_P = F_P + V diag(sig) V^T F_P (HS:676)
        float Fp[9], Fpn[9], W[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Fp[k] = cur.Fp[k][pj];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                W[3 * a + b] = V[3 * a] * sig[0] * V[3 * b] + V[3 * a + 1] * sig[1] * V[3 * b + 1] +
                               V[3 * a + 2] * sig[2] * V[3 * b + 2];
        mat_mul(W, Fp, Fpn);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            Fpn[k] += Fp[k];
            nxt.Fp[k][j] = Fpn[k];
        }
        if (mat == kSnow) q = mat_det(Fpn);
    } else if (P.track_fp) {
        // F_P = V S^-1 U^T F_tr F_P (HS:676)
        float Fp[9], Ft[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Fp[k] = cur.Fp[k][pj];
        mat_mul(Ftr, Fp, Ft);
        float VS[9], M[9], Fpn[9];
        if (!used_fp64) {
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) VS[3 * r + c] = V[3 * r + c] / sn[c];
            mat_mul_bt(VS, U, M);
        } else {
            double VSd[9], Md[9];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) VSd[3 * r + c] = Vd[3 * r + c] / sd[c];
            mat_mul_bt(VSd, Ud, Md);
            for (int k = 0; k < 9; ++k) M[k] = (float)Md[k];
        }
        mat_mul(M, Ft, Fpn);
#pragma unroll
        for (int k = 0; k < 9; ++k) nxt.Fp[k][j] = Fpn[k];
        if (mat == kSnow) q = mat_det(Fpn);
    } else if (mat == kSnow && skind < 0) {
        q *= sprod;  // J_P = det F_P = det(F_tr) det(F_P) / det(S_new); the stretch form scaled it already
    }
    // store in the new order
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        nxt.x[a][j] = xn[a];
        nxt.v[a][j] = vp[a];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) nxt.B[k][j] = Bn[k];
    if (!deferred) {
#pragma unroll
        for (int k = 0; k < 9; ++k) nxt.F[k][j] = Fe[k];
        nxt.plastic[j] = q;
    }
    nxt.mat[j] = (uint8_t)mat;
    nxt.m[j] = kDefer ? cur.m[pj] : sm[threadIdx.x];
    nxt.vol[j] = kDefer ? cur.vol[pj] : svol[threadIdx.x];
    nxt.id[j] = kDefer ? cur.id[pj] : sid[threadIdx.x];
    int ncell[3];
    float nf[3];
    bool clamped = locate(P, xn[0], xn[1], xn[2], ncell, nf);
    keys_next[j] = make_key(P, ncell);
    if (clamped) atomicAdd(&st->out_of_domain, 1ull);
}

// ===================================================================================
// The learned return map of the rows that k_g2p<true> queued: one warp per 32
// consecutive rows runs the MLP (aep_mlp.cuh) on the tensor cores on the sorted
// trial log singular values, and each prediction is checked against the optimality
// conditions of the projection it stands for (HybridSolver.cpp:626-674), with the
// residuals in ln-strain units and accepted within max(tol_rel |ln s_pred|, tol_abs),
// relative to the projected strain the prediction gives (the stress is linear in it,
// so an accepted state's stress carries a relative error of a few tol_rel):
//   sand (the cone; the apex never reaches the network): the yield condition at the
//     prediction, |dev| + k alpha(q) tr = 0, and the flow rule: the trace kept and the
//     deviatoric part a shrunk copy of the trial's (0 <= c <= 1);
//   snow (the clamp of each log singular value to [ln(1 - theta_c), ln(1 + theta_s)]):
//     every predicted value inside the bounds, equal to its trial value where that is
//     inside and to the bound it crossed where it is outside.
// A rejected prediction is replaced by the exact projection (learned_fallbacks).
// F_E, F_P and the plastic scalar follow in the stretch form.  Persistent: the
// weights are loaded once per block.
constexpr int kFinThreads = 128;

// The residual of a predicted projection (ln units); q_new: the plastic scalar it implies
__device__ __forceinline__ float learned_residual(const KParams& P, int mat, const float ln[3], const float pred[3],
                                                  float q, float& q_new) {
    q_new = q;
    if (mat == kSnow) {
        const float lo = P.snow_lnlo, hi = P.snow_lnhi;
        float r = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float target = ln[a] < lo ? lo : (ln[a] > hi ? hi : ln[a]);
            r = fmaxf(r, fabsf(pred[a] - target));
        }
        return r;
    }
    const float tr = ln[0] + ln[1] + ln[2], trp = pred[0] + pred[1] + pred[2];
    float dev[3], devp[3], nd = 0.0f, ndp = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        dev[a] = ln[a] - tr / 3.0f;
        devp[a] = pred[a] - trp / 3.0f;
        nd += dev[a] * dev[a];
        ndp += devp[a] * devp[a];
    }
    nd = sqrtf(nd);
    ndp = sqrtf(ndp);
    const float c = nd > 0.0f ? ndp / nd : 0.0f;
    float r = fabsf(ndp + dp_k_alpha(P, q) * trp);  // yield condition at the prediction
    r = fmaxf(r, fabsf(trp - tr));                   // flow rule: the trace is kept,
#pragma unroll
    for (int a = 0; a < 3; ++a) r = fmaxf(r, fabsf(devp[a] - c * dev[a]));  // dev shrinks radially
    if (c > 1.0f) r = fmaxf(r, (c - 1.0f) * nd);
    q_new = q + (nd - ndp);  // the plastic amount grows by the projection distance dg
    return r;
}

__global__ void __launch_bounds__(kFinThreads) k_mlp_finish(KParams P, PArrays cur, PArrays nxt, MlpQueue Qu,
                                                            DevStats* st, MlpParams mlp, float tol_rel,
                                                            float tol_abs) {
    pdl_entry();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int rows = (int)min(st->mlp_rows, (unsigned)Qu.cap);
    if ((long)blockIdx.x * kFinThreads >= rows) return;  // no tile for this block (block-uniform)
    const MlpSmem W = mlp_smem_carve(smem_raw);
    mlp_load_smem(mlp, W, threadIdx.x, blockDim.x);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wbase = smem_raw + kMlpSmemBytes + warp * kMlpWarpBytes;
    __nv_bfloat16* X = reinterpret_cast<__nv_bfloat16*>(wbase);
    float* Y = reinterpret_cast<float*>(X + kMlpWarpX);
    const long cap = Qu.cap;
    unsigned n_ok = 0, n_rej = 0;
    const int nwarps = gridDim.x * (kFinThreads / 32);
    for (int t = blockIdx.x * (kFinThreads / 32) + warp; t * 32 < rows; t += nwarps) {  // warp-uniform
        const int r = t * 32 + lane;
        const bool live = r < rows;
        const int rr = live ? r : t * 32;  // a lane past the end repeats the tile's first row
        const float* f = Qu.f + rr;
        const int pj = Qu.pj[rr];
        const int mat = (int)cur.mat[pj];
        float ln[3], srt[3];
        int pm[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) ln[a] = f[(kQLn + a) * cap];
        sort3_desc(ln, srt, pm);
        float q = cur.plastic[pj];
        const float osc = mlp_features(srt, q, mat, X + lane * kStrideIn);
        mlp_forward_warp<true>(W, X, Y, lane);
        if (live) {
            float pred[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) pred[pm[k]] = srt[k] + Y[lane * kMlpOut + k] / osc;
            float q_new;
            const float res = learned_residual(P, mat, ln, pred, q, q_new);
            const float pnorm = sqrtf(pred[0] * pred[0] + pred[1] * pred[1] + pred[2] * pred[2]);
            float lnn[3];
            if (res <= fmaxf(tol_rel * pnorm, tol_abs)) {
                lnn[0] = pred[0]; lnn[1] = pred[1]; lnn[2] = pred[2];
                ++n_ok;
            } else {  // the exact projection
                q_new = q;
                stretch_project<float>(P, mat, ln, lnn, q_new);
                ++n_rej;
            }
            float F[9], D[9], V[9], Fe[9], sig[3];
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                F[k] = cur.F[k][pj];
                D[k] = f[(kQD + k) * cap];
                V[k] = f[(kQV + k) * cap];
            }
            stretch_finish<float>(mat, F, D, V, ln, lnn, true, q_new, q, Fe, sig);
            const int j = Qu.j[r];
#pragma unroll
            for (int k = 0; k < 9; ++k) nxt.F[k][j] = Fe[k];
            if (P.track_fp) {  // F_P <- F_P + V diag(sig) V^T F_P (HS:676)
                float Fp[9], Wm[9], Fpn[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) Fp[k] = cur.Fp[k][pj];
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b)
                        Wm[3 * a + b] = V[3 * a] * sig[0] * V[3 * b] + V[3 * a + 1] * sig[1] * V[3 * b + 1] +
                                        V[3 * a + 2] * sig[2] * V[3 * b + 2];
                mat_mul(Wm, Fp, Fpn);
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    Fpn[k] += Fp[k];
                    nxt.Fp[k][j] = Fpn[k];
                }
                if (mat == kSnow) q = mat_det(Fpn);
            }
            nxt.plastic[j] = q;
        }
    }
    n_ok = __reduce_add_sync(0xffffffffu, n_ok);
    n_rej = __reduce_add_sync(0xffffffffu, n_rej);
    if (lane == 0) {
        if (n_ok) atomicAdd(&st->learned_ok, (unsigned long long)n_ok);
        if (n_rej) atomicAdd(&st->learned_rejected, (unsigned long long)n_rej);
    }
}

// ===================================================================================
// cloth elements (one thread per element): APIC momenta from the element's own
// G2P velocity at its old centroid (HS:927-933), velocity = mean of the new vertex
// velocities (HS:749-756), position = centroid of the new vertex positions
// (LagrangianMesh.cpp:371-380), directions d1, d2 from the vertices and
// d3 += dt grad v^bf d3 (HS:584-607), then the QR return mapping (HS:686-720).
// With an MLP (use_mlp), the cloth return mapping of plastic elements (shear beyond
// the frictional cap) is predicted by the learned map (cloth rows of the same
// network) and checked against the cap's optimality conditions, the exact
// projection replacing a rejected prediction; the warp runs the network when any
// of its elements is plastic.  With a harvest buffer (plain steps), plastic
// elements record [r13, r23, r33 - 1, cap ratio, 2, projected - trial (3)].
__global__ void __launch_bounds__(128) k_cloth_g2p(KParams P, PArrays cur, PArrays nxt, GArrays G, MeshArrays M,
                                                   float dt, uint32_t* __restrict__ keys_next, DevStats* st,
                                                   Harvest H, MlpParams mlp, int use_mlp, float tol_rel,
                                                   float tol_abs) {
    pdl_entry();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = e < M.nf;
    dt = step_dt(P, dt, 1);
    MlpSmem W{};
    if (use_mlp) {  // block-uniform
        W = mlp_smem_carve(smem_raw);
        mlp_load_smem(mlp, W, threadIdx.x, blockDim.x);
        __syncthreads();
    }
    float Q[9], r[3] = {0, 0, 1}, rp[3] = {0, 0, 1}, cap = 0.0f;
    bool plastic = false, tension = false;
    int j = 0, pc = 0;
    if (live) {
        const int id = M.ebase + e;
        j = M.slot_of[id];
        pc = M.curidx_of[id];
        float xp[3] = {cur.x[0][pc], cur.x[1][pc], cur.x[2][pc]};
        int cell[3];
        float f[3], w[3][4], dw[3][4];
        locate(P, xp[0], xp[1], xp[2], cell, f);
        particle_weights(P, cell, f, w, dw);
        int base[3] = {cell[0] + 3, cell[1] + 3, cell[2] + 3};
        uint32_t X[4], Y[4], Z[4];
        stencil_offsets(P, base, X, Y, Z);
        float xi[3][4];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int o = 0; o < 4; ++o) xi[a][o] = ((float)(o - 1) - f[a]) * P.h[a];
        float vp[3], xs[3], C[9], Gb[9];
        g2p_gather(G.vel, G.vbf, w, dw, xi, X, Y, Z, vp, C, xs, Gb);
        float Bn[9];
        apic_damp(C, P.mesh_damp, Bn);
        float xv[3][3], vv[3][3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int sv = M.slot_of[M.vbase + M.faces[3 * e + c]];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                xv[c][a] = nxt.x[a][sv];
                vv[c][a] = nxt.v[a][sv];
            }
        }
        float D[9];
        const float d3o[3] = {cur.F[2][pc], cur.F[5][pc], cur.F[8][pc]};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            D[3 * a + 0] = xv[1][a] - xv[0][a];
            D[3 * a + 1] = xv[2][a] - xv[0][a];
            D[3 * a + 2] = dt * (Gb[3 * a] * d3o[0] + Gb[3 * a + 1] * d3o[1] + Gb[3 * a + 2] * d3o[2]) + d3o[a];
        }
        float R[9];
        gram_schmidt(D, Q, R);
        r[0] = R[2]; r[1] = R[5]; r[2] = R[8];
        rp[0] = r[0]; rp[1] = r[1]; rp[2] = r[2];
        // the trial yield check (HybridSolver.cpp:701-716): tension (r33 > 1, the
        // constant r = e3) or a shear beyond the frictional cap (plastic)
        tension = r[2] > 1.0f;
        cap = cloth_cap_ratio(r, M.shear, M.stiffness, M.friction);
        plastic = !tension && cap < 1.0f;
        // the exact projection, unless the learned map predicts this row
        if (!(use_mlp && plastic)) cloth_project(rp, M.shear, M.stiffness, M.friction);
        // records of states within 1e-5 of r = e3 would carry the FP32 rounding of
        // r33 as more than 1e-2 of their size: skipped
        if (H.buf && !use_mlp && plastic && (e % H.stride) == 0 &&
            fmaxf(fmaxf(fabsf(r[0]), fabsf(r[1])), fabsf(r[2] - 1.0f)) >= 1e-5f) {
            const unsigned long long slot = atomicAdd(H.count, 1ull);
            if ((long long)slot < H.capacity) {
                float* o = H.buf + 8ull * slot;
                o[0] = r[0]; o[1] = r[1]; o[2] = r[2] - 1.0f; o[3] = cap; o[4] = (float)kMlpCloth;
                o[5] = rp[0] - r[0]; o[6] = rp[1] - r[1]; o[7] = rp[2] - r[2];
            }
        }
        float xn[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            xn[a] = (xv[0][a] + xv[1][a] + xv[2][a]) / 3.0f;
            nxt.x[a][j] = xn[a];
            nxt.v[a][j] = (vv[0][a] + vv[1][a] + vv[2][a]) / 3.0f;
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) nxt.B[k][j] = Bn[k];
        nxt.F[0][j] = D[0]; nxt.F[1][j] = D[1];
        nxt.F[3][j] = D[3]; nxt.F[4][j] = D[4];
        nxt.F[6][j] = D[6]; nxt.F[7][j] = D[7];
        nxt.plastic[j] = cur.plastic[pc];
        nxt.mat[j] = (uint8_t)kClothElement;
        nxt.m[j] = cur.m[pc];
        nxt.vol[j] = cur.vol[pc];
        nxt.id[j] = id;
        int nc[3];
        float nf[3];
        const bool clamped = locate(P, xn[0], xn[1], xn[2], nc, nf);
        keys_next[j] = make_key(P, nc);
        if (clamped) atomicAdd(&st->out_of_domain, 1ull);
    }
    if (use_mlp) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        unsigned char* wbase = smem_raw + kMlpSmemBytes + warp * kMlpWarpBytes;
        __nv_bfloat16* MX = reinterpret_cast<__nv_bfloat16*>(wbase);
        float* MY = reinterpret_cast<float*>(MX + kMlpWarpX);
        bool ok = false;
        if (__any_sync(0xffffffffu, plastic)) {  // warp-uniform
            const float in[3] = {r[0], r[1], r[2] - 1.0f};
            const float sc = mlp_features(in, cap, plastic ? kMlpCloth : 0, MX + lane * kStrideIn);
            mlp_forward_warp<true>(W, MX, MY, lane);
            if (plastic) {
                // optimality conditions of the frictional cap: r33 kept, the shear
                // (r13, r23) a shrunk copy of the trial's, its length on the cap
                // friction * stiffness (r33 - 1)^2 / shear; residuals in r units,
                // relative to the predicted (r13, r23, r33 - 1)
                float pred[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) pred[a] = r[a] + MY[lane * kMlpOut + a] / sc;
                const float ns = sqrtf(r[0] * r[0] + r[1] * r[1]), nsp = sqrtf(pred[0] * pred[0] + pred[1] * pred[1]);
                const float c = ns > 0.0f ? nsp / ns : 0.0f;
                const float on_cap = M.friction * M.stiffness * (r[2] - 1.0f) * (r[2] - 1.0f) / M.shear;
                float res = fmaxf(fabsf(pred[2] - r[2]), fabsf(nsp - on_cap));
                res = fmaxf(res, fmaxf(fabsf(pred[0] - c * r[0]), fabsf(pred[1] - c * r[1])));
                const float ref = sqrtf(nsp * nsp + (pred[2] - 1.0f) * (pred[2] - 1.0f));
                ok = res <= fmaxf(tol_rel * ref, tol_abs);
                if (ok) {
                    rp[0] = pred[0]; rp[1] = pred[1]; rp[2] = pred[2];
                } else {
                    cloth_project(rp, M.shear, M.stiffness, M.friction);  // the exact projection
                }
            }
        }
        // warp-aggregated counters (every lane of the warp is here)
        const unsigned b_ok = __ballot_sync(0xffffffffu, plastic && ok);
        const unsigned b_rej = __ballot_sync(0xffffffffu, plastic && !ok);
        const unsigned b_ex = __ballot_sync(0xffffffffu, tension);
        if (lane == 0) {
            if (b_ok) atomicAdd(&st->learned_ok, (unsigned long long)__popc(b_ok));
            if (b_rej) atomicAdd(&st->learned_rejected, (unsigned long long)__popc(b_rej));
            if (b_ex) atomicAdd(&st->learned_exact, (unsigned long long)__popc(b_ex));
        }
    }
    if (live) {
        // d3 = Q r (HybridSolver.cpp:718-719)
#pragma unroll
        for (int a = 0; a < 3; ++a) nxt.F[3 * a + 2][j] = Q[3 * a] * rp[0] + Q[3 * a + 1] * rp[1] + Q[3 * a + 2] * rp[2];
    }
}

// ===================================================================================
// first-P2G densities and volumes (HybridSolver.cpp:242-249):
// rho_p = sum_i w_ip m_i / h^3, vol_p = m_p / rho_p; written in the current order.
__global__ void k_volumes(KParams P, PArrays cur, const int32_t* __restrict__ perm, int n, GArrays G) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int pj = perm[j];
    if (cur.mat[pj] > kSand) return;  // only the ParticleSystem gets volumes (HS:244-248)
    int cell[3];
    float f[3], w[3][4], dw[3][4];
    locate(P, cur.x[0][pj], cur.x[1][pj], cur.x[2][pj], cell, f);
    particle_weights(P, cell, f, w, dw);
    int base[3] = {cell[0] + 3, cell[1] + 3, cell[2] + 3};
    uint32_t X[4], Y[4], Z[4];
    stencil_offsets(P, base, X, Y, Z);
    float s = 0.0f;
    for (int oz = 0; oz < 4; ++oz)
        for (int oy = 0; oy < 4; ++oy)
            for (int ox = 0; ox < 4; ++ox) s += w[0][ox] * w[1][oy] * w[2][oz] * G.vel[X[ox] + Y[oy] + Z[oz]].w;
    float rho = s / P.cell_volume;
    cur.vol[pj] = cur.m[pj] / rho;
}

// ===================================================================================
// layout conversion: reference FP64 layouts <-> device FP32 structure of arrays
// mode: 0 = N x 3 column-major vector field into dst[3], 1 = 9N B rows (see aep.h),
// 2 = 9N per-particle column-major 3x3 into row-major dst[9], 3 = N scalars,
// 4 = element directions d1 | d2 | d3 (each N x 3 column-major) into the columns of dst[9]
// map (optional): item q of the source goes to slot map[q] (keeps the device order)
// Host-layout doubles -> FP32 SoA, one thread per source double (consecutive
// threads read consecutive doubles, so a source in pinned host memory streams
// over the host link at full width).  Item q goes to slot map[q] (or q).
// mode 0: N x 3 column-major; 1: affine momenta (3 blocks of N x 3, block a =
// row a); 2: 3x3 column-major per item; 3: scalar; 4: element directions
// (3 blocks of N x 3, block c = column c).
__global__ void k_upload(long total, int n, int mode, const double* __restrict__ src, float* d0, float* d1, float* d2,
                         float* d3, float* d4, float* d5, float* d6, float* d7, float* d8,
                         const int32_t* __restrict__ map) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    float* d[9] = {d0, d1, d2, d3, d4, d5, d6, d7, d8};
    int k, q;
    if (mode == 2) {
        q = (int)(e / 9);
        const int r = (int)(e % 9);
        k = 3 * (r % 3) + r / 3;
    } else if (mode == 4) {
        const int t = (int)(e / n);
        q = (int)(e % n);
        k = 3 * (t % 3) + t / 3;
    } else {
        k = (int)(e / n);
        q = (int)(e % n);
    }
    const long p = map ? map[q] : q;
    d[k][p] = (float)src[e];
}

// The whole particle upload of aep_set_particles in one launch: one thread per
// source double, over the segments x (3n), v (3n), B (9n), Fe (9n), Fp (9n, with
// track_plastic_F and a given F_P) and one thread per item for m, vol, plastic,
// material, id and snow J_P.  Consecutive threads read consecutive doubles, so a
// source in page-locked host memory streams over the host link without gaps
// between kernels.  Item q goes to slot map[q] (or q).  check = {max mass bits,
// bad mass or tag}.
__global__ void k_upload_particles(int n, UploadSrc src, PArrays P, const int32_t* __restrict__ map, int track_fp,
                                   unsigned long long* check) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long N = n;
    const long nF = (track_fp && src.Fp) ? 9 * N : 0;
    const long total = 24 * N + nF + N;
    unsigned long long mx = 0ull, bad = 0ull;
    if (e < total) {
        long r = e;
        if (r < 3 * N) {  // x: N x 3 column-major
            const int a = (int)(r / N), q = (int)(r % N);
            P.x[a][map ? map[q] : q] = (float)src.x[r];
        } else if ((r -= 3 * N) < 3 * N) {  // v
            const int a = (int)(r / N), q = (int)(r % N);
            P.v[a][map ? map[q] : q] = src.v ? (float)src.v[r] : 0.0f;
        } else if ((r -= 3 * N) < 9 * N) {  // B: block a of N x 3 = row a
            const int t = (int)(r / N), q = (int)(r % N);
            P.B[t][map ? map[q] : q] = src.B ? (float)src.B[r] : 0.0f;
        } else if ((r -= 9 * N) < 9 * N) {  // Fe: 3x3 column-major per item
            const int q = (int)(r / 9), c = (int)(r % 9);
            P.F[3 * (c % 3) + c / 3][map ? map[q] : q] = (float)src.Fe[r];
        } else if ((r -= 9 * N) < nF) {  // F_P, same layout
            const int q = (int)(r / 9), c = (int)(r % 9);
            P.Fp[3 * (c % 3) + c / 3][map ? map[q] : q] = (float)src.Fp[r];
        } else {  // item fields
            const int q = (int)(r - nF);
            const int p = map ? map[q] : q;
            const double m = src.m[q];
            if (!(m >= 0.0) || !isfinite(m)) bad = 1ull;
            else if (m > 0.0) mx = (unsigned long long)__double_as_longlong(m);
            const int mat = src.mat ? (int)src.mat[q] : kSand;
            if (mat > kSand) bad = 1ull;
            P.m[p] = (float)m;
            P.vol[p] = src.vol ? (float)src.vol[q] : 0.0f;
            P.mat[p] = (uint8_t)mat;
            P.id[p] = q;
            float pl = src.plastic ? (float)src.plastic[q] : 0.0f;
            if (track_fp && !src.Fp)
#pragma unroll
                for (int c = 0; c < 9; ++c) P.Fp[c][p] = (c % 4 == 0) ? 1.0f : 0.0f;
            if (!track_fp && mat == kSnow) {  // J_P = det F_P, else the given scalar, else 1
                if (src.Fp) {
                    double A[9];
#pragma unroll
                    for (int c = 0; c < 9; ++c) A[3 * (c % 3) + c / 3] = src.Fp[9l * q + c];
                    pl = (float)mat_det(A);
                } else if (!src.plastic) {
                    pl = 1.0f;
                }
            }
            P.plastic[p] = pl;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (mx) atomicMax(check, mx);
        if (bad) atomicOr(check + 1, bad);
    }
}

// The particle readback of aep_get_particles in one launch: one thread per
// destination double over the requested fields (coalesced writes into
// page-locked host memory); inv[id] = slot.
__global__ void k_download_particles(int n, DownloadDst dst, PArrays P, const int32_t* __restrict__ inv) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long N = n;
    long r = e;
    const long sx = dst.x ? 3 * N : 0, sv = dst.v ? 3 * N : 0, sB = dst.B ? 9 * N : 0, sF = dst.Fe ? 9 * N : 0,
               sP = dst.Fp ? 9 * N : 0, sV = dst.vol ? N : 0, sQ = dst.plastic ? N : 0;
    if (r < sx) {
        dst.x[r] = (double)P.x[r / N][inv[r % N]];
    } else if ((r -= sx) < sv) {
        dst.v[r] = (double)P.v[r / N][inv[r % N]];
    } else if ((r -= sv) < sB) {
        dst.B[r] = (double)P.B[r / N][inv[r % N]];
    } else if ((r -= sB) < sF) {
        const int c = (int)(r % 9);
        dst.Fe[r] = (double)P.F[3 * (c % 3) + c / 3][inv[r / 9]];
    } else if ((r -= sF) < sP) {
        const int c = (int)(r % 9);
        dst.Fp[r] = (double)P.Fp[3 * (c % 3) + c / 3][inv[r / 9]];
    } else if ((r -= sP) < sV) {
        dst.vol[r] = (double)P.vol[inv[r]];
    } else if ((r -= sV) < sQ) {
        dst.plastic[r] = (double)P.plastic[inv[r]];
    }
}

// FP32 SoA -> host-layout doubles for ids [id_lo, id_lo + count), one thread per
// destination double (coalesced writes into pinned host memory); inv[id] = slot.
__global__ void k_download(long total, int count, int mode, const int32_t* __restrict__ inv, int id_lo,
                           double* __restrict__ dst, const float* s0, const float* s1, const float* s2,
                           const float* s3, const float* s4, const float* s5, const float* s6, const float* s7,
                           const float* s8) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const float* s[9] = {s0, s1, s2, s3, s4, s5, s6, s7, s8};
    int k, p;
    if (mode == 2) {
        p = (int)(e / 9);
        const int r = (int)(e % 9);
        k = 3 * (r % 3) + r / 3;
    } else if (mode == 4) {
        const int t = (int)(e / count);
        p = (int)(e % count);
        k = 3 * (t % 3) + t / 3;
    } else {
        k = (int)(e / count);
        p = (int)(e % count);
    }
    dst[e] = (double)s[k][inv[id_lo + p]];
}

__global__ void k_init_particles(int n, PArrays cur, const uint8_t* __restrict__ mat_in, int has_fp, int track_fp,
                                 int id0, int fixed_mat, const int32_t* __restrict__ map) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int p = map ? map[q] : id0 + q;  // slot
    cur.id[p] = id0 + q;
    int mat = fixed_mat >= 0 ? fixed_mat : (mat_in ? mat_in[q] : kSand);
    cur.mat[p] = (uint8_t)mat;
    if (!has_fp && track_fp)
        for (int k = 0; k < 9; ++k) cur.Fp[k][p] = (k % 4 == 0) ? 1.0f : 0.0f;
}

// snow particles carry J_P = det F_P in `plastic` when F_P is not tracked
__global__ void k_snow_jp(int n, PArrays cur, const double* __restrict__ Fp, const int32_t* __restrict__ map) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int p = map ? map[q] : q;
    if (cur.mat[p] != kSnow) return;
    double A[9];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) A[3 * a + b] = Fp ? Fp[9l * q + a + 3 * b] : (a == b ? 1.0 : 0.0);
    cur.plastic[p] = (float)mat_det(A);
}

// upload validation: largest mass (bit pattern of a non-negative double is monotonic),
// bad masses (negative, NaN, inf) and unknown material tags; out = {max bits, bad}
__global__ void k_check_upload(int n, const double* __restrict__ m, const uint8_t* __restrict__ mat,
                               unsigned long long* out) {
    unsigned long long mx = 0ull, bad = 0ull;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = m[i];
        if (!(v >= 0.0) || !isfinite(v)) bad = 1ull;
        else if (v > 0.0) mx = max(mx, (unsigned long long)__double_as_longlong(v));
        if (mat && mat[i] > kSand) bad = 1ull;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (mx) atomicMax(out, mx);
        if (bad) atomicOr(out + 1, bad);
    }
}

// inverse of the id map of the current order: inv[id[j]] = j
__global__ void k_inverse_ids(int n, const int32_t* __restrict__ id, int32_t* __restrict__ inv) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) inv[id[j]] = j;
}

// dense grid readback in reference order (mode 0: P2G state; 1: after grid update)
__global__ void k_grid_dense(KParams P, GArrays G, double* mass, double* vel, double* vbf) {
    const int nact = *G.nactive;
    const long total = (long)nact * 64;
    const long ng = (long)P.res[0] * P.res[1] * P.res[2];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const uint32_t blk = (uint32_t)G.active[i >> 6];
        const uint32_t node = (blk << 6) | (uint32_t)(i & 63);
        uint32_t bx = blk % (uint32_t)P.nb[0], r = blk / (uint32_t)P.nb[0];
        uint32_t by = r % (uint32_t)P.nb[1], bz = r / (uint32_t)P.nb[1];
        int ix = (int)(4 * bx + (i & 3)) - 4, iy = (int)(4 * by + ((i >> 2) & 3)) - 4,
            iz = (int)(4 * bz + ((i >> 4) & 3)) - 4;
        if (ix < 0 || iy < 0 || iz < 0 || ix >= P.res[0] || iy >= P.res[1] || iz >= P.res[2]) continue;
        long idx = ((long)iz * P.res[1] + iy) * P.res[0] + ix;
        float4 v = G.vel[node];
        if (mass) mass[idx] = v.w;
        if (vel) { vel[idx] = v.x; vel[ng + idx] = v.y; vel[2 * ng + idx] = v.z; }
        if (vbf) {
            float4 b = G.vbf[node];
            vbf[idx] = b.x; vbf[ng + idx] = b.y; vbf[2 * ng + idx] = b.z;
        }
    }
}

// ===================================================================================
// host launchers
static inline int blocks_for(long n, int t) { return (int)((n + t - 1) / t); }

// A launch that may overlap the tail of the previous kernel in the stream (the
// kernel waits for it in pdl_entry before touching memory): hides the launch
// latency between the kernels of a step.
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

void launch_keys(const KParams& P, const PArrays& cur, int n, uint32_t* keys, DevStats* st, cudaStream_t s) {
    if (n > 0) k_keys<<<blocks_for(n, 256), 256, 0, s>>>(P, cur, n, keys, st);
}
void launch_p2g(const KParams& P, const PArrays& cur, const uint32_t* keys, const int32_t* perm, int n,
                const GArrays& G, int32_t* slot_of, int32_t* curidx_of, cudaStream_t s) {
    // particles per warp: the particles spread evenly over the fewest waves of the
    // device's resident warps with at most kP2GMaxChunk each, rounded up to a
    // multiple of 32 (whole batches)
    static const long slots = [] {  // resident warps of k_p2g on the device
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_p2g, kP2GThreads, 0);
        return (long)std::max(1, sms * per) * (kP2GThreads / 32);
    }();
    const long waves = std::max(1L, ((long)n + slots * kP2GMaxChunk - 1) / (slots * kP2GMaxChunk));
    const long per_warp = ((long)n + waves * slots - 1) / (waves * slots);
    const int chunk = (int)std::min((long)kP2GMaxChunk, std::max(32L, (per_warp + 31) / 32 * 32));
    const long hw = ((long)n + chunk - 1) / chunk;
    if (n > 0)
        k_p2g<<<blocks_for(hw, kP2GThreads / 32), kP2GThreads, 0, s>>>(P, cur, keys, perm, n, chunk, G, slot_of,
                                                                        curidx_of);
}
void launch_normalize(const KParams& P, const GArrays& G, DevStats* st, int grid_blocks, cudaStream_t s) {
    launch_pdl(k_normalize, grid_blocks, 256, 0, s, P, G, st);
}
void launch_cloth_force(const KParams& P, const PArrays& cur, const MeshArrays& M, float dt_force, cudaStream_t s) {
    // the cloth forces launch after the normalisation has completed: early, their
    // small blocks filled the SMs beside the one-wave normalisation and slowed the
    // 8,388,608-item sand + cloth step by 2% (and the cloth drape's by 3%)
    if (M.nf > 0) k_cloth_force<<<blocks_for(M.nf, 128), 128, 0, s>>>(P, cur, M, dt_force);
}
void launch_force(const KParams& P, const PArrays& cur, const uint32_t* keys, const int32_t* perm, int n,
                  const GArrays& G, float dt_force, DevStats* st, const MeshArrays& M, cudaStream_t s,
                  int32_t* fp64_list) {
    long warps = (n + 31) / 32;
    if (n > 0) {
        launch_pdl(k_force, blocks_for(warps, kFrcThreads / 32), kFrcThreads, 0, s, P, cur, keys, perm, n, G, dt_force,
                   st, M, fp64_list, n);
        launch_pdl(k_force_fp64, 8, 128, 0, s, P, cur, G, dt_force, st, (const int32_t*)fp64_list, n);
    }
}
void launch_grid(const KParams& P, const GArrays& G, float dt_force, int write_force, double* force_out,
                 int grid_blocks, cudaStream_t s) {
    launch_pdl(k_grid, grid_blocks, 256, 0, s, P, G, dt_force, write_force, force_out);
}
void launch_grid_clear(const GArrays& G, int grid_blocks, cudaStream_t s) {
    k_grid_clear<<<grid_blocks, 256, 0, s>>>(G);
}
void launch_g2p(const KParams& P, const PArrays& cur, const PArrays& nxt, const int32_t* perm, int n,
                const GArrays& G, float dt, uint32_t* keys_next, DevStats* st, cudaStream_t s, const Harvest& H,
                bool learned, const uint32_t* keys_sorted, const MlpQueue& Qu) {
    if (n <= 0) return;
    if (learned)
        launch_pdl(k_g2p<true>, blocks_for(n, 128), 128, 0, s, P, cur, nxt, perm, n, G, dt, keys_next, st, H,
                   keys_sorted, Qu);
    else
        launch_pdl(k_g2p<false>, blocks_for(n, 128), 128, 0, s, P, cur, nxt, perm, n, G, dt, keys_next, st, H,
                   keys_sorted, Qu);
}
void launch_mlp_finish(const KParams& P, const PArrays& cur, const PArrays& nxt, const MlpQueue& Qu, DevStats* st,
                       const MlpParams& mlp, float tol_rel, float tol_abs, cudaStream_t s) {
    constexpr int smem = kMlpSmemBytes + (kFinThreads / 32) * kMlpWarpBytes;
    // resident finisher blocks of the device, looked up once (the attribute is set
    // with it, before the first launch)
    static const int resident = [] {
        cudaFuncSetAttribute(k_mlp_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlp_finish, kFinThreads, smem);
        return std::max(1, sms * std::max(per_sm, 1));
    }();
    const int blocks = std::min(blocks_for(Qu.cap, kFinThreads), resident);
    launch_pdl(k_mlp_finish, blocks, kFinThreads, smem, s, P, cur, nxt, Qu, st, mlp, tol_rel, tol_abs);
}
void launch_cloth_g2p(const KParams& P, const PArrays& cur, const PArrays& nxt, const GArrays& G, const MeshArrays& M,
                      float dt, uint32_t* keys_next, DevStats* st, const Harvest& H, const MlpParams* mlp,
                      float tol_rel, float tol_abs, cudaStream_t s) {
    if (M.nf <= 0) return;
    constexpr int kClothMlpSmem = kMlpSmemBytes + 4 * kMlpWarpBytes;
    const int smem = mlp ? kClothMlpSmem : 0;
    if (mlp) {
        static const bool attr_set = [] {  // once per process, before the first learned launch
            cudaFuncSetAttribute(k_cloth_g2p, cudaFuncAttributeMaxDynamicSharedMemorySize, kClothMlpSmem);
            return true;
        }();
        (void)attr_set;
    }
    launch_pdl(k_cloth_g2p, blocks_for(M.nf, 128), 128, smem, s, P, cur, nxt, G, M, dt, keys_next, st, H,
               mlp ? *mlp : MlpParams{}, mlp ? 1 : 0, tol_rel, tol_abs);
}
void launch_volumes(const KParams& P, const PArrays& cur, const int32_t* perm, int n, const GArrays& G,
                    cudaStream_t s) {
    if (n > 0) k_volumes<<<blocks_for(n, 128), 128, 0, s>>>(P, cur, perm, n, G);
}
void launch_upload(int n, int mode, const double* src, float* const* dst, cudaStream_t s, const int32_t* map) {
    const int per = mode == 3 ? 1 : (mode == 0 ? 3 : 9);
    const long total = (long)per * n;
    if (total > 0)
        k_upload<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(total, n, mode, src, dst[0], dst[1], dst[2], dst[3],
                                                                 dst[4], dst[5], dst[6], dst[7], dst[8], map);
}
void launch_upload_particles(int n, const UploadSrc& src, const PArrays& P, const int32_t* map, int track_fp,
                             unsigned long long* check, cudaStream_t s) {
    const long total = 25l * n + ((track_fp && src.Fp) ? 9l * n : 0);
    if (n > 0)
        k_upload_particles<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n, src, P, map, track_fp, check);
}
void launch_download_particles(int n, const DownloadDst& dst, const PArrays& P, const int32_t* inv, cudaStream_t s) {
    const long total = (long)n * ((dst.x ? 3 : 0) + (dst.v ? 3 : 0) + (dst.B ? 9 : 0) + (dst.Fe ? 9 : 0) +
                                  (dst.Fp ? 9 : 0) + (dst.vol ? 1 : 0) + (dst.plastic ? 1 : 0));
    if (total > 0) k_download_particles<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n, dst, P, inv);
}
void launch_fixed_vertices(const KParams& P, const PArrays& cur, const GArrays& G, const MeshArrays& M,
                           const int32_t* fixed, int nfixed, cudaStream_t s) {
    const long threads = (long)nfixed * 64 * 27;
    if (threads > 0) k_fixed_vertices<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(P, cur, G, M, fixed, nfixed);
}
void launch_solve_dt(SolveState* S, int phase, cudaStream_t s) { k_solve_dt<<<1, 1, 0, s>>>(S, phase); }
void launch_query_weights(const KParams& P, const PArrays& cur, const int32_t* inv, const int64_t* ids, int count,
                          int64_t* nodes, double* w, double* g, cudaStream_t s) {
    const long threads = (long)count * 64;
    if (threads > 0) k_query_weights<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(P, cur, inv, ids, count, nodes, w, g);
}
void launch_check_upload(int n, const double* m, const uint8_t* mat, unsigned long long* out, cudaStream_t s) {
    if (n > 0) k_check_upload<<<std::min(1024, blocks_for(n, 256)), 256, 0, s>>>(n, m, mat, out);
}
void launch_inverse_ids(int n, const int32_t* id, int32_t* inv, cudaStream_t s) {
    if (n > 0) k_inverse_ids<<<blocks_for(n, 256), 256, 0, s>>>(n, id, inv);
}
void launch_download(int count, int mode, const int32_t* inv, int id_lo, double* dst, float* const* src,
                     cudaStream_t s) {
    const int per = mode == 3 ? 1 : (mode == 0 ? 3 : 9);
    const long total = (long)per * count;
    if (total > 0)
        k_download<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(total, count, mode, inv, id_lo, dst, src[0], src[1],
                                                                   src[2], src[3], src[4], src[5], src[6], src[7],
                                                                   src[8]);
}
void launch_init_particles(int n, const PArrays& cur, const uint8_t* mat, int has_fp, int track_fp, cudaStream_t s,
                           int id0, int fixed_mat, const int32_t* map) {
    if (n > 0) k_init_particles<<<blocks_for(n, 256), 256, 0, s>>>(n, cur, mat, has_fp, track_fp, id0, fixed_mat, map);
}
void launch_snow_jp(int n, const PArrays& cur, const double* Fp, cudaStream_t s, const int32_t* map) {
    if (n > 0) k_snow_jp<<<blocks_for(n, 256), 256, 0, s>>>(n, cur, Fp, map);
}
void launch_grid_dense(const KParams& P, const GArrays& G, double* mass, double* vel, double* vbf, int grid_blocks,
                       cudaStream_t s) {
    k_grid_dense<<<grid_blocks, 256, 0, s>>>(P, G, mass, vel, vbf);
}

}  // namespace aep
