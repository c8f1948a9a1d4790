// aep_noalloc.cu -- aep_p2g_noalloc: particle-to-grid transfer into buffers the
// caller already owns, for callers that must not allocate GPU memory.
//
// Who needs it: code that runs inside a host application which owns every byte
// of device memory through its own pool (a renderer or another framework with a
// caching allocator, where a stray cudaMalloc breaks its budget or fragments its
// heap), and real-time loops that cannot pay for the device-wide synchronisation
// a cudaMalloc/cudaFree implies.  Such callers pass
// their particle arrays and their output grid as device pointers; the only other
// memory this path touches is a fixed scratch array compiled into the library.
//
// The scratch is a file-scope __device__ array: each GPU that loads libaep.so
// holds it (AEP_NOALLOC_MAX_NODES * 32 bytes, about 12 MB) until the process
// exits.  Host code never uses the array's name as a pointer (on the host it is
// only a stand-in, not a device address); its device address is looked up once
// per device with cudaGetSymbolAddress and passed to the kernels.
#include <cmath>
#include <mutex>

#include "../../include/aep.h"
#include "aep_device.cuh"

namespace {

using namespace aep;

// int64 fixed-point accumulators (mass, momentum x, y, z) of the padded, blocked grid
__device__ __align__(256) unsigned long long g_p2g_noalloc_scratch[4ull * AEP_NOALLOC_MAX_NODES];

constexpr int kMaxDevices = 256;
std::mutex g_setup_mutex;
unsigned long long* g_scratch_on_device[kMaxDevices] = {};

// Device address of the scratch on the current device; looked up on the first
// call made on each device (with that device current) and kept for the life of
// the process (not valid after a cudaDeviceReset of that device).
cudaError_t scratch_for_current_device(unsigned long long** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_on_device[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_p2g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_on_device[dev] = static_cast<unsigned long long*>(p);
    }
    *out = g_scratch_on_device[dev];
    return cudaSuccess;
}

constexpr int kThreads = 128;
constexpr int kChunk = 64;  // particles per half-warp stream

struct alignas(16) Prep {
    float b[3];
    float m;
    float Mh[9];
    float pad0;
    long long T;
    float wx[4], wy[4], wz[4];
    int base[3];
    uint32_t key;
};

// Particles arrive in the caller's order, so equal keys need not be adjacent: a
// particle starts a new run whenever its key differs from the previous one's.
__device__ __forceinline__ unsigned heads_of(unsigned hmask, int l, uint32_t key, uint32_t carried) {
    const uint32_t prev = __shfl_up_sync(hmask, key, 1, 16);
    const bool head = key != (l == 0 ? carried : prev);
    return __ballot_sync(hmask, head) >> (threadIdx.x & 16);
}

// Same transfer as the step's P2G (HybridSolver.cpp:113-231), for particles in the
// caller's order (no sort): runs of equal base node are simply shorter.
__global__ void __launch_bounds__(kThreads) k_p2g_noalloc(KParams P, const float* __restrict__ x,
                                                          const float* __restrict__ v, const float* __restrict__ B,
                                                          const float* __restrict__ m, int n,
                                                          unsigned long long* __restrict__ acc) {
    __shared__ Prep sm[kThreads / 16][16];
    const int hw = threadIdx.x >> 4, l = threadIdx.x & 15;
    const unsigned hmask = 0xFFFFu << (threadIdx.x & 16);
    const int ox = l & 3, oy = l >> 2;
    const long chunk0 = ((long)blockIdx.x * (kThreads / 16) + hw) * kChunk;
    if (chunk0 >= n) return;
    const int cnt_total = (int)min((long)kChunk, (long)n - chunk0);
    float am[4] = {0, 0, 0, 0}, ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0}, az[4] = {0, 0, 0, 0};
    uint32_t run_key = kInvalidKey;
    int rb[3] = {0, 0, 0};
    long long run_T = 0;
    auto flush = [&]() {
        if (run_key == kInvalidKey) return;
        long long mf[4], S = 0;
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) {
            mf[oz] = __float2ll_rn(am[oz] * P.mass_scale);
            S += mf[oz];
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) S += __shfl_xor_sync(hmask, S, o, 16);
        if (l == 5) mf[1] += run_T - S;  // exact mass, as in the step's P2G
        run_T = 0;
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) {
            if (mf[oz] != 0) {
                unsigned long long* a = acc + 4ull * node_index(P, rb[0] + ox, rb[1] + oy, rb[2] + oz);
                atomicAdd(a + 0, (unsigned long long)mf[oz]);
                atomicAdd(a + 1, to_fixed(ax[oz], P.mom_scale));
                atomicAdd(a + 2, to_fixed(ay[oz], P.mom_scale));
                atomicAdd(a + 3, to_fixed(az[oz], P.mom_scale));
            }
            am[oz] = ax[oz] = ay[oz] = az[oz] = 0.0f;
        }
    };
    for (int b0 = 0; b0 < cnt_total; b0 += 16) {
        const long j = chunk0 + b0 + l;
        if (b0 + l < cnt_total) {
            Prep& s = sm[hw][l];
            const float xp[3] = {x[j], x[n + j], x[2l * n + j]};
            const float mp = m[j];
            int cell[3];
            float f[3], w[3][4], dw[3][4];
            locate(P, xp[0], xp[1], xp[2], cell, f);
            const bool trunc = particle_weights(P, cell, f, w, dw);
            float wsum = 1.0f;
            if (trunc)
                wsum = (w[0][0] + w[0][1] + w[0][2] + w[0][3]) * (w[1][0] + w[1][1] + w[1][2] + w[1][3]) *
                       (w[2][0] + w[2][1] + w[2][2] + w[2][3]);
            s.T = __float2ll_rn(mp * wsum * P.mass_scale);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                float t = mp * v[(long)a * n + j];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float mh = mp * P.apic[c] * B[(long)a * 3 * n + (long)c * n + j];
                    s.Mh[3 * a + c] = mh;
                    t -= mh * (1.0f + f[c]);
                }
                s.b[a] = t;
            }
            s.m = mp;
#pragma unroll
            for (int o = 0; o < 4; ++o) { s.wx[o] = w[0][o]; s.wy[o] = w[1][o]; s.wz[o] = w[2][o]; }
#pragma unroll
            for (int a = 0; a < 3; ++a) s.base[a] = cell[a] + 3;
            s.key = make_key(P, cell);
        }
        __syncwarp(hmask);
        const int cnt = min(16, cnt_total - b0);
        const unsigned heads = heads_of(hmask, l, b0 + l < cnt_total ? sm[hw][l].key : kInvalidKey, run_key);
        for (int t = 0; t < cnt; ++t) {
            const Prep& s = sm[hw][t];
            if ((heads >> t) & 1u) {
                flush();
                run_key = s.key;
                rb[0] = s.base[0]; rb[1] = s.base[1]; rb[2] = s.base[2];
            }
            run_T += s.T;
            const float wxy = s.wx[ox] * s.wy[oy];
            const float fx = (float)ox, fy = (float)oy;
            float tx = s.b[0] + s.Mh[0] * fx + s.Mh[1] * fy;
            float ty = s.b[1] + s.Mh[3] * fx + s.Mh[4] * fy;
            float tz = s.b[2] + s.Mh[6] * fx + s.Mh[7] * fy;
#pragma unroll
            for (int oz = 0; oz < 4; ++oz) {
                const float w = wxy * s.wz[oz];
                am[oz] = fmaf(w, s.m, am[oz]);
                ax[oz] = fmaf(w, tx, ax[oz]);
                ay[oz] = fmaf(w, ty, ay[oz]);
                az[oz] = fmaf(w, tz, az[oz]);
                tx += s.Mh[2];
                ty += s.Mh[5];
                tz += s.Mh[8];
            }
        }
        __syncwarp(hmask);
    }
    flush();
}

// dense outputs in reference node order: mass and v = p / m (HybridSolver.cpp:233-240)
__global__ void k_dense_out(KParams P, const unsigned long long* __restrict__ acc, float* __restrict__ mass_out,
                            float* __restrict__ vel_out) {
    const long ng = (long)P.res[0] * P.res[1] * P.res[2];
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < ng; idx += (long)gridDim.x * blockDim.x) {
        const int i = (int)(idx % P.res[0]);
        const int j = (int)((idx / P.res[0]) % P.res[1]);
        const int k = (int)(idx / ((long)P.res[0] * P.res[1]));
        const longlong2* a2 = reinterpret_cast<const longlong2*>(acc + 4ull * node_index(P, i + 4, j + 4, k + 4));
        const longlong2 a = a2[0], b = a2[1];
        float mass = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
        if (a.x > 0) {
            mass = __ll2float_rn(a.x) * P.inv_mass_scale;
            const float inv = 1.0f / mass;
            vx = __ll2float_rn(a.y) * P.inv_mom_scale * inv;
            vy = __ll2float_rn(b.x) * P.inv_mom_scale * inv;
            vz = __ll2float_rn(b.y) * P.inv_mom_scale * inv;
        }
        mass_out[idx] = mass;
        vel_out[idx] = vx;
        vel_out[ng + idx] = vy;
        vel_out[2 * ng + idx] = vz;
    }
}

}  // namespace

extern "C" aep_status aep_p2g_noalloc(const aep_grid_desc* grid, int64_t n, const float* x, const float* v,
                                      const float* B, const float* m, double mass_ref, float* mass_out,
                                      float* vel_out, void* cuda_stream) {
    if (!grid || !x || !v || !B || !m || !mass_out || !vel_out) return AEP_INVALID_ARG;
    if (n <= 0 || n > (int64_t)INT32_MAX / 2 || !(mass_ref > 0.0) || !std::isfinite(mass_ref)) return AEP_INVALID_ARG;
    KParams P{};
    double h[3], hmin = 1e300;
    long long padded_nodes = 64;
    for (int a = 0; a < 3; ++a) {
        if (grid->res[a] < 1 || !(grid->max[a] > grid->min[a])) return AEP_INVALID_ARG;
        h[a] = (grid->max[a] - grid->min[a]) / grid->res[a];
        hmin = std::fmin(hmin, h[a]);
        P.min[a] = (float)grid->min[a];
        P.h[a] = (float)h[a];
        P.inv_h[a] = (float)(1.0 / h[a]);
        P.res[a] = grid->res[a];
        P.nb[a] = ((grid->res[a] + 2) >> 2) + 2;  // same padded layout as the step
        padded_nodes *= P.nb[a];
    }
    if (padded_nodes > (long long)AEP_NOALLOC_MAX_NODES) return AEP_CAPACITY;
    for (int a = 0; a < 3; ++a) P.apic[a] = (float)(3.0 / hmin / hmin * h[a]);
    aep_params prm;
    aep_default_params(&prm);
    const double ml = std::ldexp(1.0, prm.mass_bits) / mass_ref, pl = std::ldexp(1.0, prm.momentum_bits) / mass_ref;
    P.mass_scale = (float)ml;
    P.inv_mass_scale = (float)(1.0 / ml);
    P.mom_scale = (float)pl;
    P.inv_mom_scale = (float)(1.0 / pl);

    unsigned long long* scratch = nullptr;
    if (scratch_for_current_device(&scratch) != cudaSuccess) return AEP_CUDA_ERROR;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    // the array keeps the previous call's sums: clear the part this grid uses
    if (cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * 4ull * (size_t)padded_nodes, s) != cudaSuccess)
        return AEP_CUDA_ERROR;
    const long halfwarps = (n + kChunk - 1) / kChunk;
    k_p2g_noalloc<<<(int)((halfwarps + kThreads / 16 - 1) / (kThreads / 16)), kThreads, 0, s>>>(P, x, v, B, m, (int)n,
                                                                                             scratch);
    const long ng = (long)grid->res[0] * grid->res[1] * grid->res[2];
    k_dense_out<<<(int)std::fmin(4096.0, (double)((ng + 255) / 256)), 256, 0, s>>>(P, scratch, mass_out, vel_out);
    return cudaGetLastError() == cudaSuccess ? AEP_OK : AEP_CUDA_ERROR;
}
