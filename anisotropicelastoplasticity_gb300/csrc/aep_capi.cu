// aep_capi.cu -- the C-ABI of include/aep.h: solver handle, device memory,
// layout conversion at the boundary, and the per-step launch sequence.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/aep.h"
#include "aep_kernels.h"

using namespace aep;

namespace {

constexpr int kFloatArrays = 3 + 3 + 9 + 9 + 3;  // x, v, B, F, m, vol, plastic
constexpr int kFpArrays = 9;

struct ParticleSet {
    float* f = nullptr;
    uint8_t* mat = nullptr;
    int32_t* id = nullptr;
};

}  // namespace

struct aep_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    aep_grid_desc grid{};
    aep_params prm{};
    KParams kp{};
    int64_t n = 0, cap = 0;   // n = np + nv + nf particle slots
    int64_t np = 0, nv = 0, nf = 0;
    bool stepped_since_upload = false;
    // LagrangianMesh device state
    int32_t* faces = nullptr;
    float* rest = nullptr;
    float* estress = nullptr;
    unsigned long long* vforce = nullptr;
    int32_t* slot_of = nullptr;
    int32_t* curidx_of = nullptr;
    double cloth[5] = {0, 0, 0, 0, 0};  // mu, lambda, shear, stiffness, friction
    // training-pair harvest and learned return map
    float* harvest = nullptr;
    unsigned long long* harvest_count = nullptr;
    int64_t harvest_cap = 0;
    int32_t harvest_stride = 1;
    const aep_mlp* mlp = nullptr;
    double learned_tol = 1e-3;  // learned-map check: relative bound
    double learned_abs = 0x1p-23;  // and absolute bound (ln-strain units)
    void* queue_mem = nullptr;     // rows queued for the network (MlpQueue), one per particle
    MlpQueue queue{};
    ParticleSet set[2];
    PArrays P[2];
    int cur = 0;
    uint32_t* keys = nullptr;
    uint32_t* keys_sorted = nullptr;
    int32_t* iota = nullptr;
    int32_t* perm = nullptr;
    int32_t* inv = nullptr;  // id -> slot of the current order (readback); during a step, the
                             // force pass's list of particles redone in FP64
    void* sort_tmp = nullptr;
    size_t sort_bytes = 0;
    int key_bits = 0;
    // incremental ordering (aep_sort.cu): mover list, sorted mover keys, scratch
    uint32_t* order_mem = nullptr;  // one allocation for the arrays below
    uint32_t* mk = nullptr;
    int32_t* mj = nullptr;
    uint32_t* mkeys = nullptr;
    int32_t* mslot = nullptr;
    int32_t* mpos = nullptr;
    uint32_t* order_scratch = nullptr;
    unsigned long long* check_host = nullptr;  // pinned, 2 words: upload validation result
    bool prev_sorted = false;  // keys_sorted holds an ascending array of the current n
    int since_order = 0;       // steps since the last ordering (reorder_interval)
    int64_t orderings = 0;     // orderings run (stats)
    const uint32_t* step_keys = nullptr;  // this step's keys and permutation: the new
    const int32_t* step_perm = nullptr;   // ordering's, or the current keys and identity
    void* order_graph = nullptr;  // the incremental ordering, captured (aep_sort.cu)
    int order_graph_n = -1;
    cudaStream_t capture_stream = nullptr;
    GArrays G{};
    size_t nnodes = 0;
    int nblocks = 0;
    DevStats* dstats = nullptr;
    double* staging = nullptr;
    size_t staging_bytes = 0;
    double* dforce = nullptr;  // dense f_i after a force-stage stop
    bool have_particles = false, keys_valid = false, dirty_grid = false;
    int last_stage = 0;
    double m_max = 1.0;
    double mesh_m_max = 0.0;  // heaviest mesh vertex or element (aep_set_mesh)
    int64_t steps = 0;
    int grid_blocks = 1024;
    cudaStream_t own_stream = nullptr;
    // phase timing: a ring of per-step event sets, folded into `phase_ms` lazily
    bool profiling = false;
    static constexpr int kRing = 32;
    cudaEvent_t ev[kRing][AEP_NUM_PHASES + 1] = {};
    bool ev_pending[kRing] = {};
    int ev_slot = 0;
    double phase_ms[AEP_NUM_PHASES] = {};
    int64_t timed_steps = 0;
    unsigned long long* check = nullptr;  // upload validation result
    // fixed cloth vertices (vertex indices 0..nv-1)
    int32_t* fixed = nullptr;
    int nfixed = 0;
    // adaptive solve loop: device state, its pinned host copy, callback
    SolveState* solve = nullptr;
    SolveState* solve_host = nullptr;
    DevStats* stats_host = nullptr;
    aep_solve_fn solve_fn = nullptr;
    void* solve_user = nullptr;
    int64_t max_steps = 0;
    aep_solve_state solve_last{};
    std::string err;
};

namespace {

aep_status fail(aep_solver* s, aep_status st, const std::string& msg) {
    if (s) s->err = msg;
    return st;
}

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(s, e_ == cudaErrorMemoryAllocation ? AEP_OUT_OF_MEMORY : AEP_CUDA_ERROR,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                            \
    } while (0)

#define CKLAUNCH() CK(cudaGetLastError())

void lame(double E, double nu, double& lambda, double& mu) {
    lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
    mu = E / 2.0 / (1.0 + nu);
}

void fill_kparams(aep_solver* s) {
    KParams& k = s->kp;
    const aep_grid_desc& g = s->grid;
    const aep_params& p = s->prm;
    double h[3], hmin = 1e300;
    for (int a = 0; a < 3; ++a) {
        h[a] = (g.max[a] - g.min[a]) / g.res[a];
        hmin = std::min(hmin, h[a]);
        k.min[a] = (float)g.min[a];
        k.h[a] = (float)h[a];
        k.inv_h[a] = (float)(1.0 / h[a]);
        k.res[a] = g.res[a];
        // base node (padded) <= res + 2; its block and the next one must exist
        k.nb[a] = ((g.res[a] + 2) >> 2) + 2;
    }
    for (int a = 0; a < 3; ++a) k.apic[a] = (float)(3.0 / hmin / hmin * h[a]);
    k.cell_volume = (float)(h[0] * h[1] * h[2]);
    double ml = std::ldexp(1.0, p.mass_bits) / s->m_max, pl = std::ldexp(1.0, p.momentum_bits) / s->m_max;
    k.mass_scale = (float)ml;
    k.inv_mass_scale = (float)(1.0 / ml);
    k.mom_scale = (float)pl;
    k.inv_mom_scale = (float)(1.0 / pl);
    double l, m;
    lame(p.snow.E, p.snow.nu, l, m);
    k.snow_mu = (float)m;
    k.snow_lambda = (float)l;
    k.snow_xi = (float)p.snow.xi;
    k.snow_lo = (float)(1.0 - p.snow.theta_c);
    k.snow_hi = (float)(1.0 + p.snow.theta_s);
    k.snow_lnlo = (float)std::log((double)k.snow_lo);
    k.snow_lnhi = (float)std::log((double)k.snow_hi);
    lame(p.sand.E, p.sand.nu, l, m);
    k.sand_mu = (float)m;
    k.sand_lambda = (float)l;
    k.sand_h0 = (float)p.sand.h0;
    k.sand_h1 = (float)p.sand.h1;
    k.sand_h2 = (float)p.sand.h2;
    k.sand_h3 = (float)p.sand.h3;
    k.sand_k = (float)((3.0 * l + 2.0 * m) / 2.0 / m);
    for (int a = 0; a < 3; ++a) k.gravity[a] = (float)p.gravity[a];
    k.friction = (float)p.friction;
    k.friction_bug = p.friction_bug;
    k.particle_damp = (float)p.particle_damp;
    k.mesh_damp = (float)p.mesh_damp;
    k.track_fp = p.track_plastic_F;
    k.fp64_apex = p.fp64_apex;
}

MeshArrays mesh_arrays(aep_solver* s) {
    MeshArrays M{};
    M.nv = (int)s->nv;
    M.nf = (int)s->nf;
    M.vbase = (int)s->np;
    M.ebase = (int)(s->np + s->nv);
    M.faces = s->faces;
    M.rest = s->rest;
    M.estress = s->estress;
    M.vforce = s->vforce;
    M.slot_of = s->slot_of;
    M.curidx_of = s->curidx_of;
    M.mu = (float)s->cloth[0];
    M.lambda = (float)s->cloth[1];
    M.shear = (float)s->cloth[2];
    M.stiffness = (float)s->cloth[3];
    M.friction = (float)s->cloth[4];
    M.damp = (float)s->prm.mesh_damp;
    M.volume_weighting = s->prm.cloth_volume_weighting;
    return M;
}

void free_mesh(aep_solver* s) {
    cudaFree(s->faces);
    cudaFree(s->rest);
    cudaFree(s->estress);
    cudaFree(s->vforce);
    cudaFree(s->slot_of);
    cudaFree(s->curidx_of);
    s->faces = nullptr;
    s->rest = s->estress = nullptr;
    s->vforce = nullptr;
    s->slot_of = s->curidx_of = nullptr;
    s->nv = s->nf = 0;
    s->mesh_m_max = 0.0;
    cudaFree(s->fixed);
    s->fixed = nullptr;
    s->nfixed = 0;
}

void build_parrays(aep_solver* s, int which) {
    PArrays& P = s->P[which];
    float* f = s->set[which].f;
    size_t c = (size_t)s->cap;
    int k = 0;
    for (int a = 0; a < 3; ++a) P.x[a] = f + c * k++;
    for (int a = 0; a < 3; ++a) P.v[a] = f + c * k++;
    for (int a = 0; a < 9; ++a) P.B[a] = f + c * k++;
    for (int a = 0; a < 9; ++a) P.F[a] = f + c * k++;
    P.m = f + c * k++;
    P.vol = f + c * k++;
    P.plastic = f + c * k++;
    for (int a = 0; a < 9; ++a) P.Fp[a] = s->prm.track_plastic_F ? f + c * k++ : nullptr;
    P.mat = s->set[which].mat;
    P.id = s->set[which].id;
}

void free_particles(aep_solver* s) {
    for (int i = 0; i < 2; ++i) {
        cudaFree(s->set[i].f);
        cudaFree(s->set[i].mat);
        cudaFree(s->set[i].id);
        s->set[i] = ParticleSet{};
    }
    cudaFree(s->keys);
    cudaFree(s->keys_sorted);
    cudaFree(s->iota);
    cudaFree(s->perm);
    cudaFree(s->sort_tmp);
    cudaFree(s->staging);
    order_graph_destroy(s->order_graph);
    s->order_graph = nullptr;
    s->order_graph_n = -1;
    cudaFree(s->order_mem);
    cudaFree(s->inv);
    s->inv = nullptr;
    s->keys = s->keys_sorted = nullptr;
    s->iota = s->perm = nullptr;
    s->sort_tmp = nullptr;
    s->staging = nullptr;
    s->order_mem = s->mk = s->mkeys = s->order_scratch = nullptr;
    s->mj = s->mslot = s->mpos = nullptr;
    s->prev_sorted = false;
    s->cap = 0;
}

// Grow the particle buffers to n slots.  The first `keep` slots of set 0 (in id
// order, i.e. before any step) survive the reallocation.
aep_status ensure_capacity(aep_solver* s, int64_t n, int64_t keep = 0) {
    if (n <= s->cap) return AEP_OK;
    size_t nf = kFloatArrays + (s->prm.track_plastic_F ? kFpArrays : 0);
    ParticleSet old = s->set[0];
    int64_t oldcap = s->cap;
    s->set[0] = ParticleSet{};  // keep the old set 0 alive until copied
    free_particles(s);
    s->cap = n;
    for (int i = 0; i < 2; ++i) {
        CK(cudaMalloc(&s->set[i].f, sizeof(float) * nf * (size_t)n));
        CK(cudaMalloc(&s->set[i].mat, (size_t)n));
        CK(cudaMalloc(&s->set[i].id, sizeof(int32_t) * (size_t)n));
    }
    if (keep > 0 && old.f) {
        for (size_t k = 0; k < nf; ++k)
            CK(cudaMemcpy(s->set[0].f + k * (size_t)n, old.f + k * (size_t)oldcap, sizeof(float) * (size_t)keep,
                          cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(s->set[0].mat, old.mat, (size_t)keep, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(s->set[0].id, old.id, sizeof(int32_t) * (size_t)keep, cudaMemcpyDeviceToDevice));
    }
    cudaFree(old.f);
    cudaFree(old.mat);
    cudaFree(old.id);
    CK(cudaMalloc(&s->keys, sizeof(uint32_t) * (size_t)n));
    CK(cudaMalloc(&s->keys_sorted, sizeof(uint32_t) * (size_t)n));
    CK(cudaMalloc(&s->iota, sizeof(int32_t) * (size_t)n));
    CK(cudaMalloc(&s->perm, sizeof(int32_t) * (size_t)n));
    CK(cudaMalloc(&s->inv, sizeof(int32_t) * (size_t)n));
    s->sort_bytes = sort_temp_bytes((int)n, s->key_bits);
    CK(cudaMalloc(&s->sort_tmp, s->sort_bytes));
    // mover list and sorted mover keys (n / 4 + 1 each: more movers take the full sort)
    // and the ordering scratch
    const size_t mcap = (size_t)n / 4 + 1;
    CK(cudaMalloc(&s->order_mem, sizeof(uint32_t) * (5 * mcap + order_scratch_words((int)n))));
    s->mk = s->order_mem;
    s->mj = reinterpret_cast<int32_t*>(s->order_mem + mcap);
    s->mkeys = s->order_mem + 2 * mcap;
    s->mslot = reinterpret_cast<int32_t*>(s->order_mem + 3 * mcap);
    s->mpos = reinterpret_cast<int32_t*>(s->order_mem + 4 * mcap);
    s->order_scratch = s->order_mem + 5 * mcap;
    if (!s->check_host) CK(cudaMallocHost(&s->check_host, 2 * sizeof(unsigned long long)));
    s->prev_sorted = false;
    s->staging_bytes = sizeof(double) * 37 * (size_t)n;  // every field of one particle set at once
    CK(cudaMalloc(&s->staging, s->staging_bytes));
    if (!s->check) CK(cudaMalloc(&s->check, 2 * sizeof(unsigned long long)));
    std::vector<int32_t> io((size_t)n);
    for (int64_t i = 0; i < n; ++i) io[(size_t)i] = (int32_t)i;
    CK(cudaMemcpy(s->iota, io.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice));
    build_parrays(s, 0);
    build_parrays(s, 1);
    return AEP_OK;
}

// A device-usable alias of a caller pointer: page-locked host memory (read and
// written by the conversion kernels directly over the host link), device and
// managed memory; nullptr for pageable host memory, which goes through the
// staging buffer.
const void* device_alias(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged) return a.devicePointer;
    if (a.type == cudaMemoryTypeDevice) return p;
    return nullptr;
}

// A device pointer with the caller's `bytes` at `p`: the alias, or a copy in the
// staging buffer at `off` doubles
const void* device_source(aep_solver* s, const void* p, size_t bytes, size_t off, cudaError_t* err) {
    const void* a = device_alias(p);
    if (a) return a;
    double* st = s->staging + off;
    *err = cudaMemcpyAsync(st, p, bytes, cudaMemcpyHostToDevice, s->stream);
    return st;
}

// upload `count` doubles per item for items [id0, id0 + n) of set 0
// src: caller array of `count` doubles per item; `off` doubles into the staging
// buffer when src is pageable (distinct offsets let consecutive uploads proceed
// without waiting on each other)
aep_status upload(aep_solver* s, const double* src, int count, int mode, float* const* dst, int64_t n = -1,
                  int64_t id0 = 0, const int32_t* map = nullptr, size_t off = 0) {
    if (n < 0) n = s->n;
    cudaError_t e = cudaSuccess;
    const double* d_src =
        static_cast<const double*>(device_source(s, src, sizeof(double) * count * (size_t)n, off, &e));
    CK(e);
    float* d[9] = {};
    int nd = mode == 3 ? 1 : (mode == 0 ? 3 : 9);
    for (int k = 0; k < nd; ++k) d[k] = dst[k] + id0;
    launch_upload((int)n, mode, d_src, d, s->stream, map);
    CKLAUNCH();
    return AEP_OK;
}

// inverse of the current order's id map (inv[id] = slot), used by download()
aep_status prepare_download(aep_solver* s) {
    launch_inverse_ids((int)s->n, s->P[s->cur].id, s->inv, s->stream);
    CKLAUNCH();
    return AEP_OK;
}

// download ids [id_lo, id_hi) in id order (after prepare_download): straight into
// dst when it is page-locked or device memory, else through staging offset `off`
// (doubles) and a copy; the caller synchronises once after all fields
aep_status download(aep_solver* s, double* dst, int count, int mode, float* const* src, int64_t id_lo = 0,
                    int64_t id_hi = -1, size_t off = 0, bool sync = true) {
    if (id_hi < 0) id_hi = s->n;
    const int cnt = (int)(id_hi - id_lo);
    double* alias = static_cast<double*>(const_cast<void*>(device_alias(dst)));
    double* out = alias ? alias : s->staging + off;
    launch_download(cnt, mode, s->inv, (int)id_lo, out, src, s->stream);
    CKLAUNCH();
    if (!alias)
        CK(cudaMemcpyAsync(dst, out, sizeof(double) * count * (size_t)cnt, cudaMemcpyDeviceToHost, s->stream));
    if (sync) CK(cudaStreamSynchronize(s->stream));
    return AEP_OK;
}

aep_status check_overflow(aep_solver* s) {
    DevStats h;
    CK(cudaMemcpy(&h, s->dstats, sizeof(h), cudaMemcpyDeviceToHost));
    if (h.overflow) return fail(s, AEP_OVERFLOW, "fixed-point grid accumulator overflow");
    return AEP_OK;
}

aep_status fold_slot(aep_solver* s, int slot) {
    if (!s->ev_pending[slot]) return AEP_OK;
    CK(cudaEventSynchronize(s->ev[slot][AEP_NUM_PHASES]));
    for (int p = 0; p < AEP_NUM_PHASES; ++p) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->ev[slot][p], s->ev[slot][p + 1]));
        s->phase_ms[p] += ms;
    }
    s->ev_pending[slot] = false;
    s->timed_steps++;
    return AEP_OK;
}

inline void mark(aep_solver* s, int boundary) {
    if (s->profiling) cudaEventRecord(s->ev[s->ev_slot][boundary], s->stream);
}

// Order the current particles by key into keys_sorted / perm: incrementally from
// the last sorted keys (a captured graph whose branch is chosen on the device,
// aep_sort.cu), or a full radix sort when there are no sorted keys yet.
cudaError_t order_particles(aep_solver* s) {
    const int n = (int)s->n;
    if (!s->prm.full_sort && s->prev_sorted && n >= 4096) {
        if (!s->order_graph || s->order_graph_n != n) {
            order_graph_destroy(s->order_graph);
            s->order_graph = nullptr;
            if (!s->capture_stream) {
                cudaError_t e = cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking);
                if (e != cudaSuccess) return e;
            }
            OrderBuffers b{s->keys, s->keys_sorted, s->perm, s->iota, s->mk, s->mj, s->mkeys, s->mslot, s->mpos,
                           s->order_scratch, s->sort_tmp, s->sort_bytes, n, n / 4, s->key_bits, s->dstats};
            cudaError_t e = order_graph_build(&s->order_graph, s->capture_stream, b);
            if (e != cudaSuccess) return e;
            s->order_graph_n = n;
        }
        return order_graph_launch(s->order_graph, s->stream);
    }
    cudaError_t e = sort_pairs(s->sort_tmp, s->sort_bytes, s->keys, s->keys_sorted, s->iota, s->perm, n,
                               s->key_bits, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(&s->dstats->movers, 0xFF, sizeof(long long), s->stream);  // -1
    if (e == cudaSuccess) s->prev_sorted = true;
    return e;
}

// P2G of the current particle order (sort + scatter + normalisation)
aep_status run_p2g(aep_solver* s) {
    if (s->dirty_grid) {
        launch_grid_clear(s->G, s->grid_blocks, s->stream);
        CKLAUNCH();
        s->dirty_grid = false;
    }
    const PArrays& P = s->P[s->cur];
    CK(cudaMemsetAsync(s->dstats, 0, sizeof(DevStats), s->stream));
    mark(s, AEP_PHASE_SORT);
    if (!s->keys_valid) {
        launch_keys(s->kp, P, (int)s->n, s->keys, s->dstats, s->stream);
        CKLAUNCH();
        s->keys_valid = true;
    }
    // reorder_interval: the steps between two orderings keep the particles in their
    // slots (identity permutation) with the keys G2P wrote for the current positions
    const int interval = std::max(1, (int)s->prm.reorder_interval);
    if (s->prev_sorted && !s->prm.full_sort && s->n >= 4096 && s->since_order + 1 < interval) {
        ++s->since_order;
        s->step_keys = s->keys;
        s->step_perm = s->iota;
    } else {
        CK(order_particles(s));
        s->since_order = 0;
        ++s->orderings;
        s->step_keys = s->keys_sorted;
        s->step_perm = s->perm;
    }
    mark(s, AEP_PHASE_P2G);
    launch_p2g(s->kp, P, s->step_keys, s->step_perm, (int)s->n, s->G, s->slot_of, s->curidx_of, s->stream);
    CKLAUNCH();
    mark(s, AEP_PHASE_NORMALIZE);
    launch_normalize(s->kp, s->G, s->dstats, s->grid_blocks, s->stream);
    CKLAUNCH();
    mark(s, AEP_PHASE_CLOTH_FORCE);
    return AEP_OK;
}

}  // namespace

// =====================================================================================
extern "C" {

int32_t aep_abi_version(void) { return AEP_ABI_VERSION; }

void aep_default_params(aep_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->snow.E = 1.4e5;  // ParticleSystem.cpp:173-176
    p->snow.nu = 0.2;
    p->snow.theta_c = 2.5e-2;
    p->snow.theta_s = 7.5e-3;
    p->snow.xi = 10.0;  // HybridSolver.cpp:267
    p->sand.E = 3.537e5;  // ParticleSystem.cpp:233-234
    p->sand.nu = 0.3;
    p->sand.h0 = 35.0;  // HybridSolver.cpp:641-644
    p->sand.h1 = 9.0;
    p->sand.h2 = 0.2;
    p->sand.h3 = 10.0;
    p->gravity[0] = 0.0;
    p->gravity[1] = 0.0;
    p->gravity[2] = -9.8;  // HybridSolver.cpp:457
    p->friction = 0.2;     // HybridSolver.cpp:465
    p->friction_bug = 1;   // HybridSolver.cpp:500-501
    p->track_plastic_F = 0;
    p->particle_damp = 0.0;  // HybridSolver.cpp:916
    p->mesh_damp = 1.0;      // HybridSolver.cpp:926,932
    p->mass_bits = 34;
    p->momentum_bits = 40;
    p->reorder_interval = 4;  // ordering every 4th step: 281 vs 306 us per step on the
                              // 524,288-particle sand column, the same physics
}

aep_status aep_solver_create(const aep_grid_desc* grid, const aep_params* params, aep_solver** out) {
    aep_solver* s = nullptr;
    if (!grid || !out) return AEP_INVALID_ARG;
    *out = nullptr;
    for (int a = 0; a < 3; ++a) {
        if (grid->res[a] < 1 || grid->res[a] > 1400 || !(grid->max[a] > grid->min[a])) return AEP_INVALID_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return AEP_NO_DEVICE;
    s = new aep_solver();
    s->grid = *grid;
    if (params) s->prm = *params;
    else aep_default_params(&s->prm);
    if (s->prm.mass_bits <= 0 || s->prm.mass_bits > 50 || s->prm.momentum_bits <= 0 || s->prm.momentum_bits > 50) {
        delete s;
        return AEP_INVALID_ARG;
    }
    CK(cudaGetDevice(&s->device));
    CK(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking));
    s->stream = s->own_stream;
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
    s->grid_blocks = std::max(1, sms) * 8;
    fill_kparams(s);
    s->nblocks = s->kp.nb[0] * s->kp.nb[1] * s->kp.nb[2];
    s->nnodes = (size_t)s->nblocks * 64;
    uint64_t maxkey = (uint64_t)s->nblocks * 64;
    s->key_bits = 1;
    while ((1ull << s->key_bits) < maxkey) ++s->key_bits;
    CK(cudaMalloc(&s->G.acc, sizeof(unsigned long long) * 4 * s->nnodes));
    CK(cudaMalloc(&s->G.vel, sizeof(float4) * s->nnodes));
    CK(cudaMalloc(&s->G.vbf, sizeof(float4) * s->nnodes));
    CK(cudaMalloc(&s->G.flag, sizeof(uint32_t) * (size_t)s->nblocks));
    CK(cudaMalloc(&s->G.active, sizeof(int32_t) * (size_t)s->nblocks));
    CK(cudaMalloc(&s->dstats, sizeof(DevStats)));
    s->G.nactive = &s->dstats->nactive;  // device address inside the counters
    CK(cudaMemsetAsync(s->G.acc, 0, sizeof(unsigned long long) * 4 * s->nnodes, s->stream));
    CK(cudaMemsetAsync(s->G.vel, 0, sizeof(float4) * s->nnodes, s->stream));
    CK(cudaMemsetAsync(s->G.vbf, 0, sizeof(float4) * s->nnodes, s->stream));
    CK(cudaMemsetAsync(s->G.flag, 0, sizeof(uint32_t) * (size_t)s->nblocks, s->stream));
    CK(cudaMemsetAsync(s->dstats, 0, sizeof(DevStats), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *out = s;
    return AEP_OK;
}

aep_status aep_solver_destroy(aep_solver* s) {
    if (!s) return AEP_INVALID_ARG;
    cudaStreamSynchronize(s->stream);
    free_particles(s);
    free_mesh(s);
    cudaFree(s->G.acc);
    cudaFree(s->G.vel);
    cudaFree(s->G.vbf);
    cudaFree(s->G.flag);
    cudaFree(s->G.active);
    cudaFree(s->dstats);
    cudaFree(s->dforce);
    cudaFree(s->harvest_count);
    cudaFree(s->queue_mem);
    cudaFree(s->check);
    cudaFreeHost(s->check_host);
    cudaFree(s->solve);
    cudaFreeHost(s->solve_host);
    cudaFreeHost(s->stats_host);
    for (int r = 0; r < aep_solver::kRing; ++r)
        for (int p = 0; p <= AEP_NUM_PHASES; ++p)
            if (s->ev[r][p]) cudaEventDestroy(s->ev[r][p]);
    cudaStreamDestroy(s->own_stream);
    if (s->capture_stream) cudaStreamDestroy(s->capture_stream);
    delete s;
    return AEP_OK;
}

aep_status aep_set_particles(aep_solver* s, int64_t n, const double* x, const double* v, const double* B,
                             const double* Fe, const double* Fp, const double* m, const double* vol,
                             const double* plastic, const uint8_t* material) {
    if (!s) return AEP_INVALID_ARG;
    if (n <= 0 || n > (int64_t)INT32_MAX / 2 || !x || !Fe || !m)
        return fail(s, AEP_INVALID_ARG, "aep_set_particles: need n > 0 and non-null x, Fe, m");
    // Re-uploading the same particle set keeps the device's current (sorted) order
    // and an attached mesh: item q goes to the slot its id occupies now, so the next
    // ordering sees nearly sorted keys and the permuted particle reads stay coalesced.
    const bool keep_order = s->have_particles && s->np == n && s->n == s->np + s->nv + s->nf;
    if (!keep_order) {
        CK(cudaStreamSynchronize(s->stream));
        free_mesh(s);  // a mesh must be (re)attached after the particles
        s->have_particles = false;
        s->n = s->np = 0;
        aep_status st0 = ensure_capacity(s, n);
        if (st0 != AEP_OK) return st0;
        s->prev_sorted = false;
        s->cur = 0;
    }
    const int32_t* map = nullptr;
    if (keep_order) {
        launch_inverse_ids((int)s->n, s->P[s->cur].id, s->perm, s->stream);  // over every item: ids 0..n-1 first
        CKLAUNCH();
        map = s->perm;
    } else {
        s->n = n;
    }
    s->np = n;
    PArrays& P = s->P[s->cur];
    // Arrays in page-locked host or device memory are read by the conversion
    // kernel directly; pageable ones are staged first (doubles): x 0, v 3n, B 6n,
    // Fe 15n, Fp 24n, m 33n, vol 34n, plastic 35n, material bytes at 36n.
    const size_t N = (size_t)n;
    cudaError_t e = cudaSuccess;
    auto dsrc = [&](const void* p, size_t bytes, size_t off) -> const void* {
        if (!p || e != cudaSuccess) return nullptr;
        return device_source(s, p, bytes, off, &e);
    };
    UploadSrc src{static_cast<const double*>(dsrc(x, sizeof(double) * 3 * N, 0)),
                  static_cast<const double*>(dsrc(v, sizeof(double) * 3 * N, 3 * N)),
                  static_cast<const double*>(dsrc(B, sizeof(double) * 9 * N, 6 * N)),
                  static_cast<const double*>(dsrc(Fe, sizeof(double) * 9 * N, 15 * N)),
                  static_cast<const double*>(dsrc(Fp, sizeof(double) * 9 * N, 24 * N)),
                  static_cast<const double*>(dsrc(m, sizeof(double) * N, 33 * N)),
                  static_cast<const double*>(dsrc(vol, sizeof(double) * N, 34 * N)),
                  static_cast<const double*>(dsrc(plastic, sizeof(double) * N, 35 * N)),
                  static_cast<const uint8_t*>(dsrc(material, N, 36 * N))};
    CK(e);
    // the whole upload and its validation (bad masses, unknown tags, largest mass)
    // in one launch, read back with the final synchronisation
    CK(cudaMemsetAsync(s->check, 0, 2 * sizeof(unsigned long long), s->stream));
    launch_upload_particles((int)n, src, P, map, s->prm.track_plastic_F, s->check, s->stream);
    CKLAUNCH();
    unsigned long long* chk = s->check_host;
    CK(cudaMemcpyAsync(chk, s->check, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    double mm = 0.0;
    std::memcpy(&mm, &chk[0], sizeof(mm));
    if (chk[1] || !(mm > 0.0)) {
        s->have_particles = false;  // the device arrays are partly overwritten
        free_mesh(s);
        s->n = s->np = 0;
        return fail(s, AEP_INVALID_ARG, chk[1] ? "aep_set_particles: bad mass or unknown material tag"
                                               : "aep_set_particles: all masses are zero");
    }
    s->m_max = std::max(mm, s->mesh_m_max);
    fill_kparams(s);
    s->have_particles = true;
    s->keys_valid = false;
    s->stepped_since_upload = false;
    s->last_stage = 0;
    return AEP_OK;
}

// LagrangianMesh(vertexPositions, faces, vertexVelocities, elementVelocities, vertexMasses,
// vertexVolumes, elementMasses, elementVolumes, elementDirections_1..3, elementRestDirections_1..3,
// mu, lambda, shearStiffness, stiffness, frictionCoeff)   (LagrangianMesh.cpp:127-195)
aep_status aep_set_mesh(aep_solver* s, int64_t nv, int64_t nf, const double* xv, const int32_t* faces,
                        const double* vv, const double* ve, const double* mv, const double* volv, const double* me,
                        const double* vole, const double* d, const double* drest, double mu, double lambda,
                        double shear_stiffness, double stiffness, double friction_coeff) {
    if (!s) return AEP_INVALID_ARG;
    if (nv <= 0 || nf <= 0 || !xv || !faces || !mv || !me || !vole || !d || !drest)
        return fail(s, AEP_INVALID_ARG, "aep_set_mesh: need nv, nf > 0 and non-null xv, faces, masses, "
                                        "element volumes and directions");
    if (s->have_particles && s->stepped_since_upload)
        return fail(s, AEP_NOT_READY, "aep_set_mesh: attach the mesh before the first step");
    if (s->np + nv + nf > (int64_t)INT32_MAX / 2) return fail(s, AEP_INVALID_ARG, "aep_set_mesh: too many items");
    for (int64_t e = 0; e < nf; ++e)
        for (int c = 0; c < 3; ++c) {
            int32_t v = faces[c * nf + e];
            if (v < 0 || v >= nv) return fail(s, AEP_INVALID_ARG, "aep_set_mesh: face index out of range");
        }
    double mm = s->have_particles ? s->m_max : 0.0, mesh_mm = 0.0;
    for (int64_t i = 0; i < nv; ++i) {
        if (!(mv[i] >= 0.0) || !std::isfinite(mv[i])) return fail(s, AEP_INVALID_ARG, "aep_set_mesh: bad mass");
        mesh_mm = std::max(mesh_mm, mv[i]);
    }
    for (int64_t e = 0; e < nf; ++e) {
        if (!(me[e] >= 0.0) || !std::isfinite(me[e])) return fail(s, AEP_INVALID_ARG, "aep_set_mesh: bad mass");
        mesh_mm = std::max(mesh_mm, me[e]);
    }
    mm = std::max(mm, mesh_mm);
    if (!(mm > 0.0)) return fail(s, AEP_INVALID_ARG, "aep_set_mesh: all masses are zero");
    // rest data per element: inverseR of the rest in-plane R (geometry.cpp:67-73, from the
    // Gram-Schmidt QR of the rest directions, LagrangianMesh.cpp:421-429) and the third
    // row of the rest direction matrix (HybridSolver.cpp:427)
    std::vector<float> rest((size_t)6 * nf);
    for (int64_t e = 0; e < nf; ++e) {
        double D1[3], D2[3], D3[3];
        for (int a = 0; a < 3; ++a) {
            D1[a] = drest[0 * 3 * nf + a * nf + e];
            D2[a] = drest[1 * 3 * nf + a * nf + e];
            D3[a] = drest[2 * 3 * nf + a * nf + e];
        }
        double r11 = std::sqrt(D1[0] * D1[0] + D1[1] * D1[1] + D1[2] * D1[2]);
        double r12 = (D2[0] * D1[0] + D2[1] * D1[1] + D2[2] * D1[2]) / r11;
        double q2[3];
        for (int a = 0; a < 3; ++a) q2[a] = D2[a] - r12 * D1[a] / r11;
        double r22 = std::sqrt(q2[0] * q2[0] + q2[1] * q2[1] + q2[2] * q2[2]);
        if (!(r11 > 0.0) || !(r22 > 0.0)) return fail(s, AEP_INVALID_ARG, "aep_set_mesh: degenerate rest element");
        rest[6 * e + 0] = (float)(1.0 / r11);
        rest[6 * e + 1] = (float)(-r12 / r11 / r22);
        rest[6 * e + 2] = (float)(1.0 / r22);
        rest[6 * e + 3] = (float)D1[2];
        rest[6 * e + 4] = (float)D2[2];
        rest[6 * e + 5] = (float)D3[2];
    }
    CK(cudaStreamSynchronize(s->stream));
    const int64_t np = s->have_particles ? s->np : 0;
    free_mesh(s);
    const int64_t total = np + nv + nf;
    aep_status st = ensure_capacity(s, total, np);
    if (st != AEP_OK) return st;
    s->np = np;
    s->nv = nv;
    s->nf = nf;
    s->n = total;
    s->prev_sorted = false;
    s->cur = 0;
    s->m_max = mm;
    s->mesh_m_max = mesh_mm;
    s->cloth[0] = mu;
    s->cloth[1] = lambda;
    s->cloth[2] = shear_stiffness;
    s->cloth[3] = stiffness;
    s->cloth[4] = friction_coeff;
    fill_kparams(s);
    PArrays& P = s->P[0];
    const int64_t vb = np, eb = np + nv;
    std::vector<double> tmp((size_t)9 * std::max(nv, nf), 0.0);
    // vertices
    st = upload(s, xv, 3, 0, P.x, nv, vb);
    if (st) return st;
    if (vv) { st = upload(s, vv, 3, 0, P.v, nv, vb); if (st) return st; }
    else for (int a = 0; a < 3; ++a) CK(cudaMemsetAsync(P.v[a] + vb, 0, sizeof(float) * nv, s->stream));
    for (int a = 0; a < 9; ++a) CK(cudaMemsetAsync(P.B[a] + vb, 0, sizeof(float) * (nv + nf), s->stream));
    for (int64_t i = 0; i < nv; ++i)
        for (int k = 0; k < 9; ++k) tmp[9 * i + k] = (k % 4 == 0) ? 1.0 : 0.0;
    st = upload(s, tmp.data(), 9, 2, P.F, nv, vb);
    if (st) return st;
    st = upload(s, mv, 1, 3, &P.m, nv, vb);
    if (st) return st;
    if (volv) { st = upload(s, volv, 1, 3, &P.vol, nv, vb); if (st) return st; }
    else CK(cudaMemsetAsync(P.vol + vb, 0, sizeof(float) * nv, s->stream));
    CK(cudaMemsetAsync(P.plastic + vb, 0, sizeof(float) * (nv + nf), s->stream));
    launch_init_particles((int)nv, P, nullptr, 0, 0, s->stream, (int)vb, AEP_CLOTH_VERTEX);
    CKLAUNCH();
    // elements: positions are the centroids of their vertices (LagrangianMesh.cpp:186-187)
    for (int64_t e = 0; e < nf; ++e)
        for (int a = 0; a < 3; ++a) {
            double c = 0.0;
            for (int k = 0; k < 3; ++k) c += xv[a * nv + faces[k * nf + e]];
            tmp[a * nf + e] = c / 3.0;
        }
    CK(cudaStreamSynchronize(s->stream));
    st = upload(s, tmp.data(), 3, 0, P.x, nf, eb);
    if (st) return st;
    if (ve) { st = upload(s, ve, 3, 0, P.v, nf, eb); if (st) return st; }
    else for (int a = 0; a < 3; ++a) CK(cudaMemsetAsync(P.v[a] + eb, 0, sizeof(float) * nf, s->stream));
    st = upload(s, d, 9, 4, P.F, nf, eb);
    if (st) return st;
    st = upload(s, me, 1, 3, &P.m, nf, eb);
    if (st) return st;
    st = upload(s, vole, 1, 3, &P.vol, nf, eb);
    if (st) return st;
    launch_init_particles((int)nf, P, nullptr, 0, 0, s->stream, (int)eb, AEP_CLOTH_ELEMENT);
    CKLAUNCH();
    // mesh buffers
    std::vector<int32_t> fem((size_t)3 * nf);
    for (int64_t e = 0; e < nf; ++e)
        for (int c = 0; c < 3; ++c) fem[3 * e + c] = faces[c * nf + e];
    CK(cudaMalloc(&s->faces, sizeof(int32_t) * 3 * nf));
    CK(cudaMalloc(&s->rest, sizeof(float) * 6 * nf));
    CK(cudaMalloc(&s->estress, sizeof(float) * 9 * nf));
    CK(cudaMalloc(&s->vforce, sizeof(unsigned long long) * 3 * nv));
    CK(cudaMalloc(&s->slot_of, sizeof(int32_t) * total));
    CK(cudaMalloc(&s->curidx_of, sizeof(int32_t) * total));
    CK(cudaMemcpy(s->faces, fem.data(), sizeof(int32_t) * 3 * nf, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->rest, rest.data(), sizeof(float) * 6 * nf, cudaMemcpyHostToDevice));
    CK(cudaMemset(s->vforce, 0, sizeof(unsigned long long) * 3 * nv));
    CK(cudaStreamSynchronize(s->stream));
    s->have_particles = true;
    s->keys_valid = false;
    s->stepped_since_upload = false;
    s->last_stage = 0;
    return AEP_OK;
}

// LagrangianMesh public members (LagrangianMesh.h:37-61) in the layouts of aep_set_mesh;
// any pointer may be NULL.
aep_status aep_get_mesh(aep_solver* s, double* xv, double* vv, double* Bv, double* xe, double* ve, double* Be,
                        double* d) {
    if (!s) return AEP_INVALID_ARG;
    if (s->nf == 0) return fail(s, AEP_NOT_READY, "aep_get_mesh: no mesh");
    PArrays& P = s->P[s->cur];
    const int64_t vb = s->np, eb = s->np + s->nv, ee = s->n;
    const size_t V = (size_t)s->nv, F = (size_t)s->nf;
    aep_status st = prepare_download(s);
    if (st) return st;
    if (xv && (st = download(s, xv, 3, 0, P.x, vb, eb, 0, false))) return st;
    if (vv && (st = download(s, vv, 3, 0, P.v, vb, eb, 3 * V, false))) return st;
    if (Bv && (st = download(s, Bv, 9, 1, P.B, vb, eb, 6 * V, false))) return st;
    if (xe && (st = download(s, xe, 3, 0, P.x, eb, ee, 15 * V, false))) return st;
    if (ve && (st = download(s, ve, 3, 0, P.v, eb, ee, 15 * V + 3 * F, false))) return st;
    if (Be && (st = download(s, Be, 9, 1, P.B, eb, ee, 15 * V + 6 * F, false))) return st;
    if (d && (st = download(s, d, 9, 4, P.F, eb, ee, 15 * V + 15 * F, false))) return st;
    CK(cudaStreamSynchronize(s->stream));
    return AEP_OK;
}

// Writes to LagrangianMesh's public members between steps (LagrangianMesh.h:37-61), the
// counterpart of aep_get_mesh: any pointer may be NULL (kept).  Items go to the slots
// they occupy now, so the device order survives.
aep_status aep_set_mesh_state(aep_solver* s, int64_t nv, int64_t nf, const double* xv, const double* vv,
                              const double* Bv, const double* xe, const double* ve, const double* Be,
                              const double* d) {
    if (!s) return AEP_INVALID_ARG;
    if (s->nf == 0) return fail(s, AEP_NOT_READY, "aep_set_mesh_state: no mesh");
    if (nv != s->nv || nf != s->nf) return fail(s, AEP_INVALID_ARG, "aep_set_mesh_state: sizes differ from the mesh's");
    PArrays& P = s->P[s->cur];
    const int64_t vb = s->np, eb = s->np + s->nv;
    const size_t V = (size_t)s->nv, F = (size_t)s->nf;
    launch_inverse_ids((int)s->n, P.id, s->perm, s->stream);  // perm[id] = slot
    CKLAUNCH();
    const int32_t* mv = s->perm + vb;
    const int32_t* me = s->perm + eb;
    aep_status st;
    // staging offsets (doubles) as in aep_get_mesh, so that pageable sources do not overlap
    if (xv && (st = upload(s, xv, 3, 0, P.x, nv, 0, mv, 0))) return st;
    if (vv && (st = upload(s, vv, 3, 0, P.v, nv, 0, mv, 3 * V))) return st;
    if (Bv && (st = upload(s, Bv, 9, 1, P.B, nv, 0, mv, 6 * V))) return st;
    if (xe && (st = upload(s, xe, 3, 0, P.x, nf, 0, me, 15 * V))) return st;
    if (ve && (st = upload(s, ve, 3, 0, P.v, nf, 0, me, 15 * V + 3 * F))) return st;
    if (Be && (st = upload(s, Be, 9, 1, P.B, nf, 0, me, 15 * V + 6 * F))) return st;
    if (d && (st = upload(s, d, 9, 4, P.F, nf, 0, me, 15 * V + 15 * F))) return st;
    if (xv || xe) s->keys_valid = false;  // positions changed: fresh keys at the next step
    CK(cudaStreamSynchronize(s->stream));
    return AEP_OK;
}

aep_status aep_set_levelset(aep_solver* s, const aep_sdf* shapes, int32_t n) {
    if (!s) return AEP_INVALID_ARG;
    if (n < 0 || n > kMaxShapes || (n > 0 && !shapes))
        return fail(s, AEP_INVALID_ARG, "aep_set_levelset: 0..8 shapes");
    for (int i = 0; i < n; ++i) {
        if (shapes[i].type < AEP_SDF_PLANE || shapes[i].type > AEP_SDF_WALL2GROUND)
            return fail(s, AEP_INVALID_ARG, "aep_set_levelset: unknown shape type");
        s->kp.shapes[i].type = shapes[i].type;
        for (int k = 0; k < 6; ++k) s->kp.shapes[i].p[k] = (float)shapes[i].p[k];
    }
    s->kp.nshapes = n;
    return AEP_OK;
}

aep_status aep_init_volumes(aep_solver* s) {
    if (!s) return AEP_INVALID_ARG;
    if (!s->have_particles) return fail(s, AEP_NOT_READY, "aep_init_volumes: no particles");
    aep_status st = run_p2g(s);
    if (st) return st;
    launch_volumes(s->kp, s->P[s->cur], s->step_perm, (int)s->n, s->G, s->stream);
    CKLAUNCH();
    // no G2P applied this ordering to the particle arrays: the next step orders
    s->since_order = std::max(1, (int)s->prm.reorder_interval);
    s->dirty_grid = true;
    s->last_stage = AEP_STAGE_P2G;
    CK(cudaStreamSynchronize(s->stream));
    return check_overflow(s);
}

namespace {

// One step up to `stage`.  adaptive: the kernels read Dt from the solve state
// and reduce max |v| into it (aep_solve); otherwise dt_force / dt are used.
aep_status step_impl(aep_solver* s, double dt_force, double dt, int32_t stage, bool adaptive) {
    if (!s->have_particles) return fail(s, AEP_NOT_READY, "aep_step: no particles");
    if (!adaptive && (!(dt > 0.0) || !std::isfinite(dt) || !(dt_force > 0.0) || !std::isfinite(dt_force)))
        return fail(s, AEP_INVALID_ARG, "aep_step: dt must be > 0");
    if (stage < AEP_STAGE_P2G || stage > AEP_STAGE_FULL) return fail(s, AEP_INVALID_ARG, "aep_step: bad stage");
    if (adaptive) {
        s->kp.dt_dev = s->solve->dt;
        s->kp.vmax2 = s->solve->vmax2;
    }
    struct Restore {
        KParams& k;
        ~Restore() { k.dt_dev = nullptr; k.vmax2 = nullptr; }
    } restore{s->kp};
    const bool timed = s->profiling && stage == AEP_STAGE_FULL;
    const bool prof_saved = s->profiling;
    if (s->profiling && !timed) s->profiling = false;  // only whole steps are timed
    if (timed) {
        aep_status fs = fold_slot(s, s->ev_slot);
        if (fs) return fs;
    }
    aep_status st = run_p2g(s);
    s->profiling = prof_saved;
    if (st) return st;
    s->last_stage = stage;
    // a call that stops before G2P leaves the particle arrays in their order: the
    // next step orders them
    if (stage != AEP_STAGE_FULL) s->since_order = std::max(1, (int)s->prm.reorder_interval);
    if (stage == AEP_STAGE_P2G) {
        s->dirty_grid = true;
        return AEP_OK;
    }
    if (adaptive) {
        launch_solve_dt(s->solve, 0, s->stream);
        CKLAUNCH();
    }
    const float dtf = (float)dt_force;
    const PArrays& P = s->P[s->cur];
    const MeshArrays M = mesh_arrays(s);
    launch_cloth_force(s->kp, P, M, dtf, s->stream);
    CKLAUNCH();
    if (timed) mark(s, AEP_PHASE_FORCE);
    launch_force(s->kp, P, s->step_keys, s->step_perm, (int)s->n, s->G, dtf, s->dstats, M, s->stream, s->inv);
    CKLAUNCH();
    if (timed) mark(s, AEP_PHASE_GRID);
    if (stage == AEP_STAGE_FORCES) {
        size_t ng = (size_t)s->grid.res[0] * s->grid.res[1] * s->grid.res[2];
        if (!s->dforce) CK(cudaMalloc(&s->dforce, sizeof(double) * 3 * ng));
        CK(cudaMemsetAsync(s->dforce, 0, sizeof(double) * 3 * ng, s->stream));
        launch_grid(s->kp, s->G, dtf, 1, s->dforce, s->grid_blocks, s->stream);
        CKLAUNCH();
        s->dirty_grid = true;
        return AEP_OK;
    }
    launch_grid(s->kp, s->G, dtf, 0, nullptr, s->grid_blocks, s->stream);
    CKLAUNCH();
    if (s->nfixed > 0) {
        launch_fixed_vertices(s->kp, P, s->G, M, s->fixed, s->nfixed, s->stream);
        CKLAUNCH();
    }
    if (adaptive) {
        launch_solve_dt(s->solve, 1, s->stream);
        CKLAUNCH();
    }
    if (stage == AEP_STAGE_GRID) return AEP_OK;
    if (timed) mark(s, AEP_PHASE_G2P);
    const int nx = 1 - s->cur;
    Harvest H{s->harvest, s->harvest_count, s->harvest_cap, s->harvest_stride};
    MlpParams mp{};
    if (s->mlp) {
        mp = mlp_device_params(s->mlp);
        if (s->queue.cap < s->n) {  // room for every particle: (int32 j, pj, kQueueFields floats) per row
            CK(cudaStreamSynchronize(s->stream));
            cudaFree(s->queue_mem);
            s->queue_mem = nullptr;
            s->queue = MlpQueue{};
            const size_t cap = (size_t)s->n;
            CK(cudaMalloc(&s->queue_mem, cap * (2 * sizeof(int32_t) + kQueueFields * sizeof(float))));
            s->queue.j = static_cast<int32_t*>(s->queue_mem);
            s->queue.pj = s->queue.j + cap;
            s->queue.f = reinterpret_cast<float*>(s->queue.pj + cap);
            s->queue.cap = (int)cap;
        }
    }
    launch_g2p(s->kp, P, s->P[nx], s->step_perm, (int)s->n, s->G, (float)dt, s->keys, s->dstats, s->stream, H,
               s->mlp != nullptr, s->step_keys, s->queue);
    CKLAUNCH();
    if (timed) mark(s, AEP_PHASE_MLP);
    if (s->mlp) {
        launch_mlp_finish(s->kp, P, s->P[nx], s->queue, s->dstats, mp, (float)s->learned_tol, (float)s->learned_abs,
                          s->stream);
        CKLAUNCH();
    }
    if (timed) mark(s, AEP_PHASE_CLOTH_G2P);
    launch_cloth_g2p(s->kp, P, s->P[nx], s->G, M, (float)dt, s->keys, s->dstats, H, s->mlp ? &mp : nullptr,
                     (float)s->learned_tol, (float)s->learned_abs, s->stream);
    CKLAUNCH();
    if (timed) {
        mark(s, AEP_NUM_PHASES);
        s->ev_pending[s->ev_slot] = true;
        s->ev_slot = (s->ev_slot + 1) % aep_solver::kRing;
    }
    s->cur = nx;
    s->keys_valid = true;
    s->stepped_since_upload = true;
    s->steps++;
    return AEP_OK;
}

}  // namespace

aep_status aep_step_stage(aep_solver* s, double dt, int32_t stage) {
    if (!s) return AEP_INVALID_ARG;
    return step_impl(s, dt, dt, stage, false);
}

aep_status aep_step(aep_solver* s, double dt) {
    if (!s) return AEP_INVALID_ARG;
    return step_impl(s, dt, dt, AEP_STAGE_FULL, false);
}

aep_status aep_step_split(aep_solver* s, double dt_force, double dt) {
    if (!s) return AEP_INVALID_ARG;
    return step_impl(s, dt_force, dt, AEP_STAGE_FULL, false);
}

aep_status aep_set_solve_callback(aep_solver* s, aep_solve_fn fn, void* user) {
    if (!s) return AEP_INVALID_ARG;
    s->solve_fn = fn;
    s->solve_user = user;
    return AEP_OK;
}

aep_status aep_set_max_steps(aep_solver* s, int64_t max_steps) {
    if (!s) return AEP_INVALID_ARG;
    if (max_steps < 0) return fail(s, AEP_INVALID_ARG, "aep_set_max_steps: max_steps must be >= 0");
    s->max_steps = max_steps;
    return AEP_OK;
}

aep_status aep_get_solve_state(aep_solver* s, aep_solve_state* out) {
    if (!s || !out) return AEP_INVALID_ARG;
    *out = s->solve_last;
    return AEP_OK;
}

aep_status aep_solve(aep_solver* s, double cfl, double maxt, double alpha) {
    (void)alpha;  // HybridSolver::updateParticleVelocities_ ignores it (:739-758)
    if (!s) return AEP_INVALID_ARG;
    if (!(cfl > 0.0) || !std::isfinite(cfl) || !std::isfinite(maxt))
        return fail(s, AEP_INVALID_ARG, "aep_solve: need cfl > 0 and a finite maxt");
    if (!s->have_particles) return fail(s, AEP_NOT_READY, "aep_solve: no particles");
    if (!s->solve) {
        CK(cudaMalloc(&s->solve, sizeof(SolveState)));
        CK(cudaMallocHost(&s->solve_host, sizeof(SolveState)));
        CK(cudaMallocHost(&s->stats_host, sizeof(DevStats)));
    }
    // the first P2G of solve computes densities and volumes (:853-855)
    aep_status st = aep_init_volumes(s);
    if (st) return st;
    double hmin = 1e300;
    for (int a = 0; a < 3; ++a) hmin = std::min(hmin, (s->grid.max[a] - s->grid.min[a]) / s->grid.res[a]);
    SolveState init{};
    init.cfl = cfl;
    init.inv_hmin = 1.0 / hmin;
    CK(cudaMemcpyAsync(s->solve, &init, sizeof(init), cudaMemcpyHostToDevice, s->stream));
    s->solve_last = aep_solve_state{};
    double t = 0.0;
    int64_t it = 0;
    while (t <= maxt && (s->max_steps <= 0 || it < s->max_steps)) {
        st = step_impl(s, 0.0, 0.0, AEP_STAGE_FULL, true);
        if (st) return st;
        CK(cudaMemcpyAsync(s->solve_host, s->solve, sizeof(SolveState), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(s->stats_host, s->dstats, sizeof(DevStats), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (s->stats_host->overflow) return fail(s, AEP_OVERFLOW, "fixed-point grid accumulator overflow");
        const SolveState& h = *s->solve_host;
        t = h.t;
        ++it;
        aep_solve_state& o = s->solve_last;
        o.t = h.t;
        o.inner_t = h.inner;
        o.dt = h.Dt;
        o.steps = it;
        o.frames = h.frame;
        o.frame_done = h.frame_flag;
        if (s->solve_fn && s->solve_fn(s, &o, s->solve_user) != 0) break;
    }
    return AEP_OK;
}

aep_status aep_set_fixed_vertices(aep_solver* s, int64_t nv, const double* vertex_is_fixed) {
    if (!s) return AEP_INVALID_ARG;
    cudaFree(s->fixed);
    s->fixed = nullptr;
    s->nfixed = 0;
    if (!vertex_is_fixed) return AEP_OK;
    if (s->nv <= 0 || nv != s->nv)
        return fail(s, AEP_INVALID_ARG, "aep_set_fixed_vertices: need one value per mesh vertex (set the mesh first)");
    std::vector<int32_t> ids;
    for (int64_t v = 0; v < nv; ++v)
        if (vertex_is_fixed[v] != 0.0) ids.push_back((int32_t)v);
    if (ids.empty()) return AEP_OK;
    CK(cudaMalloc(&s->fixed, sizeof(int32_t) * ids.size()));
    CK(cudaMemcpy(s->fixed, ids.data(), sizeof(int32_t) * ids.size(), cudaMemcpyHostToDevice));
    s->nfixed = (int)ids.size();
    return AEP_OK;
}

aep_status aep_get_weights(aep_solver* s, int64_t count, const int64_t* ids, int64_t* nodes, double* w,
                           double* grad) {
    if (!s) return AEP_INVALID_ARG;
    if (!s->have_particles) return fail(s, AEP_NOT_READY, "aep_get_weights: no particles");
    if (count < 0 || (count > 0 && (!ids || !nodes || !w || !grad)) || count > (int64_t)INT32_MAX / 64)
        return fail(s, AEP_INVALID_ARG, "aep_get_weights: need count >= 0 and non-null arrays");
    for (int64_t q = 0; q < count; ++q)
        if (ids[q] < 0 || ids[q] >= s->n) return fail(s, AEP_INVALID_ARG, "aep_get_weights: id out of range");
    if (count == 0) return AEP_OK;
    CK(cudaStreamSynchronize(s->stream));
    // scratch: inverse id map, ids, then the three outputs
    const size_t b_inv = sizeof(int32_t) * (size_t)s->n, b_ids = sizeof(int64_t) * (size_t)count;
    const size_t b_nodes = sizeof(int64_t) * 64 * (size_t)count, b_w = sizeof(double) * 64 * (size_t)count;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char* buf = nullptr;
    CK(cudaMalloc(&buf, up(b_inv) + up(b_ids) + up(b_nodes) + up(b_w) + 3 * b_w));
    int32_t* inv = reinterpret_cast<int32_t*>(buf);
    int64_t* dids = reinterpret_cast<int64_t*>(buf + up(b_inv));
    int64_t* dn = reinterpret_cast<int64_t*>(buf + up(b_inv) + up(b_ids));
    double* dw = reinterpret_cast<double*>(buf + up(b_inv) + up(b_ids) + up(b_nodes));
    double* dg = reinterpret_cast<double*>(buf + up(b_inv) + up(b_ids) + up(b_nodes) + up(b_w));
    aep_status st = AEP_OK;
    cudaError_t e = cudaSuccess;
    launch_inverse_ids((int)s->n, s->P[s->cur].id, inv, s->stream);
    if ((e = cudaMemcpyAsync(dids, ids, b_ids, cudaMemcpyHostToDevice, s->stream)) == cudaSuccess) {
        launch_query_weights(s->kp, s->P[s->cur], inv, dids, (int)count, dn, dw, dg, s->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(nodes, dn, b_nodes, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w, dw, b_w, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad, dg, 3 * b_w, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) st = fail(s, AEP_CUDA_ERROR, cudaGetErrorString(e));
    cudaFree(buf);
    return st;
}

namespace {

// checkpoint blob: header, then per item the float arrays of the current set
// (n floats each), material tags, ids; the mesh faces and rest data; the fixed
// vertex list
struct CkptHeader {
    char magic[8];
    int32_t version, float_arrays;
    int64_t n, np, nv, nf, steps;
    aep_grid_desc grid;
    aep_params prm;
    double m_max;
    double cloth[5];
    int32_t nshapes, nfixed;
    int32_t prev_sorted, since_order;
    DevShape shapes[kMaxShapes];
};
constexpr char kCkptMagic[8] = {'A', 'E', 'P', 'C', 'K', 'P', 'T', '1'};
constexpr int32_t kCkptVersion = 2;

int float_arrays(const aep_params& p) { return kFloatArrays + (p.track_plastic_F ? kFpArrays : 0); }

size_t ckpt_bytes(int64_t n, int64_t nf, int nfixed, int nfa) {
    return sizeof(CkptHeader) + (size_t)n * (sizeof(float) * nfa + 1 + 2 * sizeof(int32_t)) +
           (size_t)nf * (3 * sizeof(int32_t) + 6 * sizeof(float)) + (size_t)nfixed * sizeof(int32_t);
}

// Host-side check of a checkpoint blob whose header and size are consistent, with
// the rules the uploads apply (aep_solver_create's parameter bounds, aep_set_particles'
// material tags, aep_set_mesh's face indices, aep_set_levelset's shape types) plus
// the invariants the kernels index with: ids a permutation of [0, n) with the tag
// their range implies, the saved ordering keys ascending inside the padded grid, and
// fixed vertices inside the mesh.  Nothing reaches the device before it passes.
const char* ckpt_invalid(const CkptHeader& h, const char* body, int nblocks) {
    const aep_params& p = h.prm;
    if (p.mass_bits <= 0 || p.mass_bits > 50 || p.momentum_bits <= 0 || p.momentum_bits > 50)
        return "fixed-point bits out of range";
    if (p.reorder_interval < 0 || (p.friction_bug | 1) != 1 || (p.track_plastic_F | 1) != 1 ||
        (p.full_sort | 1) != 1 || (p.cloth_volume_weighting | 1) != 1 || (p.fp64_apex | 1) != 1)
        return "bad parameter flags";
    if (h.steps < 0 || h.since_order < 0 || (h.prev_sorted | 1) != 1) return "bad step counters";
    for (int k = 0; k < h.nshapes; ++k)
        if (h.shapes[k].type < kSdfPlane || h.shapes[k].type > kSdfWall2Ground) return "unknown level-set shape";
    const size_t n = (size_t)h.n;
    const uint8_t* mat = reinterpret_cast<const uint8_t*>(body + sizeof(float) * n * (size_t)h.float_arrays);
    const char* ids_raw = reinterpret_cast<const char*>(mat + n);
    const char* keys_raw = ids_raw + sizeof(int32_t) * n;
    std::vector<uint8_t> seen(n, 0);
    for (size_t j = 0; j < n; ++j) {
        int32_t id;
        std::memcpy(&id, ids_raw + sizeof(int32_t) * j, sizeof(id));
        if (id < 0 || (int64_t)id >= h.n || seen[(size_t)id]) return "particle ids are not a permutation";
        seen[(size_t)id] = 1;
        const int want = id < h.np ? -1 : (id < h.np + h.nv ? kClothVertex : kClothElement);
        if (want < 0 ? mat[j] > kSand : mat[j] != want) return "material tag does not match the item";
    }
    if (h.prev_sorted) {
        const uint64_t key_end = (uint64_t)nblocks * 64;
        uint32_t last = 0;
        for (size_t j = 0; j < n; ++j) {
            uint32_t k;
            std::memcpy(&k, keys_raw + sizeof(uint32_t) * j, sizeof(k));
            if ((uint64_t)k >= key_end || (j > 0 && k < last)) return "ordering keys not ascending inside the grid";
            last = k;
        }
    }
    const char* q = keys_raw + sizeof(uint32_t) * n;
    if (h.nf > 0) {
        for (int64_t i = 0; i < 3 * h.nf; ++i) {
            int32_t v;
            std::memcpy(&v, q + sizeof(int32_t) * i, sizeof(v));
            if (v < 0 || v >= h.nv) return "face index out of range";
        }
        for (int k = 0; k < 5; ++k)
            if (!std::isfinite(h.cloth[k])) return "bad cloth parameters";
        q += sizeof(int32_t) * 3 * h.nf + sizeof(float) * 6 * h.nf;
    }
    for (int i = 0; i < h.nfixed; ++i) {
        int32_t v;
        std::memcpy(&v, q + sizeof(int32_t) * i, sizeof(v));
        if (v < 0 || v >= h.nv) return "fixed vertex out of range";
    }
    return nullptr;
}

}  // namespace

aep_status aep_checkpoint_size(aep_solver* s, int64_t* bytes) {
    if (!s || !bytes) return AEP_INVALID_ARG;
    if (!s->have_particles) return fail(s, AEP_NOT_READY, "aep_checkpoint_size: no particles");
    *bytes = (int64_t)ckpt_bytes(s->n, s->nf, s->nfixed, float_arrays(s->prm));
    return AEP_OK;
}

aep_status aep_checkpoint_save(aep_solver* s, void* buf, int64_t bytes) {
    if (!s || !buf) return AEP_INVALID_ARG;
    if (!s->have_particles) return fail(s, AEP_NOT_READY, "aep_checkpoint_save: no particles");
    const int nfa = float_arrays(s->prm);
    if (bytes != (int64_t)ckpt_bytes(s->n, s->nf, s->nfixed, nfa))
        return fail(s, AEP_INVALID_ARG, "aep_checkpoint_save: bytes must be aep_checkpoint_size");
    CK(cudaStreamSynchronize(s->stream));
    CkptHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kCkptMagic, 8);
    h.version = kCkptVersion;
    h.float_arrays = nfa;
    h.n = s->n;
    h.np = s->np;
    h.nv = s->nv;
    h.nf = s->nf;
    h.steps = s->steps;
    h.grid = s->grid;
    h.prm = s->prm;
    h.m_max = s->m_max;
    for (int k = 0; k < 5; ++k) h.cloth[k] = s->cloth[k];
    h.nshapes = s->kp.nshapes;
    h.nfixed = s->nfixed;
    h.prev_sorted = s->prev_sorted ? 1 : 0;
    h.since_order = s->since_order;
    for (int k = 0; k < kMaxShapes; ++k) h.shapes[k] = s->kp.shapes[k];
    char* p = static_cast<char*>(buf);
    std::memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    const ParticleSet& set = s->set[s->cur];
    const size_t n = (size_t)s->n;
    for (int k = 0; k < nfa; ++k, p += sizeof(float) * n)
        CK(cudaMemcpy(p, set.f + (size_t)k * s->cap, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(p, set.mat, n, cudaMemcpyDeviceToHost));
    p += n;
    CK(cudaMemcpy(p, set.id, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    p += sizeof(int32_t) * n;
    // the last sorted keys: the next ordering starts from them (incremental path)
    if (s->prev_sorted) CK(cudaMemcpy(p, s->keys_sorted, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    else std::memset(p, 0, sizeof(uint32_t) * n);
    p += sizeof(uint32_t) * n;
    if (s->nf > 0) {
        CK(cudaMemcpy(p, s->faces, sizeof(int32_t) * 3 * s->nf, cudaMemcpyDeviceToHost));
        p += sizeof(int32_t) * 3 * s->nf;
        CK(cudaMemcpy(p, s->rest, sizeof(float) * 6 * s->nf, cudaMemcpyDeviceToHost));
        p += sizeof(float) * 6 * s->nf;
    }
    if (s->nfixed > 0) CK(cudaMemcpy(p, s->fixed, sizeof(int32_t) * s->nfixed, cudaMemcpyDeviceToHost));
    return AEP_OK;
}

aep_status aep_checkpoint_load(aep_solver* s, const void* buf, int64_t bytes) {
    if (!s || !buf) return AEP_INVALID_ARG;
    CkptHeader h;
    if (bytes < (int64_t)sizeof(h)) return fail(s, AEP_INVALID_ARG, "aep_checkpoint_load: truncated");
    std::memcpy(&h, buf, sizeof(h));
    if (std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != kCkptVersion)
        return fail(s, AEP_INVALID_ARG, "aep_checkpoint_load: not a checkpoint of this version");
    if (h.float_arrays != float_arrays(h.prm) || h.n <= 0 || h.n != h.np + h.nv + h.nf || h.np < 0 || h.nv < 0 ||
        h.nf < 0 || (h.nf > 0) != (h.nv > 0) || h.nshapes < 0 || h.nshapes > kMaxShapes || h.nfixed < 0 ||
        h.nfixed > h.nv || h.n > (int64_t)INT32_MAX / 2 || !(h.m_max > 0.0))
        return fail(s, AEP_INVALID_ARG, "aep_checkpoint_load: inconsistent header");
    if (bytes != (int64_t)ckpt_bytes(h.n, h.nf, h.nfixed, h.float_arrays))
        return fail(s, AEP_INVALID_ARG, "aep_checkpoint_load: size does not match the header");
    for (int a = 0; a < 3; ++a)
        if (h.grid.res[a] != s->grid.res[a] || h.grid.min[a] != s->grid.min[a] || h.grid.max[a] != s->grid.max[a])
            return fail(s, AEP_INVALID_ARG, "aep_checkpoint_load: the grid differs from the handle's");
    if (const char* why = ckpt_invalid(h, static_cast<const char*>(buf) + sizeof(h), s->nblocks))
        return fail(s, AEP_INVALID_ARG, std::string("aep_checkpoint_load: ") + why);
    CK(cudaStreamSynchronize(s->stream));
    free_mesh(s);
    free_particles(s);
    s->cap = 0;
    s->have_particles = false;
    s->n = s->np = 0;
    s->prm = h.prm;
    s->m_max = h.m_max;
    aep_status st = ensure_capacity(s, h.n);
    if (st != AEP_OK) return st;
    s->n = h.n;
    s->np = h.np;
    s->cur = 0;
    fill_kparams(s);
    s->kp.nshapes = h.nshapes;
    for (int k = 0; k < kMaxShapes; ++k) s->kp.shapes[k] = h.shapes[k];
    const char* p = static_cast<const char*>(buf) + sizeof(h);
    const ParticleSet& set = s->set[0];
    const size_t n = (size_t)h.n;
    for (int k = 0; k < h.float_arrays; ++k, p += sizeof(float) * n)
        CK(cudaMemcpy(set.f + (size_t)k * s->cap, p, sizeof(float) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(set.mat, p, n, cudaMemcpyHostToDevice));
    p += n;
    CK(cudaMemcpy(set.id, p, sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    p += sizeof(int32_t) * n;
    CK(cudaMemcpy(s->keys_sorted, p, sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    p += sizeof(uint32_t) * n;
    if (h.nf > 0) {
        s->nv = h.nv;
        s->nf = h.nf;
        s->mesh_m_max = h.m_max;  // not stored separately: the combined bound stands in
        for (int k = 0; k < 5; ++k) s->cloth[k] = h.cloth[k];
        CK(cudaMalloc(&s->faces, sizeof(int32_t) * 3 * h.nf));
        CK(cudaMalloc(&s->rest, sizeof(float) * 6 * h.nf));
        CK(cudaMalloc(&s->estress, sizeof(float) * 9 * h.nf));
        CK(cudaMalloc(&s->vforce, sizeof(unsigned long long) * 3 * h.nv));
        CK(cudaMalloc(&s->slot_of, sizeof(int32_t) * n));
        CK(cudaMalloc(&s->curidx_of, sizeof(int32_t) * n));
        CK(cudaMemcpy(s->faces, p, sizeof(int32_t) * 3 * h.nf, cudaMemcpyHostToDevice));
        p += sizeof(int32_t) * 3 * h.nf;
        CK(cudaMemcpy(s->rest, p, sizeof(float) * 6 * h.nf, cudaMemcpyHostToDevice));
        p += sizeof(float) * 6 * h.nf;
        CK(cudaMemset(s->vforce, 0, sizeof(unsigned long long) * 3 * h.nv));
    }
    if (h.nfixed > 0) {
        CK(cudaMalloc(&s->fixed, sizeof(int32_t) * h.nfixed));
        CK(cudaMemcpy(s->fixed, p, sizeof(int32_t) * h.nfixed, cudaMemcpyHostToDevice));
        s->nfixed = h.nfixed;
    }
    s->steps = h.steps;
    s->prev_sorted = h.prev_sorted != 0;
    s->since_order = h.since_order;
    s->have_particles = true;
    s->keys_valid = false;
    s->stepped_since_upload = h.steps > 0;
    s->last_stage = 0;
    return AEP_OK;
}

aep_status aep_synchronize(aep_solver* s) {
    if (!s) return AEP_INVALID_ARG;
    CK(cudaStreamSynchronize(s->stream));
    return check_overflow(s);
}

aep_status aep_get_particles(aep_solver* s, int64_t n, double* x, double* v, double* B, double* Fe, double* Fp,
                             double* vol, double* plastic) {
    if (!s) return AEP_INVALID_ARG;
    if (!s->have_particles) return fail(s, AEP_NOT_READY, "aep_get_particles: no particles");
    if (n != s->np) return fail(s, AEP_INVALID_ARG, "aep_get_particles: n mismatch");
    if (Fp && !s->prm.track_plastic_F) return fail(s, AEP_INVALID_ARG, "aep_get_particles: Fp needs track_plastic_F");
    PArrays& P = s->P[s->cur];
    aep_status st;
    const int64_t np = s->np;
    const size_t N = (size_t)np;
    if ((st = prepare_download(s))) return st;
    // one conversion launch for all requested fields: straight into page-locked or
    // device destinations, through staging (doubles: x 0, v 3N, B 6N, Fe 15N,
    // Fp 24N, vol 33N, plastic 34N) and one copy each for pageable ones
    double* const req[7] = {x, v, B, Fe, Fp, vol, plastic};
    const size_t cnt[7] = {3, 3, 9, 9, 9, 1, 1}, off[7] = {0, 3, 6, 15, 24, 33, 34};
    double* dev[7] = {};
    for (int f = 0; f < 7; ++f)
        if (req[f]) {
            double* a = static_cast<double*>(const_cast<void*>(device_alias(req[f])));
            dev[f] = a ? a : s->staging + off[f] * N;
        }
    DownloadDst dst{dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], dev[6]};
    launch_download_particles((int)np, dst, P, s->inv, s->stream);
    CKLAUNCH();
    for (int f = 0; f < 7; ++f)
        if (req[f] && dev[f] == s->staging + off[f] * N)
            CK(cudaMemcpyAsync(req[f], dev[f], sizeof(double) * cnt[f] * N, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return AEP_OK;
}

aep_status aep_get_grid(aep_solver* s, double* mass, double* vel, double* vbf, double* force) {
    if (!s) return AEP_INVALID_ARG;
    CK(cudaStreamSynchronize(s->stream));
    size_t ng = (size_t)s->grid.res[0] * s->grid.res[1] * s->grid.res[2];
    double* d = nullptr;
    CK(cudaMalloc(&d, sizeof(double) * 7 * ng));
    CK(cudaMemsetAsync(d, 0, sizeof(double) * 7 * ng, s->stream));
    if (s->last_stage > 0) {
        bool has_vbf = s->last_stage >= AEP_STAGE_GRID;
        launch_grid_dense(s->kp, s->G, d, d + ng, has_vbf ? d + 4 * ng : nullptr, s->grid_blocks, s->stream);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { cudaFree(d); return fail(s, AEP_CUDA_ERROR, cudaGetErrorString(e)); }
    }
    cudaError_t e = cudaSuccess;
    if (mass && e == cudaSuccess) e = cudaMemcpyAsync(mass, d, sizeof(double) * ng, cudaMemcpyDeviceToHost, s->stream);
    if (vel && e == cudaSuccess) e = cudaMemcpyAsync(vel, d + ng, sizeof(double) * 3 * ng, cudaMemcpyDeviceToHost, s->stream);
    if (vbf && e == cudaSuccess) e = cudaMemcpyAsync(vbf, d + 4 * ng, sizeof(double) * 3 * ng, cudaMemcpyDeviceToHost, s->stream);
    if (force && e == cudaSuccess) {
        if (s->last_stage == AEP_STAGE_FORCES && s->dforce)
            e = cudaMemcpyAsync(force, s->dforce, sizeof(double) * 3 * ng, cudaMemcpyDeviceToHost, s->stream);
        else
            std::memset(force, 0, sizeof(double) * 3 * ng);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(s, AEP_CUDA_ERROR, cudaGetErrorString(e));
    return AEP_OK;
}

aep_status aep_get_stats(aep_solver* s, aep_stats* out) {
    if (!s || !out) return AEP_INVALID_ARG;
    CK(cudaStreamSynchronize(s->stream));
    DevStats h;
    CK(cudaMemcpy(&h, s->dstats, sizeof(h), cudaMemcpyDeviceToHost));
    int32_t nact = 0;
    CK(cudaMemcpy(&nact, s->G.nactive, sizeof(nact), cudaMemcpyDeviceToHost));
    std::memset(out, 0, sizeof(*out));
    out->steps = s->steps;
    out->num_particles = s->n;
    out->active_blocks = nact;
    out->out_of_domain = (int64_t)h.out_of_domain;
    out->fp64_fallbacks = (int64_t)h.fallbacks;
    out->overflow = (int64_t)h.overflow;
    out->active_nodes = (int64_t)h.nodes;
    out->learned_accepted = (int64_t)h.learned_ok;
    out->learned_fallbacks = (int64_t)h.learned_rejected;
    out->sort_movers = (int64_t)h.movers;
    out->learned_exact = (int64_t)h.learned_exact;
    out->orderings = s->orderings;
    out->fp64_apex = (int64_t)h.fp64_apex;
    double im = std::ldexp(s->m_max, -s->prm.mass_bits), ip = std::ldexp(s->m_max, -s->prm.momentum_bits);
    out->total_mass = (double)(long long)h.mass * im;
    for (int a = 0; a < 3; ++a) out->total_momentum[a] = (double)(long long)h.mom[a] * ip;
    return AEP_OK;
}

aep_status aep_set_harvest(aep_solver* s, float* d_records, int64_t capacity, int32_t stride) {
    if (!s) return AEP_INVALID_ARG;
    if (d_records && (capacity <= 0 || stride < 1))
        return fail(s, AEP_INVALID_ARG, "aep_set_harvest: capacity > 0, stride >= 1");
    CK(cudaStreamSynchronize(s->stream));
    s->harvest = d_records;
    s->harvest_cap = d_records ? capacity : 0;
    s->harvest_stride = stride < 1 ? 1 : stride;
    if (!s->harvest_count) CK(cudaMalloc(&s->harvest_count, sizeof(unsigned long long)));
    CK(cudaMemset(s->harvest_count, 0, sizeof(unsigned long long)));
    return AEP_OK;
}

aep_status aep_get_harvest_count(aep_solver* s, int64_t* count) {
    if (!s || !count) return AEP_INVALID_ARG;
    CK(cudaStreamSynchronize(s->stream));
    unsigned long long c = 0;
    if (s->harvest_count) CK(cudaMemcpy(&c, s->harvest_count, sizeof(c), cudaMemcpyDeviceToHost));
    *count = (int64_t)std::min<unsigned long long>(c, (unsigned long long)s->harvest_cap);
    return AEP_OK;
}

aep_status aep_set_return_map(aep_solver* s, const aep_mlp* m, double tolerance) {
    if (!s) return AEP_INVALID_ARG;
    if (m && !(tolerance >= 0.0)) return fail(s, AEP_INVALID_ARG, "aep_set_return_map: tolerance >= 0");
    s->mlp = m;
    s->learned_tol = tolerance;
    s->learned_abs = std::ldexp(1.0, -24);  // FP32 spacing below 1: the rounding of a stretch near 1, in ln s
    return AEP_OK;
}

aep_status aep_set_return_map_bounds(aep_solver* s, double rel_tol, double abs_tol) {
    if (!s) return AEP_INVALID_ARG;
    if (!(rel_tol >= 0.0) || !(abs_tol >= 0.0))
        return fail(s, AEP_INVALID_ARG, "aep_set_return_map_bounds: tolerances >= 0");
    s->learned_tol = rel_tol;
    s->learned_abs = abs_tol;
    return AEP_OK;
}

aep_status aep_set_stream(aep_solver* s, void* cuda_stream) {
    if (!s) return AEP_INVALID_ARG;
    CK(cudaStreamSynchronize(s->stream));
    s->stream = cuda_stream ? (cudaStream_t)cuda_stream : s->own_stream;
    return AEP_OK;
}

aep_status aep_set_profiling(aep_solver* s, int32_t on) {
    if (!s) return AEP_INVALID_ARG;
    CK(cudaStreamSynchronize(s->stream));
    if (on && !s->ev[0][0]) {
        for (int r = 0; r < aep_solver::kRing; ++r)
            for (int p = 0; p <= AEP_NUM_PHASES; ++p) CK(cudaEventCreate(&s->ev[r][p]));
    }
    for (int r = 0; r < aep_solver::kRing; ++r) s->ev_pending[r] = false;
    for (int p = 0; p < AEP_NUM_PHASES; ++p) s->phase_ms[p] = 0.0;
    s->timed_steps = 0;
    s->ev_slot = 0;
    s->profiling = on != 0;
    return AEP_OK;
}

aep_status aep_get_phase_times(aep_solver* s, double* ms, int64_t* steps) {
    if (!s || !ms) return AEP_INVALID_ARG;
    CK(cudaStreamSynchronize(s->stream));
    for (int r = 0; r < aep_solver::kRing; ++r) {
        aep_status st = fold_slot(s, r);
        if (st) return st;
    }
    for (int p = 0; p < AEP_NUM_PHASES; ++p) ms[p] = s->phase_ms[p];
    if (steps) *steps = s->timed_steps;
    return AEP_OK;
}

int64_t aep_sort_pairs_temp_bytes(int64_t n, int32_t key_bits) {
    if (n < 0 || n > (int64_t)INT32_MAX / 2 || key_bits < 1 || key_bits > 32) return -1;
    return (int64_t)sort_temp_bytes((int)n, key_bits);
}

aep_status aep_sort_pairs(const uint32_t* keys_in, uint32_t* keys_out, const int32_t* vals_in, int32_t* vals_out,
                          int64_t n, int32_t key_bits, void* temp, int64_t temp_bytes, void* cuda_stream) {
    if (n < 0 || n > (int64_t)INT32_MAX / 2 || key_bits < 1 || key_bits > 32) return AEP_INVALID_ARG;
    if (n == 0) return AEP_OK;
    if (!keys_in || !keys_out || !vals_in || !vals_out || !temp ||
        temp_bytes < (int64_t)sort_temp_bytes((int)n, key_bits))
        return AEP_INVALID_ARG;
    const cudaError_t e = sort_pairs(temp, (size_t)temp_bytes, keys_in, keys_out, vals_in, vals_out, (int)n, key_bits,
                                     static_cast<cudaStream_t>(cuda_stream));
    return e == cudaSuccess ? AEP_OK : AEP_CUDA_ERROR;
}

const char* aep_last_error(aep_solver* s) {
    if (!s) return "null solver";
    return s->err.c_str();
}

}  // extern "C"
