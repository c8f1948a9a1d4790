// aep_kernels.h -- host launchers of the kernels in aep_kernels.cu.
#pragma once

#include "../../include/aep.h"
#include "aep_device.cuh"
#include "aep_mlp.cuh"

namespace aep {

void launch_keys(const KParams& P, const PArrays& cur, int n, uint32_t* keys, DevStats* st, cudaStream_t s);
void launch_p2g(const KParams& P, const PArrays& cur, const uint32_t* keys, const int32_t* perm, int n,
                const GArrays& G, int32_t* slot_of, int32_t* curidx_of, cudaStream_t s);
void launch_normalize(const KParams& P, const GArrays& G, DevStats* st, int grid_blocks, cudaStream_t s);
void launch_cloth_force(const KParams& P, const PArrays& cur, const MeshArrays& M, float dt_force, cudaStream_t s);
void launch_force(const KParams& P, const PArrays& cur, const uint32_t* keys, const int32_t* perm, int n,
                  const GArrays& G, float dt_force, DevStats* st, const MeshArrays& M, cudaStream_t s,
                  int32_t* fp64_list);
void launch_grid(const KParams& P, const GArrays& G, float dt_force, int write_force, double* force_out,
                 int grid_blocks, cudaStream_t s);
void launch_grid_clear(const GArrays& G, int grid_blocks, cudaStream_t s);
// G2P of the particle system and the cloth vertices (learned: the plastic rows are
// queued for the finisher), the learned map's finisher, the cloth elements' G2P
void launch_g2p(const KParams& P, const PArrays& cur, const PArrays& nxt, const int32_t* perm, int n,
                const GArrays& G, float dt, uint32_t* keys_next, DevStats* st, cudaStream_t s, const Harvest& H,
                bool learned, const uint32_t* keys_sorted, const MlpQueue& queue);
void launch_mlp_finish(const KParams& P, const PArrays& cur, const PArrays& nxt, const MlpQueue& queue, DevStats* st,
                       const MlpParams& mlp, float tol_rel, float tol_abs, cudaStream_t s);
void launch_cloth_g2p(const KParams& P, const PArrays& cur, const PArrays& nxt, const GArrays& G, const MeshArrays& M,
                      float dt, uint32_t* keys_next, DevStats* st, const Harvest& H, const MlpParams* mlp,
                      float tol_rel, float tol_abs, cudaStream_t s);
void launch_volumes(const KParams& P, const PArrays& cur, const int32_t* perm, int n, const GArrays& G,
                    cudaStream_t s);
void launch_upload(int n, int mode, const double* src, float* const* dst, cudaStream_t s,
                   const int32_t* map = nullptr);
void launch_inverse_ids(int n, const int32_t* id, int32_t* inv, cudaStream_t s);
// one-launch particle upload / readback (device-usable source / destination pointers)
struct UploadSrc {
    const double *x, *v, *B, *Fe, *Fp, *m, *vol, *plastic;
    const uint8_t* mat;
};
struct DownloadDst {
    double *x, *v, *B, *Fe, *Fp, *vol, *plastic;
};
void launch_upload_particles(int n, const UploadSrc& src, const PArrays& P, const int32_t* map, int track_fp,
                             unsigned long long* check, cudaStream_t s);
void launch_download_particles(int n, const DownloadDst& dst, const PArrays& P, const int32_t* inv, cudaStream_t s);
void launch_fixed_vertices(const KParams& P, const PArrays& cur, const GArrays& G, const MeshArrays& M,
                           const int32_t* fixed, int nfixed, cudaStream_t s);
void launch_solve_dt(SolveState* S, int phase, cudaStream_t s);
void launch_query_weights(const KParams& P, const PArrays& cur, const int32_t* inv, const int64_t* ids, int count,
                          int64_t* nodes, double* w, double* g, cudaStream_t s);
void launch_check_upload(int n, const double* m, const uint8_t* mat, unsigned long long* out, cudaStream_t s);
void launch_download(int count, int mode, const int32_t* inv, int id_lo, double* dst, float* const* src,
                     cudaStream_t s);
void launch_init_particles(int n, const PArrays& cur, const uint8_t* mat, int has_fp, int track_fp,
                           cudaStream_t s, int id0 = 0, int fixed_mat = -1, const int32_t* map = nullptr);
void launch_snow_jp(int n, const PArrays& cur, const double* Fp, cudaStream_t s, const int32_t* map = nullptr);
void launch_grid_dense(const KParams& P, const GArrays& G, double* mass, double* vel, double* vbf,
                       int grid_blocks, cudaStream_t s);

// device view of a trained MLP (aep_mlp.cu)
MlpParams mlp_device_params(const aep_mlp* m);

// incremental ordering (aep_sort.cu): movers flagged and listed, placed by their
// (key, slot) rank, stayers placed from block offsets; captured as a CUDA graph
// whose if/else node runs the full sort when the movers are too many
constexpr int kBruteMovers = 8192;  // movers placed by brute-force rank up to this count
struct OrderBuffers {
    const uint32_t* keys;  // new keys in the current order
    uint32_t* keys_sorted; // in: the last sorted keys (ascending); out: this ordering's keys
    int32_t* perm;         // out: current slot of each sorted position
    const int32_t* iota;
    uint32_t* mk;          // mover list: keys and slots (cap entries)
    int32_t* mj;
    uint32_t* mkeys;       // movers sorted by (key, slot): keys, slots, final positions
    int32_t* mslot;
    int32_t* mpos;
    uint32_t* scratch;     // order_scratch_words(n) words
    void* sort_tmp;
    size_t sort_bytes;
    int n, cap, key_bits;
    DevStats* st;
};
size_t order_scratch_words(int n);
cudaError_t order_graph_build(void** out, cudaStream_t capture_stream, const OrderBuffers& b);
cudaError_t order_graph_launch(void* graph, cudaStream_t s);
void order_graph_destroy(void* graph);

// stable LSD radix sort of (key, value) pairs on the low key_bits bits (aep_sort.cu)
size_t sort_temp_bytes(int n, int key_bits);
cudaError_t sort_pairs(void* temp, size_t temp_bytes, const uint32_t* keys_in, uint32_t* keys_out,
                       const int32_t* vals_in, int32_t* vals_out, int n, int key_bits, cudaStream_t s);

}  // namespace aep
