/*
 * aep.h -- C-ABI of the GB300 MPM step (APIC transfers, cubic B-spline weights,
 * snow / Drucker-Prager sand / anisotropic cloth elastoplasticity, level-set
 * collision).  Plain pointers and sizes only; no CUDA or C++ types cross it.
 *
 * The reference has no C API: its boundary is the C++ class surface of
 * HybridSolver / ParticleSystem / RegularGrid / LagrangianMesh (public Eigen
 * members, read and written in place).  Each entry point below names the
 * reference interface it replaces.  All host arrays use the reference's memory
 * layouts so that a caller can pass Eigen's data() pointers unchanged:
 *
 *   "N x 3 column-major"  = Eigen::MatrixX3d: all x, then all y, then all z.
 *   "3x3 column-major"    = Eigen::Matrix3d: M(a,b) at [a + 3*b]; a
 *                           std::vector<Matrix3d> of N is 9*N doubles.
 *   affine momenta B      = affineMomenta_1 | affineMomenta_2 | affineMomenta_3
 *                           (each N x 3 column-major; row p of affineMomenta_a
 *                           is row a of the particle's 3x3 B), 9*N doubles.
 *   grid node index       = k*Rx*Ry + j*Rx + i (RegularGrid.cpp:164-168).
 *
 * Errors: every function returns an aep_status; the reference instead spins
 * in while(1) or calls exit() (RegularGrid.cpp:134, LagrangianMesh.cpp:213,360,474).
 * Threading: one host thread per handle; work is ordered on the handle's stream.
 */
#ifndef AEP_H
#define AEP_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AEP_ABI_VERSION 2

/* Opaque solver handle: device state of one particle system on one grid. */
typedef struct aep_solver aep_solver;

typedef enum aep_status {
    AEP_OK = 0,
    AEP_INVALID_ARG = 1,     /* bad size, null pointer, bad enum value            */
    AEP_CUDA_ERROR = 2,      /* a CUDA runtime call failed                        */
    AEP_OVERFLOW = 3,        /* a fixed-point grid accumulator left its range     */
    AEP_OUT_OF_DOMAIN = 4,   /* reserved: particles are clamped and counted       */
    AEP_NOT_READY = 5,       /* call order violated (e.g. step before particles)  */
    AEP_OUT_OF_MEMORY = 6,   /* device allocation failed                          */
    AEP_NO_DEVICE = 7,       /* no CUDA device visible                            */
    AEP_CAPACITY = 8         /* request exceeds the fixed scratch of aep_p2g_noalloc */
} aep_status;

/* Particle material tags (the reference hard-codes one MaterialType for the
 * whole system, HybridSolver.h:21-25 and HybridSolver.cpp:873,955,959; here
 * the tag is per particle). */
enum { AEP_SNOW = 0, AEP_SAND = 1 };
/* Tags of the LagrangianMesh vertices and elements inside the solver (set by
 * aep_set_mesh; not accepted by aep_set_particles). */
enum { AEP_CLOTH_VERTEX = 2, AEP_CLOTH_ELEMENT = 3 };

/* Level-set shapes (replaces the LevelSet/DLevelSet std::function pair,
 * HybridSolver.h:18-19, LevelSet.cpp:8-42).  Several shapes are unioned:
 * phi = min over shapes, normal = the normal of the minimising shape. */
enum {
    AEP_SDF_PLANE = 0,       /* p[0..2] = unit normal n, p[3] = offset: phi = n.x - p[3]
                                (groundLevelSet(x, g) is n=(0,0,1), offset g)        */
    AEP_SDF_SPHERE = 1,      /* p[0..2] = centre, p[3] = radius: phi = |x-c| - r    */
    AEP_SDF_WALL2GROUND = 2  /* p[0] = wallX, p[1] = wallY, p[2] = groundZ
                                (wall2groundLevelSet / Dwall2groundLevelSet)        */
};

typedef struct aep_sdf {
    int32_t type;
    int32_t reserved;
    double p[6];
} aep_sdf;

/* RegularGrid(minBound, maxBound, resolution), RegularGrid.cpp:117-162:
 * h = (max - min) / res per axis; node (i,j,k) sits at min + (i,j,k)*h. */
typedef struct aep_grid_desc {
    double min[3];
    double max[3];
    int32_t res[3];
    int32_t reserved;
} aep_grid_desc;

/* Fixed-corotated snow with hardening (HybridSolver.cpp:281-287,314-325,626-631). */
typedef struct aep_snow_params {
    double E, nu;            /* Young's modulus, Poisson ratio (ParticleSystem.cpp:173-174) */
    double theta_c;          /* critical compression (clamp 1 - theta_c)               */
    double theta_s;          /* critical stretch     (clamp 1 + theta_s)               */
    double xi;               /* hardening coefficient, reference literal 10 (HS:267)    */
} aep_snow_params;

/* Drucker-Prager sand (HybridSolver.cpp:326-339,632-674). */
typedef struct aep_sand_params {
    double E, nu;
    double h0, h1, h2, h3;   /* friction-angle hardening, reference 35, 9, 0.2, 10 (HS:641-644) */
} aep_sand_params;

typedef struct aep_params {
    aep_snow_params snow;
    aep_sand_params sand;
    double gravity[3];       /* reference: (0, 0, -9.8), HybridSolver.cpp:457          */
    double friction;         /* grid friction mu, reference literal 0.2 (HS:465)        */
    int32_t friction_bug;    /* 1: reproduce the dropped Coulomb term of HS:500-501
                                (sliding nodes keep the full tangential velocity);
                                0: Coulomb friction v_t + mu v_n v_t/|v_t|             */
    int32_t track_plastic_F; /* 1: keep the full 3x3 plastic gradient F_P per particle
                                (HS:676); 0: keep only J_P = det F_P, which is all the
                                step reads (HS:283)                                    */
    double particle_damp;    /* APIC symmetric-part damping, reference 0 (HS:916)      */
    int32_t mass_bits;       /* fixed-point fraction bits of the grid mass accumulator,
                                relative to the heaviest particle (default 34)         */
    int32_t momentum_bits;   /* same for momentum and force impulse, relative to
                                (heaviest particle mass) x (1 m/s)   (default 40)      */
    double mesh_damp;        /* APIC damping of cloth vertices/elements, reference 1 (HS:926,932) */
    int32_t cloth_volume_weighting; /* 0: in-plane vertex forces as the reference computes
                                       them, without the element volume (LagrangianMesh.cpp:
                                       452-458); 1: multiplied by the element volume        */
    int32_t full_sort;       /* 1: radix-sort every step; 0 (default): order incrementally
                                from the last sorted keys when at most a quarter of the
                                particles changed cell (same result up to the order of
                                equal keys)                                            */
    int32_t reorder_interval; /* order the particles every this many steps (default 4;
                                1 or 0: every step); the steps between keep the last order, and
                                the few particles that changed cell since are scattered
                                and gathered out of order (same physics; the FP32 sums
                                of a run take its particles in another order)           */
    int32_t fp64_apex;       /* 1: sand return mappings near the Drucker-Prager apex (projected
                                onto it, or |tr ln s| within 1e-3 |ln s| of the switch between
                                apex and cone, HybridSolver.cpp:652-663) run again in FP64,
                                counted in aep_stats.fp64_apex; 0 (default): FP32 throughout */
    int64_t reserved[5];
} aep_params;

/* Counters of the last step (all zero until a step ran). */
typedef struct aep_stats {
    int64_t steps;              /* steps taken by this handle                            */
    int64_t num_particles;
    int64_t active_blocks;      /* 4x4x4 node blocks touched by the last P2G             */
    int64_t out_of_domain;      /* particles clamped into the grid in the last step     */
    int64_t fp64_fallbacks;     /* particles whose SVD / projection ran in FP64          */
    int64_t overflow;           /* nonzero if a fixed-point accumulator overflowed       */
    int64_t active_nodes;       /* grid nodes with mass after the last P2G               */
    double total_mass;          /* grid mass after the last P2G (exact fixed-point sum)  */
    double total_momentum[3];   /* grid momentum after the last P2G                      */
    int64_t learned_accepted;   /* learned return maps used in the last step             */
    int64_t learned_fallbacks;  /* learned outputs replaced by the exact mapping         */
    int64_t sort_movers;        /* particles that changed cell key in the last ordering,
                                   -1 when it was a full radix sort                      */
    int64_t learned_exact;      /* plastic states with a constant projection (sand apex,
                                   cloth in tension), taken exactly by the learned path  */
    int64_t orderings;          /* particle orderings run by this handle (reorder_interval) */
    int64_t fp64_apex;          /* sand return mappings redone in FP64 near the apex
                                   (aep_params.fp64_apex) in the last step               */
    double reserved[1];
} aep_stats;

/* ---- version / defaults ------------------------------------------------------- */

int32_t aep_abi_version(void);

/* Reference literal values (see field comments above). */
void aep_default_params(aep_params* params);

/* ---- lifetime ------------------------------------------------------------------ */

/* Replaces HybridSolver(ParticleSystem*, RegularGrid*) + RegularGrid(min,max,res)
 * (HybridSolver.h:83-87, RegularGrid.cpp:117-162).  Picks the current CUDA device. */
aep_status aep_solver_create(const aep_grid_desc* grid, const aep_params* params,
                             aep_solver** out);
aep_status aep_solver_destroy(aep_solver* s);

/* ---- state upload (by copy, reference layouts) ------------------------------------ */

/* Replaces the ParticleSystem constructor / HybridSolver::setParticleSystem
 * (ParticleSystem.cpp:81-117, HybridSolver.h:86).  x, v: N x 3 column-major;
 * B: 9N (see top), may be NULL (zero); Fe, Fp: 9N (3x3 column-major per
 * particle), Fp may be NULL (identity); m, vol: N; plastic: N, the sand
 * plasticAmount (ParticleSystem.h:31), may be NULL (zero); material: N tags.
 * For snow particles the scalar J_P is det(Fp) when Fp is given, else `plastic`
 * (what aep_get_particles returns for snow), else 1.  Re-uploading the same
 * number of particles keeps the device's current particle order and an attached
 * mesh (a different number removes the mesh: attach it again after the upload). */
aep_status aep_set_particles(aep_solver* s, int64_t n,
                             const double* x, const double* v, const double* B,
                             const double* Fe, const double* Fp,
                             const double* m, const double* vol,
                             const double* plastic, const uint8_t* material);

/* Replaces the LagrangianMesh constructor + HybridSolver::setLagrangianMesh
 * (LagrangianMesh.cpp:127-195, HybridSolver.h:88).  Vertices and elements (one
 * per triangle) become MPM particles.  xv: Nv x 3 column-major; faces: Nf x 3
 * column-major int32 (0-based vertex indices); vv (Nv x 3), ve (Nf x 3) may be
 * NULL; mv, volv (Nv); me, vole (Nf), volv may be NULL; d, drest: element
 * directions d1 | d2 | d3 and rest directions, each Nf x 3 column-major (9Nf);
 * mu, lambda: in-plane Lame parameters; shear_stiffness, stiffness: the shear
 * and normal stiffness of the normal-direction response; friction_coeff: the
 * frictional cap of the cloth return mapping.  Element positions start at the
 * centroids of their vertices.  Call after aep_set_particles (or without
 * particles) and before the first step; aep_set_particles with a different
 * particle count removes the mesh.                                             */
aep_status aep_set_mesh(aep_solver* s, int64_t nv, int64_t nf, const double* xv, const int32_t* faces,
                        const double* vv, const double* ve, const double* mv, const double* volv,
                        const double* me, const double* vole, const double* d, const double* drest,
                        double mu, double lambda, double shear_stiffness, double stiffness,
                        double friction_coeff);

/* Replaces reading LagrangianMesh's public members (LagrangianMesh.h:37-61):
 * vertex positions/velocities/affine momenta, element positions/velocities/
 * affine momenta and element directions, in the layouts of aep_set_mesh; any
 * pointer may be NULL.                                                          */
aep_status aep_get_mesh(aep_solver* s, double* xv, double* vv, double* Bv, double* xe,
                        double* ve, double* Be, double* d);

/* Replaces writing LagrangianMesh's public members between steps (LagrangianMesh.h:
 * 37-61, which the reference's caller may edit in place): the same arrays and layouts
 * as aep_get_mesh; nv, nf must be the attached mesh's sizes; any pointer may be NULL
 * (that member is kept).  Masses, volumes, rest directions and faces stay as
 * aep_set_mesh set them; the device order of the items is kept.                 */
aep_status aep_set_mesh_state(aep_solver* s, int64_t nv, int64_t nf, const double* xv,
                              const double* vv, const double* Bv, const double* xe,
                              const double* ve, const double* Be, const double* d);

/* Replaces LagrangianMesh::bindConstraints(VectorXd* vertexIsFixed)
 * (LagrangianMesh.cpp:354-363): one value per mesh vertex, nonzero = fixed
 * (LagrangianMesh::vertexIsFixed, :462-475).  After the collision pass, every
 * grid node in the stencil of a fixed vertex zeroes the velocity and the
 * before-friction velocity of its 3x3x3 neighbours (HybridSolver.cpp:513-550).
 * nv must equal the mesh's vertex count; vertex_is_fixed == NULL removes the
 * constraints.  aep_set_mesh removes them too.                                 */
aep_status aep_set_fixed_vertices(aep_solver* s, int64_t nv, const double* vertex_is_fixed);

/* Replaces HybridSolver::setLevelSet(phi, dphi) (HybridSolver.h:89). */
aep_status aep_set_levelset(aep_solver* s, const aep_sdf* shapes, int32_t n);

/* ---- stepping -------------------------------------------------------------------- */

/* The first P2G of HybridSolver::solve with evaluateVolumesAndDensities = true
 * (HybridSolver.cpp:242-249, called at :854): rho_p = sum_i w_ip m_i / h^3,
 * vol_p = m_p / rho_p.  Overwrites the uploaded volumes.                       */
aep_status aep_init_volumes(aep_solver* s);

/* One MPM time step: the body of the while loop of HybridSolver::solve
 * (HybridSolver.cpp:867-989) with a fixed dt, rotated so that the P2G that
 * the reference runs last (:987) runs first: P2G -> grid forces -> grid
 * velocity update + gravity -> collision/friction -> G2P (velocity, APIC
 * affine, advection) -> F update -> return mapping.  Stream-ordered, returns
 * without waiting for the GPU.                                                 */
aep_status aep_step(aep_solver* s, double dt);

/* One step with the two time steps of the reference loop: the force pass and
 * the grid update take dt_force (the Dt of the previous iteration, :873, :877),
 * the grid-to-particle part takes dt (the Dt computed at :878).  aep_step(dt)
 * is aep_step_split(dt, dt).                                                   */
aep_status aep_step_split(aep_solver* s, double dt_force, double dt);

/* ---- the adaptive solve loop (HybridSolver::solve, HybridSolver.cpp:827-989) ---- */

typedef struct aep_solve_state {
    double t;                /* simulated time: advances by 1/60 per completed frame  */
    double inner_t;          /* time inside the current frame                         */
    double dt;               /* Dt of the last step                                   */
    int64_t steps;           /* steps of this solve call                              */
    int32_t frames;          /* frames completed by this solve call                   */
    int32_t frame_done;      /* the last step completed a frame (:880-887)            */
    double reserved[4];
} aep_solve_state;

/* Called by aep_solve after every step with the device state read back; the
 * frame files of the reference (:991-1030) are written from here when
 * state->frame_done (frame number = state->frames - 1).  A nonzero return ends
 * the solve (aep_solve then returns AEP_OK).                                   */
typedef int32_t (*aep_solve_fn)(aep_solver* s, const aep_solve_state* state, void* user);
aep_status aep_set_solve_callback(aep_solver* s, aep_solve_fn fn, void* user);

/* Upper bound on the steps of one aep_solve call (0: none, the default). */
aep_status aep_set_max_steps(aep_solver* s, int64_t max_steps);

/* Replaces HybridSolver::solve(CFL, maxt, alpha) (HybridSolver.h:90,
 * HybridSolver.cpp:827-989): the first P2G with volumes (:854, as
 * aep_init_volumes), Dt = CFL / max(300, max|v_i| / hmin) from the P2G
 * velocities (:860), then while t <= maxt: a step whose force pass and grid
 * update use the previous Dt, whose Dt is recomputed from the updated grid
 * velocities before collision (:878, RegularGrid.cpp:188-200) and clamped to
 * end the 1/60 s frame (:880-892).  Dt and the frame clock live on the device;
 * the host reads them once per step.  alpha is accepted and unused, as in the
 * reference (:739).                                                            */
aep_status aep_solve(aep_solver* s, double cfl, double maxt, double alpha);

/* The state after the last step of the current or last aep_solve call. */
aep_status aep_get_solve_state(aep_solver* s, aep_solve_state* out);

/* ---- interpolation weights ------------------------------------------------------- */

/* One row per item of the reference's weight matrices omegas_ and domegas_1..3
 * (HybridSolver::evaluateInterpolationWeights_, HybridSolver.cpp:18-97) at the
 * current positions, as the GPU step evaluates them (FP32, widened to double).
 * ids: `count` item indices (particles 0..Np-1, then mesh vertices Np..Np+Nv-1,
 * then mesh elements); per id 64 entries in ascending node order: nodes (the
 * reference index k*Rx*Ry + j*Rx + i, or -1 where the weight is zero or the node
 * is outside the grid), w, and grad (3 per entry: d/dx, d/dy, d/dz).          */
aep_status aep_get_weights(aep_solver* s, int64_t count, const int64_t* ids, int64_t* nodes,
                           double* w, double* grad);

/* ---- checkpoint (full device state, bit-exact resume) --------------------------- */

/* Bytes of a checkpoint of the current state. */
aep_status aep_checkpoint_size(aep_solver* s, int64_t* bytes);
/* Copy the particle and mesh state in the device's current order, the
 * parameters, level set and fixed vertices into buf (`bytes` from
 * aep_checkpoint_size).  Steps after aep_checkpoint_load of this buffer repeat
 * the steps after the save bit for bit.  The learned return map, harvest and
 * stream settings are not part of it.                                           */
aep_status aep_checkpoint_save(aep_solver* s, void* buf, int64_t bytes);
/* Restore a checkpoint into a handle created with the same grid description;
 * replaces particles, mesh, parameters, level set and fixed vertices.          */
aep_status aep_checkpoint_load(aep_solver* s, const void* buf, int64_t bytes);

/* Wait for all work of the handle; returns the status of the work (overflow). */
aep_status aep_synchronize(aep_solver* s);

/* ---- readback ------------------------------------------------------------------- */

/* Replaces reading ParticleSystem's public members (ParticleSystem.h:28-41).
 * Arrays in the layout of aep_set_particles, in the caller's original particle
 * order; any pointer may be NULL.  Fp is only available with track_plastic_F.
 * plastic returns the sand plasticAmount for sand particles and J_P for snow. */
aep_status aep_get_particles(aep_solver* s, int64_t n,
                             double* x, double* v, double* B,
                             double* Fe, double* Fp, double* vol, double* plastic);

/* Replaces reading RegularGrid::masses / velocities (RegularGrid.h:49-55).
 * Dense arrays in reference node order; mass: Ng, vel: Ng x 3 column-major
 * (the grid velocity after the last grid update and collision, or after the
 * last P2G when stage == AEP_STAGE_P2G), vbf: the before-friction velocity
 * (HybridSolver.cpp:460-511), force: f_i without gravity after the force
 * stage.  Any pointer may be NULL.                                             */
aep_status aep_get_grid(aep_solver* s, double* mass, double* vel, double* vbf,
                        double* force);

aep_status aep_get_stats(aep_solver* s, aep_stats* out);

/* ---- staged stepping for parity tests ----------------------------------------------- */

enum {
    AEP_STAGE_P2G = 1,       /* stop after P2G + velocity normalisation          */
    AEP_STAGE_FORCES = 2,    /* stop after the force scatter                      */
    AEP_STAGE_GRID = 3,      /* stop after grid update + collision                */
    AEP_STAGE_FULL = 4       /* the whole step (same as aep_step)                 */
};

/* Run one step up to `stage` (inclusive).  A partial step leaves the particle
 * state untouched; the next call starts a fresh step.                          */
aep_status aep_step_stage(aep_solver* s, double dt, int32_t stage);

/* ---- streams and timing ----------------------------------------------------------- */

/* Order all later work of the handle on `cuda_stream` (a cudaStream_t of the
 * handle's device; NULL restores the handle's own stream).  The reference has
 * no counterpart (it is single-threaded CPU code).                            */
aep_status aep_set_stream(aep_solver* s, void* cuda_stream);

/* Kernel phases of one step, in launch order (a phase without work, e.g. the
 * cloth phases without a mesh, takes ~0 ms). */
enum {
    AEP_PHASE_SORT = 0,        /* particle ordering by grid block                     */
    AEP_PHASE_P2G = 1,         /* mass + APIC momentum scatter                        */
    AEP_PHASE_NORMALIZE = 2,   /* v = p / m on touched nodes                          */
    AEP_PHASE_CLOTH_FORCE = 3, /* per-element cloth in-plane forces, normal stress    */
    AEP_PHASE_FORCE = 4,       /* grad v gather, SVD, stress, impulse scatter         */
    AEP_PHASE_GRID = 5,        /* grid update, gravity, collision (+ fixed vertices)  */
    AEP_PHASE_G2P = 6,         /* G2P, APIC, advection, F update, return mapping      */
    AEP_PHASE_MLP = 7,         /* learned return map: network, check, finish          */
    AEP_PHASE_CLOTH_G2P = 8,   /* cloth elements: G2P, directions, QR return mapping  */
    AEP_NUM_PHASES = 9
};

/* Enable (1) or disable (0) CUDA-event timing of every phase on the handle's
 * stream.  Enabling resets the accumulated times.                             */
aep_status aep_set_profiling(aep_solver* s, int32_t on);

/* Accumulated milliseconds per phase since profiling was enabled, and the
 * number of timed steps.  Synchronises the handle's stream.                  */
aep_status aep_get_phase_times(aep_solver* s, double ms[AEP_NUM_PHASES], int64_t* steps);

/* ---- learned return map ----------------------------------------------------------- */

/* No counterpart in the reference.  A small MLP (6 -> 64 -> 64 -> 64 -> 3, SiLU,
 * BF16 weights on the tensor cores, FP32 accumulation) that maps the trial log
 * singular values (sorted, descending), the sand plastic amount and the material
 * to the projected log singular values of the return mapping
 * (HybridSolver.cpp:626-674).  It is trained on the device from (trial, projected)
 * pairs that the exact mapping produces during plain steps (aep_set_harvest).
 *
 * Training records: 8 floats each, [ln s0, ln s1, ln s2 (trial, sorted desc),
 * q, material, d0, d1, d2] with d = ln s_projected - ln s_trial.                 */
typedef struct aep_mlp aep_mlp;
#define AEP_MLP_NUM_PARAMS 9928  /* f32 master parameters: W1^T, W2^T, W3^T, W4^T, b1..b4 */

aep_status aep_mlp_create(uint64_t seed, aep_mlp** out);
aep_status aep_mlp_destroy(aep_mlp* m);
aep_status aep_mlp_get_params(aep_mlp* m, float* host_params, int64_t count);
aep_status aep_mlp_set_params(aep_mlp* m, const float* host_params, int64_t count);
/* Gradient of the mean squared error (outputs scaled by 50) over n device records,
 * with respect to the packed f32 parameters; also returns the loss.           */
aep_status aep_mlp_gradient(aep_mlp* m, const float* d_records, int64_t n, float* host_grad, double* loss);
/* Adam steps over batches drawn cyclically from n device records; the learning
 * rate decays from lr to lr_final (cosine).  Returns the last batch's loss.   */
aep_status aep_mlp_train(aep_mlp* m, const float* d_records, int64_t n, int64_t steps, int32_t batch,
                         double lr, double lr_final, double* final_loss, void* cuda_stream);
/* Predicted corrections d (3 floats per record, ln units) for n device records. */
aep_status aep_mlp_forward(aep_mlp* m, const float* d_records, int64_t n, float* d_out, void* cuda_stream);
/* The same predictions with the arithmetic of the step's learned return map: its
 * SiLU is z/2 + (z/2) tanh(z/2) with the hardware tanh (relative error ~2^-11)
 * instead of an exponential and a reciprocal.  For checking that arithmetic
 * against aep_mlp_forward.                                                      */
aep_status aep_mlp_forward_step_form(aep_mlp* m, const float* d_records, int64_t n, float* d_out,
                                     void* cuda_stream);
const char* aep_mlp_last_error(aep_mlp* m);

/* Collect training records from the exact return mapping of every `stride`-th
 * particle slot during later plain steps into the caller's device buffer
 * d_records (8 floats per record), up to `capacity` records; d_records = NULL
 * stops collecting.  The buffer must stay valid while collecting.              */
aep_status aep_set_harvest(aep_solver* s, float* d_records, int64_t capacity, int32_t stride);
/* Number of records written so far (capped at the capacity). */
aep_status aep_get_harvest_count(aep_solver* s, int64_t* count);
/* Use the learned return map in later steps (NULL: the exact mapping).  The G2P
 * pass checks each trial state's yield condition; a plastic state whose projection
 * is not a constant is predicted by the network, and the prediction is checked in
 * the kernel against the optimality conditions of the projection it stands for:
 * sand, the yield condition at the prediction (|dev ln s| + k alpha(q) tr ln s = 0)
 * and the flow rule (trace kept, deviatoric part shrunk radially); snow, each value
 * inside the clamp bounds, kept where the trial is inside and on the bound it
 * crossed; cloth, r33 kept and the shear shrunk radially onto the frictional cap.
 * A prediction whose largest residual (ln-strain units; cloth: QR units) exceeds
 * max(tolerance x |prediction|, 2^-24) is replaced by the exact projection
 * (aep_stats.learned_fallbacks).  Constant projections (sand apex, cloth in
 * tension) are taken exactly (aep_stats.learned_exact).  The handle must outlive
 * its use.                                                                     */
aep_status aep_set_return_map(aep_solver* s, const aep_mlp* m, double tolerance);
/* The two bounds of that check: relative to the predicted projected strain
 * (rel_tol; the stress is linear in it) and absolute (abs_tol, in ln-strain
 * units; 2^-24 after aep_set_return_map, the spacing of FP32 numbers just below 1,
 * what rounding a stretch near 1 to FP32 costs in ln s).  A residual bound of
 * 1e-4 is rel_tol = 0, abs_tol = 1e-4.                                          */
aep_status aep_set_return_map_bounds(aep_solver* s, double rel_tol, double abs_tol);

/* ---- particle-to-grid without allocation --------------------------------------------- */

/* No counterpart in the reference.  For callers that must not allocate GPU memory:
 * code running inside a host application that owns all device memory through its
 * own pool (a stray cudaMalloc breaks its budget or fragments its heap), or
 * real-time loops that cannot afford the device-wide synchronisation of
 * cudaMalloc/cudaFree.  It performs the
 * step's particle-to-grid transfer (mass and APIC momentum, then v = p / m) from
 * the caller's device arrays into the caller's device output arrays, and allocates
 * nothing: its only working memory is a fixed array compiled into the library
 * (AEP_NOALLOC_MAX_NODES * 32 bytes, about 12 MB, held on every GPU that loads the
 * library until the process exits).
 *
 * Inputs (device pointers, FP32, the C-ABI layouts above): x, v are N x 3
 * column-major; B is 9N (affineMomenta_1 | _2 | _3); m is N.  mass_ref > 0 sets the
 * fixed-point unit and should be the largest particle mass.  Outputs (device
 * pointers, FP32, reference node order): mass_out (Ng), vel_out (Ng x 3
 * column-major); nodes without mass get 0.  Work is queued on cuda_stream (NULL =
 * the default stream) and the call returns without waiting.
 *
 * Limits: the padded grid, ((res+2)/4 + 2)^3 * 64 nodes, must not exceed
 * AEP_NOALLOC_MAX_NODES (a 64^3 grid fits); larger grids return AEP_CAPACITY.
 * The first call on a device looks up the device address of the fixed array
 * (cudaGetSymbolAddress) and keeps it for the life of the process.  The kept
 * address is not valid
 * after cudaDeviceReset on that device: a process that resets a device must not
 * call this entry point on it again.  Every call shares the one array and clears
 * the part it uses at its start, so calls that can overlap on the GPU (different
 * streams, or different host threads) race and must be serialised by the caller. */
#define AEP_NOALLOC_MAX_NODES 373248
aep_status aep_p2g_noalloc(const aep_grid_desc* grid, int64_t n,
                           const float* x, const float* v, const float* B, const float* m,
                           double mass_ref, float* mass_out, float* vel_out, void* cuda_stream);

/* ---- ordering -------------------------------------------------------------------------- */

/* The stable radix sort that orders the particles by grid block every
 * reorder_interval-th step (its counterpart in the reference is the sort inside
 * Eigen's setFromTriplets, HybridSolver.cpp:92-95), for device arrays: sorts n
 * (key, value) pairs by the low key_bits bits of the key (1..32), pairs with equal
 * keys keeping their input order.  Inputs and outputs must not overlap; temp is a
 * device buffer of aep_sort_pairs_temp_bytes(n, key_bits) bytes.  Queued on
 * cuda_stream (NULL = the default stream), returns without waiting.               */
int64_t aep_sort_pairs_temp_bytes(int64_t n, int32_t key_bits);
aep_status aep_sort_pairs(const uint32_t* keys_in, uint32_t* keys_out, const int32_t* vals_in,
                          int32_t* vals_out, int64_t n, int32_t key_bits, void* temp,
                          int64_t temp_bytes, void* cuda_stream);

/* Human-readable text of the last error on this handle (static storage). */
const char* aep_last_error(aep_solver* s);

#ifdef __cplusplus
}
#endif

#endif /* AEP_H */
