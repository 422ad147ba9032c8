/* mpm_gb300.h — C ABI of the GB300-native implicit MPM snow substep.
 *
 * One context owns the device state of one or more independent scenes on one GPU and
 * advances all of them together, one fused pipeline of sm_103a kernels per substep.
 * Every entry point takes plain pointers and sizes and returns an mpm_status; host
 * memory stays caller-owned and is copied, device memory is library-owned. One CUDA
 * stream per context; a context is not thread-safe.
 *
 * Reference boundary (SoldierDown/Non_Ficks_Diffusion): the MPM_Example<T,d> method set
 * that MPM_Driver::Advance_Step calls in order (MPM_Driver.cpp:103-116), plus
 * Initialize (MPM_Driver.cpp:18-32), Max_Particle_Velocity (MPM_Example.cpp:375-387) and
 * the particle half of Write/Read_Output_Files (MPM_Example.cpp:1049-1079). Each
 * declaration below names the reference interface it replaces.
 */
#ifndef MPM_GB300_H
#define MPM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MPM_API __attribute__((visibility("default")))
#else
#define MPM_API
#endif

#define MPM_MAX_BARRIERS 16
#define MPM_MAX_SCENES 256

/* The reference has no error channel (assert only, MPM_CG_System.h:233-234); every call
 * here reports one. MPM_CG_NOT_CONVERGED is a warning: the substep still completed. */
typedef enum mpm_status {
    MPM_OK = 0,
    MPM_CG_NOT_CONVERGED = 1, /* some scene's CG stopped at cg_max_iters */
    MPM_NONFINITE = 2,        /* NaN or Inf reached a particle position */
    MPM_CAPACITY = 3,         /* particle, node-block or work-item capacity exceeded; the results of
                                 the call are not valid (recreate the context with larger capacities) */
    MPM_BAD_ARG = 4,          /* invalid argument (null pointer, bad size, bad index) */
    MPM_CUDA_ERROR = 5,       /* a CUDA runtime call failed; see mpm_last_error */
    MPM_NOT_READY = 6         /* call order violated (e.g. advance before initialize) */
} mpm_status;

typedef enum mpm_precision {
    MPM_PRECISION_FP32 = 0,  /* everything FP32 (the reference's shipped T=float) */
    MPM_PRECISION_MIXED = 1, /* FP32 state, transfers and CG vectors; FP64 SVD/polar, CG dots and norms */
    MPM_PRECISION_FP64 = 2   /* everything FP64 (the reference built with T=double) */
} mpm_precision;

typedef enum mpm_dtype { MPM_F32 = 0, MPM_F64 = 1 } mpm_dtype;

typedef struct mpm_config {
    int precision;            /* mpm_precision */
    int device;               /* CUDA device ordinal */
    int use_graphs;           /* 1: each substep is one CUDA graph launch with a device-side CG loop */
    int max_scenes;           /* <= MPM_MAX_SCENES */
    long long max_particles;  /* particle capacity over all scenes */
    long long max_blocks;     /* capacity of active 4x4x4 node blocks over all scenes; 0: derived */
    int chunk;                /* max particles per transfer work item (32..4096); 0: default 1024 */
} mpm_config;

/* MPM_Plane_Barrier (MPM_Plane_Barrier.h:13-32): grid velocities at cell centres with
 * (x - surface).normal < 0 are projected (Grid_Based_Collision_Helper.h:57-85). The
 * reference stores but never reads `sticky`; here sticky=1 zeroes the velocity there. */
typedef struct mpm_barrier {
    double normal[3];
    double surface[3];
    double mu;
    int sticky;
} mpm_barrier;

/* One scene: a cell-centred grid over [0,1]^3 with counts[a] cells per axis (each a
 * multiple of 4), plus the solver and material constants the reference hard-codes in
 * MPM_Example's constructor (MPM_Example.cpp:73-82) and sets per particle in
 * Standard_Tests (mpm_3d/Standard_Tests/Standard_Tests.h:81-85). */
/* Material of a scene's particles. Snow: fixed-corotated elasticity with Stomakhin
 * plasticity (MPM_Constitutive_Model). EOS fluid: the reference's particle.eos branch
 * (MPM_Example.cpp:599, 737-745, 774-782; MPM_CG_System.h:102-107, 138-140), pressure
 * from density through bulk_modulus and eos_gamma; the density is carried in the Jp slot. */
typedef enum mpm_material { MPM_MATERIAL_SNOW = 0, MPM_MATERIAL_EOS_FLUID = 1 } mpm_material;

typedef struct mpm_scene_desc {
    int counts[3];
    double gravity[3];        /* reference default (0,-2,0) */
    double flip;              /* FLIP/PIC blend, reference 0.9 */
    double cg_abs_tol;        /* reference 1e-7 (absolute, on the max-norm of the residual) */
    double cg_rel_tol;        /* tolerance = max(abs, rel * max-norm of the right-hand side) */
    int cg_max_iters;         /* reference 10000 */
    int cg_min_iters;         /* reference 0 */
    int project;              /* 1: zero CG vectors at nodes inside a barrier half-space */
    int plastic;              /* snow plasticity on (reference per particle: constitutive_model.plastic) */
    double hardening;         /* xi */
    double compression_yield; /* 1 - theta_c */
    double stretching_yield;  /* 1 + theta_s */
    double hardening_max;     /* cap on xi(1-Jp); reference FLT_MAX */
    int n_barriers;
    mpm_barrier barriers[MPM_MAX_BARRIERS];
    int material;             /* mpm_material of every particle of the scene */
    double bulk_modulus;      /* EOS fluid (MPM_Particle.h:36, default 1e7) */
    double eos_gamma;         /* EOS fluid exponent (MPM_Particle.h:37, default 7) */
} mpm_scene_desc;

/* Particle arrays, particle-major (AoS rows): X and V n*3, Fe n*9 (row-major 3x3).
 * Element type of every array is `dtype`. Inputs: Fe NULL = identity, Jp NULL = 1,
 * V0 NULL (or entries <= 0) = computed by mpm_initialize from the grid density; for
 * mpm_add_particles and mpm_set_particles a non-NULL `valid` marks particles with 0 as
 * removed (and the others as simulated): removed slots added up front are a reserve for
 * mpm_allocate_particles. Outputs: any NULL array is skipped; `valid` (int) marks
 * particles still simulated. */
typedef struct mpm_particle_arrays {
    long long n;
    int dtype;                /* mpm_dtype */
    void* X;
    void* V;
    void* mass;
    void* lambda0;            /* Lame parameters from Compute_Lame_Parameters (MPM_Constitutive_Model.cpp:23-28) */
    void* mu0;
    void* Fe;
    void* Jp;                 /* det of the plastic deformation gradient */
    void* V0;                 /* initial particle volume */
    int* valid;
} mpm_particle_arrays;

typedef struct mpm_stats {
    long long n_particles;    /* particles in the scene, valid or not */
    long long n_valid;        /* particles still simulated */
    long long n_active_blocks;/* 4x4x4 node blocks allocated this substep */
    long long n_interior;     /* grid nodes with mass (Cell_Type_Interior) */
    int cg_iterations;        /* CG iterations of the last substep */
    int cg_converged;
    double cg_residual;       /* max-norm of the final residual */
    double cg_tolerance;
    long long substeps;       /* substeps completed */
    long long gpu_launches;   /* kernels launched by this context so far (graph nodes included) */
} mpm_stats;

MPM_API const char* mpm_status_string(mpm_status s);
MPM_API void mpm_default_config(mpm_config* cfg);
/* Reference constants (MPM_Example.cpp:73-82, MPM_Driver.cpp:58-60, Standard_Tests.h:81-85). */
MPM_API void mpm_default_scene(mpm_scene_desc* desc);

/* Allocates the device state. Replaces MPM_Example's constructor and the hierarchy it
 * rebuilds every substep (MPM_Example.cpp:73-119, :325-331). */
MPM_API mpm_status mpm_create(const mpm_config* cfg, struct mpm_context** out);
MPM_API mpm_status mpm_destroy(struct mpm_context* ctx);
MPM_API const char* mpm_last_error(const struct mpm_context* ctx);

/* Registers a scene. Replaces the Example options (-size, MPM_Example.cpp:856-864) and
 * the barrier list Standard_Tests appends (Standard_Tests.h:56-57). */
MPM_API mpm_status mpm_add_scene(struct mpm_context* ctx, const mpm_scene_desc* desc, int* scene_id);

/* Appends particles to a scene. Replaces Standard_Tests::Initialize_Particles appending
 * to MPM_Example::particles (Standard_Tests.h:47-110) and Allocate_Particle
 * (MPM_Example.cpp:959-975). */
MPM_API mpm_status mpm_add_particles(struct mpm_context* ctx, int scene, const mpm_particle_arrays* p);

/* First grid build and first-touch particle volumes. Replaces MPM_Driver::Initialize
 * (MPM_Driver.cpp:18-32): Rasterize + Process_Waiting_Particles (MPM_Example.cpp:827-840). */
MPM_API mpm_status mpm_initialize(struct mpm_context* ctx);

/* One substep of every scene. Replaces MPM_Driver::Advance_Step (MPM_Driver.cpp:103-116):
 * grid build, P2G, plasticity, explicit force, collision, implicit CG, G2P. Returns after
 * the substep has completed on the device. */
MPM_API mpm_status mpm_advance_step(struct mpm_context* ctx, double dt);
/* k substeps with one host synchronisation at the end. */
MPM_API mpm_status mpm_advance_steps(struct mpm_context* ctx, int k, double dt);
/* A substep stopped after a phase, for phase-by-phase checks: 1 after Rasterize (m, v),
 * 2 after explicit force and collision (v*), 3 after the CG solve. The particle state is
 * not advanced; the next call rebuilds the grid. */
MPM_API mpm_status mpm_advance_step_partial(struct mpm_context* ctx, double dt, int stop_after);

/* Replaces MPM_Example::Max_Particle_Velocity (MPM_Example.cpp:375-387). */
MPM_API mpm_status mpm_max_particle_velocity(struct mpm_context* ctx, int scene, double* vmax);

/* Particle state of a scene in insertion order. Replaces the particle output of
 * Write_Output_Files (MPM_Example.cpp:1049-1063, Read_Write_MPM_Particles.h:33-46). */
MPM_API mpm_status mpm_get_particles(struct mpm_context* ctx, int scene, mpm_particle_arrays* out);
/* Overwrites the state of a scene's particles (same count, insertion order). Replaces
 * Read_Output_Files (MPM_Example.cpp:1075-1079); mass/lambda0/mu0/V0 NULL keep the
 * current values. */
MPM_API mpm_status mpm_set_particles(struct mpm_context* ctx, int scene, const mpm_particle_arrays* p);
/* mpm_get_particles / mpm_set_particles for `count` scenes (scenes[k] with arrays[k]) in one
 * call, for a driver that holds a batch of scenes (each the reference's Write_Output_Files /
 * Read_Output_Files of one example). Scenes whose host arrays the device reads and writes in
 * place are queued back to back and waited for once; the call returns when every copy is
 * complete, as the single-scene calls do. On an error the scenes before it are done. */
MPM_API mpm_status mpm_get_particles_batch(struct mpm_context* ctx, int count, const int* scenes, mpm_particle_arrays* arrays);
MPM_API mpm_status mpm_set_particles_batch(struct mpm_context* ctx, int count, const int* scenes, const mpm_particle_arrays* arrays);
/* New particles in a running scene. Replaces Allocate_Particle(true) (MPM_Example.cpp:
 * 959-975), which reuses the slot of a removed particle (invalid_particles) before it
 * appends one. A scene's slots are fixed when mpm_initialize runs, so here every new
 * particle takes the slot of one of the scene's removed particles, lowest insertion index
 * first (the reference takes the most recently removed one); MPM_CAPACITY when the scene
 * has fewer removed particles than p->n (add reserve slots with mpm_add_particles and
 * valid = 0). X, V, mass, lambda0, mu0 are required; Fe NULL = identity, Jp NULL = 1 (the
 * reference resets the particle); V0 NULL or <= 0 is computed at once from the grid
 * density at the current positions (Process_Waiting_Particles, MPM_Example.cpp:827-840,
 * which the reference runs at the start of the next substep, before any particle has
 * moved). ids (may be NULL) receives each new particle's insertion index in the scene. */
MPM_API mpm_status mpm_allocate_particles(struct mpm_context* ctx, int scene, const mpm_particle_arrays* p, int* ids);

MPM_API mpm_status mpm_get_stats(struct mpm_context* ctx, int scene, mpm_stats* out);

/* Flag_Helper counts (Flag_Helper.h:31-60) over the last grid: [0] cells of the particle
 * bounding box (Rasterize_Voxels' Dirichlet set, MPM_Example.cpp:291-302), [1] Interior
 * nodes (mass > 0, Flag_Setup_Helper.h:25-35), [2] both. */
MPM_API mpm_status mpm_flag_counts(struct mpm_context* ctx, int scene, long long out[3]);

/* Interior nodes of the last grid build: cell coordinates (n*3), mass, v, v* (n*3) in
 * FP64. *n returns the count; pass capacity 0 to query it. */
MPM_API mpm_status mpm_get_interior_nodes(struct mpm_context* ctx, int scene, long long capacity,
                                          int* coords, double* mass, double* v, double* vstar, long long* n);
/* Active 4x4x4 blocks of the last grid build, as block coordinates (n*3, cells/4). */
MPM_API mpm_status mpm_get_active_blocks(struct mpm_context* ctx, int scene, long long capacity,
                                         int* coords, long long* n);
/* Sorted cell keys and the particle order of the last sort (all scenes). The key of a
 * particle in cell (i,j,k) of scene s is ((base_s + bx + nbx*(by + nby*bz)) << 6) |
 * (lx + 4*ly + 16*lz) with (b,l) = divmod(cell + 4, 4), nb = counts/4 + 2 blocks per axis,
 * base_s the sum of the block counts of earlier scenes; removed particles sort last with
 * key 0xFFFFFFFF. The sort is stable and orders by block (key >> 6) only: inside a block the
 * particles keep their previous order. order[i] is the insertion index (within its scene)
 * of sorted particle i. */
MPM_API mpm_status mpm_get_sort(struct mpm_context* ctx, long long capacity, uint32_t* keys, int* order,
                                int* scene_of, long long* n);

MPM_API mpm_status mpm_synchronize(struct mpm_context* ctx);
MPM_API void* mpm_stream(struct mpm_context* ctx);

/* Per-phase device timing (CUDA events on the context stream). While enabled, substeps
 * run eagerly with events around each phase. */
MPM_API mpm_status mpm_set_timing(struct mpm_context* ctx, int enabled);
/* Phase names and accumulated milliseconds and launch counts since timing was enabled;
 * returns the number of phases. */
MPM_API int mpm_get_phase_times(struct mpm_context* ctx, int capacity, const char** names, double* ms,
                                long long* launches);
/* Device time of k substeps measured with CUDA events on the context stream. */
MPM_API mpm_status mpm_time_steps(struct mpm_context* ctx, int k, double dt, double* ms);

/* CG iterations and Interior node counts of every scene's last substep in one device read
 * (per scene, mpm_get_stats reports the same with more fields). *n_scenes (may be NULL)
 * receives the scene count; pass capacity 0 to query it. No counterpart in the reference,
 * whose CG is silent (MPM_CG_System.h:233-234). */
MPM_API mpm_status mpm_get_cg_iterations(struct mpm_context* ctx, int capacity, int* iterations,
                                         long long* interior_nodes, int* n_scenes);

/* Check of the bounded waits (no counterpart in the reference, whose OpenMP loops never
 * wait on another thread's flag). The block sort and the binning scans find their offsets
 * by a decoupled look-back: a CTA waits for an earlier CTA's published word, and every such
 * wait gives up after a bounded number of polls. This runs one look-back on a status array
 * whose predecessor never publishes, with the wait limited to spin_limit polls (1..2^22,
 * about 40 ns each): the wait gives up, sets the context's device error flag and returns,
 * and the call reports MPM_CUDA_ERROR ("sort look-back wait exceeded its limit"), as a
 * substep whose wait ran out would. The context stays usable; the next call clears the
 * flag. Needs mpm_initialize. */
MPM_API mpm_status mpm_selftest_lookback_wait(struct mpm_context* ctx, int spin_limit);

/* Simulation clock: seconds simulated since mpm_initialize (or the last mpm_set_time).
 * Fixed-dt substeps advance it by dt; mpm_advance_to_time by its substeps. */
MPM_API mpm_status mpm_get_time(struct mpm_context* ctx, double* time);
MPM_API mpm_status mpm_set_time(struct mpm_context* ctx, double time);
/* Replaces MPM_Driver::Advance_To_Target_Time (MPM_Driver.cpp:55-80) with
 * Max_Particle_Velocity (MPM_Example.cpp:375-387): substeps from the clock to
 * `target_time`, each of size clamp(cfl dx / max(max_v, 1e-2), 1e-6, 5e-3) computed on the
 * device from the current particle velocities, the last one landing on the target and the
 * one before it halving the rest when less than two remain. With several scenes the
 * substep takes the smallest scene dt. With CUDA graphs the whole advance is one graph
 * launch (the loop is a conditional node; no host round trip per substep). Stops after
 * max_substeps substeps (the clock then stops short of the target). *substeps_done (may
 * be NULL) receives the number of substeps. */
MPM_API mpm_status mpm_advance_to_time(struct mpm_context* ctx, double target_time, double cfl, int max_substeps,
                                       int* substeps_done);

/* Launch configuration of the transfer kernels (P2G, the Hessian product, G2P). */
typedef struct mpm_launch_config {
    int chunk;            /* particles per work item (the "particles per block" of a CTA) */
    int ctas_hessian;     /* occupancy variant: resident CTAs per SM the registers are capped */
    int ctas_p2g;         /*   for (3, 4, 5, 6 or 8) */
    int ctas_g2p;
    int grid_per_sm;      /* CTAs per SM launched for the grid-stride loop over work items */
    int node_grid_per_sm; /* CTAs per SM of the node kernels (grid update, CG vector updates) */
    int hessian_warp_items; /* form of the Hessian product: 1 each work item handled by one warp
                               (no CTA barriers; for launches with many work items per SM), 0 by
                               a whole CTA, 2 chosen per launch on the device: a warp per item
                               when the launch has at least as many work items as warps can be
                               resident (the first product and the early CG trips of a large
                               scene or batch), else a CTA per item (small scenes, and the last
                               trips when few scenes still iterate).
                               Default 2 */
    int incremental_sort; /* binning of a substep: 0 a full stable radix sort of the cell keys;
                             1 the same order obtained by sorting only the particles whose
                             block changed since the previous substep and merging them into
                             the previous order (bit-identical; cheaper when few move).
                             Default 0; MPM_SORT_INCREMENTAL=1 in the environment sets 1 */
} mpm_launch_config;

typedef struct mpm_tune_result {
    mpm_launch_config chosen;
    mpm_launch_config initial;
    double ms_per_substep;          /* median device time per substep of the chosen configuration */
    double ms_per_substep_initial;  /* the same for the configuration before tuning */
    int trials;                     /* configurations timed */
} mpm_tune_result;

/* The context's current launch configuration. */
MPM_API mpm_status mpm_get_launch_config(struct mpm_context* ctx, mpm_launch_config* out);
/* Sets the launch configuration (validated; the CUDA graphs are rebuilt at the next substep). */
MPM_API mpm_status mpm_set_launch_config(struct mpm_context* ctx, const mpm_launch_config* cfg);
/* Autotuner; no counterpart in the reference, whose OpenMP loops have nothing to tune.
 * Times candidate launch configurations on the context's own scenes and keeps the
 * fastest: the Hessian's form (work items per warp or per CTA), the work-item size
 * (256..2048 particles), the occupancy variant of each transfer kernel, the transfer grid
 * size, the node-kernel grid size and the binning (full or incremental sort), one
 * coordinate at a time, in two sweeps (the second from the first one's best, timing only
 * configurations not yet timed). Each trial starts
 * from the same saved particle state, runs one untimed substep of size dt (graph build)
 * and then `substeps` timed substeps; the median per-substep time ranks the candidates.
 * The particle state, the buffer parity and the substep counters are restored afterwards,
 * so tuning consumes no simulated time. Needs mpm_initialize; allocates a temporary copy
 * of the particle state. `out` may be NULL. */
MPM_API mpm_status mpm_autotune(struct mpm_context* ctx, double dt, int substeps, mpm_tune_result* out);

/* Stable LSD radix sort of n (key, value) pairs that allocates no device memory. It has no
 * counterpart in the reference (whose Group_Particles bins particles on the host); it is
 * the pair sort of the substep's particle binning, offered for callers that cannot
 * allocate when they sort: a host recording its loop into a CUDA graph (cudaMalloc is not
 * allowed during stream capture), a real-time loop that cannot take cudaMalloc's device
 * synchronisation, or a framework that owns all device memory.
 * keys_in, vals_in (NULL: the values are 0..n-1), keys_out and vals_out are device arrays
 * of n entries; outputs must not overlap inputs. Pairs are ordered by the key bits from
 * begin_bit upward in ceil((end_bit-begin_bit)/8) 8-bit digits, ties keeping input order.
 * Work runs on `stream` (NULL: the default stream) and is not waited for.
 * Limit: n <= MPM_NOALLOC_SORT_MAX (1,048,576); larger n returns MPM_BAD_ARG.
 * The working memory is one fixed static device area of about 8.3 MB per GPU, held from
 * library load to process exit and shared by every call on that GPU: calls that overlap
 * on the GPU (different streams, other threads) race and must be serialised by the
 * caller. Every byte of it is rewritten before it is read, so a call does not depend on
 * what an earlier call left. The first call on a device looks up the area's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before any stream
 * capture. */
#define MPM_NOALLOC_SORT_MAX (1LL<<20)
MPM_API mpm_status mpm_sort_pairs_noalloc(const uint32_t* keys_in, const int32_t* vals_in, uint32_t* keys_out,
                                          int32_t* vals_out, long long n, int begin_bit, int end_bit, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MPM_GB300_H */
