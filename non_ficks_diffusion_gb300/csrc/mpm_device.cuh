// mpm_device.cuh — device data layout shared by every kernel.
//
// Particles: structure-of-arrays, 20 fields per particle in one allocation, field-major
// ([field][capacity]): X0..2, V0..2, Fe00..Fe22 (row-major), Jp, m, V0, lambda0, mu0.
// Two such buffers alternate every substep: the transfer kernel reads particle i of the
// old buffer through the sort permutation and writes it to slot i of the new one, so the
// state is always stored in cell order. A per-particle cache of 11 fields (Re, lambda, mu)
// is written by the same kernel for the CG's Hessian action.
//
// Grid: 4x4x4 node blocks. Cell (i,j,k) of a scene with counts n is stored at block
// (b = (i+4)>>2, ...), local (l = (i+4)&3, ...); each scene owns a dense range of
// nb = n/4+2 blocks per axis starting at its global block base, so the guard layer
// -1..n of every particle stencil always has a block. A bitmap over all global blocks
// marks the blocks some stencil touches; active blocks get consecutive indices in global
// block order and their 64 nodes are stored contiguously per channel (node = idx*64 + l).
#pragma once
#include "mpm_math.cuh"

namespace mpm {

constexpr int NB_FIELDS=20;
enum { FX=0, FV=3, FF=6, FJP=15, FM=16, FV0=17, FLAM0=18, FMU0=19 };
constexpr int NC_FIELDS=11;
enum { CR=0, CLAM=9, CMU=10 };
constexpr unsigned KEY_SENTINEL=0xFFFFFFFFu;
constexpr int MAX_BARRIERS=16;
constexpr int MAX_SCENES=256;

template<class T> struct alignas(4*sizeof(T)) V4 { T x,y,z,w; };

template<class T> struct SceneDev {
    int counts[3];
    int nb[3];
    long long block_base;           // first global block id of the scene
    long long pid_base;             // first insertion index of the scene
    T dx[3],inv_dx[3];
    T gravity[3];
    T flip;
    int plastic; T hardening,cy,sy,hmax;
    int project;
    int n_barriers;
    T bn[MAX_BARRIERS][3],bs[MAX_BARRIERS][3],bmu[MAX_BARRIERS];
    int bsticky[MAX_BARRIERS];
    double cg_abs_tol,cg_rel_tol;
    int cg_max_iters,cg_min_iters;
    int eos; T bulk,eos_gamma;      // EOS fluid scene (density in the Jp slot)
};

// Per-scene solver state, written only by the last CTA of a reduction kernel.
struct CGState {
    double rho;                // <r,r>_M of the current residual
    double alpha,beta;
    double tol;                // absolute tolerance of this substep
    double residual;           // max-norm of the residual at the last check
    int iters;                 // completed CG iterations
    int done,converged;
    int n_interior;            // nodes with mass this substep
};
// Per-scene accumulators, zeroed by the consumer after use.
struct SceneAcc {
    double sum0,sum1;          // dot products
    unsigned long long max0;   // bit pattern of a non-negative double max
    unsigned long long count0;
};

// Where each scene's entries sit in this substep's work-item list [c0, c1) and active-block
// list [b0, b1). Both lists are in global block order and scenes own consecutive global
// block ranges, so each scene's entries are contiguous. Zeroed before every substep (a
// scene without particles keeps empty ranges).
struct SceneRange { int c0,c1,b0,b1; };
// The scenes whose CG still iterates, in scene order, with exclusive prefix sums of their
// work-item and active-block counts (cpre[n], bpre[n] are the totals). Written by the last
// CTA of the kernel that checks convergence; the next loop trip's kernels walk only these
// scenes' work items and nodes.
struct ActiveList { int n; int scene[MAX_SCENES]; int cpre[MAX_SCENES+1]; int bpre[MAX_SCENES+1]; };

struct Counters {
    unsigned n_valid;          // valid particles after the key pass
    unsigned n_chunks;
    unsigned n_active;         // active node blocks
    unsigned error;            // MPM_ERR_* bits
    unsigned bad_scene1;       // 1 + the highest scene index that had a non-finite position
    unsigned ticket[8];        // last-CTA detection, one per reduction kernel
    int any_active;            // some scene's CG still runs
    int loop_iters;            // CG loop trips this substep
    unsigned long long total_trips;   // CG loop trips since the context was created
};
enum { ERR_CAPACITY=1u, ERR_NONFINITE=2u, ERR_OUT_OF_GRID=4u, ERR_CG_NOT_CONVERGED=8u, ERR_SORT_WAIT=16u };

// Device-side time stepping of mpm_advance_to_time: the reference's CFL rule and
// end-of-frame split (MPM_Driver.cpp:55-80), evaluated on the device before every substep.
struct FrameState {
    double time;          // simulation clock
    double target;        // end of this advance
    double cfl,dt_min,dt_max;
    double dt_last;       // size of the latest substep
    int done;             // the latest substep ends the advance
    int substeps;         // substeps taken by this advance
    int max_substeps;     // bound on them
    int pad;
};

// Everything a kernel needs, passed by value.
template<class T> struct DevState {
    // particles
    T* pcur; T* pnxt;               // [NB_FIELDS][pcap]
    int* pid_cur; int* pid_nxt;     // insertion index (global)
    int* scn_cur; int* scn_nxt;     // scene id s, or -(s+1) once removed
    T* cache;                       // [NC_FIELDS][pcap]
    long long pcap;
    long long n_total;              // particle slots in use (host-known)
    unsigned* keys; int* perm;      // sorted keys and source slots (output of the sort)
    // work items
    int* chunk_start; long long chunk_cap;
    // blocks
    unsigned* bitmap; long long bitmap_words;
    int* blockmap;                  // global block id -> active index (valid where the bitmap bit is set)
    int* active_gb;                 // active index -> global block id
    int* active_scene;
    long long block_cap;
    // nodes (block_cap*64)
    V4<T>* gv;                      // (mv, m) while rasterizing, then (v, m)
    V4<T>* gf;                      // explicit force, then CG q
    V4<T>* gx;                      // v* / CG solution x
    V4<T>* gr;                      // CG residual (right-hand side before the solve)
    V4<T>* gs;                      // CG search direction
    T* gm;                          // node mass (0 where not Interior)
    unsigned char* gproj;           // 1 where Project zeroes the CG vectors (set by the grid update)
    // scenes
    const SceneDev<T>* scenes; int n_scenes;
    const long long* scene_block_base;   // n_scenes+1 ascending
    CGState* cg; SceneAcc* acc; SceneAcc* acc2;
    SceneRange* srange;             // per scene, this substep
    ActiveList* alist;              // scenes of the next CG loop trip
    Counters* ctr;
    const double* dtp;              // substep size, set on the stream before each substep
    int chunk;                      // particles per work item
};

// Programmatic dependent launch. A kernel of the substep may be scheduled while the one
// before it in the stream drains (once all of that grid's CTAs have exited): it first
// waits until that grid has completed and its writes are visible (at once when it was
// launched without the attribute).
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ int scene_of_block(const long long* base,int n,long long gb)
{
    int lo=0,hi=n-1;
    while(lo<hi){int mid=(lo+hi+1)>>1;if(base[mid]<=gb) lo=mid;else hi=mid-1;}
    return lo;
}
__device__ __forceinline__ bool bit_set(const unsigned* bm,long long gb)
{return (bm[gb>>5]>>(gb&31))&1u;}

} // namespace mpm
