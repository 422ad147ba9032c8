/* mpm_scenes.h — scene presets (the Standard_Tests surface) for the implicit MPM snow path.
 *
 * Replaces Standard_Tests::Initialize_Particles (mpm_3d/Standard_Tests/Standard_Tests.h:47-154,
 * mpm_2d/Standard_Tests/Standard_Tests.h:47-327): each test number yields a scene
 * description and its particles. Sampling is a jittered grid (ppc = k^d stratified
 * samples per cell) from a counter-based hash of (seed, scene, cell, sample), so the same
 * arguments give the same particles on every machine.
 *
 * Test numbers:
 *   100  2D snowball: 64^2, disk r=.12 at (.5,.7), V=(0,-2), 16 ppc.
 *   101  3D snowball: 128^3, sphere r=.15 at (.5,.6,.5), V=(0,-3,0), 8 ppc.
 *   102  two colliding snowballs: 256^3, r=.12 at (.3,.5,.5) V=(+3,0,0) and (.7,.52,.5)
 *        V=(-3,0,0) with E0 x1.5, 8 ppc.
 *   103  snow slab crash: 512^3, slab .5 x .08 x .5 on y in [.4,.48], V=(0,-4,0), 8 ppc,
 *        plus a 30-degree slip plane through (.5,.2,.5).
 *   104  batch of 64 scenes drawn from the seed: extents {64,128,256}^3, 1-3 spheres or boxes,
 *        E0 in [0.8e5,2e5], xi in [5,10], 8 ppc (scene_index 0..63).
 *    18  the reference's 3D test 18 parameters (two balls of 20000 particles, E=30, nu=.4,
 *        density 2, ground at y=.1, gravity (0,-2,0)) on a 64^3 grid, sampled uniformly in
 *        the balls with this file's hash.
 * Common to 100-104: density 400, E0=1.4e5, nu=0.2, xi=10, theta_c=2.5e-2, theta_s=7.5e-3,
 * gravity (0,-9.8,0), dt=1e-4, CG relative tolerance 1e-5 with at most 50 iterations,
 * FLIP 0.9, a sticky ground plane at y=2dx and slip walls 2dx from every other face.
 */
#ifndef MPM_SCENES_H
#define MPM_SCENES_H

#include "mpm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpm_preset_info {
    int dim;                 /* 2 or 3 */
    int scene_count;         /* scenes of this test number (64 for 104, else 1) */
    long long n_particles;   /* particles of the requested scene */
    double dt;               /* fixed substep */
    double frame_dt;         /* 1/24 */
    double density;
} mpm_preset_info;

/* Scene description and sizes of test `test_number`, scene `scene_index`. For dim 2 the
 * description's counts[2] is 1 and barrier normals have a zero z component. */
MPM_API mpm_status mpm_preset_scene(int test_number, int scene_index, unsigned long long seed,
                                    mpm_scene_desc* desc, mpm_preset_info* info);
/* The scene's particles as FP64 arrays: X, V (n*dim), mass, lambda0, mu0 (n). capacity is
 * the row capacity of the arrays (info.n_particles rows are written). */
MPM_API mpm_status mpm_preset_particles(int test_number, int scene_index, unsigned long long seed,
                                        long long capacity, double* X, double* V, double* mass,
                                        double* lambda0, double* mu0);

#ifdef __cplusplus
}
#endif

#endif /* MPM_SCENES_H */
