/*
 * scenes.h - deterministic synthetic collision scenes (host C++).
 *
 * The reference measures on external OBJ/PLY trajectory pairs that are not
 * distributed with it; these generators produce seeded scenes with the
 * shapes of its benchmark configurations instead. Every generator is plain
 * C++ with its own PRNG (splitmix64 seeding a xoshiro256** stream, Gaussian
 * draws by Box-Muller), so the same seed gives the same bytes on one machine.
 *
 * Mesh layout follows the reference's inputs to constructBoxes
 * (src/io.cuh:9-13): V0/V1 row-major [nV x 3] fp64, E [nE x 2] int32,
 * F [nF x 3] int32; sheets are concatenated, vertex indices global.
 */
#ifndef STQ_SCENES_H
#define STQ_SCENES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Vertex, edge and face counts of one g x g cloth grid (2 triangles/cell). */
void stq_grid_counts(int g, int64_t *nV, int64_t *nE, int64_t *nF);

/* Cloth pair (sheet + copy offset in z and rotated about z around the sheet
 * centre): t0 z = 0.02 sin(6 pi x) cos(4 pi y); t1 = t0 + N(0, sigma^2).
 * Buffers sized 2*nV x 3, 2*nE x 2, 2*nF x 3 for the grid size g. */
void stq_scene_cloth_pair(int g, double z_offset, double angle_deg,
                          double sigma, uint64_t seed, double *V0, double *V1,
                          int32_t *E, int32_t *F);

/* `sheets` crumpled g x g unit sheets: 3-octave value noise z (amplitude
 * `amp`), random rotation, centre uniform in [0.5, 1.0]^3 (the sheets lie in
 * a 1.5^3 cube), t1 = t0 + N(0, sigma^2). Buffers sized sheets*nV etc. */
void stq_scene_crumpled(int sheets, int g, double amp, double sigma,
                        uint64_t seed, double *V0, double *V1, int32_t *E,
                        int32_t *F);

/* n random boxes: centres uniform in the unit cube, per-axis extents
 * lognormal(ln 0.002, 0.5); a fraction `sliver_frac` is stretched 200x
 * along a random axis. Box k is a vertex, edge or face box in the ratio
 * 1:3:2 (k mod 6) with vertex ids drawn from n/6 vertices; id = k. */
void stq_scene_random_boxes(int64_t n, double sliver_frac, uint64_t seed,
                            void *boxes /* stq_aabb[n] */);

/* Grid side g for a cloth pair of about `boxes` boxes. */
int stq_cloth_pair_grid_for(int64_t boxes);

/* Advances every t1 position by N(0, sigma^2) and moves t1 to t0
 * (one time step of a serving request): V0 <- V1, V1 <- V1 + noise. */
void stq_scene_step(int64_t nV, double sigma, uint64_t seed, double *V0,
                    double *V1);

/* splitmix64 of x: the per-scene seed derivation. */
uint64_t stq_splitmix64(uint64_t x);

#ifdef __cplusplus
}
#endif

#endif /* STQ_SCENES_H */
