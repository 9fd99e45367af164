/*
 * stq_io.h - host-side mesh input and ground-truth comparison of the STQ
 * broad phase (plain C, implemented in libstq_gb300.so).
 *
 * Reference interfaces replaced (Ahdhn/broadphase-gpu):
 *   stq_read_mesh           <- igl::readOBJ / igl::readPLY in parseMesh
 *                              src/io.cu:30-51, src/cpu/io.cpp:16-37
 *   stq_mesh_edges          <- igl::edges(F, E) in parseMesh (libigl bf079eb,
 *                              a FetchContent dependency, cmake/recipes/libigl.cmake)
 *   stq_compare_truth_json  <- compare_mathematica src/groundtruth.cu:24-67
 *                              (and app/main.cpp:65-96)
 */
#ifndef STQ_IO_H
#define STQ_IO_H

#include <stdint.h>

#include "stq_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Reads a triangle mesh: Wavefront OBJ ("v x y z", "f a b c" with 1-based
 * indices, optional "/vt/vn" parts) or PLY (ascii or binary_little_endian;
 * vertex x, y, z as float or double; faces as a list of 3 indices), chosen by
 * the file extension. Two calls: with V and F NULL it only sets *nV and *nF;
 * then with buffers of nV x 3 doubles and nF x 3 int32. Returns STQ_OK or
 * STQ_ERR_INVALID_INPUT (unreadable, malformed, non-triangle face, index out
 * of range). */
int stq_read_mesh(const char *path, double *V, int64_t *nV, int32_t *F, int64_t *nF);

/* Unique undirected edges of a triangle list, each written (smaller, larger)
 * and ordered by (larger, smaller) index, the order libigl's edges() produces
 * from its column-major adjacency matrix. Two calls: E NULL sets *nE. */
int stq_mesh_edges(const int32_t *F, int64_t nF, int32_t *E, int64_t *nE);

/* Ground truth: reads a JSON array of pairs [[a, b], ...] and counts how many
 * of them occur in h_pairs[0..count) (both sides compared as (min, max)).
 * *found = truth pairs found, *truth = distinct truth pairs, *extra = distinct
 * pairs of h_pairs not in the truth (the reference reports only found/truth). */
int stq_compare_truth_json(const char *path, const stq_pair *h_pairs, int64_t count, int64_t *found,
                           int64_t *truth, int64_t *extra);

#ifdef __cplusplus
}
#endif

#endif /* STQ_IO_H */
