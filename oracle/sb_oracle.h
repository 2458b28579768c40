/*
 * Dump interface shared by the two CPU checkers (test infrastructure only; never linked into the product):
 *   - libsb_oracle.so : our C++ restatement of the reference's boolean path (sb_oracle.cpp)
 *   - libsbref.so     : the reference's own sources compiled here, wrapped by ref_harness.cpp
 *
 * A run returns an opaque handle holding named arrays (int64 or float64). Names:
 *   status            [1]   combine() result (1 = true)
 *   cand              [C*2] candidate (AABB-overlap) pairs (first tri, second tri), in the reference's order
 *   isect             [C]   1 where the pair intersects non-coplanarly
 *   seg               [C*6] segment (source xyz, target xyz) for intersecting pairs, 0 otherwise
 *   newv              [V*3] resultVertices()
 *   newt              [T*3] every triangle of the combined arrangement (m_newTriangles)
 *   groups_a_off/_a   CSR triangle groups of the first mesh; groups_b_off/_b of the second
 *   sides_a, sides_b  group sides (1 = inside the other mesh)
 *   union, diff, intersect  [n*3] the three fetch results
 *   leaforder_a/_b    triangles in leaf order of each mesh's AABB tree
 *   ctx_a, ctx_b      (restatement only) cut faces of each mesh in their context map's iteration order
 *   loops_a_off/_a    (restatement only) CSR of the first mesh's cut loops, as buildPolygonsFromEdges lists them
 *   tri_ranges        (restatement only) [4] arrangement triangles: uncut first, uncut second, re-triangulated
 *                     first, re-triangulated second
 *   time_ms           per-stage wall times (prepareA, prepareB, search, process, addUnint, retri, loops,
 *                     groups, sides)
 */
#ifndef SB_ORACLE_H
#define SB_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

void *sbo_run(const double *va, size_t nva, const uint32_t *ta, size_t nta,
              const double *vb, size_t nvb, const uint32_t *tb, size_t ntb, long quantum);
/* The same with the robust mode's flags (sb_robust in include/solidboolean_gb300.h; not the reference). */
void *sbo_run_robust(const double *va, size_t nva, const uint32_t *ta, size_t nta,
                     const double *vb, size_t nvb, const uint32_t *tb, size_t ntb, long quantum, int flags);
long sbo_len(void *h, const char *name);
int sbo_get_i64(void *h, const char *name, int64_t *out);
int sbo_get_f64(void *h, const char *name, double *out);
void sbo_free(void *h);

/* earcut of one polygon with holes; xy is [n*2], ring_off is [nrings+1]. Returns the index count
 * written to out (or needed, when larger than cap). */
long sbo_earcut(const double *xy, const int64_t *ring_off, long nrings, int64_t *out, long cap);

/* Guigue-Devillers intersection of one pair: returns the function value, writes coplanar and the
 * segment (6 doubles). */
int sbo_tritri(const double *p1, const double *q1, const double *r1, const double *p2,
               const double *q2, const double *r2, int *coplanar, double *seg);

#ifdef __cplusplus
}
#endif
#endif
