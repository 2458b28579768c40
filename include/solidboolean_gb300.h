/*
 * solidboolean_gb300 — C ABI of the GB300 mesh-boolean path.
 *
 * Drop-in for the reference's call sequence (huxingyi/solidboolean):
 *
 *   reference (C++)                                         this library
 *   SolidMesh m; m.setVertices(&v); m.setTriangles(&t);     sb_mesh_create(xyz, nv, tris, nt, &m)
 *     (src/solidmesh.h:33-34, src/solidmesh.cpp:32-40)
 *   m.prepare()            (src/solidmesh.cpp:42-76)        sb_mesh_prepare(m, &opts)
 *   SolidBoolean b(&m1, &m2) (src/solidboolean.h:36-37)     sb_boolean_create(m1, m2, &opts, &b)
 *   bool ok = b.combine()  (src/solidboolean.cpp:288-480)   sb_combine(b, &stats) == SB_OK
 *   b.fetchUnion(tris)     (src/solidboolean.cpp:512-527)   sb_fetch(b, SB_UNION, ...)
 *   b.fetchDiff(tris)      (src/solidboolean.cpp:529-548)   sb_fetch(b, SB_DIFF, ...)
 *   b.fetchIntersect(tris) (src/solidboolean.cpp:550-565)   sb_fetch(b, SB_INTERSECT, ...)
 *   b.resultVertices()     (src/solidboolean.cpp:567-570)   sb_result_vertices(b, ...)
 *
 * Every call returns an sb_status; no exception crosses the ABI. Handles own their device memory until
 * the matching *_destroy. A handle is not thread-safe; distinct handles are independent. Work is ordered
 * on the stream given in sb_options (0 = the legacy default stream); functions that return host data
 * synchronise that stream.
 */
#ifndef SOLIDBOOLEAN_GB300_H
#define SOLIDBOOLEAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sb_mesh sb_mesh;
typedef struct sb_boolean sb_boolean;

typedef enum sb_status {
    SB_OK = 0,
    /* combine() returned false in the reference (src/solidboolean.cpp:368-370, 427-445) */
    SB_FAIL_ATTACH = 1,      /* "Attach point to triangle edge failed" (src/retriangulator.cpp:149-152) */
    SB_FAIL_LINK = 2,        /* "linkTo failed" (src/retriangulator.cpp:227-229) */
    SB_FAIL_LOOP = 3,        /* cut edges do not form closed loops (src/solidboolean.cpp:150-158) */
    /* library errors */
    SB_ERR_INVALID = 10,     /* bad argument, index out of range, call out of order */
    SB_ERR_CUDA = 11,        /* a CUDA runtime call failed; see sb_last_error() */
    SB_ERR_CAPACITY = 12,    /* a per-face scratch bound was exceeded (never expected; reported, not hidden) */
    SB_ERR_NOT_COMBINED = 13 /* fetch before a successful combine */
} sb_status;

typedef enum sb_op { SB_UNION = 0, SB_DIFF = 1, SB_INTERSECT = 2 } sb_op;

/* Arithmetic of the orientation predicates and box tests. Both give identical results. */
typedef enum sb_precision {
    SB_PRECISION_FILTERED = 0, /* FP32 with static forward-error bounds; FP64 only where not certified */
    SB_PRECISION_FP64 = 1      /* plain FP64 everywhere */
} sb_precision;

/* How the pairs of one cut face are ordered before its cut points are numbered. */
typedef enum sb_order {
    SB_ORDER_REFERENCE = 0, /* the reference's order (its AABB tree's leaf order), for bit-exact output */
    SB_ORDER_INDEX = 1      /* ascending triangle index (skips building the reference leaf order) */
} sb_order;

/* Robustness beyond the reference (bit flags of sb_options.robust). With 0, the default, every result is
 * the reference's. With any flag set, results may differ from the reference's where it would fail. */
typedef enum sb_robust {
    /* Point-on-edge test of the re-triangulation with a scale-relative bound, |cross| <= 256 eps L (L + S)
     * (L: the edge's larger 2D extent, S: the face's largest absolute coordinate), instead of the
     * reference's absolute |cross| <= eps (src/vector2.h:212-215 with src/double.h:30-33). A cut point
     * computed on the edge of a large face misses that absolute bound by rounding alone, and the reference
     * then fails with "Attach point to triangle edge failed" (src/retriangulator.cpp:149-152). */
    SB_ROBUST_EDGE_TOLERANCE = 1,
    /* When a combine fails (an SB_FAIL_* status), combine again with the weld factor ten times finer, while
     * the factor stays <= 1e12 and the largest absolute input coordinate times the factor stays below 2^52
     * (the quantum must stay coarser than FP64's resolution): cut points that a coarse quantum merges
     * break the reference's loops (src/solidboolean.cpp:150-158). */
    SB_ROBUST_WELD_RETRY = 2
} sb_robust;

typedef struct sb_options {
    int64_t weld_factor; /* PositionKey quantisation factor; the reference uses 100000 (src/positionkey.cpp:25) */
    int32_t precision;   /* sb_precision */
    int32_t order;       /* sb_order */
    void *stream;        /* cudaStream_t */
    uint32_t robust;     /* sb_robust flags; 0 (default) = the reference's behaviour */
    uint32_t stage_results; /* 1: sb_combine also copies the result vertices and the three fetch results to
                               page-locked host memory (see sb_take_staged); 0 (default): results stay on the
                               device until sb_fetch / sb_result_vertices copy them */
} sb_options;

typedef struct sb_stats {
    uint64_t candidate_pairs;    /* AABB-overlapping triangle pairs */
    uint64_t intersecting_pairs; /* non-coplanar intersecting pairs */
    uint64_t cut_faces_first, cut_faces_second;
    uint64_t new_points;         /* welded cut points appended after the input vertices */
    uint64_t result_vertices, result_triangles; /* arrangement sizes */
    uint64_t sign_tests;         /* orientation signs decided (filtered form) */
    uint64_t sign_fallbacks;     /* of those, re-evaluated in FP64 */
    uint64_t box_tests, box_fallbacks; /* leaf box tests and FP64 re-tests */
    uint32_t regions_first, regions_second;
    uint32_t failed_faces;       /* cut faces whose re-triangulation failed */
    uint32_t loop_vertices;      /* vertices of the cut loops */
    uint32_t loop_bad_degree;    /* loop vertices whose degree is not 2 */
    uint32_t duplicate_halfedges;
    uint32_t loops;              /* cut loops of the first mesh */
    uint32_t order_fallbacks;    /* cut faces whose place in the reference's processing order could not be
                                    derived (they keep triangle-index order; 0 when the order is exact) */
    uint32_t attempts;           /* combines run by this call: 1, more after SB_ROBUST_WELD_RETRY retries */
    uint32_t robust;             /* the sb_robust flags in effect */
    int64_t weld_factor_used;    /* the weld factor of the last attempt */
    double stage_ms[8];          /* broad, narrow, faces, weld, assemble, groups, sides, fetch (device time) */
} sb_stats;

void sb_default_options(sb_options *opts);
const char *sb_status_string(sb_status s);
const char *sb_last_error(void);
/* Number of this library's own kernel launches since load (sort/scan primitives excluded). */
uint64_t sb_kernel_launches(void);
/* Diagnostic device timing of the main kernels: enable (clears earlier records), then read the summed
 * event time and launch count of one kernel by name (synchronises), or the comma-separated names seen. */
void sb_kernel_timing(int enable);
int sb_kernel_timing_read(const char *name, double *total_ms, uint64_t *launches);
int sb_kernel_timing_names(char *buf, size_t cap);
/* Restrict the timing to the named kernels (comma-separated; NULL or "" for all). Each timed launch adds an
 * event pair to its stream, so a timed run is slower the more kernels it times. */
void sb_kernel_timing_select(const char *names);

/* Mesh: vertices are FP64 xyz triplets, triangles are uint32 index triplets. The host variant copies
 * the arrays; the device variant copies from device pointers on opts->stream. */
sb_status sb_mesh_create(const double *xyz, size_t nv, const uint32_t *tris, size_t nt, sb_mesh **out);
sb_status sb_mesh_create_device(const double *d_xyz, size_t nv, const uint32_t *d_tris, size_t nt,
                                const sb_options *opts, sb_mesh **out);
/* Replace the vertex positions (same count, device pointer) without rebuilding the handle. */
sb_status sb_mesh_update_vertices_device(sb_mesh *m, const double *d_xyz, const sb_options *opts);
/* Builds the mesh's search structures (LBVH, the reference tree's leaf order, edge adjacency) on
 * opts->stream and returns without waiting for them; sb_combine orders itself after the build, whatever its
 * stream, and reports a failure of the build as its own status. (sb_combine prepares unprepared meshes
 * itself, both at once.) */
sb_status sb_mesh_prepare(sb_mesh *m, const sb_options *opts);
void sb_mesh_destroy(sb_mesh *m);

sb_status sb_boolean_create(const sb_mesh *first, const sb_mesh *second, const sb_options *opts,
                            sb_boolean **out);
sb_status sb_combine(sb_boolean *b, sb_stats *stats);
/* Host results. Pass tris == NULL to query the count; cap is in triangles / vertices. */
sb_status sb_fetch(sb_boolean *b, sb_op op, uint32_t *tris, size_t cap, size_t *count);
sb_status sb_result_vertices(sb_boolean *b, double *xyz, size_t cap, size_t *count);
/* Device results: pointers stay valid until the next combine or destroy; counts are host values. */
sb_status sb_fetch_device(sb_boolean *b, sb_op op, const uint32_t **d_tris, size_t *count);
sb_status sb_result_vertices_device(sb_boolean *b, const double **d_xyz, size_t *count);
/* Stage dumps for parity checks (host copies). Names: "candidates" (uint32 pairs, in emission order),
 * "intersection_pairs" (uint32 pairs), "intersection_segments" (6 doubles per intersecting pair),
 * "arrangement" (uint32 triangles), "labels" (int8 per arrangement triangle: 0 outside, 1 inside, -1 in no
 * group), "tri_mesh" (int8 per arrangement triangle: 0 first mesh, 1 second), "new_sources" (int32 per
 * appended result vertex: 2 x its intersecting pair + the end of that pair's segment it was built from),
 * "rank_first" / "rank_second" (int32 per triangle: position in the reference tree's leaf order),
 * "loop_order_ns" (8 uint64: device time stamps at the phase boundaries of the loop-order stage),
 * "leaf_order_ns_first" / "_second" (96 uint64: per large-node level of the leaf-order build, the device
 * time at its start, after its classification and after its split; zero past the last level) (diagnostics). *bytes receives the size; out may be NULL. */
sb_status sb_debug_dump(sb_boolean *b, const char *name, void *out, size_t cap_bytes, size_t *bytes);
void sb_boolean_destroy(sb_boolean *b);

/* Diagnostic; its counterpart is mapbox::earcut (thirdparty/earcut.hpp/include/mapbox/earcut.hpp:833-838)
 * as the reference's ReTriangulator calls it. Runs the device ear-clipper that sb_combine uses inside cut
 * faces on one polygon with holes: xy [ring_off[n_rings] * 2] host doubles, rings back to back (the first
 * is the outer ring), ring_off [n_rings + 1] CSR offsets. Writes the triangle vertex indices (into the
 * concatenated rings, three per triangle) to indices (host, cap entries; NULL to query the count). Returns
 * SB_ERR_CAPACITY when the device's fixed scratch or iteration budget for the polygon's size is exceeded.
 * Allocates device memory and synchronises the device. */
sb_status sb_debug_earcut(const double *xy, const int64_t *ring_off, size_t n_rings, int64_t *indices, size_t cap,
                          size_t *count);

/* No counterpart in the reference. Re-triangulates cut faces exactly as sb_combine does, for callers that
 * cannot allocate device memory: code inside a framework that owns all device memory through its own pool
 * (an allocation behind its back breaks its accounting and can fail once the pool holds the free memory),
 * and real-time loops where a cudaMalloc or cudaFree could stall. It calls no cudaMalloc/cudaFree and no
 * allocating library routine; its workspace is a 64 MiB static device array inside the library (held by
 * every GPU that loads the library until exit). A request whose fixed layout does not fit returns
 * SB_ERR_CAPACITY before launching anything; one whose per-face workspace does not fit returns
 * SB_ERR_CAPACITY after a sizing pass that writes into the shared array (the call reads that size back and
 * synchronises its stream), without re-triangulating.
 *   d_corners   [n_faces*9]      three corners (xyz) of each face, in the face's vertex order
 *   d_seg_begin [n_faces+1]      CSR offsets of each face's segments (0 .. n_segments)
 *   d_segments  [n_segments*6]   cut segments (source xyz, target xyz) in the face's processing order
 *   d_tris      [n_faces*tri_cap*3] output: per face, local ids (0..2 corners, 3+k the face's k-th point)
 *   d_tri_count, d_point_count, d_status [n_faces] outputs (status 0 ok, 1 attach, 2 link, 3 capacity)
 *   d_points    [2*n_segments*3] output: the face's welded points at offset 2*seg_begin[f]
 * The first call on a device (with that device current) looks up the array's address and caches it: make
 * it before any stream capture. cudaDeviceReset invalidates the cached address. All calls share the array,
 * so calls that overlap on the GPU race; serialise them. */
sb_status sb_retriangulate_faces_noalloc(const double *d_corners, const int *d_seg_begin, const double *d_segments,
                                         int n_faces, int n_segments, int64_t weld_factor, int *d_tris, int tri_cap,
                                         int *d_tri_count, double *d_points, int *d_point_count, int *d_status,
                                         void *stream);

/* No counterpart in the reference, which combines one pair per call: many independent pairs in one call.
 * Inputs are host arrays in CSR form: pair i's first mesh has the vertices xyz_a[3*v_off_a[i] ..
 * 3*v_off_a[i+1]) and the triangles tris_a[3*t_off_a[i] .. 3*t_off_a[i+1]) (vertex indices local to that
 * mesh); likewise the second mesh; ops[i] (an sb_op) names the result kept for the pair. statuses[i]
 * receives what sb_combine would return for the pair. Pairs run on `workers` concurrent streams (at most 64),
 * each with reusable handles; workers <= 0 tunes the count: with at least 512 pairs, three runs of 64 pairs
 * on 4, 8 and 16 workers (their results are kept like any other) pick the fastest for the rest, else 8. With out non-NULL the results (all result vertices, the op's triangles) are kept
 * for sb_batch_result_size / sb_batch_result; with out NULL only the statuses are produced. The return value
 * reports failures of the batch itself (invalid arguments, stream or handle creation). */
/* No counterpart in the reference. Adjoint of the last sb_combine with its combinatorics held fixed: given
 * d_grad_result, the gradient of a loss with respect to every result vertex ([n*3] doubles on the device, in
 * sb_result_vertices order), adds the loss's gradient with respect to the input vertices to d_grad_first
 * ([nv_first*3]) and d_grad_second ([nv_second*3]) on the device (the caller zeroes them). An input vertex
 * passes its own gradient through; an appended vertex passes its gradient through the construction of the
 * intersection point that represents it (segment end p - a (p - r), a a ratio of dot products with a
 * triangle normal) to the six vertices of that triangle pair. Requires a combine that returned SB_OK;
 * runs on `stream` and does not synchronise. */
sb_status sb_adjoint(sb_boolean *b, const double *d_grad_result, double *d_grad_first, double *d_grad_second,
                     void *stream);

typedef struct sb_batch sb_batch;
sb_status sb_batch_combine(size_t n, const double *xyz_a, const uint64_t *v_off_a, const uint32_t *tris_a,
                           const uint64_t *t_off_a, const double *xyz_b, const uint64_t *v_off_b,
                           const uint32_t *tris_b, const uint64_t *t_off_b, const int32_t *ops,
                           const sb_options *opts, int32_t workers, int32_t *statuses, sb_batch **out);
sb_status sb_batch_result_size(const sb_batch *b, size_t i, size_t *n_vertices, size_t *n_triangles);
sb_status sb_batch_result(const sb_batch *b, size_t i, double *xyz, uint32_t *tris);
void sb_batch_destroy(sb_batch *b);

/* No counterpart in the reference. Page-locked host memory from a cache kept by the library, for result
 * buffers that sb_fetch / sb_result_vertices fill at DMA speed (a pageable destination is copied through the
 * driver's staging buffers and, when freshly allocated, first faulted in page by page). sb_host_alloc returns
 * SB_ERR_CUDA when no page-locked memory can be had; sb_host_free(NULL) does nothing. Thread-safe. */
sb_status sb_host_alloc(size_t bytes, void **ptr);
void sb_host_free(void *ptr);

/* No counterpart in the reference. With sb_options.stage_results set, sb_combine copies the result vertices
 * to page-locked host memory as soon as the weld has numbered them (on a copy stream, beside the rest of the
 * combine) and the three fetch results once their sizes are known, and returns with all four on the host.
 * sb_take_staged hands one of them over: what = SB_UNION, SB_DIFF or SB_INTERSECT (uint32 index triplets) or
 * SB_STAGED_VERTICES (FP64 xyz triplets); *count = its rows. The caller owns *host afterwards and releases it
 * with sb_host_free. *host is NULL when nothing is staged (staging off, already taken, zero rows, or no
 * page-locked memory): sb_fetch / sb_result_vertices still copy from the device. Buffers not taken are
 * released by the next combine and by sb_boolean_destroy. */
#define SB_STAGED_VERTICES 3
sb_status sb_take_staged(sb_boolean *b, int32_t what, void **host, size_t *count);

#ifdef __cplusplus
}
#endif
#endif
