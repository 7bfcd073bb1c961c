/*
 * isoext_gb300.h -- C ABI of libisoext_gb300.so (GB300 / sm_103a iso-surface
 * extraction).
 *
 * The library replaces the compute behind isoext's Python extension module
 * (src/isoext_ext.cu in the isoext project, NB_MODULE(isoext_ext) at :93-384).
 * Each entry point below names the binding function it stands in for.
 *
 * Conventions
 *   - All array arguments are DEVICE pointers (cudaMalloc / torch CUDA memory),
 *     C-contiguous, except aabb_min / aabb_max which are HOST float[3].
 *   - Every call is asynchronous on `stream` (a cudaStream_t passed as void*;
 *     NULL = legacy default stream).  Sizes are known once the stream has
 *     reached the end of the call: read `counts` then.
 *   - Return value: 0 on success, otherwise an IsoStatus code for argument or
 *     launch errors; iso_last_error() gives the message (thread-local).
 *   - Errors found on the device are written to `*status` (device int, which
 *     the caller zeroes before the call): 3 = a bounded device wait ran out,
 *     4 = internal vertex lookup failure, 6 = output capacity exceeded (counts
 *     still hold the exact sizes, so the caller can retry with bigger buffers).
 *   - Grid values are float32 [nx, ny, nz] (z fastest); `nx, ny, nz` are POINTS
 *     per axis, as isoext's UniformGrid shape.  The value buffer must be 16-byte
 *     aligned and readable up to the next 16-byte boundary (true for any
 *     cudaMalloc / torch allocation).
 */
#ifndef ISOEXT_GB300_H
#define ISOEXT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define ISO_OK 0
#define ISO_ERR_ARG 1
#define ISO_ERR_CUDA 2
#define ISO_ERR_TIMEOUT 3
#define ISO_ERR_LOOKUP 4
#define ISO_ERR_WORKSPACE 5
#define ISO_ERR_OVERFLOW 6

/* Message of the last failed call on this thread. */
const char *iso_last_error(void);

/* ABI version of this library (2). */
int iso_abi_version(void);

/* Which reading of isoext's FP32 expressions the kernels compute, process-wide
 * (read at each launch).  No counterpart in the reference, which has one per
 * build:
 *   1 (default) -- its CUDA build: nvcc's default FMA contraction of its source
 *                  (grid positions, lerp, the normal stencil, norms), so
 *                  vertices, intersection points and normals equal that
 *                  build's, bit for bit.
 *   0           -- its host build: every operation rounded on its own.
 * Returns ISO_ERR_ARG for other values. */
int iso_set_arith(int mode);
int iso_get_arith(void);

/* Coordinates of the n points of one grid axis, amin + (i / (float)(n - 1)) *
 * (amax - amin), in the current reading: out is DEVICE float [n].  Replaces
 * the position arithmetic behind UniformGrid.get_points (src/isoext_ext.cu:
 * 149-156 -> src/grid/uniform.cu get_points -> include/utils.cuh:62-80,
 * get_vtx_pos_op); the grid of points is their outer product. */
int iso_axis_coords(float *out, int n, float amin, float amax, void *stream);

/* Threads per CTA of iso_mc_dense's emit kernel (128 or 256; default 256).
 * Process-wide; the autotuner sets it.  No counterpart in the reference (it
 * has no tunables). */
int iso_mc_set_config(int threads);
int iso_mc_get_config(int *threads);

/* Launch parameters for the autotuner (isoext_gb300.tune; process-wide; no
 * counterpart in the reference).  Keys and values:
 *   "mc.emit_threads"     128 | 256   threads per CTA of the MC emit kernel
 *   "mc.sign_ctas_per_sm" 1 .. 64     CTAs per SM of the sign pass (MC and DC)
 *   "dc.cell_threads"     64 | 128 | 256  threads per CTA of the per-cell DC kernels
 *   "mc.count_threads"    128 | 256   threads per CTA of the MC count kernel (its
 *                                     scan segment is 4 words per thread)
 * Results do not depend on them. */
int iso_tune_set(const char *key, int value);
int iso_tune_get(const char *key, int *value);

/* Test hook of the bounded device waits (no counterpart in the reference):
 * the scan's decoupled look-back over states that are never published
 * (state: device, >= 32 zeroed u64) gives up after spin_limit polls
 * (<= 2^20) and writes ISO_ERR_TIMEOUT to *status; out (device u64[2]). */
int iso_test_wait_timeout(unsigned spin_limit, unsigned long long *state, int *status,
                          unsigned long long *out, void *stream);

/* Kernel timing for benchmarks (no counterpart in the reference).  While
 * enabled, each kernel (or short group of kernels) the library launches is
 * bracketed by CUDA events on its stream.  iso_profile_read synchronises on the
 * recorded events and returns the number of timed groups and their total
 * device time in ms for one name ("mc_signs", "mc_count", "mc_scan", "mc_emit",
 * "dc_classify", ...; NULL = all); iso_profile_kernels returns how many kernels
 * those groups launched. */
int iso_profile_enable(int on);
void iso_profile_reset(void);
int iso_profile_read(const char *kernel, long long *launches, double *total_ms);
int iso_profile_kernels(const char *kernel, long long *kernels);

/* Workspace bytes iso_mc_dense needs for a grid and output capacities. */
size_t iso_mc_dense_workspace_size(int nx, int ny, int nz, long long vertex_capacity,
                                   long long face_capacity);

/* Marching cubes on a dense grid.
 * Replaces isoext_ext.marching_cubes(grid: UniformGrid, level, method)
 * (src/isoext_ext.cu:95-109 -> mc::marching_cubes, src/mc/mc.cu:17-68).
 *   method: 0 = "nagae" (default in isoext), 1 = "lorensen".
 *   vertices: float32 [vertex_capacity, 3]; faces: int32 [face_capacity, 3].
 *   counts: device int64[2] <- (V, F).  Faces come in the reference's order
 *   (ascending cell id, table slot order).  Vertices come in grid-edge order; they
 *   are the same vertices as the reference's, whose order is by position.
 *   workspace: iso_mc_dense_workspace_size bytes (any alignment).
 *   Unknown method -> ISO_ERR_ARG (isoext raises "Unknown method: ...").
 *   More than 2^31-1 points -> ISO_ERR_ARG (isoext: src/grid/uniform.cu:13-16). */
int iso_mc_dense(const float *values, int nx, int ny, int nz, const float *aabb_min,
                 const float *aabb_max, float level, int method, float *vertices,
                 long long vertex_capacity, int *faces, long long face_capacity, void *workspace,
                 size_t workspace_bytes, long long *counts, int *status, void *stream);

/* Marching cubes with no caller workspace. This has NO counterpart in the
 * reference: isoext allocates per call.  It is for callers that cannot give
 * the library device memory. One example is a host with only a stream and no
 * device allocator. Another is a frame loop that must not call cudaMalloc or
 * cudaFree, because cudaFree synchronises the device and either call can fail
 * mid-frame.
 * Arguments and results are iso_mc_dense's, without workspace/workspace_bytes.
 * The workspace is a fixed array inside the library, ISO_MC_NOALLOC_SCRATCH_BYTES
 * (32 MiB) per device. The call allocates nothing.
 *   - A grid plus capacities whose iso_mc_dense_workspace_size exceeds the
 *     limit -> ISO_ERR_WORKSPACE with a message; nothing is queued. 256^3 with
 *     capacities near its mesh size fits.
 *   - Each call looks up the array's address in the CUDA context current on
 *     the calling thread (a context made after cudaDeviceReset, or the
 *     caller's own driver context, has its own copy). The first call in a
 *     context can load the module that holds the array: make it before any
 *     stream capture.
 *   - All calls in one context share the array. Calls not ordered on the
 *     device (different streams or threads without events) race. Each call
 *     clears, on its stream, what must start at zero. */
#define ISO_MC_NOALLOC_SCRATCH_BYTES (32u << 20)
int iso_mc_dense_noalloc(const float *values, int nx, int ny, int nz, const float *aabb_min,
                         const float *aabb_max, float level, int method, float *vertices,
                         long long vertex_capacity, int *faces, long long face_capacity,
                         long long *counts, int *status, void *stream);

/* ---- dual contouring on a dense grid --------------------------------------
 * Replaces isoext_ext.get_intersection / dual_contouring (src/isoext_ext.cu:
 * 329-378 -> get_intersection src/its.cu:94-159, compute_intersection_normals
 * :272-283, dual_contouring src/dc.cu:162-218).  The caller runs the steps in
 * order on one stream and sizes buffers from the counts between them:
 *   classify -> (A active cells, K crossings) -> intersect -> [normals] ->
 *   solve -> quads_count -> (Q quads) -> quads_emit -> weld_count -> (V) ->
 *   weld_write.  `ws` is one workspace of iso_dc_workspace_size bytes shared by
 *   classify / intersect / cells / quads. */
size_t iso_dc_workspace_size(int nx, int ny, int nz);
/* Sign bitmap and per-word counts; counts (device int64[2]) <- (A, K). */
int iso_dc_classify(const float *values, int nx, int ny, int nz, float level, void *ws,
                    size_t ws_bytes, long long *counts, void *stream);
/* Crossing points [K,3], optional normals [K,3] (NULL: none), active cell ids
 * [A] and CSR offsets [A+1] -- isoext's Intersection arrays. */
int iso_dc_intersect(const float *values, int nx, int ny, int nz, const float *aabb_min,
                     const float *aabb_max, float level, void *ws, long long A, long long K,
                     float *points, float *normals, int *cell_ids, int *cell_offsets, void *stream);
/* intersect + solve in one step for dual_contouring without a caller
 * intersection: active cell ids [A], CSR offsets [A+1] and dual vertices [A, 3]
 * (bit-equal to iso_dc_intersect with normals followed by iso_dc_solve); the
 * crossing points and normals are not written. */
int iso_dc_intersect_solve(const float *values, int nx, int ny, int nz, const float *aabb_min,
                           const float *aabb_max, float level, void *ws, long long A, long long K,
                           int *cell_ids, int *cell_offsets, float reg, float svd_tol, float *dual,
                           void *stream);
/* Dual contouring in one call with no host synchronisation, the dense path of
 * isoext_ext.dual_contouring(grid, level, None, reg, svd_tol) (src/dc.cu:162-218
 * with intersections from the grid, src/its.cu:94-283).  Vertices [V, 3] and
 * faces [F, 3] as the step-by-step entry points give them (bit for bit).
 *   vertex_capacity bounds the active cells A (one dual vertex each, V <= A);
 *   face_capacity the faces F = 2 Q (two per quad).
 *   counts: device int64[5] <- (V, F, A, K, Q), K the crossings.  When A or F
 *   exceed the capacities the status is 6 (ISO_ERR_OVERFLOW), no vertex or face
 *   is written, and counts[2..4] give the sizes for a retry.
 *   workspace: iso_dc_dense_workspace_size bytes.  Capturable in a CUDA graph. */
size_t iso_dc_dense_workspace_size(int nx, int ny, int nz, long long vertex_capacity,
                                   long long face_capacity);
int iso_dc_dense(const float *values, int nx, int ny, int nz, const float *aabb_min,
                 const float *aabb_max, float level, float reg, float svd_tol, float *vertices,
                 long long vertex_capacity, int *faces, long long face_capacity, void *workspace,
                 size_t workspace_bytes, long long *counts, int *status, void *stream);
/* iso_dc_dense, and (each optional) the active cell ids [vertex_capacity] and
 * their crossing offsets [vertex_capacity + 1] (isoext's Intersection cells
 * and offsets), and the active cell each vertex came from [vertex_capacity]:
 * what iso_dc_backward needs. */
int iso_dc_dense_ex(const float *values, int nx, int ny, int nz, const float *aabb_min,
                    const float *aabb_max, float level, float reg, float svd_tol, float *vertices,
                    long long vertex_capacity, int *faces, long long face_capacity, void *workspace,
                    size_t workspace_bytes, long long *counts, int *status, int *cell_ids,
                    int *cell_offsets, int *vertex_source, void *stream);
/* Normals of existing crossings from the grid (src/its.cu:186-268). */
int iso_dc_normals(const float *values, int nx, int ny, int nz, const float *aabb_min,
                   const float *aabb_max, const float *points, const int *cell_ids,
                   const int *cell_offsets, long long A, float *normals, void *stream);
/* Dual vertex per active cell: QEF (src/dc.cu:14-65), pseudo-inverse with the
 * s > svd_tol * s_max rule (src/batched_la.cu:152-178), clip (src/dc.cu:82-99). */
int iso_dc_solve(int nx, int ny, int nz, const float *aabb_min, const float *aabb_max,
                 const float *points, const float *normals, const int *cell_ids,
                 const int *cell_offsets, long long A, float reg, float svd_tol, float *dual,
                 void *stream);
/* Active-cell masks only (an intersection computed by an earlier call). */
int iso_dc_cells(const float *values, int nx, int ny, int nz, float level, void *ws, void *stream);
/* Quads: count (counts[0] <- Q), then 6 dual indices per quad in isoext's
 * order (src/grid/uniform.cu:60-83, src/dc.cu:101-157). */
int iso_dc_quads_count(int nx, int ny, int nz, void *ws, long long *counts, void *stream);
int iso_dc_quads_emit(int nx, int ny, int nz, void *ws, const float *dual, int *tri, void *stream);
/* Weld dual vertices by exact position (src/utils.cu:32-59): count V
 * (counts[0]), then write vertices [V,3] and faces [ntri/3,3]. */
size_t iso_dc_weld_workspace_size(long long A);
int iso_dc_weld_count(const float *dual, long long A, const int *tri, long long ntri, void *ws,
                      size_t ws_bytes, long long *counts, int *status, void *stream);
int iso_dc_weld_write(const float *dual, long long A, const int *tri, long long ntri, void *ws,
                      float *vout, int *fout, void *stream);
/* The same, and vertex_source[i] <- the dual vertex (active cell) vertex i came
 * from (for the backward pass). */
int iso_dc_weld_write_src(const float *dual, long long A, const int *tri, long long ntri, void *ws,
                          float *vout, int *fout, int *vertex_source, void *stream);

/* ---- sparse grids -----------------------------------------------------------
 * Replaces isoext's SparseGrid paths (src/grid/sparse.cu:9-246 with
 * src/mc/mc.cu:17-68, src/its.cu:94-283, src/dc.cu:162-218).  A sparse grid is
 * `ids` (int32 [n] cell ids of an nx*ny*nz-point lattice, ascending as uint32,
 * unique) and `vals` (float32 [n, 8], corner k = 4x + 2y + z, 16-byte aligned).
 * `blk` is a block-sum workspace of iso_sparse_blocks_size(n) bytes; counting
 * calls write totals to device int64 counts[2]. */
size_t iso_sparse_blocks_size(long long n);
/* MC: counts[0] <- F; then a triangle soup [3F, 3] in the reference's order
 * (cell order, table slots; triangles with two equal positions dropped,
 * src/mc/nagae.cu:71).  Weld it with iso_dc_weld_count / iso_dc_weld_write
 * (A = 3F, tri = 0 .. 3F-1), which merges equal positions as isoext does. */
int iso_sparse_mc_count(const int *ids, const float *vals, long long n, int nx, int ny, int nz,
                        const float *aabb_min, const float *aabb_max, float level, int method,
                        void *blk, long long *counts, void *stream);
int iso_sparse_mc_emit(const int *ids, const float *vals, long long n, int nx, int ny, int nz,
                       const float *aabb_min, const float *aabb_max, float level, int method,
                       const void *blk, float *soup, void *stream);
/* Intersection: counts <- (A, K); then points [K,3], optional normals, active
 * cells as sparse indices [A] (isoext's Intersection.cell_indices) and as
 * lattice ids [A] (for iso_dc_solve), offsets [A+1], and rank [n] (active
 * index of each sparse cell, -1 if inactive). */
int iso_sparse_its_count(const float *vals, long long n, float level, void *blk, long long *counts,
                         void *stream);
int iso_sparse_its_emit(const int *ids, const float *vals, long long n, int nx, int ny, int nz,
                        const float *aabb_min, const float *aabb_max, float level, const void *blk,
                        long long A, long long K, float *points, float *normals, int *act_sparse,
                        int *act_lattice, int *offsets, int *rank, void *stream);
/* Normals of existing crossings (src/its.cu:186-268). */
int iso_sparse_normals(const int *ids, const float *vals, int nx, int ny, int nz, const float *aabb_min,
                       const float *aabb_max, const int *act_sparse, const int *offsets, long long A,
                       const float *points, float *normals, void *stream);
/* DC quads (src/grid/sparse.cu:181-246, src/dc.cu:101-157): counts[0] <- Q,
 * then 6 dual indices per quad.  A quad needs its 4 cells present and active;
 * its orientation comes from the first of them (sparse order) that crosses. */
int iso_sparse_quads_count(const int *ids, const float *vals, long long n, int nx, int ny, int nz,
                           float level, const int *rank, void *blk, long long *counts, void *stream);
int iso_sparse_quads_emit(const int *ids, const float *vals, long long n, int nx, int ny, int nz,
                          float level, const int *rank, const void *blk, const float *dual, int *tri,
                          void *stream);
/* Sparse MC in one call with no host synchronisation: the soup of
 * iso_sparse_mc_count/emit welded as iso_dc_weld_* does, into vertices
 * [vertex_capacity, 3] and faces [face_capacity, 3].  counts (device
 * int64[3]) <- (V, F, F needed); status 6 when F or V exceed the capacities
 * (the outputs are then incomplete; retry with the sizes from counts). */
size_t iso_sparse_mc_workspace_size(long long n, long long vertex_capacity, long long face_capacity);
int iso_sparse_mc(const int *ids, const float *vals, long long n, int nx, int ny, int nz,
                  const float *aabb_min, const float *aabb_max, float level, int method, float *vertices,
                  long long vertex_capacity, int *faces, long long face_capacity, void *workspace,
                  size_t workspace_bytes, long long *counts, int *status, void *stream);
/* Corner positions [m, 8, 3] of cell ids (get_points / get_points_by_cell_indices,
 * src/grid/sparse.cu:21-43). */
int iso_sparse_points(const int *ids, long long m, int nx, int ny, int nz, const float *aabb_min,
                      const float *aabb_max, float *out, void *stream);
/* filter_cell_indices (src/grid/sparse.cu:150-179): counts[0] <- kept; then the
 * kept ids in input order. */
int iso_sparse_filter_count(const float *vals, long long m, float level, void *blk, long long *counts,
                            void *stream);
int iso_sparse_filter_write(const int *ids, const float *vals, long long m, float level, const void *blk,
                            int *out, void *stream);

/* ---- backward passes ---------------------------------------------------------
 * No counterpart in isoext (its extraction is not differentiable).  Gradients
 * of vertex positions are sent to the grid values; topology has no gradient.
 * grad_values [nx, ny, nz] is ACCUMULATED into (zero it first). */

/* iso_mc_dense, and vertex_edges[i] <- 3 * (point id of vertex i's low edge
 * endpoint) + axis (0 x, 1 y, 2 z); vertex_edges has vertex_capacity entries. */
int iso_mc_dense_edges(const float *values, int nx, int ny, int nz, const float *aabb_min,
                       const float *aabb_max, float level, int method, float *vertices,
                       long long vertex_capacity, int *faces, long long face_capacity, void *workspace,
                       size_t workspace_bytes, long long *counts, int *status,
                       long long *vertex_edges, void *stream);
/* Through the interpolation weights of each vertex (src/mc/nagae.cu:52-56). */
int iso_mc_backward(const float *values, int nx, int ny, int nz, const float *aabb_min,
                    const float *aabb_max, float level, const long long *vertex_edges, long long V,
                    const float *grad_vertices, float *grad_values, void *stream);
/* Implicit differentiation of the QEF solve (src/dc.cu:14-99) per active cell:
 * grad_dual [A, 3] is the gradient of the unclipped-then-clipped dual vertices
 * (zero in clipped coordinates).  normals NULL: the normals were computed from
 * the grid (iso_dc_intersect), and the gradient flows through them; otherwise
 * the caller's normals [K, 3] were used, and grad_normals (optional) receives
 * their gradient. */
int iso_dc_backward(const float *values, int nx, int ny, int nz, const float *aabb_min,
                    const float *aabb_max, float level, const int *cell_ids, const int *cell_offsets,
                    long long A, float reg, float svd_tol, const float *normals, const float *grad_dual,
                    float *grad_values, float *grad_normals, void *stream);
/* iso_dc_backward from the gradient of the welded vertices: vertex i came from
 * active cell vertex_source[i] (iso_dc_dense_ex), grad_vertices [V, 3];
 * grad_dual_ws is a device scratch of A * 3 floats.  grad_values is zeroed
 * first, then written (not accumulated). */
int iso_dc_backward_src(const float *values, int nx, int ny, int nz, const float *aabb_min,
                        const float *aabb_max, float level, const int *cell_ids, const int *cell_offsets,
                        long long A, float reg, float svd_tol, const int *vertex_source, long long V,
                        const float *grad_vertices, float *grad_dual_ws, float *grad_values, void *stream);

/* ------------------------------------------------------------------------- */
/* Grid values of a union of spheres and boxes, for the served request stream
 * (no counterpart in isoext, which builds grids with torch expressions; the
 * distances are src/isoext/sdf.py:70-116's sphere and box formulas, the point
 * positions the grid's own, include/utils.cuh:62-80).
 * prims: DEVICE float [1 + 7 * count]: prims[0] = count (1 .. 32), then rows of
 * kind (0 sphere, 1 box), centre xyz, radius | half-extents xyz.  Reading them
 * from device memory lets a captured CUDA graph evaluate each new request.
 * out: device float [nx, ny, nz], the minimum over the primitives. */
int iso_sdf_union_grid(const float *prims, int nx, int ny, int nz, const float *aabb_min,
                       const float *aabb_max, float *out, void *stream);

/* ---- exact-position weld of a mesh -------------------------------------------
 * isoext welds its triangle soup by exact position (src/utils.cu:32-59: sort,
 * unique) after dropping triangles with two equal vertex positions
 * (src/mc/nagae.cu:71).  The extraction kernels weld by grid edge, which is the
 * same mesh while neighbouring grid coordinates are many ulps apart; on a grid
 * whose spacing comes within a few ulps of its coordinates, vertices of
 * distinct edges can round to one position, and this pass gives isoext's mesh:
 * vertices with bit-equal positions (-0 and +0 equal) merge into the first of
 * them, faces with two equal vertices are dropped, and vertices no remaining
 * face uses are dropped; the survivors keep their order.  vertices: device
 * float [V, 3]; faces: device int32 [F, 3]; vout / fout: device, room for V and
 * F; vertex_source (optional): device int32 [V], each output vertex's index in
 * the input; counts: device int64 [2] <- (V', F'); status: device int, 0 or
 * ISO_ERR_OVERFLOW (a hash probe limit; not reached when V fits the table).
 * workspace: iso_weld_mesh_workspace_size(V, F) bytes. */
size_t iso_weld_mesh_workspace_size(long long num_vertices, long long num_faces);
int iso_weld_mesh(const float *vertices, long long num_vertices, const int *faces, long long num_faces,
                  float *vout, int *fout, int *vertex_source, long long *counts, int *status,
                  void *workspace, size_t workspace_bytes, void *stream);

/* ---- isoext's vertex order --------------------------------------------------
 * The extraction entry points number vertices by grid edge (MC) or by cell
 * (DC); isoext sorts its welded vertices by position (src/utils.cu:32-59:
 * thrust::sort with float3_less_pred, then unique), and the faces' order is
 * the same either way.  This pass renumbers a mesh in isoext's order, in
 * place: vertices (device float [V, 3], distinct positions) sorted
 * lexicographically by (x, y, z), -0 and +0 equal; faces (device int32
 * [F, 3]) renumbered to match.  Two stable radix sorts (CUB).
 * workspace: iso_sort_vertices_workspace_size(V) bytes. */
size_t iso_sort_vertices_workspace_size(long long num_vertices);
int iso_sort_vertices(float *vertices, long long num_vertices, int *faces, long long num_faces, void *workspace,
                      size_t workspace_bytes, void *stream);

/* ---- native serving loop -------------------------------------------------
 * No counterpart in isoext.  A server keeps `slots` worker threads on the
 * current device, each with its own stream and a cache of entries: device
 * buffers and a CUDA graph of iso_sdf_union_grid + iso_mc_dense / iso_dc_dense
 * per (kind, n, method, level).  Requests are taken first come, first served
 * by free workers.  Every device byte the server holds counts against
 * budget_bytes: a new entry evicts least-recently-used idle entries to fit, or
 * waits for running requests.  A new entry is sized from a count pass on its
 * request (the extraction at capacity 1 reports the exact sizes); a larger
 * mesh later grows its entry from the sizes it reported.  Results come back in
 * host memory.  Thread-safe. */
typedef struct IsoServer IsoServer;
typedef struct {
    int kind;            /* 0 marching cubes, 1 dual contouring (reg 1e-2, svd_tol 1e-6) */
    int n;               /* points per axis of the cubic grid over [-1, 1]^3 (2 .. 1290) */
    int method;          /* marching cubes: 0 nagae, 1 lorensen */
    float level;
    int num_prims;       /* 1 .. 32 */
    const float *prims;  /* host [num_prims][7]: kind (0 sphere, 1 box), centre xyz, radius | half-extents xyz */
} IsoServeRequest;
typedef struct {
    long long ticket;
    int status;                    /* 0, or an ISO_ERR_* code */
    int slot;                      /* the worker that ran it */
    long long num_vertices, num_faces;
    float *vertices;               /* host [V, 3] (malloc); release with iso_serve_free_result */
    int *faces;                    /* host [F, 3] */
    double t_submit, t_start, t_done;  /* steady-clock seconds */
} IsoServeResult;
/* warm_sizes: grid sizes whose entries (both kinds, nagae, level 0) every
 * slot builds up front, with capacities of the closed-surface bound
 * (24 (n - 1)^2 + 4096 faces); other keys are built on first use. */
int iso_serve_create(int slots, long long budget_bytes, const int *warm_sizes, int num_warm_sizes,
                     IsoServer **server);
/* Returns the request's ticket (>= 0), or -ISO_ERR_ARG / -ISO_ERR_WORKSPACE
 * (larger than the budget).  The primitives are copied. */
long long iso_serve_submit(IsoServer *server, const IsoServeRequest *request);
/* Blocks until the ticket's request is done (timeout_s < 0: no limit;
 * ISO_ERR_TIMEOUT when it runs out) and moves its result out. */
int iso_serve_wait(IsoServer *server, long long ticket, double timeout_s, IsoServeResult *result);
void iso_serve_free_result(IsoServeResult *result);
/* stats[0] completed, [1] most workers running at once (a worker runs one
 * request, or one bucket of them), [2] most device bytes the server held at
 * once (never above budget_bytes), [3] queued now. */
int iso_serve_stats(IsoServer *server, long long *stats);
/* The first `count` (<= 12) of: the four above, [4] device bytes held now,
 * [5] entries evicted, [6] entries cached, [7] count passes run, [8] entries
 * grown for a larger mesh, [9] the budget, [10] launches that ran more than
 * one request, [11] the requests they ran. */
int iso_serve_stats_ex(IsoServer *server, long long *stats, int count);
/* Length buckets: a worker takes, with the request at the head of the queue,
 * up to max_requests - 1 queued requests of the same kind, grid size, method
 * and level, and runs them with one launch of a graph with one parallel branch
 * per request (max_requests 1, 2, 4 or 8; with fewer matching requests the
 * largest power of two of them runs).  1 (the default): one launch per
 * request. */
int iso_serve_set_bucket(IsoServer *server, int max_requests);
/* Finishes the queued requests, then frees everything. */
int iso_serve_destroy(IsoServer *server);
/* Capacities of the entries built after the call, as a fraction (0, 1] of the
 * counted sizes; meshes that do not fit grow their entry and run again (tests). */
int iso_serve_set_capacity_scale(IsoServer *server, double scale);

#ifdef __cplusplus
}
#endif

#endif /* ISOEXT_GB300_H */
