/*
 * pamo_gb300 — C ABI of the GB300-native PaMO simplifier: stage 2 (parallel QEM edge collapse with LBVH
 * self-intersection rollback) and stage 3 (barrier/CCD Newton-CG safe projection onto the input mesh).
 *
 * Every pointer argument named points/triangles/verts/tris/verts_* is a DEVICE pointer on the context's
 * GPU unless stated otherwise; sizes are element counts (points = rows of 3 float32, triangles = rows of 3
 * int32). Every call returns a pamo_status; the message of the last failure is pamo_ctx_last_error().
 * A context is not thread-safe: use one context per host thread / stream.
 */
#ifndef PAMO_GB300_H
#define PAMO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pamo_ctx pamo_ctx;
typedef void* pamo_stream; /* a cudaStream_t; NULL is the legacy default stream */

typedef enum pamo_status {
    PAMO_OK = 0,
    PAMO_ERR_INVALID_ARG = 1, /* bad size, null pointer or out-of-range vertex index */
    PAMO_ERR_OOM = 2,         /* device allocation failed */
    PAMO_ERR_CAPACITY = 3,    /* an internal list overflowed (reported, never clipped silently) */
    PAMO_ERR_ITER_LIMIT = 4,  /* a bounded device loop or traversal ran out of room */
    PAMO_ERR_CUDA = 5,        /* a CUDA runtime call failed */
    PAMO_ERR_STATE = 6        /* call order: e.g. outputs requested before a round ran */
} pamo_status;

const char* pamo_status_string(int status);

/* Create a context on CUDA device `device`. Replaces the default construction of the reference's
 * pybind class CUDSP_Free (simp_cuda/src/pybind.cpp:16-19, 189-193). */
int pamo_ctx_create(pamo_ctx** out, int device);

/* Release every device buffer of the context (simp_cuda/src/pybind.cpp:21-49). */
int pamo_ctx_destroy(pamo_ctx* ctx);

/* Message of the last failed call on this context ("" when none). */
const char* pamo_ctx_last_error(const pamo_ctx* ctx);

/* Put the context in the state of a newly created one (as constructing a new CUDSP_Free does,
 * simp_cuda/src/pybind.cpp:16-19): the state the reference carries between calls (stale edge costs,
 * invalid-vertex table, previous compaction map, undo list, capacity bookkeeping) is dropped; device
 * buffers are kept for reuse. Lets one context serve independent jobs with the results of fresh instances. */
int pamo_ctx_reset(pamo_ctx* ctx, pamo_stream stream);

/* Device memory the context currently holds, in bytes (no reference counterpart; used for admission). */
int64_t pamo_ctx_device_bytes(const pamo_ctx* ctx);

/* Options of the stage-2 rounds (the execution options give the same results with any setting):
 *   "device_rounds" (default 1): rounds after the first read their sizes and loop state from device memory
 *                                and synchronise once per round (plus once per extra undo pass);
 *   "graphs"        (default 1): those rounds run as CUDA graphs cached per size class;
 *   "bvh_reuse"     (default 1): those rounds refit the LBVH carried from the previous round (rebuilt when a
 *                                quarter of its leaves lost their faces) instead of building it each round;
 *   "precision"     (default 0): 0 the reference's float arithmetic; 1 (precision mode) quadric, ring-length,
 *                                skinny and cost sums compensated (TwoSum/TwoProd, rounded once); 2 as 1 with each
 *                                collapse placed at the edge quadric's minimiser instead of the reference's midpoint
 *                                (float solve, double for near-singular quadrics, midpoint for singular ones);
 *                                modes 1 and 2 change results and are not the reference's arithmetic;
 *   "skinny_pow"    (default 0): 1 squares the skinny term's lengths with the device's pow(float, int), the
 *                                reference's call (cusimp_free.cu:533,573), where 0 multiplies; the device function
 *                                differs from the product by one ulp on a few floats in a million and costs the
 *                                edge-cost kernel about 12x; every job measured so far is bit-identical either way.
 * The phase timers (pamo_profile_enable) use the host-sized path. */
int pamo_ctx_set_option(pamo_ctx* ctx, const char* name, int64_t value);

/*
 * One simplification round: CUDSP_Free.forward(points, triangles, verts_undo, n_verts_undo, scale,
 * threshold, is_stuck, init) (simp_cuda/src/pybind.cpp:52-72 -> CUSimp_Free::forward,
 * simp_cuda/src/cusimp_free.cu:891-1048). Inputs are only read. State that the reference keeps between
 * calls (stale edge costs, the invalid-vertex table, the previous compaction map, the undo list) is kept
 * in the context with the same semantics. Synchronises `stream` before returning.
 */
int pamo_forward_round(pamo_ctx* ctx, const float* points, const int32_t* triangles, const int32_t* verts_undo,
                       int32_t n_verts_undo, int32_t n_points, int32_t n_triangles, float scale, float threshold,
                       int32_t is_stuck, int32_t init, pamo_stream stream);

/*
 * One round of the legacy simplifier without rollback, _C.CUDSP().forward(points, triangles, scale,
 * threshold, init) (simp_cuda/src/pybind.cpp:140-182, CUSimp::forward at simp_cuda/src/cusimp.cu:587-720):
 * the same selection and collapse as pamo_forward_round with the legacy cost (the mean ring length counted
 * twice, no skinny penalty factor), no invalid table, stuck mode, face clean-up, self-intersection check or
 * undo. Outputs through pamo_round_sizes / pamo_round_outputs (verts, tris, verts_occ, verts_map; no undo
 * list). Use a context of its own: the stale edge costs it keeps are those of this variant.
 */
int pamo_legacy_round(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                      int32_t n_triangles, float scale, float threshold, int32_t init, pamo_stream stream);

/* Shapes of the five outputs of the last round: verts [n_points,3], tris [n_triangles,3],
 * verts_occ [n_points,1], verts_map [n_points,1], verts_undo [n_verts_undo] (simp_cuda/src/pybind.cpp:74-102). */
/* Precision probe (no reference counterpart): one round up to the edge costs (no shuffle, no collapse, fresh state)
 * on device arrays, with precision mode 0 (the reference's float arithmetic), 1 (quadric, length, skinny and cost sums
 * compensated by TwoSum/TwoProd) or 2 (as 1, placement at the edge quadric's minimiser: a float solve when well
 * conditioned, a double solve when near-singular, the midpoint when singular). Writes n_edges and, when capacity
 * allows, out_edges [n,2] (the reference's edge numbering), out_cost [n] (cost before clamp and quantisation, NaN
 * where the edge is invalid) and out_place [n,3] (device arrays; any may be NULL). Overwrites the context's round
 * state: use a context of its own. Synchronises `stream`. */
int pamo_cost_probe(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                    int32_t n_triangles, float scale, float threshold, int32_t precision, int32_t* out_edges,
                    float* out_cost, float* out_place, int32_t capacity, int32_t* n_edges, pamo_stream stream);

int pamo_round_sizes(const pamo_ctx* ctx, int32_t* n_points, int32_t* n_triangles, int32_t* n_verts_undo);

/* Copy the last round's outputs into caller-owned device buffers (any may be NULL to skip it). Removed
 * faces are (-1, -1, -1); verts_map is the exclusive scan of verts_occ. */
int pamo_round_outputs(pamo_ctx* ctx, float* verts, int32_t* tris, int32_t* verts_occ, int32_t* verts_map,
                       int32_t* verts_undo, pamo_stream stream);

/* Diagnostics of the last round, written to out[0..n): n_edges, n_win, n_collapsed, n_considered,
 * n_query, passes, n_vertices_undo, status bits, candidate pairs, fp64 pairs, undo per pass [8]. */
int pamo_round_stats(const pamo_ctx* ctx, int64_t* out, int32_t n);

/*
 * The whole stage-2 loop of PaMO.run(points, triangles, ratio, tolerance, threshold, iter, min_verts) with
 * stage 1 and stage 3 off (simp_cuda/pamo/__init__.py:95-163): centring by the mean of the face centroids,
 * rounds with compaction on the device, stuck/tolerance termination. Results stay in the context; fetch
 * them with pamo_simplify_result. Returns the output sizes and the number of rounds run.
 */
int pamo_simplify_device(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                         int32_t n_triangles, double ratio, int32_t tolerance, float threshold, int32_t iter,
                         int64_t min_verts, int32_t* out_n_points, int32_t* out_n_triangles, int32_t* out_rounds,
                         pamo_stream stream);

/*
 * The Blender add-on's whole-loop entry point (pamo_blender/cusimpinterface.cu:55-161) with HOST pointers:
 * in_verts [n_verts*3] float32, in_tris [n_tris*3] int32, in_out_nv_ni = {n_verts, n_tris} on entry and the
 * output sizes on return; out_verts/out_tris must hold at least the input sizes. Scale = the largest extent of
 * the input bounding box, no centring, rounds until 4 rounds in a row remove no face (no target), as the
 * reference. One context per device is kept between calls, like the reference's static CUSimp_Free.
 * Uses the current device and the legacy default stream; returns a pamo_status (the reference returns void).
 */
int pamo_simplify(float* in_verts, int* in_tris, float* out_verts, int* out_tris, int* in_out_nv_ni, float threshold);

/* Copy the result of pamo_simplify_device (centring undone, as the reference's run() returns it). */
int pamo_simplify_result(pamo_ctx* ctx, float* verts, int32_t* tris, pamo_stream stream);

/* Face count after each round of the last pamo_simplify_device call (host array of `capacity`). */
int pamo_simplify_round_faces(const pamo_ctx* ctx, int32_t* faces_per_round, int32_t capacity);

/* Host wall-clock milliseconds of each round of the last pamo_simplify_device call (every round ends with a
 * synchronisation); returns the number written. No reference counterpart (diagnostics). */
int pamo_simplify_round_ms(const pamo_ctx* ctx, double* ms, int32_t capacity);

/* Device time of each round of the last loop, with pamo_ctx_set_option(ctx, "time_rounds", 1): the time between
 * events recorded around the round's graph launches (0 for rounds launched without graphs or with the option
 * off); the gap to pamo_simplify_round_ms is host turnaround. Returns the number written. Diagnostics. */
int pamo_simplify_round_gpu_ms(const pamo_ctx* ctx, double* ms, int32_t capacity);

/* With pamo_ctx_set_option(ctx, "time_edge_cost", 1), events are recorded around every edge-cost kernel launch
 * (also inside the cached round graphs); this returns their summed duration in ms and the number of launches
 * since the option was set or the last reset (reset != 0 clears them). Diagnostics. */
int pamo_kernel_time(pamo_ctx* ctx, double* ms, int64_t* launches, int32_t reset);

/*
 * The centre PaMO.run subtracts before simplifying: preprocess_mesh's tris_mean (simp_cuda/pamo/__init__.py:
 * 60-64), numpy float32 semantics: per face ((a + b) + c) / 3, then the sequential float32 sum over faces in
 * face order divided by the face count. Device points/triangles; out3 is a host array of 3 floats.
 * Synchronises `stream`.
 */
int pamo_tris_mean(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                   int32_t n_triangles, float* out3, pamo_stream stream);

/*
 * The reference's self-intersection check over a whole mesh (selfx::self_intersect,
 * simp_cuda/src/bvh/self_intersect.cuh:151-392): face_hit[f] = 1 iff face f takes part in a (query, hit)
 * pair the reference's tri-tri filter reports, else 0 (uint8, device buffer of n_triangles). Faces equal
 * to (-1, -1, -1) are skipped. Synchronises `stream`.
 */
int pamo_self_intersect(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                        int32_t n_triangles, uint8_t* face_hit, pamo_stream stream);

/*
 * pamo_self_intersect without any device allocation, for callers that must not allocate device memory
 * (hosts that own a fixed memory budget and forbid cudaMalloc/cudaFree by plug-ins, or code that cannot
 * afford the device synchronisation an allocation may cause). No counterpart in the reference.
 * Same result as pamo_self_intersect; needs no context. Scratch is a 24 MiB array in device memory that
 * the library holds on every GPU that loads it; its address is looked up on the first call made in each CUDA
 * context (a new context, e.g. after cudaDeviceReset, gets a new lookup), so make that first call before any
 * stream capture. Limits: n_points <= 65536 and n_triangles <= 65536, else PAMO_ERR_CAPACITY. All calls
 * share the scratch: calls that overlap on the GPU race. A CUDA error already pending from earlier work
 * returns PAMO_ERR_CUDA before any GPU work (and stays pending). Uses the current device and context; every
 * return after work was queued synchronises `stream` first.
 */
int pamo_self_intersect_noalloc(const float* points, const int32_t* triangles, int32_t n_points,
                                int32_t n_triangles, uint8_t* face_hit, pamo_stream stream);

/* Totals over the rounds of the last pamo_simplify_device call, written to out[0..n): vertices, faces,
 * edges, winners, query-face tests (query faces x checks), candidate pairs, pairs that took the fp64 path,
 * intersection checks, live faces indexed by the LBVH (x checks), collapsed edges. Returns 10. No reference
 * counterpart (diagnostics). */
int pamo_run_totals(const pamo_ctx* ctx, int64_t* out, int32_t n);

/* Number of kernels this library has launched since it was loaded (all contexts). No reference
 * counterpart (launch accounting for benchmarks). */
int64_t pamo_launch_count(void);

/* Phase timers: when enabled, CUDA events on the call's stream bracket each phase of every round
 * (0 load/shuffle, 1 adjacency, 2 quadrics, 3 edge cost, 4 selection+collapse, 5 cleanup+query marks,
 * 6 LBVH build, 7 LBVH query + pair tests, 8 undo, 9 compaction, 10 centring). Enabling resets them.
 * No reference counterpart (the reference only prints wall-clock times, simp_cuda/pamo/__init__.py:121,160). */
int pamo_profile_enable(pamo_ctx* ctx, int32_t enable);

/* Accumulated milliseconds and launch counts per phase; returns the number of phases. */
int pamo_profile_read(const pamo_ctx* ctx, double* ms, int64_t* counts, int32_t n);

/* ------------------------------------------------------------------------------------------------------
 * Many meshes on one GPU (no reference counterpart: the reference runs one PaMO object at a time). A pool of
 * worker contexts, each on its own CUDA stream and host thread, runs the whole PaMO.run loop
 * (pamo_simplify_device) per mesh. Every job starts from the state of a new context (pamo_ctx_reset), so each
 * result equals the mesh's result alone.
 * ------------------------------------------------------------------------------------------------------ */
typedef struct pamo_batch pamo_batch;
typedef struct pamo_server pamo_server;

int pamo_batch_create(pamo_batch** out, int device, int32_t n_workers);
int pamo_batch_destroy(pamo_batch* b);
const char* pamo_batch_last_error(const pamo_batch* b);

/* Simplify n_meshes meshes given in CSR form: points [V_total*3] float32 and triangles [F_total*3] int32 (device),
 * mesh m owning rows vert_offsets[m]..vert_offsets[m+1] and face_offsets[m]..face_offsets[m+1] (host arrays of
 * n_meshes+1), its triangle indices local to its own vertices; ratios[m] per mesh (host); tolerance, threshold,
 * iter and min_verts as PaMO.run. Results (centring undone) are written packed in mesh order into out_points
 * and out_triangles (device, room for the input sizes), with their CSR offsets in out_vert_offsets and
 * out_face_offsets (host, n_meshes+1). Synchronises `stream`. */
int pamo_batch_simplify(pamo_batch* b, const float* points, const int32_t* triangles, const int64_t* vert_offsets,
                        const int64_t* face_offsets, int32_t n_meshes, const double* ratios, int32_t tolerance,
                        float threshold, int32_t iter, int64_t min_verts, float* out_points, int32_t* out_triangles,
                        int64_t* out_vert_offsets, int64_t* out_face_offsets, pamo_stream stream);

/* Rounds each mesh of the last batch ran (host array); returns the number written. */
int pamo_batch_rounds(const pamo_batch* b, int32_t* rounds, int32_t capacity);

/* ------------------------------------------------------------------------------------------------------
 * Batched rounds (no reference counterpart): many meshes concatenated in CSR form run the PaMO.run loop together
 * on one stream, every round being one pass of the round's kernels over all live meshes (CUSimp_Free::forward,
 * cusimp_free.cu:891-1048, once per mesh). The state the reference carries between rounds lives in fixed regions
 * per mesh, each mesh gets its own LBVH subtree, loop control is per mesh, and a finished mesh leaves the next
 * round: each result equals the mesh's result alone.
 * ------------------------------------------------------------------------------------------------------ */
typedef struct pamo_csr pamo_csr;
int pamo_csr_create(pamo_csr** out, int device);
int pamo_csr_destroy(pamo_csr* b);
const char* pamo_csr_last_error(const pamo_csr* b);
/* "skinny_pow" (default 0): as pamo_ctx_set_option's option of the same name. */
int pamo_csr_set_option(pamo_csr* b, const char* name, int64_t value);
/* Same contract as pamo_batch_simplify (at most 65,536 meshes and 2^29 faces per call); synchronises `stream`. */
int pamo_csr_simplify(pamo_csr* b, const float* points, const int32_t* triangles, const int64_t* vert_offsets,
                      const int64_t* face_offsets, int32_t n_meshes, const double* ratios, int32_t tolerance,
                      float threshold, int32_t iter, int64_t min_verts, float* out_points, int32_t* out_triangles,
                      int64_t* out_vert_offsets, int64_t* out_face_offsets, pamo_stream stream);
/* Rounds each mesh of the last call ran (host array); returns the number written. */
int pamo_csr_rounds(const pamo_csr* b, int32_t* rounds, int32_t capacity);

/* A request loop: n_workers workers; requests queue in arrival order and are admitted while the device bytes
 * they are estimated to need (pamo_server_job_bytes) fit hbm_budget_bytes (a request larger than the budget
 * runs alone). */
int pamo_server_create(pamo_server** out, int device, int32_t n_workers, int64_t hbm_budget_bytes);
int pamo_server_destroy(pamo_server* s);
const char* pamo_server_last_error(const pamo_server* s);

/* Submit one PaMO.run job (stage 2, min_verts 0) on HOST arrays (copied before returning). */
int pamo_server_submit(pamo_server* s, const float* points, const int32_t* triangles, int32_t n_points,
                       int32_t n_triangles, double ratio, int32_t tolerance, float threshold, int64_t* request_id);

/* pamo_server_submit with use_stage3 != 0: after stage 2 the job runs PaMO.run's stage 3 (trimesh's processing of
 * the stage-2 mesh, then pamo_safe_project onto the request's own input mesh, 5 steps, default parameters), and its
 * result has float64 positions (pamo_server_fetch_f64). */
int pamo_server_submit_ex(pamo_server* s, const float* points, const int32_t* triangles, int32_t n_points,
                          int32_t n_triangles, double ratio, int32_t tolerance, float threshold, int32_t use_stage3,
                          int64_t* request_id);

/* Wait up to timeout_ms for a finished request: returns 1 with its id, status, output sizes and times_ms[3]
 * (queued until admitted, admitted until finished, submitted until finished), or 0 on time-out. */
int pamo_server_wait(pamo_server* s, int32_t timeout_ms, int64_t* request_id, int32_t* status, int32_t* out_n_points,
                     int32_t* out_n_triangles, double* times_ms);

/* Copy a finished request's result into host arrays (sizes from pamo_server_wait) and release it. */
int pamo_server_fetch(pamo_server* s, int64_t request_id, float* points, int32_t* triangles);
/* The same with float64 positions (a stage-3 result's own precision). */
int pamo_server_fetch_f64(pamo_server* s, int64_t request_id, double* points, int32_t* triangles);

/* Counters, out[0..n): bytes in use, most bytes in use so far, requests admitted, finished, queued, budget,
 * stage-3 projections run a second time without cooperative kernels (after a bounded grid-wide wait gave up).
 * Returns 7. */
int pamo_server_stats(pamo_server* s, int64_t* out, int32_t n);

/* The admission estimate of a job's device bytes. */
int64_t pamo_server_job_bytes(int32_t n_points, int32_t n_triangles);

/* The processing a stage-3 request's stage-2 mesh goes through before the projection (host code, no GPU):
 * trimesh.Trimesh(V, F)'s default processing as PaMO.run applies it (simp_cuda/pamo/__init__.py:165-176):
 * faces on non-finite vertices dropped, vertices equal after rounding to 8 decimals merged (first occurrence
 * kept), unreferenced vertices dropped, first-occurrence order. Outputs have room for the input sizes; returns
 * PAMO_ERR_INVALID_ARG for an index outside [0, n_points). */
int pamo_mesh_process(const double* points, int32_t n_points, const int32_t* triangles, int32_t n_triangles,
                      double* out_points, int32_t* out_n_points, int32_t* out_triangles, int32_t* out_n_triangles);

/* ------------------------------------------------------------------------------------------------------
 * Stage 3: safe projection of the simplified mesh onto the input ("GT") mesh.
 * A pamo_stage3 handle replaces the reference's Stage3System (simp_cuda/safe_project/src/pamo_safe_project/
 * system.py:28-110), which PaMO builds once and reuses across run() calls (simp_cuda/pamo/__init__.py:34-36).
 * ------------------------------------------------------------------------------------------------------ */
typedef struct pamo_stage3 pamo_stage3;

/* Stage3System(Stage3Config(), device) with the default configuration (config.py:6-73). */
int pamo_stage3_create(pamo_stage3** out, int device);

/* Release the handle and its device buffers. */
int pamo_stage3_destroy(pamo_stage3* s);

/* Message of the last failed stage-3 call ("" when none). */
const char* pamo_stage3_last_error(const pamo_stage3* s);

/* Set one Stage3Config field by its reference name (config.py:6-73): n_newton_iters, n_cg_iters,
 * n_line_search_iters, d_hat, coll_stiffness, contact_detection_radius, ee_classify_thres, ccd_slackness,
 * ccd_thickness, ccd_max_iters, spd_max_iters, elas_young_modulus, elas_poisson_ratio, hinge_stiffness,
 * mesh2gt_dist_stiffness, min_angle_thres (degrees), max_blocks. Execution knobs that leave the method
 * unchanged: use_cuda_graph (0/1), ccd_fp64 (1: float64 CCD step, the default; 0: float32 like the reference),
 * cg_mode (PCG launch shape: 0 cooperative 128-thread blocks, 2 one thread-block cluster, 3/4 256/512-thread
 * blocks, 5/6 at least one/two blocks per SM), ls_mode (1: the line search as one cooperative launch, 0: a
 * launch pair per trial). Unknown names: PAMO_ERR_INVALID_ARG. */
int pamo_stage3_set_param(pamo_stage3* s, const char* name, double value);

/*
 * pamo_safe_project.process(gt_V, gt_F, stage2_V, stage2_F, n_iters) (processing.py:23-106): normalise by
 * the GT mesh's mean and largest extent, register the mesh (Voronoi weights, StVK rest shapes, hinges),
 * then n_iters steps of closest-point targets + n_newton_iters Newton iterations (contact detection,
 * Jacobi PCG, step clamp, additive CCD, backtracking line search) (system.py:411-470). gt_points and
 * points are float64 rows of 3 (device), triangles int32 rows of 3 (device); out_points receives the
 * n_points x 3 float64 result in the input frame (device). The faces are unchanged. Synchronises `stream`.
 */
int pamo_safe_project(pamo_stage3* s, const double* gt_points, const int32_t* gt_triangles, int32_t n_gt_points,
                      int32_t n_gt_triangles, const double* points, const int32_t* triangles, int32_t n_points,
                      int32_t n_triangles, int32_t n_iters, double* out_points, pamo_stream stream);

/* Diagnostics of the last pamo_safe_project call, out[0..n): particles, triangles, edges, hinges, steps,
 * Newton iterations, most contacts in one detection, detection-radius halvings, do-nothing flag, final
 * energy, contacts summed over detections, rebuilds of the contact candidate lists, 1 when a grid barrier of a
 * cooperative kernel gave up and the run was made again without cooperative kernels (same bits). Returns 13. No reference
 * counterpart (the reference logs these). */
int pamo_stage3_stats(const pamo_stage3* s, double* out, int32_t n);

/* The topology a stage-3 call builds on the host (no GPU): the unique edges in trimesh's edges_unique order
 * (2 ints per edge, smaller endpoint first, ordered by (larger, smaller); room for 3 n_triangles edges) and the
 * hinges of hinge_preprocess_slow_kernel (safe_project/.../hinge_energy.py:21-57; 4 ints per hinge: opposite
 * vertex in t0, a, b, opposite vertex in t1, for every directed edge (a, b), a < b, of a face t0 and every face t1
 * holding (b, a)). *n_hinges is the full count; PAMO_ERR_CAPACITY when it exceeds hinge_capacity. */
int pamo_stage3_topology(const int32_t* triangles, int32_t n_points, int32_t n_triangles, int32_t* edges,
                         int32_t* n_edges, int32_t* hinges, int32_t hinge_capacity, int32_t* n_hinges);

/* ---------------------------------------------------------------- evaluation (metrics.py:7-107)
 * Squared distances from points to a triangle mesh, as igl.point_mesh_squared_distance and
 * trimesh.proximity.closest_point compute them for the reference's Chamfer and Hausdorff distances
 * (simp_cuda/safe_project/src/pamo_safe_project/metrics.py:7-50): out_sqdist[i] = min over faces of the
 * squared float64 distance from points[i] to the face, out_face[i] = that face (lowest index on ties; may be
 * NULL). All arrays are device arrays (float64 [n,3], int32 [m,3]). Synchronises `stream`. */
int pamo_point_mesh_sqdist(const double* points, int32_t n_points, const double* vertices, int32_t n_vertices,
                           const int32_t* triangles, int32_t n_triangles, double* out_sqdist, int32_t* out_face,
                           pamo_stream stream);

/* Per-face minimum angles in radians (metrics.py:55-107): out_edge_form as compute_min_angle_VF computes
 * the corner angles (from the face's edge vectors, cosines clipped to [-1, 1]), out_igl_form as
 * igl.internal_angles does (law of cosines on the edge lengths), NaN for a face with a repeated index. Either
 * output may be NULL. Device arrays; synchronises `stream`. */
int pamo_face_min_angles(const double* vertices, const int32_t* triangles, int32_t n_triangles, double* out_edge_form,
                         double* out_igl_form, pamo_stream stream);

/* ---------------------------------------------------------------- stage 1 (remeshing)
 * PaMO.remesh (simp_cuda/pamo/__init__.py:58-93): preprocess_mesh's normalisation into the unit cube, a
 * narrow-band distance field of the triangles on a resolution^3 grid (band 3 / R) with the inside found by a
 * flood fill from the grid boundary, its level set at 0.9 voxel extracted as a closed triangle mesh, mapped
 * back to the input's frame minus mean3 (the tris_mean of pamo_tris_mean, as the reference's remesh output
 * is). The reference calls torchcumesh2sdf and pdmc for this; both are absent, so the construction is this
 * library's own (dual extraction, one vertex per sign-changing cell). Device points/triangles; sizes out;
 * fetch the mesh with pamo_remesh_result. */
typedef struct pamo_remesher pamo_remesher;
int pamo_remesher_create(pamo_remesher** out, int32_t device);
int pamo_remesher_destroy(pamo_remesher* m);
int pamo_remesh(pamo_remesher* m, const float* points, const int32_t* triangles, int32_t n_points, int32_t n_triangles,
                int32_t resolution, const float* mean3, int32_t* out_n_points, int32_t* out_n_triangles,
                pamo_stream stream);
int pamo_remesh_result(pamo_remesher* m, float* verts, int32_t* tris, pamo_stream stream);

/* The stage-2 loop of PaMO.run with an explicit face target (target_faces computed by the caller, e.g. from the
 * input's face count when stage 1 replaced the mesh) and centring optional (off when the points are already
 * centred, as after stage 1). Otherwise as pamo_simplify_device. */
int pamo_simplify_device_target(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                                int32_t n_triangles, int64_t target_faces, int32_t tolerance, float threshold,
                                int32_t iter, int32_t centre, int32_t* out_n_points, int32_t* out_n_triangles,
                                int32_t* out_rounds, pamo_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* PAMO_GB300_H */
