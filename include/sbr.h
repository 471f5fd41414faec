/* sbr.h - C ABI of the GB300 shoot-bounce-reflect (SBR) propagation path.
 *
 * Drop-in boundary for SBRSolver's hot path.  Each entry point replaces one
 * piece of the reference's C++ interface (paths relative to SBRSolver_rev2/):
 *
 *   sbr_scene_create / _from_stl  Preprocessor::StlToGeometry (Preprocessor.h:24-31,
 *                                 Preprocessor.cpp:69-114) + BVH<Triangle>::ConstructBVH
 *                                 (BVH/BVH.h:25,51-55) + RTSolver::Init (RTSolver.h:23,
 *                                 RTSolver.cpp:13-22): triangles, coplanar ids, SAH BVH and
 *                                 the material table, resident on the GPU.
 *   sbr_solve                     RTSolver::ExecuteRayTracing (RTSolver.h:25-37,
 *                                 RTSolver.cpp:52-126): ray launch, bounces, reception
 *                                 spheres, image correction, duplicate removal, field.
 *   sbr_solve_batch               many ExecuteRayTracing calls (one per transmitter) in one
 *                                 device pass; no reference counterpart (the reference runs
 *                                 one transmitter per call).
 *   sbr_result_field              FieldCompute::FieldAtReceiver (FieldCompute.h:37,
 *                                 FieldCompute.cpp:11-25) for every receiver.
 *   sbr_result_paths              RTSolver::_rayPaths after duplicate removal (the data
 *                                 SavePathsAsVtk writes, RTSolver.cpp:510-610).
 *   sbr_last_error                none in the reference (it reports no errors); every call
 *                                 here returns an sbr_status and leaves a message.
 *
 * Conventions: plain pointers and sizes, host memory unless a field says
 * otherwise, row-major 3x3 matrices, no exceptions across the boundary.
 * Results match the reference's FP64 CPU code: identical path sets
 * (facet-id sequences, launch ids, ray counts) and received fields within
 * 1e-4 relative magnitude / 1e-3 rad phase in the default precision mode.
 */
#ifndef SBR_H
#define SBR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sbr_status {
  SBR_OK = 0,
  SBR_ERR_INVALID_ARG = 1,
  SBR_ERR_OOM = 2,           /* device or host allocation failed, or over the memory budget */
  SBR_ERR_CAPACITY = 3,      /* a work queue or table stayed full after the allowed regrowth */
  SBR_ERR_TIMEOUT = 4,
  SBR_ERR_CUDA = 5,
  SBR_ERR_IO = 6,
  SBR_ERR_NOT_READY = 7
} sbr_status;

/* MaterialProperties (common/DataStructures.h:20-28), same field order.
 * The field uses rel_permittivity_re and rel_conductivity only, like the
 * reference (FieldCompute.cpp:185-235).
 * width: wall thickness in metres for the slab coefficients
 * (FieldCompute.cpp:255-262,284-291), used when use_fresnel is 0.  The
 * reference always passes 0 (FieldCompute.cpp:131,138), which gives
 * reflection 0 and transmission 1; width 0 reproduces that. */
typedef struct sbr_material {
  double frequency, transmission_loss, reflection_loss;
  double rel_permittivity_re, rel_permittivity_im, rel_conductivity;
  double width;
} sbr_material;

/* Antenna patterns of FieldCompute::GetAnalyticEfieldPattern
 * (FieldCompute.cpp:153-183); the reference always uses SBR_ANTENNA_HERTZIAN. */
enum { SBR_ANTENNA_ISOTROPIC = 0, SBR_ANTENNA_HERTZIAN = 1, SBR_ANTENNA_HALF_WAVE = 2,
       SBR_ANTENNA_TABULATED = 3 /* sbr_request.pattern: see sbr_pattern_create */ };
typedef struct sbr_pattern sbr_pattern;

/* Field precision: FP64 everywhere, or FP32 Fresnel/rotation arithmetic
 * with FP64 path length and phase and a compensated FP32 per-receiver sum.
 * SBR_FIELD_FP32_PHASE also takes path length and phase k*L in FP32; it
 * exists to measure the phase error that FP64 length/phase avoids. */
enum { SBR_FIELD_FP64 = 0, SBR_FIELD_FP32 = 1, SBR_FIELD_FP32_PHASE = 2 };

typedef struct sbr_scene sbr_scene;
typedef struct sbr_result sbr_result;

typedef struct sbr_scene_info {
  int n_triangles, n_bvh_nodes, bvh_depth, n_coplanar;
  double extent;          /* max |coordinate| of the scene */
  long long device_bytes; /* resident scene size */
  /* wall time of the scene's preparation (ms): the whole of sbr_scene_create;
   * the host's part (triangle records; every table with SBR_SCENE_HOST_PREP);
   * on the device: vertex merge, coplanar groups and frames; the search BVH;
   * the reference BVH; then the upload of the finished tables */
  double prep_total_ms, prep_host_ms, prep_device_tables_ms, prep_search_bvh_ms,
      prep_reference_bvh_ms, prep_upload_ms;
} sbr_scene_info;

/* Arguments of RTSolver::ExecuteRayTracing (RTSolver.h:25-37) plus the
 * pattern and precision knobs the reference hard-codes. */
typedef struct sbr_request {
  double tx[3];
  double tx_coord_sys[9];  /* row-major; the reference's txCoordSys */
  int max_reflection, max_transmission;
  double frequency, pt;
  int use_fresnel;         /* useFresnelCoeff */
  int tessellation;        /* icosahedron subdivision level (txTesslation) */
  int antenna;             /* SBR_ANTENNA_*; SBR_ANTENNA_HERTZIAN reproduces the reference */
  int field_precision;     /* SBR_FIELD_* */
  int n_rx;
  const double* rx;        /* 3 doubles per receiver */
  int rx_on_device;        /* rx is a device pointer (already resident) */
  int stage_counts;        /* also count captures before correction (sbr_counts.captured);
                              costs time, results are identical either way */
  int field_check;         /* FP32 field precisions: also compute the FP64 field on the
                              GPU so sbr_result_field_error can state the error */
  const sbr_pattern* pattern; /* antenna SBR_ANTENNA_TABULATED; must outlive the solve */
} sbr_request;

typedef struct sbr_counts {
  long long segments;      /* executed ray segments = closest-hit queries (rays x bounces) */
  long long captured;      /* receiver captures before image correction (-1 unless
                              the request set stage_counts) */
  long long corrected;     /* captures whose image correction succeeded */
  long long paths;         /* surviving paths after duplicate removal */
  long long rays;          /* rays over all surviving paths */
  long long fp64_triangle_tests, fallback_rays, fp64_capture_tests;
  long long launches;
  long long capture_candidates; /* receivers tested against a reception sphere */
  long long ancestor_tests;     /* re-tests of ancestors for capture suppression */
  long long classes;            /* distinct (facet, interaction) prefixes traced */
  long long groups;             /* unused, -1 */
  long long keys;               /* distinct (receiver, coplanar key) after correction */
  long long near_edge_paths;    /* surviving paths with an interaction point within 1e-6
                                   (barycentric) of its triangle's edge */
  long long gpu_kernels;        /* kernel launches of the solve (a batch's, for its parts) */
  long long fp64_field_paths;   /* SBR_FIELD_FP32: paths whose field was taken in FP64 (an
                                   ill-conditioned path, or one of an uncertified receiver) */
  long long fp64_field_receivers; /* SBR_FIELD_FP32: receivers whose error bound could not
                                     certify the tolerance, recomputed and summed in FP64 */
  long long pipeline_graph;     /* 1: the device pipeline ran as one CUDA graph launch (the
                                   same pipeline, i.e. request structure, capacities and
                                   launch shapes, ran before on this scene: captured the
                                   second time, replayed after) */
} sbr_counts;

/* One surviving path; its rays are [ray_offset, ray_offset + n_rays) in the
 * flat arrays of sbr_result_paths. */
typedef struct sbr_path {
  int request, receiver, n_rays, heap;  /* heap: BFS position in the launch's ray tree */
  long long launch;
  long long ray_offset;
  double field[6];                      /* this path's contribution (Ex re, im, Ey, Ez) */
  int near_edge;                        /* 1: an interaction point lies within 1e-6
                                           (barycentric) of its triangle's edge */
  int reserved;
} sbr_path;

/* Error of an FP32-precision field against the FP64 field of the same path
 * set (requests with field_check).  Components compared: those whose FP64
 * magnitude exceeds 1e-6 of the receiver's largest component. */
typedef struct sbr_field_error {
  long long components;      /* receiver field components compared */
  long long over_tolerance;  /* of those, outside 1e-4 relative magnitude or 1e-3 rad */
  double max_rel_mag;        /* max | |E| - |E64| | / |E64| */
  double max_phase_rad;      /* max |arg(E / E64)| */
  double max_rel_vec;        /* max |E - E64| / |E64| */
} sbr_field_error;

/* Stage times from CUDA events on the engine's stream.  device_ms spans
 * everything after the receivers are on the device (grid, trace, capture,
 * correction, field) and before results are copied back; capture_kernel_ms
 * is the capture kernel alone (inside capture_ms), trace_kernel_ms the
 * FP64 resolution-and-spawn kernel alone over its trace_kernel_launches
 * launches (inside trace_ms, which also holds the FP32 candidate search),
 * trace_kernel_first_ms its first launch alone (the launch rays: one
 * segment per launch direction of every request). */
typedef struct sbr_timing {
  double total_ms, trace_ms, capture_ms, correct_ms, field_ms, h2d_ms, d2h_ms, device_ms;
  double capture_kernel_ms, trace_kernel_ms, trace_kernel_launches, trace_kernel_first_ms;
} sbr_timing;

/* ---- scene ---------------------------------------------------------- */
/* vertices: 9 floats per triangle (v1, v2, v3); normals: 3 floats per
 * triangle (facet normals as in the STL); material_ids may be NULL (all 0). */
sbr_status sbr_scene_create(int n_triangles, const float* vertices, const float* normals,
                            const int* material_ids, const sbr_material* materials,
                            int n_materials, sbr_scene** out);
/* As sbr_scene_create, with flags.  By default the GPU builds the coplanar
 * groups (Preprocessor.cpp:116-246), the triangle frames and boxes
 * (Triangle.cpp:37-70) and the search BVH, while the host builds the
 * reference BVH (BVH.h:135-230, whose tie order only the host's std::sort
 * reproduces); SBR_SCENE_HOST_PREP builds everything on the host.  Both give
 * identical tables. */
#define SBR_SCENE_HOST_PREP 1u
sbr_status sbr_scene_create_ex(int n_triangles, const float* vertices, const float* normals,
                               const int* material_ids, const sbr_material* materials,
                               int n_materials, unsigned flags, sbr_scene** out);
/* The scene's prepared tables, by triangle id (file order): frame rows
 * (9 doubles: x, y, z rows), box (6: min xyz, max xyz), box centre (3);
 * any pointer may be NULL. */
sbr_status sbr_scene_triangle_frames(const sbr_scene* scene, double* frames, double* boxes,
                                     double* centers);
/* The search BVH: *n_nodes in: capacity of nodes (14 4-byte words per node:
 * lo[2][3], hi[2][3] floats, child[2] ints, a child < 0 being the leaf
 * ~(first << 3 | count)), out: node count; order: the depth-first rank of
 * each leaf slot (as many as triangles).  NULL nodes/order: sizes only. */
sbr_status sbr_scene_search_bvh(const sbr_scene* scene, int* n_nodes, int* max_depth,
                                float* nodes, int* order);
/* The reference BVH (BVH/BVH.h:135-230), nodes in depth-first order
 * (children[0] subtree first): *n_nodes in: capacity, out: node count;
 * boxes: 6 doubles per node (min xyz, max xyz); links: 6 ints per node
 * (child 0, child 1 (-1 for a leaf), first, count (leaf range of order),
 * parent, depth); order: the triangle ids of the leaves in visit order (as
 * many as triangles).  NULL boxes/links/order: sizes only. */
sbr_status sbr_scene_reference_bvh(const sbr_scene* scene, int* n_nodes, int* max_depth,
                                   double* boxes, int* links, int* order);
sbr_status sbr_scene_create_from_stl(const char* path, const int* material_ids,
                                     const sbr_material* materials, int n_materials,
                                     sbr_scene** out);
sbr_status sbr_scene_info_get(const sbr_scene* scene, sbr_scene_info* out);
/* Triangle id at each position of the caller's triangle vector once
 * BVH::ConstructBVH has sorted it (BVH/BVH.h:152,214).  The reference indexes
 * that vector by triangle id during image correction and the field stage
 * (RTSolver.cpp:356,415; FieldCompute.cpp:107), so this order is part of its
 * result; sbr_scene_create installs it by default. */
sbr_status sbr_scene_mesh_order(const sbr_scene* scene, int* out);
/* Replace that order (e.g. identity for a caller whose vector is in file order). */
sbr_status sbr_scene_set_mesh_order(sbr_scene* scene, const int* order);
sbr_status sbr_scene_coplanar_ids(const sbr_scene* scene, int* out);
/* Replace the per-triangle material ids (NULL = all 0) and the material
 * table, as RTSolver::Init (RTSolver.cpp:13-22) binds materials after
 * BVH::ConstructBVH.  Not while solves on the scene are running. */
sbr_status sbr_scene_set_materials(sbr_scene* scene, const int* material_ids,
                                   const sbr_material* materials, int n_materials);
sbr_status sbr_scene_destroy(sbr_scene* scene);
/* The facets of a binary or ASCII STL file in file order (StlReader.h, as
 * Preprocessor::StlToGeometry reads it, Preprocessor.cpp:69-114): 9 floats
 * of vertices and 3 of normal per facet.  With vertices or normals NULL only
 * *n_triangles is set; otherwise *n_triangles is the buffers' capacity on
 * entry (SBR_ERR_CAPACITY if too small) and the facet count on return.  No
 * GPU needed. */
sbr_status sbr_stl_read(const char* path, int* n_triangles, float* vertices, float* normals);

/* ---- solve ---------------------------------------------------------- */
sbr_status sbr_solve(sbr_scene* scene, const sbr_request* request, sbr_result** out);
sbr_status sbr_solve_batch(sbr_scene* scene, const sbr_request* requests, int n_requests,
                           sbr_result** out);

sbr_status sbr_result_counts(const sbr_result* result, sbr_counts* out);
/* 6 doubles per receiver (Ex re, Ex im, Ey re, Ey im, Ez re, Ez im), requests
 * concatenated in order. */
sbr_status sbr_result_field(const sbr_result* result, double* out);
/* Per receiver, a bound on the absolute error of each of its three complex
 * field components (n_rx doubles).  SBR_FIELD_FP32 requests: every path's
 * FP32 error is bounded by (16 kappa + 1) FP32 ulps of its field, kappa its
 * condition number (largest field it could carry over the field it ends
 * with; paths with kappa > 32 or a Fresnel coefficient near a pole of its
 * formula are computed in FP64); a receiver's bound is the sum over its
 * paths plus 2 ulps of the summed field.  A receiver whose bound exceeds half
 * the tolerance (1e-4 relative magnitude) of a component is recomputed and
 * summed in FP64 (bound 0), so every FP32 component meets 1e-4 / 1e-3 rad.
 * 0 for SBR_FIELD_FP64 (the reference's arithmetic), -1 for
 * SBR_FIELD_FP32_PHASE (no bound: a study mode). */
sbr_status sbr_result_field_bound(const sbr_result* result, double* out);
/* Field error of an FP32-precision result against FP64 (request field_check);
 * SBR_ERR_NOT_READY when the result carries no FP64 field. */
sbr_status sbr_result_field_error(const sbr_result* result, sbr_field_error* out);
/* The FP64 field of a field_check result, in sbr_result_field's layout. */
sbr_status sbr_result_field_fp64(const sbr_result* result, double* out);
/* paths: counts.paths entries; tri/cop/kind: counts.rays entries
 * (kind 0 = launch, 1 = reflected, 2 = transmitted; tri/cop -1 on the last
 * ray); points: 6 doubles per ray (corrected source, target).  Any output
 * pointer may be NULL. */
sbr_status sbr_result_paths(const sbr_result* result, sbr_path* paths, int* tri, int* cop,
                            int* kind, double* points);
sbr_status sbr_result_timing(const sbr_result* result, sbr_timing* out);
sbr_status sbr_result_destroy(sbr_result* result);

const char* sbr_last_error(void);
const char* sbr_version(void);

/* ---- request server ------------------------------------------------- */
/* No reference counterpart (the reference's main() runs one solve).  A
 * server runs `slots` solves at a time over resident scenes: submitted
 * requests queue in arrival order and each starts as soon as a slot is free
 * and its device-memory estimate fits in the HBM budget next to the requests
 * already running (hbm_budget_bytes <= 0: 60% of free memory at creation).
 * Requests admitted while others run overlap with them on the GPU (separate
 * streams); each result equals sbr_solve of that request alone. */
typedef struct sbr_server sbr_server;
typedef struct sbr_completion {
  long long tag;           /* the caller's tag from sbr_server_submit */
  int status;              /* sbr_status of the solve */
  int scene;
  double queue_ms;         /* submit -> start */
  double latency_ms;       /* submit -> result ready */
  double device_ms;        /* sbr_timing.device_ms */
  sbr_counts counts;
  sbr_result* result;      /* caller destroys with sbr_result_destroy (NULL on error) */
} sbr_completion;
sbr_status sbr_server_create(sbr_scene* const* scenes, int n_scenes, int slots,
                             long long hbm_budget_bytes, sbr_server** out);
/* Copies the request and its receivers (host memory); returns at once. */
sbr_status sbr_server_submit(sbr_server* server, int scene, const sbr_request* request,
                             long long tag);
/* Up to max finished requests; waits up to timeout_ms when none is ready. */
sbr_status sbr_server_poll(sbr_server* server, sbr_completion* out, int max, int* n_out,
                           int timeout_ms);
sbr_status sbr_server_pending(sbr_server* server, int* queued, long long* in_flight_bytes);
/* Admission and batching policy (takes effect for the next request a worker
 * picks): requests whose device-memory estimate is at most batch_bytes are
 * solved together with the queued ones of the same scene that are also that
 * small, up to max_batch per device pass (1 = never batch); a request's
 * priority is its estimate minus aging_bytes_per_s for every second it has
 * waited (0 = smallest first, large = arrival order); at most max_large
 * requests larger than batch_bytes run at once (0 = as many as the slots;
 * small batches still run beside them).  Defaults: 2 GiB, 64, 16e9, 0. */
sbr_status sbr_server_set_policy(sbr_server* server, long long batch_bytes, int max_batch,
                                double aging_bytes_per_s, int max_large);
/* Finishes queued and running requests, then stops. */
sbr_status sbr_server_destroy(sbr_server* server);

/* ---- tabulated antenna patterns -------------------------------------- */
/* The reference ships data/TXPattern.dat and reads it with
 * Preprocessor::ReadPatternFile (Preprocessor.cpp:3-35) into a GainMap, but
 * never applies it.  Antenna SBR_ANTENNA_TABULATED applies such a table to
 * the launch direction (theta, phi in the txCoordSys frame, as the analytic
 * patterns): E_theta = sqrt(60 Pt) 10^(g_theta/20) e^(j arg_theta), E_phi
 * likewise, gains in dB, phases in degrees, bilinear on the grid.
 * gain_phase: 4 floats per grid point (g_theta, arg_theta, g_phi, arg_phi),
 * theta-major, theta = i * d_theta (i < n_theta, at most 180 degrees), phi =
 * j * d_phi with n_phi * d_phi = 360.  The table is copied to the current
 * device. */
sbr_status sbr_pattern_create(int n_theta, int n_phi, double d_theta, double d_phi,
                              const float* gain_phase, sbr_pattern** out);
/* TXPattern.dat: lines of six numbers (theta phi g_theta arg_theta g_phi
 * arg_phi) on a regular grid from (0, 0); other lines are skipped. */
sbr_status sbr_pattern_read(const char* path, sbr_pattern** out);
sbr_status sbr_pattern_info(const sbr_pattern* pattern, int* n_theta, int* n_phi,
                            double* d_theta, double* d_phi);
sbr_status sbr_pattern_destroy(sbr_pattern* pattern);

/* ---- receiver layouts ---------------------------------------------- */
/* Preprocessor::GenerateRXLine (Preprocessor.cpp:270-284): floor(|end-start|
 * / resolution) points start + i*resolution*unit(end-start).  With out NULL
 * only *n_out is set; otherwise `capacity` points fit in out (3 doubles each,
 * SBR_ERR_CAPACITY if fewer).  No GPU needed. */
sbr_status sbr_generate_rx_line(const double* start, const double* end, double resolution,
                                double* out, int capacity, int* n_out);
/* Preprocessor::GenerateRxPlane (Preprocessor.cpp:254-268): an
 * (int((xMax-xMin)/res)+1) x (int((yMax-yMin)/res)+1) grid at `height`,
 * x-major; same buffer convention. */
sbr_status sbr_generate_rx_plane(double x_min, double y_min, double x_max, double y_max,
                                 double height, double resolution, double* out, int capacity,
                                 int* n_out);

/* ---- result files --------------------------------------------------- */
/* The reference's output files, byte for byte (default six-digit stream
 * formatting, the sticky '+' sign of its CSV writer, Phase columns holding
 * the sum of the component phases in radians).  Arrays are host memory in
 * the layouts of sbr_result_field / sbr_result_paths.  Return SBR_ERR_IO when
 * the file cannot be written. */
/* RTSolver::SaveFieldAsCsv (RTSolver.cpp:692-717): X,Y,Z,Ex,Ey,Ez rows. */
sbr_status sbr_write_field_csv(const char* path, const double* rx, int n_rx, const double* field);
/* RTSolver::SaveReceiversAsVtk (RTSolver.cpp:612-690). */
sbr_status sbr_write_receivers_vtk(const char* path, const double* rx, int n_rx,
                                   const double* field);
/* RTSolver::SavePathsAsVtk (RTSolver.cpp:510-610): one polyline per path,
 * ordered by launch, receiver, then breadth-first tree position; `points`
 * holds 6 doubles (source, target) per ray; field is per receiver. */
sbr_status sbr_write_paths_vtk(const char* path, const sbr_path* paths, int n_paths,
                               const double* points, const double* field, int n_rx);
/* RTSolver::SaveIcosahedronAsVtk (RTSolver.cpp:719-766): the launch rays of
 * an icosahedron level as unit segments from `origin` (3 doubles). */
sbr_status sbr_write_launch_rays_vtk(const char* path, const double* origin, int tessellation);
/* GenerateRaysOnIcosahedron (Icosahedron.cpp:80-109, whose origin argument
 * is unused): the unit launch directions of subdivision level `tessellation`
 * (0..12), 3 doubles per ray in the reference's vertex order, the directions
 * sbr_solve launches.  *n_rays receives 10*4^level + 2; directions may be NULL
 * to query it, else it needs room for cap >= *n_rays rays.  Host only. */
sbr_status sbr_launch_directions(int tessellation, double* directions, long long cap,
                                 long long* n_rays);

/* ---- launch shapes and the autotuner ------------------------------------ */
/* No counterpart in the reference, whose solve is one single-threaded CPU
 * loop (RTSolver.cpp:82-121).  The launch shapes of the trace and capture
 * kernels; 0 in a field means the library's default. */
typedef struct sbr_tuning {
  int find_steps;            /* FP32 search: traversal steps between refills (32) */
  int find_refill;           /* FP32 search: idle lanes that trigger a warp's refill, <= 32 (16) */
  int find_blocks_per_sm;    /* FP32 search: resident 128-thread blocks per SM (all that fit) */
  int trace_blocks_per_sm;   /* FP64 resolution: resident 128-thread blocks per SM (all that fit) */
  int capture_blocks_per_sm; /* capture: resident blocks per SM (all that fit) */
  int trace_chunk_log2;      /* rays per search/resolution launch pair = 2^this, 16..26 (25) */
  int trace_kernel;          /* FP64 resolution: 1 = one ray per lane (registers), 2 = 64 rays
                                per warp in shared memory, tests handed out to full warps */
  int pipeline_graph;        /* 0 (default) or 1: a device pipeline that ran before (same
                                request structure, capacities and shapes) is captured as a
                                CUDA graph and replayed from then on; -1: every solve issues
                                its operations one by one */
  int find_tris_per_step;    /* FP32 search: triangles of a leaf tested per step, 1 or 2 (2) */
} sbr_tuning;
/* The scene's default shapes, used by request mixes sbr_autotune has not
 * tuned.  Values above what fits on an SM are clamped. */
sbr_status sbr_scene_set_tuning(sbr_scene* scene, const sbr_tuning* tuning);
/* The shapes a solve of this request mix would use, defaults filled in
 * (requests may be NULL with n_requests 0: the scene's default). */
sbr_status sbr_scene_get_tuning(sbr_scene* scene, const sbr_request* requests, int n_requests,
                                sbr_tuning* out);
/* Autotuner: solves the batch repeatedly, changing one shape at a time over
 * its candidates and keeping a change that cuts the batch's device time
 * (sbr_timing.device_ms, the better of two solves) by at least 1 %, for up
 * to `rounds` passes over the shapes (1..8).  The choice is kept for this
 * request mix (its requests' levels and bounce limits) and used by every
 * later solve of the same mix on this scene; out / best_ms (may be NULL)
 * receive it and its device time.  Other solves on the same scene while it
 * runs see the candidate shapes. */
sbr_status sbr_autotune(sbr_scene* scene, const sbr_request* requests, int n_requests, int rounds,
                        sbr_tuning* out, double* best_ms);

/* ---- fault injection (tests) ------------------------------------------ */
/* No counterpart in the reference, which reports no errors from the solve.
 * Lets a caller's tests see how the library and its server behave when the
 * device runs out of memory, without exhausting a shared GPU: with after >= 0
 * the (after+1)-th device allocation the library attempts from now on fails
 * as cudaMalloc fails on a full device (the call is not made), so the entry
 * point that needed it returns SBR_ERR_OOM; after < 0 disarms.  The count is
 * process-wide and covers every thread.  No GPU needed. */
sbr_status sbr_fault_inject_alloc(long long after);

/* ---- allocation-free field sum -------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory: processes whose device memory is held by another framework's
 * caching allocator, services that must keep a fixed device footprint after
 * start-up, and latency-bound loops that cannot afford cudaMalloc/cudaFree
 * (which may synchronise the device).  Sums per-path fields into
 * per-receiver fields in each receiver's (launch, BFS) rank order, with the
 * arithmetic sbr_solve's own sum uses (FP64 for SBR_FIELD_FP64, compensated
 * FP32 for both FP32 precisions, where sbr_solve itself switches to FP64 for
 * the receivers its FP32 error bound cannot certify; paths of equal rank are
 * added in path-index order), using only a fixed 4 MiB array compiled into the library (held on
 * every GPU that loads it until exit).  All pointers are device pointers
 * owned by the caller: path_receiver[n_paths] (0-based), path_rank[n_paths]
 * (launch << 17 | heap, see sbr_path), path_field[6 * n_paths],
 * field_out[6 * n_rx].  Limits: 1 <= n_rx <= 262144, 0 <= n_paths <= 262144,
 * at most 2048 paths on one receiver; larger sizes, receiver indices outside
 * [0, n_rx) and precisions other than SBR_FIELD_FP64 / SBR_FIELD_FP32 /
 * SBR_FIELD_FP32_PHASE are rejected with SBR_ERR_INVALID_ARG.  Runs on
 * `stream` (a cudaStream_t of the current device, NULL = default stream) and
 * returns after it completes.  The first call on a device looks up the
 * array's device address and must come before any stream capture.  A later
 * call on a stream that is being captured into a CUDA graph only enqueues its
 * kernels and returns SBR_OK: the host-side argument checks still apply, but
 * receiver indices outside [0, n_rx) and receivers over the per-receiver
 * limit are then skipped without a report (their fields stay zero).  Calls
 * share the array: calls (or graph launches) that overlap on the GPU race
 * and must be serialised by the caller. */
sbr_status sbr_receiver_field_sum_noalloc(const int* path_receiver, const long long* path_rank,
                                          const double* path_field, int n_paths, int n_rx,
                                          int field_precision, double* field_out,
                                          void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SBR_H */
