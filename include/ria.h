/*
 * ria.h - C ABI of the GB300 implementation of the per-tet implicit-arrangement path of
 * Robust-Implicit-Surface-Networks (duxingyi-charles).
 *
 * Plain pointers and sizes only.  Every call runs on the current CUDA device; there is no CPU
 * fallback: without a usable CUDA device the calls return RIA_ENODEVICE.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   implicit_arrangement(...)        src/implicit_arrangement.h:39-62 (stages signs, filter,
 *                                    per-tet cut, extract_iso_mesh, compute_iso_vert_xyz:
 *                                    src/implicit_arrangement.cpp:53-403)
 *   material_interface(...)          src/material_interface.h:38-61 (src/material_interface.cpp:53-448)
 *   load_functions(...)              the external implicit_functions library, called at
 *                                    app/implicit_arrangement.cpp:59 and app/material_interface.cpp:62
 *   compute_arrangement(planes)      simplicial_arrangement (external), called at
 *                                    src/implicit_arrangement.cpp:279,283
 *   compute_material_interface(m)    simplicial_arrangement (external), called at
 *                                    src/material_interface.cpp:323,327
 *   generate_tet_mesh(...)           src/io.cpp:95-152 (the *_grid_* entry points build the grid
 *                                    on the device)
 * The downstream stages (edges, patches, chains, face pairing, shells, cells) stay on the host and
 * consume the mesh returned here.
 */
#ifndef RIA_H
#define RIA_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define RIA_API __attribute__((visibility("default")))
#else
#define RIA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ria_status {
    RIA_OK = 0,
    RIA_EINVAL = 1,       /* bad argument (null pointer, n_func > 64, index out of range, ...) */
    RIA_ENOMEM = 2,       /* device or host allocation failed */
    RIA_ECAPACITY = 3,    /* a tet's arrangement exceeds the per-tet capacity (255 vertices or 254 cells: about
                             13 planes in general position; 60 active functions) */
    RIA_EDEGENERATE = 4,  /* an exact predicate exceeded its expansion capacity (extreme dynamic range) */
    RIA_ETIMEOUT = 5,     /* reserved for bounded device waits */
    RIA_ECUDA = 6,        /* a CUDA runtime call failed */
    RIA_EINTERNAL = 7,    /* an internal consistency check failed */
    RIA_ENODEVICE = 8     /* no CUDA device (the library never computes on the CPU) */
} ria_status;

/* Implicit function descriptor (one JSON object of a reference function file).
 *   RIA_FUNC_PLANE           p[0..2] point, p[3..5] normal:        n . (x - p)
 *   RIA_FUNC_SPHERE          p[0..2] centre, p[3] radius:          r - |x - c|
 *   RIA_FUNC_SPHERE_SQUARED  p[0..2] centre, p[3] radius:          r*r - |x - c|^2
 *   RIA_FUNC_CYLINDER        p[0..2] axis point, p[3..5] unit axis, p[6] radius:
 *                            v = x - a; t = v . u; r - |v - t u|
 *   RIA_FUNC_TORUS           p[0..2] centre, p[3..5] unit axis, p[6] major R, p[7] minor r:
 *                            v = x - c; h = v . u; rho = |v - h u|; r - sqrt((rho - R)^2 + h^2)
 *   RIA_FUNC_ZERO            0
 * flipped != 0 negates the value.  Every value is FP64, evaluated left to right as written with
 * each operation rounded on its own (no fused multiply-add) and a correctly rounded sqrt. */
enum {
    RIA_FUNC_ZERO = 0,
    RIA_FUNC_PLANE = 1,
    RIA_FUNC_SPHERE = 2,
    RIA_FUNC_SPHERE_SQUARED = 3,
    RIA_FUNC_CYLINDER = 4,
    RIA_FUNC_TORUS = 5
};

typedef struct ria_function {
    int32_t type;
    int32_t flipped;
    double p[12];
} ria_function;

/* Switches of the reference JSON config (src/io.h:12-28).  use_lookup = 0 forces
 * use_secondary_lookup = 0 (src/implicit_arrangement.cpp:38-40).  The lookup tables only choose
 * the code path; the result is the same either way. */
typedef struct ria_config {
    int32_t use_lookup;
    int32_t use_secondary_lookup;
    int32_t use_topo_ray_shooting; /* accepted for the downstream stages; unused here */
    int32_t robust_test;           /* -R: cut every tet in both plane orders and compare the
                                      vertex/face/cell counts (src/implicit_arrangement.cpp:137-243);
                                      the mesh then holds only the statistics, with the tets of each
                                      failure type counted (RIA_STAT_ROBUST_*), and the call returns
                                      RIA_EINTERNAL when any tet failed */
    int32_t keep_records;          /* keep the per-tet records (RIA_MESH_REC_*) */
} ria_config;

typedef struct ria_mesh ria_mesh;

/* Mesh fields.  Index values use int64 with -1 for "none" (the reference's size_t Mesh_None).
 *
 * Per-tet record layout (little endian, RIA_MESH_REC_BYTES; one record per tet with at least one
 * active function, in tet order).  Labels 0..3 are the tet faces (label b is the face opposite
 * corner b); label 4+j is the j-th active function (or material) of the tet.
 *   implicit arrangement:
 *     u8 type=1, u8 k, u16 nv, u16 nf, u16 nc, u16 nloop
 *     u8 rep[k]        representative label of the group of coincident planes (0xFF: zero plane)
 *     u8 vlab[nv][3]   sorted labels of the planes that define each vertex
 *     face[nf]         u8 supporting plane, u8 flags (bit 0: on the tet boundary),
 *                      u16 positive cell, u16 negative cell (0xFFFF: none), u16 loop length
 *     u16 loops[nloop] vertex ids, each loop starting at its smallest id, counter-clockwise seen
 *                      from the positive side
 *     u64 cells[nc]    sign vector of each cell (bit 4+j set on the positive side of plane 4+j)
 *   material interface:
 *     u8 type=2, u8 k, u16 nv, u16 nf, u16 nc, u16 nloop
 *     u8 rep[k]        representative label of the group of identical materials
 *     u8 vlab[nv][4]   sorted labels
 *     face[nf]         u8 positive label, u8 negative label, u16 loop length
 *     u16 loops[nloop]
 *     u8 cells[nc]     material label of each cell
 * Vertices are sorted by label, faces by (supporting plane, sorted vertex ids) or by
 * (positive, negative) label, cells by sign vector or label. */
typedef enum ria_mesh_field {
    RIA_MESH_POINTS = 0,          /* double [n_verts][3] */
    RIA_MESH_VERTS = 1,           /* int64 [n_verts][11]: tet_index, tet_vert_index, simplex_size,
                                     simplex_vert_indices[4], func_indices[4] (IA: 3 used;
                                     MI: material_indices) */
    RIA_MESH_FACE_OFFSETS = 2,    /* int64 [n_faces + 1] */
    RIA_MESH_FACE_VERTS = 3,      /* int64 [...] */
    RIA_MESH_FACE_TET_OFFSETS = 4,/* int64 [n_faces + 1] */
    RIA_MESH_FACE_TETS = 5,       /* int64 [...][2]: (tet, local face) */
    RIA_MESH_FACE_FUNC = 6,       /* int64 [n_faces][2]: func_index (first, second) */
    RIA_MESH_FUNC_IN_TET = 7,     /* int64 [...]: active functions per tet, ascending (CRS) */
    RIA_MESH_START_INDEX = 8,     /* int64 [n_tets + 1] */
    RIA_MESH_REC_OFFSETS = 9,     /* int64 [n_tets + 1] byte offsets into RIA_MESH_REC_BYTES */
    RIA_MESH_REC_BYTES = 10,      /* uint8 [...] */
    RIA_MESH_STATS = 11,          /* int64 [RIA_NUM_STATS] */
    RIA_MESH_TIMINGS = 12,        /* double [RIA_NUM_TIMINGS]: seconds of each device stage */
    RIA_MESH_FUNC_VALS = 13,      /* double [n_pts][n_func]: the values the mesh was computed from (device
                                     entry points: read from the caller's buffer, which must still exist) */
    /* Local-to-global maps, the outputs of the reference's extraction variants used when
     * useTopoRayShooting is off (src/extract_mesh.cpp:268-566 and 988-1443, called at
     * src/implicit_arrangement.cpp:370-385).  Computed on the device on first request; not available
     * for a batch mesh.  Local vertex and face ids are those of the per-tet records (RIA_MESH_REC_*). */
    RIA_MESH_TET_VERT_OFFSETS = 14,/* int64 [n_tets + 1] (global_vId_start_index_of_tet) */
    RIA_MESH_TET_VERTS = 15,      /* int64 [...] per record vertex: its mesh vertex, or -v-1 for tet vertex v
                                     (a record vertex on a tet corner; global_vId_of_tet_vert) */
    RIA_MESH_TET_FACE_OFFSETS = 16,/* int64 [n_tets + 1] (iso_fId_start_index_of_tet / MI_fId_...) */
    RIA_MESH_TET_FACES = 17,      /* int64 [...] per record face: its mesh face, or -1 (iso_fId_of_tet_face /
                                     MI_fId_of_tet_face: an interface face on the tet boundary is set in both
                                     tets that share it) */
    /* Mesh connectivity, the host stages that follow extraction in the reference
     * (src/mesh_connectivity.cpp:10-242, called at src/implicit_arrangement.cpp:410-440), computed on the
     * device on first request with the reference's numbering; not available for a batch mesh. */
    RIA_MESH_EDGES = 18,          /* int64 [n_edges][2]: v1 < v2, numbered by first occurrence in face order
                                     (compute_mesh_edges) */
    RIA_MESH_EDGE_FACE_OFFSETS = 19,/* int64 [n_edges + 1] */
    RIA_MESH_EDGE_FACES = 20,     /* int64 [...][2]: (face, local edge) occurrences (Edge::face_edge_indices) */
    RIA_MESH_FACE_EDGES = 21,     /* int64 [n_face_verts]: the edge of each face corner (edges_of_face; offsets
                                     are RIA_MESH_FACE_OFFSETS) */
    RIA_MESH_PATCH_OFFSETS = 22,  /* int64 [n_patches + 1] (compute_patches) */
    RIA_MESH_PATCH_FACES = 23,    /* int64 [n_faces]: each patch's faces in the reference's breadth-first order */
    RIA_MESH_PATCH_LABELS = 24,   /* int64 [n_patches][2]: func_index of each patch's first face (IA: first only) */
    RIA_MESH_CHAIN_OFFSETS = 25,  /* int64 [n_chains + 1] (compute_chains) */
    RIA_MESH_CHAIN_EDGES = 26     /* int64 [...]: non-manifold edges of each chain, in breadth-first order */
} ria_mesh_field;

/* RIA_MESH_STATS entries, named as in the reference's stats.json
 * (src/implicit_arrangement.cpp:46-49,80,119,322-327,390-393; src/material_interface.cpp) */
enum {
    RIA_STAT_NUM_PTS = 0,
    RIA_STAT_NUM_TETS = 1,
    RIA_STAT_NUM_DEGENERATE_VERTEX = 2,
    RIA_STAT_NUM_INTERSECTING_TET = 3,
    RIA_STAT_NUM_A_FUNC = 4,     /* IA: num_1_func; MI: num_2_func */
    RIA_STAT_NUM_B_FUNC = 5,     /* IA: num_2_func; MI: num_3_func */
    RIA_STAT_NUM_MORE_FUNC = 6,
    RIA_STAT_NUM_VERTS = 7,      /* num_iso_verts / num_MI_verts */
    RIA_STAT_NUM_FACES = 8,      /* num_iso_faces / num_MI_faces */
    RIA_STAT_NUM_DEFERRED = 9,   /* tets cut by the exact (slow) variant */
    RIA_STAT_ROBUST_FAILURES = 10,/* robust_test, type 1: tets cut in both plane orders whose vertex, face
                                     or cell counts differ ("inconsistency") */
    RIA_STAT_ROBUST_TYPE2 = 11,  /* robust_test, type 2: tets whose cut fails in the given order */
    RIA_STAT_ROBUST_TYPE3 = 12,  /* robust_test, type 3: tets whose cut succeeds in the given order and
                                     fails in the reversed order */
    RIA_NUM_STATS = 13
};
enum {
    RIA_TIME_SAMPLE = 0,   /* stage a (grid entry points) or upload */
    RIA_TIME_FILTER = 1,   /* stage b */
    RIA_TIME_CUT = 2,      /* stage c */
    RIA_TIME_EXTRACT = 3,  /* stage d: dedup, faces, vertex xyz */
    RIA_TIME_TOTAL = 4,
    RIA_NUM_TIMINGS = 5
};

/* ---- whole-grid entry points (host buffers) --------------------------------------------------
 * pts: n_pts x 3 doubles; tets: n_tets x 4 vertex ids; func_vals: n_pts x n_func, row major
 * (the reference's Eigen RowMajor funcVals).  n_func <= 64. */
RIA_API ria_status ria_compute_implicit_arrangement(const ria_config* cfg, const double* pts, uint64_t n_pts,
                                            const int64_t* tets, uint64_t n_tets, const double* func_vals,
                                            uint32_t n_func, ria_mesh** out);
RIA_API ria_status ria_compute_material_interface(const ria_config* cfg, const double* pts, uint64_t n_pts,
                                          const int64_t* tets, uint64_t n_tets, const double* func_vals,
                                          uint32_t n_func, ria_mesh** out);

/* Same inputs already resident on the current device; work is queued on `stream`
 * (a cudaStream_t, NULL for the default stream) and the call returns when the mesh is ready. */
RIA_API ria_status ria_compute_implicit_arrangement_device(const ria_config* cfg, const double* d_pts, uint64_t n_pts,
                                                   const int64_t* d_tets, uint64_t n_tets,
                                                   const double* d_func_vals, uint32_t n_func, void* stream,
                                                   ria_mesh** out);
RIA_API ria_status ria_compute_material_interface_device(const ria_config* cfg, const double* d_pts, uint64_t n_pts,
                                                 const int64_t* d_tets, uint64_t n_tets,
                                                 const double* d_func_vals, uint32_t n_func, void* stream,
                                                 ria_mesh** out);

/* tet5 grid of `resolution` cubes per axis over [bbox_min, bbox_max] (src/io.cpp:95-152), with the
 * functions sampled on the device (stage a).  The mesh keeps the sampled values
 * (RIA_MESH_FUNC_VALS). */
RIA_API ria_status ria_grid_implicit_arrangement(const ria_config* cfg, uint32_t resolution, const double* bbox_min,
                                         const double* bbox_max, const ria_function* funcs, uint32_t n_func,
                                         ria_mesh** out);
RIA_API ria_status ria_grid_material_interface(const ria_config* cfg, uint32_t resolution, const double* bbox_min,
                                       const double* bbox_max, const ria_function* funcs, uint32_t n_func,
                                       ria_mesh** out);

/* ---- batched grids -------------------------------------------------------------------------------
 * Many independent grid problems in one pass of every stage.  The problems' grids are concatenated
 * (vertices and tets numbered problem after problem), the general-case tets of all problems are cut
 * together in bins of equal active-function count, and the mesh numbering stays per problem: each
 * problem's fields, read with ria_batch_copy, equal those of its own ria_grid_* call.  No counterpart
 * in the reference, which solves one grid per call.  Limits: 2^31 points and tets in total. */
typedef struct ria_grid_problem {
    uint32_t resolution;        /* cubes per axis, 1..1200 */
    uint32_t n_func;            /* 1..64 */
    double bbox_min[3];
    double bbox_max[3];
    const ria_function* funcs;  /* host array of n_func */
} ria_grid_problem;

RIA_API ria_status ria_grid_batch(const ria_config* cfg, int32_t material_interface, const ria_grid_problem* problems,
                                  uint32_t n_problems, ria_mesh** out);
/* Number of problems of a batch mesh (0 for a mesh of any other entry point). */
RIA_API uint32_t ria_batch_size(const ria_mesh* mesh);
/* One problem's part of a field, with vertex, tet, mesh-vertex and offset values relative to the
 * problem.  RIA_MESH_STATS are the problem's own counts (RIA_STAT_NUM_DEFERRED and the
 * RIA_STAT_ROBUST_* counts are 0); RIA_MESH_TIMINGS are the batch's. */
RIA_API uint64_t ria_batch_count(const ria_mesh* mesh, uint32_t problem, ria_mesh_field field);
RIA_API ria_status ria_batch_copy(const ria_mesh* mesh, uint32_t problem, ria_mesh_field field, void* host_dst);

/* ---- CSG pruning (src/csg.cpp:55-116; replaces the lambda on cell labels) ----------------------------
 * For each face of an implicit-arrangement mesh: 0 if the CSG shape is on both sides or on neither,
 * 1 if its inside is on the positive side of the face's function (func_index.first), 2 if on the
 * negative side.  tree: n_units units of three int32 {op, a, b} as the reference's CSG tree files
 * (app/csg.cpp:15-52): op 0 Intersection, 1 Union, 2 Negation (b unused); an element e > 0 is unit e
 * (1-based), e < 0 is function -e-1; unit 1 is the root.  n_units = 0: the union of all functions
 * (the reference's default lambda).  Function j is inside where it is positive (positive_inside != 0)
 * or negative.  The reference instead negates every function when positive_inside is false, which
 * also reverses the faces' positive sides.  face_labels: host array of n_faces bytes (for a batch,
 * of the problem's faces).  Meshes from the *_device entry points read the caller's tets and values,
 * which must still exist. */
RIA_API ria_status ria_mesh_csg(const ria_mesh* mesh, const int32_t* tree, uint32_t n_units, int32_t positive_inside,
                                uint8_t* face_labels);
RIA_API ria_status ria_batch_csg(const ria_mesh* mesh, uint32_t problem, const int32_t* tree, uint32_t n_units,
                                 int32_t positive_inside, uint8_t* face_labels);
/* For an arbitrary membership function (the reference's std::function lambda over cell labels): the
 * sign vectors of the two sides of each face, sides[2f] on the positive and sides[2f+1] on the
 * negative side of the face's function (bit j set where function j is positive; n_func <= 64). */
RIA_API ria_status ria_mesh_face_sides(const ria_mesh* mesh, uint64_t* sides);

/* ---- served form ----------------------------------------------------------------------------------
 * A request loop for arrangement, material-interface and CSG solves.  Requests are admitted against
 * an HBM budget as they arrive; each of `streams` worker threads takes the oldest waiting request and
 * every other waiting request of the same class (material interface, or arrangement and CSG) that
 * fits the remaining budget, and solves them as one batch (ria_grid_batch) on its own stream, so
 * batches overlap on the device.  A request's result is its problem of that batch mesh, resident on
 * the device until ria_server_release; its budget share is returned when the last request of the
 * batch is released.  Results equal those of the plain calls on the same inputs.  No counterpart in
 * the reference. */
enum { RIA_REQ_IA = 0, RIA_REQ_MI = 1, RIA_REQ_CSG = 2 };
typedef struct ria_request {
    int32_t kind;              /* RIA_REQ_* */
    ria_grid_problem grid;     /* copied at submission */
    const int32_t* csg_tree;   /* CSG: n_units x 3 as ria_mesh_csg (copied); NULL: union of all */
    uint32_t csg_units;
    int32_t positive_inside;
} ria_request;
typedef struct ria_server ria_server;

RIA_API ria_status ria_server_create(const ria_config* cfg, uint64_t hbm_budget_bytes, uint32_t streams,
                                     uint32_t max_batch, ria_server** out);
RIA_API ria_status ria_server_submit(ria_server* server, const ria_request* request, uint64_t* ticket);
/* Waits up to timeout_s seconds (< 0: no limit; RIA_ETIMEOUT when it runs out) for a request; gives the
 * batch mesh holding its result (read with ria_batch_count / ria_batch_copy at `problem`) and the
 * time from submission to completion. */
RIA_API ria_status ria_server_wait(ria_server* server, uint64_t ticket, double timeout_s, const ria_mesh** mesh,
                                   uint32_t* problem, double* latency_s);
/* CSG requests: the face labels of ria_mesh_csg (host_dst may be NULL to ask for the count). */
RIA_API uint64_t ria_server_labels(ria_server* server, uint64_t ticket, uint8_t* host_dst);
RIA_API void ria_server_release(ria_server* server, uint64_t ticket);
/* Stops the workers after their current batch and frees every result.  Requests not yet started are
 * dropped.  No other thread may be inside a ria_server_* call on this server while it is destroyed. */
RIA_API void ria_server_destroy(ria_server* server);

/* ---- tuning of the per-tet cut ---------------------------------------------------------------------
 * The routing and launch shapes of stage c, per device.  The general-case tets come from the filter in
 * bins of equal active-function count, heaviest first; the heavy bins and the light bins' leftovers are
 * cut a warp per tet up to warp_route tets, the rest a thread per tet.  No counterpart in the
 * reference (its cut is serial). */
typedef struct ria_tuning {
    int64_t warp_route;         /* general-case tets cut a warp each (the bin of the warp kernel) */
    int32_t warp_blocks_per_sm; /* resident blocks of the warp kernel per SM (0: its occupancy limit) */
    int32_t fast_block;         /* threads per block of the thread-per-tet kernel: 32, 64 or 128 (0: chosen
                                   from the tet count) */
    int64_t mid_threshold;      /* deferred tets above which the mid-size variant runs before the exact one */
    int32_t cut_graph;          /* capture stage c's launches (both streams) as one CUDA graph: 0 never,
                                   1 batched grids (the default), 2 every call */
    int32_t heavy_min_k;        /* implicit arrangement: smallest active-function count of the heavy bins,
                                   cut while the lookup pass runs on the light ones: 3 to 8 (0: 4; the
                                   default record: 6) */
    int32_t mi_heavy_min_k;     /* material interface: smallest active-material count of the heavy bins,
                                   whose materials' cells are clipped in parallel: 3 to 8 (0 and the
                                   default record: 4) */
} ria_tuning;
/* The current device's tuning record. */
RIA_API ria_status ria_get_tuning(ria_tuning* tuning);
RIA_API ria_status ria_set_tuning(const ria_tuning* tuning);
/* Project-written autotuner: runs ria_grid_batch on `problems` (a sample of the caller's batches),
 * `reps` times per candidate record with the secondary lookup reset to its seeded state, in a
 * coordinate descent over the fields (heavy_min_k or mi_heavy_min_k, the one of the mode tuned;
 * warp_route, warp_blocks_per_sm, fast_block, mid_threshold, cut_graph; two sweeps, each field over a
 * few values with the others at their best so far), and installs the record with the smallest median device time on the current device.  The
 * result never depends on the record.  best_s / default_s (may be NULL): that time, and the time of
 * the record in place when the call started.  Not to be run while other calls use the device. */
RIA_API ria_status ria_autotune(const ria_config* cfg, int32_t material_interface, const ria_grid_problem* problems,
                                uint32_t n_problems, uint32_t reps, ria_tuning* best, double* best_s,
                                double* default_s);

/* Stage a alone: func_vals[n_pts][n_func] = funcs evaluated at pts (host buffers). */
RIA_API ria_status ria_sample_functions(const ria_function* funcs, uint32_t n_func, const double* pts, uint64_t n_pts,
                                double* func_vals);

/* ---- per-tet entry points (the simplicial_arrangement calls) ---------------------------------
 * values: for tet t, rows value_offsets[t] .. value_offsets[t+1]-1 of 4 corner values each
 * (a plane or a material).  records receives the canonical records back to back; record_offsets
 * (n_tets + 1 entries) their byte offsets.  Returns RIA_ECAPACITY if `capacity` is too small. */
RIA_API ria_status ria_compute_arrangement_batch(const double* values, const uint32_t* value_offsets, uint64_t n_tets,
                                         uint8_t* records, uint64_t capacity, uint64_t* record_offsets);
RIA_API ria_status ria_compute_material_interface_batch(const double* values, const uint32_t* value_offsets,
                                                uint64_t n_tets, uint8_t* records, uint64_t capacity,
                                                uint64_t* record_offsets);

/* Per-tet arrangements without any device allocation.  This entry point has no counterpart in the
 * reference; it serves callers that cannot allocate device memory: a caller whose device memory is
 * entirely held by its own allocator (a framework's caching allocator, an arena reserved at start-up)
 * or a caller in a latency-critical loop where cudaMalloc / cudaFree, which can synchronize the device,
 * are not allowed.  Inputs and outputs are the caller's device buffers (same meaning as
 * ria_compute_arrangement_batch; d_record_offsets has n_tets + 1 entries); work is queued on `stream`
 * and the call returns when it has finished.  Intermediate data lives in one fixed device array of
 * about 8.5 MB inside the library, held by every GPU that loads it until the process exits.
 * Limits: n_tets <= 4096 (RIA_EINVAL beyond) and at most 8 MiB of records per call (RIA_ECAPACITY
 * beyond).  The first call on a device looks up that array's address there; make
 * it before any stream capture.  Calls share the array: calls that overlap on the GPU race on it and
 * must be serialized by the caller. */
RIA_API ria_status ria_compute_arrangement_batch_noalloc(const double* d_values, const uint32_t* d_value_offsets,
                                                         uint64_t n_tets, uint8_t* d_records, uint64_t capacity,
                                                         uint64_t* d_record_offsets, void* stream);

/* ---- results ---------------------------------------------------------------------------------- */
RIA_API uint64_t ria_mesh_count(const ria_mesh* mesh, ria_mesh_field field); /* elements of the field */
RIA_API ria_status ria_mesh_copy(const ria_mesh* mesh, ria_mesh_field field, void* host_dst);
RIA_API void ria_mesh_free(ria_mesh* mesh);

/* Message of the last failing call on this thread. */
RIA_API const char* ria_last_error(void);
/* Diagnostics: number of kernels this library has launched in this process. */
RIA_API uint64_t ria_kernel_launches(void);
/* Resets the current device's secondary-lookup tables (two-plane and three-material records kept
 * by their combinatorial type; results never depend on them) to their seeded state: the records
 * computed once per process from synthetic configurations when the mode's table is built, like the
 * reference's precomputed tables.  Records added by later calls are dropped, so callers that must
 * not reuse work across calls (for example a benchmark timing single calls) reset them first.
 * Must not overlap with running calls on the device. */
RIA_API ria_status ria_lookup_cache_clear(void);
RIA_API int ria_device_count(void);
/* Diagnostics, no counterpart in the reference: FP64 operations per second on the current device,
 * measured with a probe kernel that keeps every SM's FP64 pipe busy (op 0: fused multiply-add, 1: add,
 * 2: multiply; each instruction counts as one operation, so the FP64 FLOP/s peak is twice the
 * multiply-add rate).  It is the denominator of the FP64 fractions of the sampling and cut stages. */
RIA_API ria_status ria_measure_fp64_rate(int32_t op, double* ops_per_s);

#ifdef __cplusplus
}
#endif
#endif /* RIA_H */
