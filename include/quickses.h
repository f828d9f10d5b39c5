/*
 * quickses_gb300 - GB300-native SES mesher, drop-in for QuickSES's library path.
 *
 * Two layers of entry points live in libquickses_gb300.so:
 *
 *  1. The QuickSES library surface, with the same symbol names, signatures and
 *     semantics as the reference (CudaSurf.h:75-83, CudaSurf.cu:778-873).  These are thin
 *     wrappers over a process-wide default context and are, like the reference, not
 *     reentrant.
 *  2. Reentrant qses_* calls: a context per caller thread/stream, explicit parameters
 *     (voxel size, smoothing passes, slice), status codes instead of exit(), and meshes
 *     owned by the caller until qses_mesh_release.
 *
 * All pointers are host pointers unless a name says "device".  No CUDA or torch types
 * appear in the signatures: qses_float3 has the layout of CUDA's float3 (3 packed floats).
 */
#ifndef QUICKSES_GB300_H
#define QUICKSES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef QSES_API
#define QSES_API
#endif

typedef struct { float x, y, z; } qses_float3;

#ifdef __cplusplus
#define QSES_BOOL bool
#else
#define QSES_BOOL _Bool
#endif

/* ------------------------------------------------------------------ status codes */
enum {
    QSES_OK = 0,
    QSES_ERR_INVALID_ARG = 1,   /* bad pointer / size / parameter */
    QSES_ERR_NO_DEVICE = 2,     /* no CUDA device, or not an sm_103 device */
    QSES_ERR_CUDA = 3,          /* a CUDA runtime call failed */
    QSES_ERR_OUT_OF_MEMORY = 4, /* device or pinned host allocation failed */
    QSES_ERR_UNSUPPORTED = 5,   /* input outside the supported envelope (see qses_status_string) */
    QSES_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up */
    QSES_ERR_INTERNAL = 7,      /* internal consistency check failed */
    QSES_ERR_CANCELLED = 8      /* a served request withdrawn before it ran (qses_server_cancel) */
};

/* --------------------------------------------- QuickSES-compatible library surface */

/* Replaces API_computeSES (CudaSurf.h:77-78, CudaSurf.cu:787-841).  Inputs are read
 * only.  out_vertices and out_triangles are ignored, as in the reference; *NVert is the
 * vertex count and *NTri the number of triangle INDICES (3 x kept triangles).  Results
 * stay in library-owned buffers reachable through API_get*.  Triangles with a repeated
 * vertex index are dropped.  doSmoothing = number of Laplacian passes.  N <= 1 gives an
 * empty mesh.  Unlike the reference, a failure does not exit(): counts are left at 0 and
 * qses_api_last_status() reports the code.  The mesh is the reference's output for one slice
 * covering the grid; with the environment variable QSES_REFERENCE_SLICES set to a slice size
 * (the reference's library uses 300) it is the reference's sliced output instead
 * (QSES_FLAG_REFERENCE_SLICES). */
QSES_API void API_computeSES(float resoSES, qses_float3 *atomPos, float *atomRad, unsigned int N,
                             qses_float3 *out_vertices, unsigned int *NVert, int *out_triangles,
                             unsigned int *NTri, int doSmoothing);
/* Replaces API_getTriangles (CudaSurf.h:79, CudaSurf.cu:845-857): when invertTriangles
 * is true the first two indices of every triangle are swapped in place (calling twice
 * toggles back).  C callers pass 0/1 in a single byte, as C++ bool. */
QSES_API int *API_getTriangles(QSES_BOOL invertTriangles);
/* Replaces API_getVertices (CudaSurf.h:80, CudaSurf.cu:858-861). */
QSES_API qses_float3 *API_getVertices(void);
/* Replaces API_freeMesh (CudaSurf.h:81, CudaSurf.cu:867-872). */
QSES_API void API_freeMesh(void);
/* Replaces API_getAtomIdPerVert (CudaSurf.h:82, CudaSurf.cu:862-865): index of the
 * closest atom in the cell-sorted atom order, as the reference returns it. */
QSES_API int *API_getAtomIdPerVert(void);

/* Exported data symbols of the reference library (CudaSurf.cu:778-785). */
extern QSES_API int NTriangles;
extern QSES_API int NVertices;
extern QSES_API int *globalTriangles;
extern QSES_API qses_float3 *globalVertices;
extern QSES_API int *globalIdAtomPerVert;

/* Status of the last API_computeSES call (no reference counterpart: the reference
 * exits the process on error, CudaSurf.h:54-62). */
QSES_API int qses_api_last_status(void);

/* ------------------------------------------------------------ reentrant interface */

typedef struct qses_context qses_context;

typedef struct {
    float voxel;        /* SES voxel size in A (CLI -v, default 0.5) */
    int smooth_passes;  /* Laplacian passes (CLI -l, default 1) */
    int slice;          /* CLI -s: slice size in voxels, default 300; used only with
                           QSES_FLAG_REFERENCE_SLICES (the reference's slicing) */
    int flags;          /* QSES_FLAG_* */
} qses_params;

#define QSES_FLAG_KEEP_DEGENERATE 1  /* keep triangles with a repeated index (CLI/OBJ path) */
/* The reference's slicing, for diffs against meshes QuickSES wrote (CudaSurf.cu:629-754,
 * the executable's -s): the grid is cut into cores of `slice` voxels, each computed in a
 * box reaching R voxels before it (refine windows clamped to the box, the box's last layer
 * outside), each slice's cells emitted by the reference's rules (two cell layers at every
 * seam from both sides), meshed, welded, given closest atoms and smoothed on its own; the
 * meshes are concatenated with vertex ids offset slice by slice, as API_computeSES does.
 * The reference never writes a slice's last triangle (MarchingCubes.cu:845 with
 * CudaSurf.cu:421) and leaves whatever the device memory held in its three vertices; here
 * that triangle and any vertex only it used are left out.  qses_compute only (host mesh);
 * device memory is bounded by one slice box, so grids of any size within 1290 neighbour
 * cells per axis are accepted.  Without this flag the result is the reference's output
 * for one slice covering the grid (slice >= grid size), whatever `slice` is. */
#define QSES_FLAG_REFERENCE_SLICES 2

typedef struct {
    unsigned n_vertices;
    unsigned n_triangles;      /* triangles (not indices) */
    qses_float3 *vertices;     /* smoothed welded vertices, lexicographic order of the
                                  quantised position */
    int *triangles;            /* 3 * n_triangles vertex indices */
    int *atom_sorted;          /* closest atom, index into the cell-sorted atom order */
    int *atom_input;           /* closest atom, index into the caller's atom array */
    int grid_dim;              /* SES grid voxels per axis */
    float origin[3];           /* grid origin (A) */
    void *_owner;              /* release with qses_mesh_release */
} qses_mesh;

/* Creates a context on CUDA device `device`; `cuda_stream` is a cudaStream_t to run on,
 * or NULL for a private non-blocking stream.  Fails with QSES_ERR_NO_DEVICE without a
 * usable sm_103 GPU. */
QSES_API int qses_context_create(int device, void *cuda_stream, qses_context **out);
QSES_API int qses_context_destroy(qses_context *ctx);
QSES_API void qses_params_default(qses_params *p);

/* Host atoms in, host mesh out (pinned, owned by *out until qses_mesh_release).  A grid too
 * large for one pass (more than 4096 voxels, or 2000 A, per axis) gets the reference's
 * sliced output for p->slice (QSES_FLAG_REFERENCE_SLICES), as the reference slices every
 * grid; qses_last_slices then reports its slices. */
QSES_API int qses_compute(qses_context *ctx, const qses_params *p, const qses_float3 *atoms,
                          const float *radii, unsigned n, qses_mesh *out);
QSES_API void qses_mesh_release(qses_mesh *m);
/* Per-slice vertex and triangle counts of the last qses_compute in the reference's slicing
 * mode (slices with a mesh, in the reference's order: x outermost); returns the number of
 * slices (at most `max` written), 0 after any other call. */
QSES_API int qses_last_slices(qses_context *ctx, unsigned *n_vertices, unsigned *n_triangles, int max);

/* Device-resident form: atoms already in device memory (3n floats, n floats); the mesh
 * stays on the device in the context's workspace (valid until the next call on `ctx`).
 * Counts are returned on the host. */
typedef struct {
    unsigned n_vertices, n_triangles;
    float *d_vertices;   /* 3 * n_vertices */
    int *d_triangles;    /* 3 * n_triangles */
    int *d_atom_sorted;
    int *d_atom_input;
} qses_device_mesh;
QSES_API int qses_compute_device(qses_context *ctx, const qses_params *p, const float *d_xyz,
                                 const float *d_radii, unsigned n, qses_device_mesh *out);

/* ------------------------------------------------------------------ batch form */

/* One SES request of a batch (no reference counterpart: QuickSES computes one molecule per
 * API_computeSES call).  atoms/radii are host arrays of n entries. */
typedef struct {
    const qses_float3 *atoms;
    const float *radii;
    unsigned n;
    float voxel;        /* SES voxel size in A */
    int smooth_passes;  /* Laplacian passes */
    int flags;          /* QSES_FLAG_* */
} qses_request;

/* Many molecules (or trajectory frames) of uneven size in one pass: every stage is one
 * launch over all of them (persistent field kernels pulling (molecule, tile) items from a
 * device work queue, one weld sort, one Gauss-Seidel dataflow), results copied into one
 * pinned block.  out[i] is exactly what qses_compute returns for request i alone; release
 * each with qses_mesh_release.  status[i] (optional) receives the request's status; a
 * request outside the supported envelope fails alone.  Requests are grouped internally by
 * smooth_passes and by weld-key width. */
QSES_API int qses_compute_batch(qses_context *ctx, const qses_request *reqs, unsigned count, qses_mesh *out,
                                int *status);

/* Pinned host memory kept for reuse by released meshes (default 16 GB): result buffers are
 * pinned for full-speed copies, and pinning is slow, so released blocks are cached. */
QSES_API void qses_set_pinned_cache(unsigned long long bytes);

/* ------------------------------------------------------------------ autotuner */

/* Picks the smoothing launch shape (threads per slab CTA, slab size aimed at) for meshes of
 * this size, and the refine tile shape for grids of this size, by running the molecule once
 * per candidate shape (`repeats` times each) and keeping the fastest; later calls of this process on meshes of the same size class (log2
 * of the vertex count) use it.  The mesh is identical for every shape: the update order is
 * fixed by the vertex ids.  No reference counterpart (QuickSES hard-codes its launches). */
QSES_API int qses_autotune(qses_context *ctx, const qses_params *p, const qses_float3 *atoms, const float *radii,
                           unsigned n, int repeats, int *threads_out, unsigned *target_out, unsigned *flags_out,
                           int *field_shape_out, float *smooth_ms_out);
/* Fixes the refine tile shape of ctx: 0 = 8 x 8 z-rows per CTA, 1 = 16 x 8, 2 = 16 x 16,
 * 3 = 32 x 16 (less halo per row, more shared memory); -1 returns to the tuned/default
 * shape.  Same codes for all. */
QSES_API int qses_set_field_shape(qses_context *ctx, int shape);
/* Fixes the smoothing launch shape of ctx: threads 512 or 1024 per slab CTA, slab size
 * aimed at (>= 256 vertices), cache_flags bit 0 = prefetch successors' neighbour lists into
 * L1 instead of L2, bit 1 = neighbour positions through L1, bit 2 = keep the positions in
 * persisting L2 lines during the pass (a window on the context's stream, cleared after it),
 * bit 3 = each slab's own positions in shared memory (slabs of at most 8192 vertices),
 * bit 4 = two vertex updates per worker warp (16 lanes each), bit 5 = four (8 lanes each;
 * not with bit 4); wave_vertices = most vertices per slab-kernel launch (0 = the whole mesh in one launch;
 * otherwise sequential waves); threads = 0 returns to the tuned/default shape.
 * Every shape gives the same mesh. */
QSES_API int qses_set_smoothing_shape(qses_context *ctx, int threads, unsigned target, unsigned cache_flags,
                                      unsigned wave_vertices);
/* Sets the process-wide smoothing shape (as qses_set_smoothing_shape, no waves) for every
 * mesh size, of single-molecule calls (batch = 0) or of batch calls and server lanes
 * (batch = 1), replacing what the autotuner recorded; contexts with a fixed shape keep it.
 * No reference counterpart.  Lets a server use a shape that shares the SMs between lanes. */
QSES_API int qses_set_default_smoothing_shape(int batch, int threads, unsigned target, unsigned cache_flags);
/* The same for the batch form, timing whole qses_compute_batch calls on `reqs`. */
QSES_API int qses_autotune_batch(qses_context *ctx, const qses_request *reqs, unsigned count, int repeats,
                                 int *threads_out, unsigned *target_out, unsigned *flags_out, float *ms_out);

/* ---------------------------------------------------------------- served form */

/* A request loop with continuous batching (no reference counterpart).  `lanes` worker
 * threads each own a context (stream + persistent workspace); a free lane takes every
 * queued request that fits its share of memory_budget (FIFO, at most max_batch) and runs
 * them as one qses_compute_batch, so requests that arrive while others run are batched as
 * lanes free up and batches overlap on the device.  Results equal qses_compute's. */
typedef struct qses_server qses_server;
typedef struct {
    int device;
    int lanes;                         /* batches in flight (default 2) */
    unsigned long long memory_budget;  /* device bytes for admitted work (default 120 GB) */
    unsigned max_batch;                /* requests per batch (default 256) */
    unsigned long long max_batch_voxels; /* grid voxels per batch, summed (default 1e9; 0 = no
                                            limit): bounds a batch's run time, so lanes take
                                            turns and late arrivals wait less */
} qses_server_config;
typedef struct {
    double queued_s;  /* submit -> start of its batch */
    double run_s;     /* its batch's run, mesh download included */
    double total_s;   /* submit -> result ready */
} qses_ticket_info;
QSES_API void qses_server_config_default(qses_server_config *c);
QSES_API int qses_server_create(const qses_server_config *cfg, qses_server **out);
/* Copies the request's atoms; returns QSES_ERR_UNSUPPORTED / QSES_ERR_OUT_OF_MEMORY at once
 * for requests that can never run (grid envelope, estimated size above the budget). */
QSES_API int qses_server_submit(qses_server *s, const qses_request *req, unsigned long long *ticket);
/* Blocks until the ticket's mesh is ready (timeout_s < 0: forever; on QSES_ERR_TIMEOUT the
 * ticket stays valid).  Returns the request's status; *out is then the caller's (release
 * with qses_mesh_release) and the ticket is consumed.  One waiter per ticket: a wait on a
 * ticket another thread is already waiting for returns QSES_ERR_INVALID_ARG.  Waits and
 * submits may come from any threads at the same time. */
QSES_API int qses_server_wait(qses_server *s, unsigned long long ticket, double timeout_s, qses_mesh *out,
                              qses_ticket_info *info);
/* [0] batches run, [1] requests served, [2] largest batch, [3] most lanes busy at once,
 * [4] requests queued now.  Returns the number of values written. */
QSES_API int qses_server_stats(qses_server *s, unsigned long long *out, int max);
/* Withdraws a request that is still queued: QSES_OK, and its qses_server_wait returns
 * QSES_ERR_CANCELLED with an empty mesh.  A request already taken into a batch runs to the
 * end: QSES_ERR_UNSUPPORTED.  An unknown or collected ticket: QSES_ERR_INVALID_ARG. */
QSES_API int qses_server_cancel(qses_server *s, unsigned long long ticket);
/* Finishes queued work, then frees everything (uncollected meshes included). */
QSES_API int qses_server_destroy(qses_server *s);

QSES_API const char *qses_status_string(int status);
QSES_API const char *qses_last_error(qses_context *ctx);

/* Per-stage device times (ms, CUDA events on the context stream) of the last call when
 * profiling is on.  Returns the number of stages written. */
QSES_API int qses_set_profiling(qses_context *ctx, int on);
QSES_API int qses_stage_times(qses_context *ctx, float *ms, const char **names, int max);
/* Number of kernels the last call launched. */
QSES_API int qses_last_launch_count(qses_context *ctx);
/* Device-to-host bytes the last qses_compute copied (the triangle download is sized by the
 * pre-filter count so it can start while the smoothing pass runs). */
QSES_API unsigned long long qses_last_download_bytes(qses_context *ctx);
/* Smoothing diagnostics of the last call: [0] slabs, [1] vertices per slab, [2] most
 * boundary polls of one slab, [3] slabs that did not finish, [4] clock cycles spent in
 * vertex updates, [5] in releasing successors, [6] vertices updated, [7] cycles until a
 * vertex's neighbour ids arrived, [8] then until their positions arrived, [9] in the
 * position store and its fence (summed over warps); [2]-[9] are counted on calls
 * made with profiling on (qses_set_profiling) and are 0 otherwise.  Returns the number of
 * values written. */
QSES_API int qses_diagnostics(qses_context *ctx, unsigned long long *out, int max);

/* Host timeline of the last pipeline run on ctx (ms; for a batch call, its last batch):
 * [0] host work before the first launch, [1] field segment from launch to its read-back,
 * [2] host work between, [3] mesh segment, [4] host work between, [5] finish segment
 * (closest atom, filter, smoothing, downloads).  No reference counterpart.  Returns the
 * number of values written. */
QSES_API int qses_host_timeline(qses_context *ctx, double *ms, int max);

/* ------------------------------------------------------------- failure tests */

/* Test hooks (no reference counterpart; QuickSES exits the process on any error).
 * qses_debug_fail_reservations: the next n device workspace reservations of any context fail
 * with QSES_ERR_OUT_OF_MEMORY, as an exhausted device would; the failing call returns that
 * code and later calls on the same context work.
 * qses_debug_wait_limit: runs the smoothing kernel on a 4-vertex mesh in which one vertex
 * waits for a hand-off from a lower slab that never comes, with its wait limited to
 * spin_cycles clock cycles (1e6 .. 4e9); *kernel_status receives the status the kernel wrote
 * (QSES_ERR_TIMEOUT: the wait gave up and every CTA returned).  Returns QSES_OK when the
 * kernel ran and the context is still usable. */
QSES_API void qses_debug_fail_reservations(unsigned n);
QSES_API int qses_debug_wait_limit(qses_context *ctx, long long spin_cycles, int *kernel_status);

/* ------------------------------------------------------------------ CUDA graphs */

/* No reference counterpart (QuickSES launches every kernel from the host, slice by slice).
 * A call runs as three segments between its host read-backs of counts (field, mesh, finish),
 * each replayed from a CUDA graph kept in ctx: launched as is when the segment's pointers,
 * counts, grid and launch shapes repeat the previous call's, captured again and updated in
 * place otherwise.  Results are identical either way.  Segments are captured on a private
 * stream of the context and launched on the context's stream (its own or the caller's).  On
 * by default; with stage timing on, or enable = 0, every kernel is launched directly. */
QSES_API int qses_set_graphs(qses_context *ctx, int enable);
/* out[0] captures, [1] instantiations, [2] in-place updates, [3] replays, counted since the
 * context was created.  Returns the number of values written. */
QSES_API int qses_graph_stats(qses_context *ctx, unsigned long long *out, int max);

/* ------------------------------------------------------- allocation-free field */

/* No counterpart in the reference.  For callers that must not allocate GPU memory while
 * they run (plugins whose host application owns every device allocation, real-time loops
 * that cannot afford cudaMalloc's implicit synchronisation, fixed memory budgets).
 * Computes the SES voxel codes of one molecule - the same bytes qses_debug_codes returns
 * after qses_compute - from device atoms (3n floats) and radii (n floats) into the caller's
 * device buffer d_codes (G*G*G bytes, x-major, z fastest; G from qses_grid_info_for), on
 * `cuda_stream` (NULL = legacy default stream).  Allocates nothing: its working memory is a
 * fixed ~3.5 MB array inside the library, reserved on every GPU that loads the library
 * until the process exits.  Limits: 2 <= n <= 4096 atoms, grid <= 128 voxels and <= 40
 * neighbour cells per axis, all returning QSES_ERR_UNSUPPORTED.  The atom count is checked
 * before any GPU work; the grid limits need the atoms' bounds, so they are checked after a
 * bounds pass on the stream, which the call waits for.  The first call on a device (and the
 * first after the device's context was replaced, e.g. by cudaDeviceReset) looks up the
 * array's device address: make it before any stream capture.  All calls share the array:
 * the function serialises host threads and, on success and on every error, waits for its
 * own GPU work before returning; work that overlapped it on the GPU would race on it. */
QSES_API int qses_field_codes_noalloc(const float *d_xyz, const float *d_radii, unsigned n, float voxel,
                                      uint8_t *d_codes, size_t codes_bytes, void *cuda_stream);

/* ---------------------------------------------------------- file front-end (CLI) */

/* PDB ATOM records -> atom centres (3n floats) and radii (n floats), malloc'd; free both
 * with qses_free.  Replaces the QuickSES executable's reading path: parsePDB
 * (cpdb/cpdb.cpp:35-158) plus the per-atom radius lookup (CudaSurf.cu:942-964,
 * CudaSurf.h:64-73): ATOM records only, stop at the first line starting with END, altLoc
 * 'A' or ' ' only, hydrogens kept, radius from the first byte of the element field.
 * Returns QSES_ERR_INVALID_ARG when the file cannot be opened (the reference exits(2)). */
QSES_API int qses_read_pdb(const char *path, float **xyz, float **radii, unsigned *n);
QSES_API void qses_free(void *p);
/* Writes an OBJ file byte-identical to QuickSES's writeToObj (CudaSurf.cu:329-371) for one
 * mesh: "v %.3f %.3f %.3f" lines, a blank line, "f b a c" lines (1-based, first two corners
 * swapped).  threads <= 0 picks the host's thread count. */
QSES_API int qses_write_obj(const char *path, const qses_float3 *vertices, unsigned nv, const int *triangles,
                            unsigned nt, int threads);
/* "%.3f" of one float, as qses_write_obj formats it; returns the length or -1. */
QSES_API int qses_format_fixed3(float v, char *out, int cap);

/* --------------------------------------------------- inspection (tests, tooling) */

typedef struct {
    float origin[3], cell, dx, probe, max_radius, max_dist;
    int gnb, G, R, Gc, W;
} qses_grid_info;

/* Grid sizing exactly as the reference computes it (CudaSurf.cu:149-174, 250-253,
 * 546-574, 629-635); host-only. */
QSES_API int qses_grid_info_for(const qses_float3 *atoms, const float *radii, unsigned n, float voxel,
                                qses_grid_info *out);
/* Voxel codes of the last qses_compute on ctx (G*G*G bytes, x-major, z fastest): n<=3R^2 =
 * squared voxel distance to the nearest outside voxel, 253 none in window, 254 inside,
 * 255 outside. */
QSES_API int qses_debug_codes(qses_context *ctx, uint8_t *codes, size_t bytes);
/* Cell-sorted atom order of the last call: sorted_to_input[n], cell hash per sorted atom. */
QSES_API int qses_debug_atom_order(qses_context *ctx, uint32_t *sorted_to_input, uint32_t *hash, unsigned n);
/* Slab plan of the smoothing pass, for tests (no reference counterpart, no GPU needed): nv
 * vertices, molecules' vertex ranges mol_off (nm + 1 entries; NULL = one molecule) and
 * depth estimates, smoothing shape (threads, target, cache_flags, wave as
 * qses_set_smoothing_shape) and
 * pmax resident slab CTAs.  launch[0..5] = ctas, smax, qcap, wsize, waves, words per wave;
 * table (cap words): the waves' slab tables [Q, Q + 1 bounds (qcap + 1 slots), Q slab ids in
 * the order CTAs take them].  Returns QSES_OK or an error code. */
QSES_API int qses_debug_slab_plan(unsigned nv, const unsigned *mol_off, const int *depth, unsigned nm, int threads,
                                  unsigned target, unsigned cache_flags, unsigned wave, int pmax, unsigned *launch,
                                  unsigned *table, size_t cap);

/* --------------------------------------------------------- synthetic molecules */
QSES_API int qses_synth_ball(unsigned N, uint64_t seed, float density, float min_dist, float *xyz,
                             float *rad, unsigned char *elem);
QSES_API int qses_synth_shell(unsigned N, uint64_t seed, float r_in, float thickness, float min_dist,
                              float *xyz, float *rad, unsigned char *elem);
QSES_API int qses_synth_jitter(const float *base_xyz, unsigned N, float sigma, uint64_t seed, float *out_xyz);

#ifdef __cplusplus
}
#endif
#endif /* QUICKSES_GB300_H */
