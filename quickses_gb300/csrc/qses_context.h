// Context state shared by the pipeline and the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <string>
#include <utility>
#include <vector>

#include "kernels.h"
#include "qses_internal.h"

namespace qses {

// Test hook (qses_debug_fail_reservations): reservations left to fail.
extern std::atomic<unsigned> g_fail_reserves;

// Bump allocator over one device allocation that persists across calls.
struct Arena {
    void *base = nullptr;
    size_t cap = 0, off = 0;
    unsigned long long gen = 0;  // bumped whenever the allocation is freed (or replaced)
    int reserve(size_t bytes);  // resets the bump pointer; grows (and invalidates) if needed
    void *take(size_t bytes);   // 256-byte aligned; null when out of room
    void release();
};

// Device-resident result of the last call (pointers into the context arenas).
struct DeviceMesh {
    bool valid = false;
    unsigned nv = 0, nt = 0, n_tri_all = 0, n_edges = 0, n_atoms = 0;
    float *vertices = nullptr;
    unsigned *triangles = nullptr;
    int *atom_sorted = nullptr, *atom_input = nullptr;
    unsigned char *codes = nullptr;
    unsigned *sorted_to_input = nullptr, *sorted_keys = nullptr;
};

// sliced: the grid of the reference's slicing mode, held one slice box at a time (no
// whole-grid size or weld-key extent limit).
int grid_from_bounds(const float mn[3], const float mx[3], float maxR, unsigned n, float dx, QGrid &g,
                     qses_grid_info *info, std::string *why, bool sliced = false);
void fill_lut(const QGrid &g, float *lut);

// One molecule of a batch call: host atoms and its grid, sized on the host.
struct BatchItem {
    const float *xyz = nullptr;  // 3n floats
    const float *r = nullptr;    // n floats
    unsigned n = 0;
    unsigned flags = 0;
    QGrid g;
};

// Device-resident result of the last batch (pointers into the context arenas) and the
// per-molecule ranges of its concatenated arrays.
struct BatchResult {
    unsigned n_mol = 0, nv = 0, nkept = 0;
    std::vector<unsigned> vtx_off, kept_off;  // n_mol + 1 entries
    float *vertices = nullptr;
    unsigned *triangles = nullptr;            // kept triangles, molecule-local vertex ids
    int *atom_sorted = nullptr, *atom_input = nullptr;
};

}  // namespace qses

namespace qses {
// Pinned host blocks from the process-wide cache (released blocks are reused).
void *pinned_take(size_t bytes, size_t *got);
void pinned_give(void *p, size_t bytes);
// Count of pinned blocks the cache has freed so far (any context's).
unsigned long long pinned_frees();

// Host destination of a qses_compute call, filled by the pipeline while the smoothing pass
// still runs: [vertices 12 nv | triangles 12 T (upper bound) | atom_sorted 4 nv | atom_input 4 nv].
struct HostDownload {
    bool want = false;
    void *block = nullptr;
    size_t bytes = 0, vb = 0, tb = 0, ab = 0;
    unsigned long long d2h = 0;  // bytes copied
};

// Host values a pipeline segment produces besides its stream work (kept with its graph).
struct SegOut {
    int launches = 0;             // kernels the segment launches
    int alt = 0;                  // which ping-pong pair holds a sort's result
};

// Launch shape of a Gauss-Seidel pass: sequential waves of wsize vertices, each a table of
// contiguous slabs (at most smax vertices, at most qcap slabs) taken by `ctas` persistent
// CTAs.  A function of the vertex count, the molecule count and the GsShape only.
struct GsLaunch {
    int ctas;
    unsigned smax, qcap, wsize, waves;
    unsigned table_words;  // per wave
};
// The plan: launch shape plus the slab tables (host words, waves x table_words), which
// follow the molecules' vertex ranges.
struct GsPlan {
    GsLaunch L;
    unsigned max_slabs = 0, max_len = 0;  // diagnostics
    std::vector<unsigned> table;
};

// One cached segment graph: its executable, the key bytes it was captured from, the host
// values the capture produced and when it was last used.
struct GraphSeg {
    cudaGraphExec_t exec = nullptr;
    std::vector<unsigned char> key;
    SegOut out;
    unsigned long long used = 0;
    unsigned long long mem = 0;  // the context's memory generation when it was captured
};
// Graphs kept per segment slot (a batch call split by smoothing passes alternates shapes).
constexpr int kSegCache = 4;
// Graph slots: per-molecule field / mesh / finish, then the batch's.
enum { kSegField = 0, kSegMesh, kSegFinish, kSegBatchField, kSegBatchMesh, kSegBatchFinish, kSegSlots };
}  // namespace qses

struct qses_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaStream_t side = nullptr;          // closest atom, filter and downloads beside the smoothing
    cudaStream_t capture = nullptr;       // private stream that pipeline segments are captured on
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    qses::HostDownload dl;
    qses::Arena input, field, mesh_ws, gs_ws;
    unsigned *h_gs = nullptr;         // pinned slab tables of the smoothing launches (grows)
    size_t h_gs_cap = 0;
    void *small = nullptr;            // 4 KB device scratch: bounds, error word, queue counters
    unsigned char *h_small = nullptr; // 4 KB pinned host scratch
    QGrid grid;
    qses_grid_info info;
    bool have_grid = false;
    qses::DeviceMesh mesh;
    qses::BatchResult batch;
    void *h_stage = nullptr;          // pinned staging for batch uploads (grows)
    size_t h_stage_cap = 0;
    std::string last_error;
    bool profiling = false;
    std::vector<std::pair<const char *, cudaEvent_t>> marks;
    std::vector<std::pair<const char *, float>> times;
    int launches = 0;
    unsigned long long last_d2h = 0;  // device-to-host bytes of the last qses_compute
    qses::GsShape gs_force{0, 0, 0, 0};  // autotuner: forced smoothing shape (threads 0 = none)
    qses::GsShape gs_used;            // shape of the last smoothing run
    int edt_force = -1;               // autotuner: forced refine tile shape (-1 = none)
    int edt_used = 0;
    unsigned long long diag[10] = {0};  // smoothing diagnostics: slabs, slab size, max/idle/total rounds
    bool use_graphs = true;           // pipeline segments through CUDA graphs
    qses::GraphSeg seg[qses::kSegSlots][qses::kSegCache];
    unsigned long long seg_clock = 0;
    // Free counters of the buffers graphs may use (see segment.h): arenas count their own;
    // host_gen counts pinned staging and slab-table reallocations; pinned_frees() the
    // process-wide pinned block cache.
    unsigned long long host_gen = 0;
    unsigned long long memory_generation() const;  // the sum of them all
    unsigned long long graph_stats[4] = {0};  // captures, instantiations, in-place updates, replays
    // host timeline of the last pipeline call (ms): host work before the first launch, field
    // segment (launch to read-back), host gap, mesh segment, host gap, finish segment
    double timeline[6] = {0};
    void tick(int k);                 // closes timeline interval k at "now"
    std::chrono::steady_clock::time_point tl_last;

    // per-slice vertex and triangle counts of the last call in the reference's slicing mode
    std::vector<unsigned> slice_nv, slice_nt;
    // the last call's grid was too large for one pass but fits the reference's slicing
    bool oversize = false;

    int fail(int code, const char *what, cudaError_t e = cudaSuccess);
    void mark(const char *name);
};

namespace qses {
// Bounds of the device atoms (one read-back) and the molecule's grid, into ctx->grid.
int molecule_grid(qses_context *ctx, const qses_params &p, const float *d_xyz, const float *d_r, unsigned n, QGrid &g,
                  bool sliced);
int run_pipeline(qses_context *ctx, const qses_params &p, const float *d_xyz, const float *d_r, unsigned n);
// The reference's slicing (QSES_FLAG_REFERENCE_SLICES): slice after slice of p.slice voxels,
// each meshed, welded and smoothed alone; the meshes concatenated on the host as
// API_computeSES does (vertex ids offset by the vertices of earlier slices).
struct SlicedMesh {
    std::vector<float> vertices;              // 3 per vertex
    std::vector<int> triangles;               // 3 per triangle (kept, or all with keep_all)
    std::vector<int> atom_sorted, atom_input;
    std::vector<unsigned> slice_nv, slice_nt;  // per slice with a mesh, in slice order
};
int run_pipeline_slices(qses_context *ctx, const qses_params &p, const float *d_xyz, const float *d_r, unsigned n,
                        SlicedMesh &out);
// `passes` exact Gauss-Seidel passes over vertices [0, nv): positions vq (3 floats each) in
// and out, CSR (deg offsets, nbr), shape sh.  The vertices run in sequential waves of at
// most the slab kernel's capacity; every dependency points to a lower id, so a wave only
// depends on earlier, finished waves.
// `before_writeback` (may be null): event the stream waits for before the smoothed
// positions overwrite vq (work on another stream that still reads the welded positions).
int run_smoothing(qses_context *ctx, const GsShape &sh, const GsLaunch &L, int passes, float *vq, float4 *pos4,
                  unsigned nv, const uint2 *deg, const unsigned *nbr, unsigned short *cnt, int *remote, uint2 *home,
                  unsigned *table, const unsigned *h_table, unsigned *inbox, unsigned *inbox_tail, int *d_err,
                  unsigned long long *stats, cudaEvent_t before_writeback = nullptr);
// Slab plan of a pass over nv vertices.  mol_off (nm + 1 entries, null for one molecule):
// the molecules' vertex ranges, never split by a slab boundary unless a molecule is larger
// than the slab size; mol_depth: a per-molecule estimate of the dependency depth (grid size),
// which orders the slabs by when their inputs are expected.  Fills pl.table.
int gs_plan(int device, const GsShape &sh, unsigned nv, const unsigned *mol_off, const int *mol_depth, unsigned nm,
            GsPlan &pl);
// The same for at most pmax resident slab CTAs (no device query).
int gs_plan_for(int pmax, const GsShape &sh, unsigned nv, const unsigned *mol_off, const int *mol_depth, unsigned nm,
                GsPlan &pl);
// The smoothing workspace of a plan (home records, slab tables, inboxes) in ctx->gs_ws and
// the plan's tables in ctx->h_gs.  Returns QSES_OK or an error code (ctx->fail called).
struct GsBuffers {
    uint2 *home;
    unsigned *table, *inbox, *inbox_tail;
};
int gs_buffers(qses_context *ctx, const GsPlan &pl, unsigned nv, GsBuffers &out);
// All items share `passes`; the weld keys of every item fit `key_bits` bits and
// key_bits + bits(count - 1) <= 64.  Results in ctx->batch.
int run_batch(qses_context *ctx, const BatchItem *items, unsigned count, int passes, int key_bits);
}
