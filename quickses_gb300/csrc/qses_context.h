// Context state shared by the pipeline and the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "qses_internal.h"

namespace qses {

// Bump allocator over one device allocation that persists across calls.
struct Arena {
    void *base = nullptr;
    size_t cap = 0, off = 0;
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

int grid_from_bounds(const float mn[3], const float mx[3], float maxR, unsigned n, float dx, QGrid &g,
                     qses_grid_info *info, std::string *why);
void fill_lut(const QGrid &g, float *lut);

}  // namespace qses

struct qses_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    qses::Arena input, field, mesh_ws;
    void *small = nullptr;            // 4 KB device scratch: bounds, error word, queue counters
    unsigned char *h_small = nullptr; // 4 KB pinned host scratch
    int gs_blocks = 16;
    QGrid grid;
    qses_grid_info info;
    bool have_grid = false;
    qses::DeviceMesh mesh;
    std::string last_error;
    bool profiling = false;
    std::vector<std::pair<const char *, cudaEvent_t>> marks;
    std::vector<std::pair<const char *, float>> times;
    int launches = 0;
    unsigned long long diag[8] = {0};  // smoothing diagnostics: slabs, slab size, max/idle/total rounds

    int fail(int code, const char *what, cudaError_t e = cudaSuccess);
    void mark(const char *name);
};

namespace qses {
int run_pipeline(qses_context *ctx, const qses_params &p, const float *d_xyz, const float *d_r, unsigned n);
}
