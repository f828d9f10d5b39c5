// C-ABI: QuickSES-compatible API_* surface (CudaSurf.h:75-83, CudaSurf.cu:778-873) and the
// reentrant qses_* interface.  No entry point exits the process; errors are status codes.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <map>
#include <new>
#include <utility>
#include <vector>

#include "kernels.h"
#include "prims.h"
#include "qses_context.h"

using qses::DeviceMesh;

namespace {

// Host result buffers are pinned so the device-to-host copies run at full link speed.
// Pinning is expensive (milliseconds for a 150 MB mesh), so released blocks go back to a
// process-wide pool and are reused by later meshes of up to the same size.
struct HostMesh {
    void *block = nullptr;
    size_t bytes = 0;
    std::atomic<int> *refs = nullptr;  // shared block of a batch: the last release returns it
};

std::atomic<unsigned long long> g_pinned_frees{0};

class PinnedPool {
  public:
    // Returns a block of at least `bytes` (rounded up to a size class), or nullptr.
    void *take(size_t bytes, size_t *got) {
        const size_t want = size_class(bytes);
        {
            std::lock_guard<std::mutex> lock(mu_);
            // smallest cached block that fits and wastes at most a factor 2; of equal ones the
            // most recently returned, so a steady loop keeps downloading into the same block
            // (and its pipeline graphs replay without a parameter update)
            size_t best = SIZE_MAX, bi = 0;
            for (size_t i = 0; i < free_.size(); i++)
                if (free_[i].second >= want && free_[i].second <= 2 * want && free_[i].second <= best) {
                    best = free_[i].second;
                    bi = i;
                }
            if (best != SIZE_MAX) {
                void *p = free_[bi].first;
                *got = best;
                cached_ -= best;
                free_.erase(free_.begin() + (long)bi);
                return p;
            }
        }
        void *p = nullptr;
        if (cudaMallocHost(&p, want) != cudaSuccess) {
            cudaGetLastError();
            trim(0);  // give cached blocks back and retry once
            if (cudaMallocHost(&p, want) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
        }
        *got = want;
        return p;
    }
    void give(void *p, size_t bytes) {
        {
            std::lock_guard<std::mutex> lock(mu_);
            if (cached_ + bytes <= cap_) {
                free_.emplace_back(p, bytes);
                cached_ += bytes;
                return;
            }
        }
        g_pinned_frees++;
        cudaFreeHost(p);
    }

  private:
    size_t cap_ = 16ull << 30;  // pinned bytes kept for reuse (qses_set_pinned_cache)

  public:
    void set_cap(size_t bytes) {
        {
            std::lock_guard<std::mutex> lock(mu_);
            cap_ = bytes;
        }
        trim(bytes);
    }

  private:
    // size classes: 64 KB granularity below 1 MB, then 1/8 steps of the next power of two
    static size_t size_class(size_t b) {
        if (b <= (1u << 20)) return (b + 65535) & ~(size_t)65535;
        size_t p2 = 1ull << 20;
        while (p2 < b) p2 <<= 1;
        const size_t step = p2 / 16;
        return (b + step - 1) / step * step;
    }
    void trim(size_t keep) {
        std::lock_guard<std::mutex> lock(mu_);
        while (cached_ > keep && !free_.empty()) {
            g_pinned_frees++;
            cudaFreeHost(free_.back().first);
            cached_ -= free_.back().second;
            free_.pop_back();
        }
    }
    std::mutex mu_;
    std::vector<std::pair<void *, size_t>> free_;
    size_t cached_ = 0;
};

PinnedPool &pinned_pool() {
    static PinnedPool *pool = new PinnedPool();  // never destroyed: meshes may outlive statics
    return *pool;
}

}  // namespace

void *qses::pinned_take(size_t bytes, size_t *got) { return pinned_pool().take(bytes, got); }
void qses::pinned_give(void *p, size_t bytes) { pinned_pool().give(p, bytes); }
unsigned long long qses::pinned_frees() { return g_pinned_frees.load(); }

namespace {

int fill_host_mesh(qses_context *ctx, qses_mesh *out) {
    const DeviceMesh &m = ctx->mesh;
    memset(out, 0, sizeof(*out));
    const size_t vb = 12ull * m.nv, tb = 12ull * m.nt, ab = 4ull * m.nv;
    const size_t total = vb + tb + 2 * ab + 64;
    HostMesh *hm = new (std::nothrow) HostMesh();
    if (!hm) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "host mesh");
    hm->block = pinned_pool().take(total, &hm->bytes);
    if (!hm->block) {
        delete hm;
        return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned host mesh");
    }
    char *p = (char *)hm->block;
    out->vertices = (qses_float3 *)p;
    out->triangles = (int *)(p + vb);
    out->atom_sorted = (int *)(p + vb + tb);
    out->atom_input = (int *)(p + vb + tb + ab);
    out->n_vertices = m.nv;
    out->n_triangles = m.nt;
    out->_owner = hm;
    if (ctx->have_grid) {
        out->grid_dim = ctx->grid.G;
        out->origin[0] = ctx->grid.ox; out->origin[1] = ctx->grid.oy; out->origin[2] = ctx->grid.oz;
    }
    ctx->last_d2h = vb + tb + 2 * ab;
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    if (vb) e = cudaMemcpyAsync(out->vertices, m.vertices, vb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && tb) e = cudaMemcpyAsync(out->triangles, m.triangles, tb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && ab) e = cudaMemcpyAsync(out->atom_sorted, m.atom_sorted, ab, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && ab) e = cudaMemcpyAsync(out->atom_input, m.atom_input, ab, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        qses_mesh_release(out);
        return ctx->fail(QSES_ERR_CUDA, "mesh download", e);
    }
    return QSES_OK;
}

int empty_mesh(qses_context *ctx, qses_mesh *out) {
    ctx->mesh = DeviceMesh();
    ctx->mesh.valid = true;
    ctx->have_grid = false;
    return fill_host_mesh(ctx, out);
}

int check_params(qses_context *ctx, const qses_params *p) {
    if (!p) return ctx->fail(QSES_ERR_INVALID_ARG, "null parameters");
    if (!(p->voxel > 0.0f)) return ctx->fail(QSES_ERR_INVALID_ARG, "voxel size must be > 0");
    if (p->smooth_passes < 0 || p->smooth_passes > 1000)
        return ctx->fail(QSES_ERR_INVALID_ARG, "smooth_passes must be in [0, 1000]");
    if ((p->flags & QSES_FLAG_REFERENCE_SLICES) && p->slice < 1)
        return ctx->fail(QSES_ERR_INVALID_ARG, "slice must be >= 1");
    return QSES_OK;
}

// The concatenated meshes of the reference's slicing mode into one pinned block.
int host_mesh_from_slices(qses_context *ctx, const qses::SlicedMesh &sm, qses_mesh *out) {
    memset(out, 0, sizeof(*out));
    const unsigned nv = (unsigned)(sm.vertices.size() / 3), nt = (unsigned)(sm.triangles.size() / 3);
    const size_t vb = 12ull * nv, tb = 12ull * nt, ab = 4ull * nv;
    HostMesh *hm = new (std::nothrow) HostMesh();
    if (!hm) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "host mesh");
    hm->block = pinned_pool().take(vb + tb + 2 * ab + 64, &hm->bytes);
    if (!hm->block) {
        delete hm;
        return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned host mesh");
    }
    char *b = (char *)hm->block;
    if (vb) memcpy(b, sm.vertices.data(), vb);
    if (tb) memcpy(b + vb, sm.triangles.data(), tb);
    if (ab) {
        memcpy(b + vb + tb, sm.atom_sorted.data(), ab);
        memcpy(b + vb + tb + ab, sm.atom_input.data(), ab);
    }
    out->vertices = (qses_float3 *)b;
    out->triangles = (int *)(b + vb);
    out->atom_sorted = (int *)(b + vb + tb);
    out->atom_input = (int *)(b + vb + tb + ab);
    out->n_vertices = nv;
    out->n_triangles = nt;
    out->grid_dim = ctx->grid.G;
    out->origin[0] = ctx->grid.ox; out->origin[1] = ctx->grid.oy; out->origin[2] = ctx->grid.oz;
    out->_owner = hm;
    ctx->last_d2h = vb + tb + 2 * ab;
    return QSES_OK;
}

}  // namespace

extern "C" {

QSES_API const char *qses_status_string(int status) {
    switch (status) {
        case QSES_OK: return "ok";
        case QSES_ERR_INVALID_ARG: return "invalid argument";
        case QSES_ERR_NO_DEVICE: return "no usable sm_103 CUDA device";
        case QSES_ERR_CUDA: return "CUDA runtime error";
        case QSES_ERR_OUT_OF_MEMORY: return "out of memory";
        case QSES_ERR_UNSUPPORTED: return "input outside the supported envelope";
        case QSES_ERR_TIMEOUT: return "bounded device wait timed out";
        case QSES_ERR_INTERNAL: return "internal error";
        case QSES_ERR_CANCELLED: return "request cancelled";
        default: return "unknown status";
    }
}

QSES_API void qses_params_default(qses_params *p) {
    if (!p) return;
    p->voxel = 0.5f;
    p->smooth_passes = 1;
    p->slice = 300;
    p->flags = 0;
}

QSES_API int qses_context_create(int device, void *cuda_stream, qses_context **out) {
    if (!out) return QSES_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return QSES_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        cudaGetLastError();
        return QSES_ERR_NO_DEVICE;
    }
    if (cudaSetDevice(device) != cudaSuccess) return QSES_ERR_CUDA;
    qses_context *ctx = new (std::nothrow) qses_context();
    if (!ctx) return QSES_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    if (cuda_stream) {
        ctx->stream = (cudaStream_t)cuda_stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            return QSES_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->capture, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        qses_context_destroy(ctx);
        return QSES_ERR_CUDA;
    }
    if (cudaMalloc(&ctx->small, 4096) != cudaSuccess || cudaMallocHost((void **)&ctx->h_small, 4096) != cudaSuccess) {
        cudaGetLastError();
        qses_context_destroy(ctx);
        return QSES_ERR_OUT_OF_MEMORY;
    }
    *out = ctx;
    return QSES_OK;
}

QSES_API int qses_context_destroy(qses_context *ctx) {
    if (!ctx) return QSES_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->input.release();
    ctx->field.release();
    ctx->mesh_ws.release();
    ctx->gs_ws.release();
    if (ctx->h_gs) cudaFreeHost(ctx->h_gs);
    if (ctx->small) cudaFree(ctx->small);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    for (auto &m : ctx->marks) cudaEventDestroy(m.second);
    for (auto &slot : ctx->seg)
        for (auto &g : slot)
            if (g.exec) cudaGraphExecDestroy(g.exec);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    if (ctx->dl.block) qses::pinned_give(ctx->dl.block, ctx->dl.bytes);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->capture) cudaStreamDestroy(ctx->capture);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return QSES_OK;
}

QSES_API int qses_compute(qses_context *ctx, const qses_params *p, const qses_float3 *atoms, const float *radii,
                          unsigned n, qses_mesh *out) {
    if (!ctx || !out) return QSES_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    int rc = check_params(ctx, p);
    if (rc) return rc;
    if (n > 0 && (!atoms || !radii)) return ctx->fail(QSES_ERR_INVALID_ARG, "null atom arrays");
    cudaSetDevice(ctx->device);
    if (n <= 1) return empty_mesh(ctx, out);  // CudaSurf.cu:539-543
    if (ctx->input.reserve(16ull * n + 512) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "input buffers");
    float *d_xyz = (float *)ctx->input.take(12ull * n);
    float *d_r = (float *)ctx->input.take(4ull * n);
    cudaError_t e = cudaMemcpyAsync(d_xyz, atoms, 12ull * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_r, radii, 4ull * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return ctx->fail(QSES_ERR_CUDA, "atom upload", e);
    if (p->flags & QSES_FLAG_REFERENCE_SLICES) {
        qses::SlicedMesh sm;
        rc = qses::run_pipeline_slices(ctx, *p, d_xyz, d_r, n, sm);
        if (rc) return rc;
        return host_mesh_from_slices(ctx, sm, out);
    }
    ctx->dl = qses::HostDownload();
    ctx->dl.want = true;
    rc = qses::run_pipeline(ctx, *p, d_xyz, d_r, n);
    qses::HostDownload dl = ctx->dl;
    ctx->dl = qses::HostDownload();
    if (rc == QSES_ERR_UNSUPPORTED && ctx->oversize && !dl.block) {
        // A grid too large for one pass (more than 4096 voxels or 2000 A per axis): the
        // reference slices every grid, so it gets the reference's sliced output
        // (CudaSurf.cu:629-754), computed one slice box at a time.
        qses_params ps = *p;
        if (ps.slice < 1) ps.slice = 300;
        ps.flags |= QSES_FLAG_REFERENCE_SLICES;
        qses::SlicedMesh sm;
        rc = qses::run_pipeline_slices(ctx, ps, d_xyz, d_r, n, sm);
        if (rc) return rc;
        return host_mesh_from_slices(ctx, sm, out);
    }
    if (rc) {
        if (dl.block) {  // copies into it may still be queued
            cudaStreamSynchronize(ctx->stream);
            cudaStreamSynchronize(ctx->side);
            qses::pinned_give(dl.block, dl.bytes);
        }
        return rc;
    }
    if (!dl.block) return fill_host_mesh(ctx, out);
    // the pipeline downloaded the mesh into dl.block while the smoothing pass ran
    HostMesh *hm = new (std::nothrow) HostMesh();
    if (!hm) {
        qses::pinned_give(dl.block, dl.bytes);
        return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "host mesh");
    }
    hm->block = dl.block;
    hm->bytes = dl.bytes;
    char *b = (char *)dl.block;
    const qses::DeviceMesh &m = ctx->mesh;
    out->vertices = (qses_float3 *)b;
    out->triangles = (int *)(b + dl.vb);
    out->atom_sorted = (int *)(b + dl.vb + dl.tb);
    out->atom_input = (int *)(b + dl.vb + dl.tb + dl.ab);
    out->n_vertices = m.nv;
    out->n_triangles = m.nt;
    out->grid_dim = ctx->grid.G;
    out->origin[0] = ctx->grid.ox; out->origin[1] = ctx->grid.oy; out->origin[2] = ctx->grid.oz;
    out->_owner = hm;
    ctx->last_d2h = dl.d2h;
    return QSES_OK;
}

QSES_API int qses_compute_device(qses_context *ctx, const qses_params *p, const float *d_xyz, const float *d_radii,
                                 unsigned n, qses_device_mesh *out) {
    if (!ctx || !out) return QSES_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    int rc = check_params(ctx, p);
    if (rc) return rc;
    if (p->flags & QSES_FLAG_REFERENCE_SLICES)
        return ctx->fail(QSES_ERR_UNSUPPORTED, "the reference's slicing mode returns host meshes (qses_compute)");
    cudaSetDevice(ctx->device);
    if (n <= 1) {
        ctx->mesh = DeviceMesh();
        ctx->mesh.valid = true;
        return QSES_OK;
    }
    if (!d_xyz || !d_radii) return ctx->fail(QSES_ERR_INVALID_ARG, "null atom arrays");
    rc = qses::run_pipeline(ctx, *p, d_xyz, d_radii, n);
    if (rc) return rc;
    out->n_vertices = ctx->mesh.nv;
    out->n_triangles = ctx->mesh.nt;
    out->d_vertices = ctx->mesh.vertices;
    out->d_triangles = (int *)ctx->mesh.triangles;
    out->d_atom_sorted = ctx->mesh.atom_sorted;
    out->d_atom_input = ctx->mesh.atom_input;
    return QSES_OK;
}

QSES_API int qses_last_slices(qses_context *ctx, unsigned *n_vertices, unsigned *n_triangles, int max) {
    if (!ctx) return -1;
    const int k = (int)ctx->slice_nv.size();
    for (int q = 0; q < k && q < max; q++) {
        if (n_vertices) n_vertices[q] = ctx->slice_nv[q];
        if (n_triangles) n_triangles[q] = ctx->slice_nt[q];
    }
    return k;
}

QSES_API void qses_mesh_release(qses_mesh *m) {
    if (!m) return;
    HostMesh *hm = (HostMesh *)m->_owner;
    if (hm) {
        if (hm->refs) {
            if (hm->refs->fetch_sub(1) == 1) {
                pinned_pool().give(hm->block, hm->bytes);
                delete hm->refs;
            }
        } else if (hm->block) {
            pinned_pool().give(hm->block, hm->bytes);
        }
        delete hm;
    }
    memset(m, 0, sizeof(*m));
}

}  // extern "C"

namespace {

// Host bounds + reference sizing of one request (the device path reads the same bounds
// with k_atom_minmax: min/max/max-radius are exact either way).
int size_request(const qses_request &r, QGrid &g) {
    float mn[3] = {100000.0f, 100000.0f, 100000.0f}, mx[3] = {-100000.0f, -100000.0f, -100000.0f}, maxR = 0.0f;
    for (unsigned a = 0; a < r.n; a++) {
        const float c[3] = {r.atoms[a].x, r.atoms[a].y, r.atoms[a].z};
        for (int q = 0; q < 3; q++) {
            mn[q] = std::min(mn[q], c[q]);
            mx[q] = std::max(mx[q], c[q]);
        }
        maxR = std::max(maxR, r.radii[a]);
    }
    return qses::grid_from_bounds(mn, mx, maxR, r.n, r.voxel, g, nullptr, nullptr);
}

// Copies one finished batch into one pinned block shared by its meshes.
int fill_batch_meshes(qses_context *ctx, const std::vector<unsigned> &reqs, const std::vector<qses::BatchItem> &items,
                      qses_mesh *out) {
    const qses::BatchResult &R = ctx->batch;
    size_t vb = 12ull * R.nv, tb = 12ull * R.nkept, ab = 4ull * R.nv, got = 0;
    void *block = nullptr;
    if (ctx->dl.block) {  // downloaded by the pipeline while the smoothing pass ran
        block = ctx->dl.block;
        got = ctx->dl.bytes;
        tb = ctx->dl.tb;  // room for the pre-filter count; the first nkept are the kept ones
        ctx->last_d2h = ctx->dl.d2h;
        ctx->dl = qses::HostDownload();
    } else {
        block = pinned_pool().take(vb + tb + 2 * ab + 256, &got);
        if (!block) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned batch meshes");
        char *p = (char *)block;
        cudaStream_t s = ctx->stream;
        cudaError_t e = cudaSuccess;
        if (vb) e = cudaMemcpyAsync(p, R.vertices, vb, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && tb) e = cudaMemcpyAsync(p + vb, R.triangles, tb, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && ab) e = cudaMemcpyAsync(p + vb + tb, R.atom_sorted, ab, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && ab)
            e = cudaMemcpyAsync(p + vb + tb + ab, R.atom_input, ab, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            pinned_pool().give(block, got);
            return ctx->fail(QSES_ERR_CUDA, "batch mesh download", e);
        }
        ctx->last_d2h = vb + tb + 2 * ab;
    }
    char *p = (char *)block;
    std::atomic<int> *refs = new std::atomic<int>((int)reqs.size());
    for (size_t m = 0; m < reqs.size(); m++) {
        qses_mesh &o = out[reqs[m]];
        HostMesh *hm = new HostMesh();
        hm->block = block;
        hm->bytes = got;
        hm->refs = refs;
        const unsigned v0 = R.vtx_off[m], v1 = R.vtx_off[m + 1], t0 = R.kept_off[m], t1 = R.kept_off[m + 1];
        o.n_vertices = v1 - v0;
        o.n_triangles = t1 - t0;
        o.vertices = (qses_float3 *)(p + 12ull * v0);
        o.triangles = (int *)(p + vb + 12ull * t0);
        o.atom_sorted = (int *)(p + vb + tb + 4ull * v0);
        o.atom_input = (int *)(p + vb + tb + ab + 4ull * v0);
        o.grid_dim = items[m].g.G;
        o.origin[0] = items[m].g.ox; o.origin[1] = items[m].g.oy; o.origin[2] = items[m].g.oz;
        o._owner = hm;
    }
    return QSES_OK;
}

}  // namespace

extern "C" {

QSES_API int qses_compute_batch(qses_context *ctx, const qses_request *reqs, unsigned count, qses_mesh *out,
                                int *status) {
    if (!ctx || (count && (!reqs || !out))) return QSES_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    std::vector<QGrid> grids(count);
    std::map<int, std::vector<unsigned>> by_passes;
    for (unsigned i = 0; i < count; i++) {
        memset(&out[i], 0, sizeof(qses_mesh));
        const qses_request &r = reqs[i];
        int rc = QSES_OK;
        if (!(r.voxel > 0.0f) || r.smooth_passes < 0 || r.smooth_passes > 1000 || (r.n > 0 && (!r.atoms || !r.radii)))
            rc = QSES_ERR_INVALID_ARG;
        else if (r.flags & QSES_FLAG_REFERENCE_SLICES)
            rc = QSES_ERR_UNSUPPORTED;  // a per-molecule compatibility mode (qses_compute)
        else if (r.n > 1)
            rc = size_request(r, grids[i]);
        if (status) status[i] = rc;
        if (rc == QSES_OK && r.n > 1) by_passes[r.smooth_passes].push_back(i);
    }
    for (auto &grp : by_passes) {
        const std::vector<unsigned> &ids = grp.second;
        size_t at = 0;
        while (at < ids.size()) {
            // Largest prefix whose molecule-tagged weld keys fit 64 bits.
            size_t end = at;
            int kb = 0;
            while (end < ids.size()) {
                const QGrid &g = grids[ids[end]];
                const int k = qses::bits_for((unsigned long long)g.Rq * g.Rq * g.Rq - 1);
                const int kb2 = std::max(kb, k);
                if (end > at && kb2 + qses::bits_for(end - at) > 64) break;
                kb = kb2;
                end++;
            }
            std::vector<unsigned> chunk(ids.begin() + (long)at, ids.begin() + (long)end);
            std::vector<qses::BatchItem> items(chunk.size());
            for (size_t m = 0; m < chunk.size(); m++) {
                const qses_request &r = reqs[chunk[m]];
                items[m].xyz = (const float *)r.atoms;
                items[m].r = r.radii;
                items[m].n = r.n;
                items[m].flags = (unsigned)r.flags;
                items[m].g = grids[chunk[m]];
            }
            ctx->dl = qses::HostDownload();
            ctx->dl.want = true;
            int rc = qses::run_batch(ctx, items.data(), (unsigned)items.size(), grp.first, kb);
            if (rc != QSES_OK && ctx->dl.block) {  // copies into it may still be queued
                cudaStreamSynchronize(ctx->stream);
                cudaStreamSynchronize(ctx->side);
                qses::pinned_give(ctx->dl.block, ctx->dl.bytes);
                ctx->dl = qses::HostDownload();
            }
            if (rc == QSES_OK) rc = fill_batch_meshes(ctx, chunk, items, out);
            ctx->dl = qses::HostDownload();
            if (rc != QSES_OK) {
                for (unsigned i : chunk) {
                    if (status) status[i] = rc;
                }
                if (rc == QSES_ERR_CUDA || rc == QSES_ERR_TIMEOUT || rc == QSES_ERR_INTERNAL) return rc;
            }
            at = end;
        }
    }
    return QSES_OK;
}

QSES_API void qses_set_pinned_cache(unsigned long long bytes) { pinned_pool().set_cap((size_t)bytes); }

QSES_API int qses_set_smoothing_shape(qses_context *ctx, int threads, unsigned target, unsigned cache_flags,
                                      unsigned wave_vertices) {
    if (!ctx) return QSES_ERR_INVALID_ARG;
    if (threads == 0) {
        ctx->gs_force = qses::GsShape{0, 0, 0, 0};
        return QSES_OK;
    }
    if ((threads != 512 && threads != 1024) || target < 256 || !qses::gs_flags_valid(cache_flags) ||
        (wave_vertices != 0 && wave_vertices < target))
        return QSES_ERR_INVALID_ARG;
    ctx->gs_force = qses::GsShape{threads, target, cache_flags, wave_vertices};
    return QSES_OK;
}

QSES_API int qses_set_default_smoothing_shape(int batch, int threads, unsigned target, unsigned cache_flags) {
    if ((threads != 512 && threads != 1024) || target < 256 || !qses::gs_flags_valid(cache_flags) ||
        (cache_flags & qses::kGsPersistL2))
        return QSES_ERR_INVALID_ARG;
    qses::gs_shape_record_all(batch != 0, qses::GsShape{threads, target, cache_flags, 0});
    return QSES_OK;
}

QSES_API int qses_set_field_shape(qses_context *ctx, int shape) {
    if (!ctx || shape < -1 || shape >= qses::kEdtShapes) return QSES_ERR_INVALID_ARG;
    ctx->edt_force = shape;
    return QSES_OK;
}

QSES_API int qses_autotune(qses_context *ctx, const qses_params *p, const qses_float3 *atoms, const float *radii,
                           unsigned n, int repeats, int *threads_out, unsigned *target_out, unsigned *flags_out,
                           int *field_shape_out, float *smooth_ms_out) {
    if (!ctx || !p || (n && (!atoms || !radii))) return QSES_ERR_INVALID_ARG;
    int rc = check_params(ctx, p);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    qses::GsShape cand[128];
    const int nc = qses::gs_shape_candidates(cand, 128);
    qses::GsShape best = cand[0];
    float best_ms = -1.0f;
    const bool prof = ctx->profiling;
    ctx->profiling = true;
    unsigned nv = 0;
    if (n > 1 && p->smooth_passes > 0) {
        for (int c = 0; c < nc && rc == QSES_OK; c++) {
            ctx->gs_force = cand[c];
            for (int r = 0; r < std::max(1, repeats) && rc == QSES_OK; r++) {
                if (ctx->input.reserve(16ull * n + 512) != QSES_OK) {
                    rc = ctx->fail(QSES_ERR_OUT_OF_MEMORY, "input buffers");
                    break;
                }
                float *d_xyz = (float *)ctx->input.take(12ull * n);
                float *d_r = (float *)ctx->input.take(4ull * n);
                cudaError_t e = cudaMemcpyAsync(d_xyz, atoms, 12ull * n, cudaMemcpyHostToDevice, ctx->stream);
                if (e == cudaSuccess) e = cudaMemcpyAsync(d_r, radii, 4ull * n, cudaMemcpyHostToDevice, ctx->stream);
                if (e != cudaSuccess) {
                    rc = ctx->fail(QSES_ERR_CUDA, "atom upload", e);
                    break;
                }
                rc = qses::run_pipeline(ctx, *p, d_xyz, d_r, n);
                if (rc) break;
                nv = ctx->mesh.nv;
                for (auto &t : ctx->times)
                    if (!strcmp(t.first, "smooth") && (best_ms < 0 || t.second < best_ms)) {
                        best_ms = t.second;
                        best = cand[c];
                    }
            }
        }
    }
    ctx->gs_force = qses::GsShape{0, 0, 0, 0};
    // refine tile shape, timed on the same molecule (the codes are the same for every shape)
    int best_edt = 0;
    float best_edt_ms = -1.0f;
    if (n > 1 && rc == QSES_OK) {
        for (int sh = 0; sh < qses::kEdtShapes && rc == QSES_OK; sh++) {
            ctx->edt_force = sh;
            for (int r = 0; r < std::max(1, repeats) && rc == QSES_OK; r++) {
                if (ctx->input.reserve(16ull * n + 512) != QSES_OK) {
                    rc = ctx->fail(QSES_ERR_OUT_OF_MEMORY, "input buffers");
                    break;
                }
                float *d_xyz = (float *)ctx->input.take(12ull * n);
                float *d_r = (float *)ctx->input.take(4ull * n);
                cudaError_t e = cudaMemcpyAsync(d_xyz, atoms, 12ull * n, cudaMemcpyHostToDevice, ctx->stream);
                if (e == cudaSuccess) e = cudaMemcpyAsync(d_r, radii, 4ull * n, cudaMemcpyHostToDevice, ctx->stream);
                if (e != cudaSuccess) {
                    rc = ctx->fail(QSES_ERR_CUDA, "atom upload", e);
                    break;
                }
                qses_params p0 = *p;
                p0.smooth_passes = 0;
                rc = qses::run_pipeline(ctx, p0, d_xyz, d_r, n);
                if (rc) break;
                for (auto &t : ctx->times)
                    if (!strcmp(t.first, "refine") && (best_edt_ms < 0 || t.second < best_edt_ms)) {
                        best_edt_ms = t.second;
                        best_edt = sh;
                    }
            }
        }
        ctx->edt_force = -1;
        if (rc == QSES_OK && ctx->have_grid) qses::edt_shape_record(ctx->grid.G, best_edt);
    }
    ctx->profiling = prof;
    if (rc) return rc;
    if (field_shape_out) *field_shape_out = best_edt;
    if (nv > 0) qses::gs_shape_record(nv, false, best);
    if (threads_out) *threads_out = best.threads;
    if (target_out) *target_out = best.target;
    if (flags_out) *flags_out = best.flags;
    if (smooth_ms_out) *smooth_ms_out = best_ms;
    return QSES_OK;
}

QSES_API int qses_autotune_batch(qses_context *ctx, const qses_request *reqs, unsigned count, int repeats,
                                 int *threads_out, unsigned *target_out, unsigned *flags_out, float *ms_out) {
    if (!ctx || (count && !reqs)) return QSES_ERR_INVALID_ARG;
    qses::GsShape cand[128];
    const int nc = qses::gs_shape_candidates(cand, 128);
    qses::GsShape best = cand[0];
    double best_s = -1.0;
    unsigned long long nv = 0;
    std::vector<qses_mesh> out(count ? count : 1);
    int rc = QSES_OK;
    for (int c = 0; c < nc && rc == QSES_OK; c++) {
        ctx->gs_force = cand[c];
        for (int r = 0; r < std::max(1, repeats) && rc == QSES_OK; r++) {
            const auto t0 = std::chrono::steady_clock::now();
            rc = qses_compute_batch(ctx, reqs, count, out.data(), nullptr);
            const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            nv = 0;
            for (unsigned i = 0; i < count; i++) {
                nv += out[i].n_vertices;
                qses_mesh_release(&out[i]);
            }
            if (rc == QSES_OK && (best_s < 0 || dt < best_s)) {
                best_s = dt;
                best = cand[c];
            }
        }
    }
    ctx->gs_force = qses::GsShape{0, 0, 0, 0};
    if (rc) return rc;
    if (nv > 0) qses::gs_shape_record((unsigned)std::min<unsigned long long>(nv, 152ull * qses::kGsSlabMaxVerts), true, best);
    if (threads_out) *threads_out = best.threads;
    if (target_out) *target_out = best.target;
    if (flags_out) *flags_out = best.flags;
    if (ms_out) *ms_out = (float)(best_s * 1e3);
    return QSES_OK;
}

QSES_API const char *qses_last_error(qses_context *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

QSES_API int qses_set_profiling(qses_context *ctx, int on) {
    if (!ctx) return QSES_ERR_INVALID_ARG;
    ctx->profiling = on != 0;
    return QSES_OK;
}

QSES_API int qses_stage_times(qses_context *ctx, float *ms, const char **names, int max) {
    if (!ctx) return 0;
    int k = 0;
    for (auto &t : ctx->times) {
        if (k >= max) break;
        if (ms) ms[k] = t.second;
        if (names) names[k] = t.first;
        k++;
    }
    return k;
}

QSES_API int qses_last_launch_count(qses_context *ctx) { return ctx ? ctx->launches : 0; }

QSES_API unsigned long long qses_last_download_bytes(qses_context *ctx) { return ctx ? ctx->last_d2h : 0ull; }

QSES_API int qses_diagnostics(qses_context *ctx, unsigned long long *out, int max) {
    if (!ctx || !out) return 0;
    int k = 0;
    for (; k < max && k < 10; k++) out[k] = ctx->diag[k];
    return k;
}

QSES_API int qses_debug_slab_plan(unsigned nv, const unsigned *mol_off, const int *depth, unsigned nm, int threads,
                                  unsigned target, unsigned cache_flags, unsigned wave, int pmax, unsigned *launch,
                                  unsigned *table, size_t cap) {
    if (!launch || (nm > 1 && !mol_off) || !qses::gs_flags_valid(cache_flags)) return QSES_ERR_INVALID_ARG;
    qses::GsPlan pl;
    const int rc =
        qses::gs_plan_for(pmax, qses::GsShape{threads, target, cache_flags, wave}, nv, mol_off, depth, nm, pl);
    if (rc != QSES_OK) return rc;
    const unsigned v[6] = {(unsigned)pl.L.ctas, pl.L.smax, pl.L.qcap, pl.L.wsize, pl.L.waves, pl.L.table_words};
    memcpy(launch, v, sizeof(v));
    if (table) {
        if (cap < pl.table.size()) return QSES_ERR_INVALID_ARG;
        memcpy(table, pl.table.data(), 4 * pl.table.size());
    }
    return QSES_OK;
}

QSES_API void qses_debug_fail_reservations(unsigned n) { qses::g_fail_reserves.store(n); }

QSES_API int qses_debug_wait_limit(qses_context *ctx, long long spin_cycles, int *kernel_status) {
    if (!ctx || !kernel_status || spin_cycles < 1000000ll || spin_cycles > 4000000000ll) return QSES_ERR_INVALID_ARG;
    *kernel_status = 0;
    cudaSetDevice(ctx->device);
    // Vertices 0-1 (slab 0) and 2-3 (slab 1), lists 0:{1} 1:{0} 2:{3} 3:{2}.  Vertex 2 is
    // marked as waiting for one lower-slab hand-off (remote count 1, +1 in its counter) that
    // no vertex ever sends, so slab 1 cannot finish and its boundary warp's wait runs out.
    const unsigned table_h[6] = {2, 0, 2, 4, 0, 1};  // Q, bounds (qcap + 1 = 3), order
    const uint2 start_h[5] = {{0, 0}, {1, 0}, {2, 0}, {3, 0}, {4, 0}};
    const unsigned nbr_h[4] = {1, 0, 3, 2};
    const unsigned short cnt_h[4] = {0, 1, 1, 1};
    const int remote_h[4] = {0, 0, 1, 0};
    const uint2 home_h[4] = {{0, 0}, {0, 0}, {1, 2}, {1, 2}};
    const float4 pos_h[4] = {{0, 0, 0, 0}, {1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}};
    char *d = nullptr;
    const size_t bytes = 4096;
    if (cudaMalloc(&d, bytes) != cudaSuccess) {
        cudaGetLastError();
        return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "wait-limit check buffers");
    }
    unsigned *table = (unsigned *)d, *nbr = (unsigned *)(d + 256), *inbox = (unsigned *)(d + 512),
             *tails = (unsigned *)(d + 768);
    uint2 *start = (uint2 *)(d + 1024), *home = (uint2 *)(d + 1280);
    unsigned short *cnt = (unsigned short *)(d + 1536);
    int *remote = (int *)(d + 1792), *err = (int *)(d + 2048);
    float4 *pos = (float4 *)(d + 2304);
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaMemsetAsync(d, 0, bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(inbox, 0xff, 256, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(table, table_h, sizeof(table_h), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(start, start_h, sizeof(start_h), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(nbr, nbr_h, sizeof(nbr_h), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, cnt_h, sizeof(cnt_h), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(remote, remote_h, sizeof(remote_h), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(home, home_h, sizeof(home_h), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pos, pos_h, sizeof(pos_h), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = qses::launch_gs_slab(pos, 0, 4, 2, table, 2, tails + 2, home, 2, 512, 0, 0, start, nbr, cnt, remote, inbox,
                                 tails, err, spin_cycles, nullptr, s);
    int h_err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d);
    if (e != cudaSuccess) return ctx->fail(QSES_ERR_CUDA, "wait-limit check", e);
    *kernel_status = h_err;
    return QSES_OK;
}

QSES_API int qses_host_timeline(qses_context *ctx, double *ms, int max) {
    if (!ctx || !ms) return 0;
    int k = 0;
    for (; k < max && k < 6; k++) ms[k] = ctx->timeline[k];
    return k;
}

QSES_API int qses_set_graphs(qses_context *ctx, int enable) {
    if (!ctx) return QSES_ERR_INVALID_ARG;
    ctx->use_graphs = enable != 0;
    return QSES_OK;
}

QSES_API int qses_graph_stats(qses_context *ctx, unsigned long long *out, int max) {
    if (!ctx || !out) return 0;
    int k = 0;
    for (; k < max && k < 4; k++) out[k] = ctx->graph_stats[k];
    return k;
}

QSES_API int qses_grid_info_for(const qses_float3 *atoms, const float *radii, unsigned n, float voxel,
                                qses_grid_info *out) {
    if (!atoms || !radii || !out || n == 0) return QSES_ERR_INVALID_ARG;
    float mn[3] = {100000.0f, 100000.0f, 100000.0f}, mx[3] = {-100000.0f, -100000.0f, -100000.0f}, maxR = 0.0f;
    for (unsigned a = 0; a < n; a++) {
        const float c[3] = {atoms[a].x, atoms[a].y, atoms[a].z};
        for (int q = 0; q < 3; q++) {
            mn[q] = std::min(mn[q], c[q]);
            mx[q] = std::max(mx[q], c[q]);
        }
        maxR = std::max(maxR, radii[a]);
    }
    QGrid g;
    return qses::grid_from_bounds(mn, mx, maxR, n, voxel, g, out, nullptr);
}

QSES_API int qses_debug_codes(qses_context *ctx, uint8_t *codes, size_t bytes) {
    if (!ctx || !codes || !ctx->mesh.valid || !ctx->have_grid || !ctx->mesh.codes) return QSES_ERR_INVALID_ARG;
    const size_t G = (size_t)ctx->grid.G;
    if (bytes < G * G * G) return QSES_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMemcpy2DAsync(codes, G, ctx->mesh.codes, (size_t)ctx->grid.Gp, G, G * G,
                                      cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? QSES_OK : ctx->fail(QSES_ERR_CUDA, "codes download", e);
}

QSES_API int qses_debug_atom_order(qses_context *ctx, uint32_t *sorted_to_input, uint32_t *hash, unsigned n) {
    if (!ctx || !ctx->mesh.valid || !ctx->mesh.sorted_to_input || n != ctx->mesh.n_atoms) return QSES_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaSuccess;
    if (sorted_to_input)
        e = cudaMemcpyAsync(sorted_to_input, ctx->mesh.sorted_to_input, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && hash)
        e = cudaMemcpyAsync(hash, ctx->mesh.sorted_keys, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? QSES_OK : ctx->fail(QSES_ERR_CUDA, "atom order download", e);
}

// ------------------------------------------------------------ QuickSES surface

QSES_API int NTriangles = 0;
QSES_API int NVertices = 0;
QSES_API int *globalTriangles = nullptr;
QSES_API qses_float3 *globalVertices = nullptr;
QSES_API int *globalIdAtomPerVert = nullptr;

}  // extern "C"

namespace {
std::mutex g_api_mu;
qses_context *g_api_ctx = nullptr;
qses_mesh g_api_mesh;
int g_api_status = QSES_OK;
}  // namespace

extern "C" {

QSES_API int qses_api_last_status(void) { return g_api_status; }

QSES_API void API_computeSES(float resoSES, qses_float3 *atomPos, float *atomRad, unsigned int N,
                             qses_float3 *out_vertices, unsigned int *NVert, int *out_triangles, unsigned int *NTri,
                             int doSmoothing) {
    (void)out_vertices;
    (void)out_triangles;  // ignored, as in the reference (CudaSurf.cu:839-840)
    std::lock_guard<std::mutex> lock(g_api_mu);
    if (NVert) *NVert = 0;
    if (NTri) *NTri = 0;
    if (!g_api_ctx) {
        g_api_status = qses_context_create(0, nullptr, &g_api_ctx);
        if (g_api_status != QSES_OK) {
            fprintf(stderr, "quickses_gb300: %s\n", qses_status_string(g_api_status));
            return;
        }
    }
    qses_params p;
    qses_params_default(&p);
    p.voxel = resoSES;
    p.smooth_passes = doSmoothing < 0 ? 0 : doSmoothing;
    // QSES_REFERENCE_SLICES=<slice voxels>: the reference's sliced output, as its library
    // computes it with SLICE = 300 (CudaSurf.cu:63, 629-754)
    if (const char *env = getenv("QSES_REFERENCE_SLICES")) {
        const long sl = strtol(env, nullptr, 10);
        if (sl > 0) {
            p.slice = (int)std::min(sl, 1l << 20);
            p.flags |= QSES_FLAG_REFERENCE_SLICES;
        }
    }
    qses_mesh m;
    g_api_status = qses_compute(g_api_ctx, &p, atomPos, atomRad, N, &m);
    if (g_api_status != QSES_OK) {
        fprintf(stderr, "quickses_gb300: %s\n", qses_last_error(g_api_ctx));
        return;
    }
    // Like the reference, a second call without API_freeMesh does not free the previous
    // buffers; the globals simply point at the new ones.
    g_api_mesh = m;
    globalVertices = m.vertices;
    globalTriangles = m.triangles;
    globalIdAtomPerVert = m.atom_sorted;
    NVertices = (int)m.n_vertices;
    NTriangles = (int)(3 * m.n_triangles);
    if (NVert) *NVert = m.n_vertices;
    if (NTri) *NTri = 3 * m.n_triangles;
}

QSES_API int *API_getTriangles(bool invertTriangles) {
    if (invertTriangles && globalTriangles) {
        for (int t = 0; t < NTriangles / 3; t++) {
            int save = globalTriangles[3 * t];
            globalTriangles[3 * t] = globalTriangles[3 * t + 1];
            globalTriangles[3 * t + 1] = save;
        }
    }
    return globalTriangles;
}

QSES_API qses_float3 *API_getVertices(void) { return globalVertices; }

QSES_API int *API_getAtomIdPerVert(void) { return globalIdAtomPerVert; }

QSES_API void API_freeMesh(void) {
    std::lock_guard<std::mutex> lock(g_api_mu);
    qses_mesh_release(&g_api_mesh);
    globalVertices = nullptr;
    globalTriangles = nullptr;
    globalIdAtomPerVert = nullptr;
    NVertices = 0;
    NTriangles = 0;
}

}  // extern "C"
