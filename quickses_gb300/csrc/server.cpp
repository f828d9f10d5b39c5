// Served form: a request loop with continuous batching (no reference counterpart; QuickSES
// serves one API_computeSES call at a time from process-global state, CudaSurf.cu:778-841).
//
// Requests are copied in at submit, sized on the host (the reference's grid formulas) and
// queued.  `lanes` worker threads each own a context (one CUDA stream, persistent device
// workspace).  A lane that is free takes every queued request that fits its share of the
// device-memory budget (FIFO, at most max_batch) and runs them as one batch; requests that
// arrive meanwhile wait for the next free lane, so work from different batches overlaps on
// the device while each batch's arithmetic is the single-molecule path's.  Workspaces and
// pinned result blocks stay allocated between batches.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "prims.h"
#include "qses_context.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    unsigned long long ticket = 0;
    std::vector<float> xyz, r;
    qses_request req;
    unsigned long long est_bytes = 0;
    unsigned long long voxels = 0;   // G^3: the work estimate used to bound a batch
    int status = QSES_OK;
    qses_mesh mesh;
    bool done = false;
    bool claimed = false;  // a qses_server_wait is waiting for (or has taken) this result
    Clock::time_point t_submit, t_start, t_done;
};

// Device bytes a request needs while it runs (field workspace + a surface-sized mesh
// workspace), from its grid alone; used only for admission.
unsigned long long estimate_bytes(const QGrid &g, unsigned n) {
    const double G = g.G;
    // codes and the refine's z distances (one byte each per padded voxel), three masks, cells
    const double field = 2.0 * G * G * (double)g.Gp + 3.0 * G * G * g.W * 4.0 + 8.0 * (double)g.gnb * g.gnb * g.gnb +
                         48.0 * n + 8.0 * (g.Gc + 1.0) * (g.Gc + 1.0);
    const double edges = 12.0 * G * G;  // active edges of a globular surface, generous
    const double mesh = edges * 220.0;  // every mesh array per edge (keys, slots, CSR, positions)
    return (unsigned long long)(field + mesh) + (1ull << 20);
}

}  // namespace

struct qses_server {
    qses_server_config cfg;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job *> pending;
    std::unordered_map<unsigned long long, std::unique_ptr<Job>> jobs;
    unsigned long long next_ticket = 1;
    bool stopping = false;
    std::vector<std::thread> workers;
    std::vector<qses_context *> ctxs;
    // statistics
    unsigned long long batches = 0, served = 0, max_batch_seen = 0;
    unsigned inflight_lanes = 0, max_inflight_lanes = 0;

    void lane_loop(int lane);
};

void qses_server::lane_loop(int lane) {
    qses_context *ctx = ctxs[(size_t)lane];
    const unsigned long long lane_budget = cfg.memory_budget / (unsigned long long)std::max(1, cfg.lanes);
    for (;;) {
        std::vector<Job *> batch;
        {
            std::unique_lock<std::mutex> lock(mu);
            cv_work.wait(lock, [&] { return stopping || !pending.empty(); });
            if (stopping && pending.empty()) return;
            unsigned long long bytes = 0, vox = 0;
            while (!pending.empty() && batch.size() < cfg.max_batch) {
                Job *j = pending.front();
                if (!batch.empty() && (bytes + j->est_bytes > lane_budget ||
                                       (cfg.max_batch_voxels && vox + j->voxels > cfg.max_batch_voxels)))
                    break;
                bytes += j->est_bytes;
                vox += j->voxels;
                batch.push_back(j);
                pending.pop_front();
            }
            batches++;
            max_batch_seen = std::max<unsigned long long>(max_batch_seen, batch.size());
            inflight_lanes++;
            max_inflight_lanes = std::max(max_inflight_lanes, inflight_lanes);
            if (!pending.empty()) cv_work.notify_one();  // more work for another free lane
        }
        const Clock::time_point t0 = Clock::now();
        std::vector<qses_request> reqs(batch.size());
        for (size_t k = 0; k < batch.size(); k++) {
            reqs[k] = batch[k]->req;
            batch[k]->t_start = t0;
        }
        std::vector<qses_mesh> out(batch.size());
        std::vector<int> st(batch.size(), QSES_OK);
        int rc = qses_compute_batch(ctx, reqs.data(), (unsigned)reqs.size(), out.data(), st.data());
        const Clock::time_point t1 = Clock::now();
        {
            std::lock_guard<std::mutex> lock(mu);
            for (size_t k = 0; k < batch.size(); k++) {
                Job *j = batch[k];
                j->status = rc != QSES_OK ? rc : st[k];
                j->mesh = out[k];
                j->t_done = t1;
                j->done = true;
                j->xyz.clear();
                j->xyz.shrink_to_fit();
                j->r.clear();
                j->r.shrink_to_fit();
            }
            served += batch.size();
            inflight_lanes--;
        }
        cv_done.notify_all();
    }
}

extern "C" {

QSES_API void qses_server_config_default(qses_server_config *c) {
    if (!c) return;
    c->device = 0;
    c->lanes = 2;
    c->memory_budget = 120ull << 30;
    c->max_batch = 256;
    c->max_batch_voxels = 1000000000ull;
}

QSES_API int qses_server_create(const qses_server_config *cfg, qses_server **out) {
    if (!out) return QSES_ERR_INVALID_ARG;
    *out = nullptr;
    qses_server_config c;
    qses_server_config_default(&c);
    if (cfg) c = *cfg;
    if (c.lanes < 1 || c.lanes > 16 || c.max_batch < 1 || c.memory_budget < (1ull << 28)) return QSES_ERR_INVALID_ARG;
    std::unique_ptr<qses_server> s(new qses_server());
    s->cfg = c;
    for (int l = 0; l < c.lanes; l++) {
        qses_context *ctx = nullptr;
        int rc = qses_context_create(c.device, nullptr, &ctx);
        if (rc != QSES_OK) {
            for (auto *x : s->ctxs) qses_context_destroy(x);
            return rc;
        }
        s->ctxs.push_back(ctx);
    }
    for (int l = 0; l < c.lanes; l++) s->workers.emplace_back([srv = s.get(), l] { srv->lane_loop(l); });
    *out = s.release();
    return QSES_OK;
}

QSES_API int qses_server_submit(qses_server *s, const qses_request *req, unsigned long long *ticket) {
    if (!s || !req || !ticket) return QSES_ERR_INVALID_ARG;
    *ticket = 0;
    if (!(req->voxel > 0.0f) || req->smooth_passes < 0 || req->smooth_passes > 1000 ||
        (req->n > 0 && (!req->atoms || !req->radii)))
        return QSES_ERR_INVALID_ARG;
    if (req->flags & QSES_FLAG_REFERENCE_SLICES) return QSES_ERR_UNSUPPORTED;  // qses_compute only
    std::unique_ptr<Job> j(new Job());
    j->xyz.assign((const float *)req->atoms, (const float *)req->atoms + 3ull * req->n);
    j->r.assign(req->radii, req->radii + req->n);
    j->req = *req;
    j->req.atoms = (const qses_float3 *)j->xyz.data();
    j->req.radii = j->r.data();
    memset(&j->mesh, 0, sizeof(j->mesh));
    j->t_submit = Clock::now();
    if (req->n > 1) {
        qses_grid_info gi;
        QGrid g;
        // bounds start at atom 0, as the device min/max pass starts from its first atom
        float mn[3] = {j->xyz[0], j->xyz[1], j->xyz[2]}, mx[3] = {j->xyz[0], j->xyz[1], j->xyz[2]}, maxR = j->r[0];
        for (unsigned a = 1; a < req->n; a++) {
            for (int q = 0; q < 3; q++) {
                mn[q] = std::min(mn[q], j->xyz[3ull * a + q]);
                mx[q] = std::max(mx[q], j->xyz[3ull * a + q]);
            }
            maxR = std::max(maxR, j->r[a]);
        }
        int rc = qses::grid_from_bounds(mn, mx, maxR, req->n, req->voxel, g, &gi, nullptr);
        if (rc != QSES_OK) return rc;  // rejected at admission, never queued
        j->est_bytes = estimate_bytes(g, req->n);
        j->voxels = (unsigned long long)g.G * g.G * g.G;
        if (j->est_bytes > s->cfg.memory_budget) return QSES_ERR_OUT_OF_MEMORY;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stopping) return QSES_ERR_INVALID_ARG;
    j->ticket = s->next_ticket++;
    *ticket = j->ticket;
    s->pending.push_back(j.get());
    s->jobs.emplace(j->ticket, std::move(j));
    s->cv_work.notify_one();
    return QSES_OK;
}

QSES_API int qses_server_wait(qses_server *s, unsigned long long ticket, double timeout_s, qses_mesh *out,
                              qses_ticket_info *info) {
    if (!s || !out) return QSES_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return QSES_ERR_INVALID_ARG;
    // The Job object itself never moves (the map holds a unique_ptr), but a submit may
    // rehash the map while this thread waits, so no iterator is kept across the wait.  One
    // waiter per ticket: a second one is refused instead of racing the first one's erase.
    Job *j = it->second.get();
    if (j->claimed) return QSES_ERR_INVALID_ARG;
    j->claimed = true;
    auto ready = [&] { return j->done; };
    if (timeout_s < 0) {
        s->cv_done.wait(lock, ready);
    } else if (!s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), ready)) {
        j->claimed = false;
        return QSES_ERR_TIMEOUT;  // still queued or running; wait again later
    }
    const int st = j->status;
    *out = j->mesh;
    if (info) {
        info->queued_s = std::chrono::duration<double>(j->t_start - j->t_submit).count();
        info->run_s = std::chrono::duration<double>(j->t_done - j->t_start).count();
        info->total_s = std::chrono::duration<double>(j->t_done - j->t_submit).count();
    }
    s->jobs.erase(ticket);  // the caller owns the mesh now
    return st;
}

QSES_API int qses_server_cancel(qses_server *s, unsigned long long ticket) {
    if (!s) return QSES_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return QSES_ERR_INVALID_ARG;
    Job *j = it->second.get();
    auto q = std::find(s->pending.begin(), s->pending.end(), j);
    if (q == s->pending.end()) return QSES_ERR_UNSUPPORTED;  // in a batch already (or done)
    s->pending.erase(q);
    j->status = QSES_ERR_CANCELLED;
    j->t_start = j->t_done = Clock::now();
    j->done = true;
    j->xyz.clear();
    j->xyz.shrink_to_fit();
    j->r.clear();
    j->r.shrink_to_fit();
    s->cv_done.notify_all();
    return QSES_OK;
}

QSES_API int qses_server_stats(qses_server *s, unsigned long long *out, int max) {
    if (!s || !out) return 0;
    std::lock_guard<std::mutex> lock(s->mu);
    const unsigned long long v[5] = {s->batches, s->served, s->max_batch_seen, s->max_inflight_lanes,
                                     (unsigned long long)s->pending.size()};
    int k = 0;
    for (; k < max && k < 5; k++) out[k] = v[k];
    return k;
}

QSES_API int qses_server_destroy(qses_server *s) {
    if (!s) return QSES_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    for (auto &kv : s->jobs) qses_mesh_release(&kv.second->mesh);  // results never collected
    for (auto *c : s->ctxs) qses_context_destroy(c);
    delete s;
    return QSES_OK;
}

}  // extern "C"
