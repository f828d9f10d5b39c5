// Pipeline segments replayed from CUDA graphs.
//
// A segment is the stream work between two host read-backs of a call (the counts that size
// the next buffers).  Its enqueue function reads nothing but a plain key struct - every
// pointer, count, grid, launch shape and flag it uses - and the context's fixed streams,
// events and pinned scratch; host values it produces besides the stream work (which
// ping-pong buffer holds a sort's result, launch counts, smoothing diagnostics) go to a
// SegOut.  So the key's bytes decide the whole segment:
//   * same bytes as one of the slot's cached graphs: that instantiated graph is launched
//     again (pinned host sources are read when the copy node runs, so fresh atoms and tables
//     flow in);
//   * different bytes: the segment is captured again and instantiated into a free cache
//     entry, or, with the slot's entries all taken, the least recently used executable is
//     updated in place (cudaGraphExecUpdate: same topology, new parameters), or
//     re-instantiated when the topology differs.
// Copy and memset nodes stay bound to the allocations they were captured with, even when a
// freed buffer comes back at the same address.  So every key also holds the sum of the
// free counters of the buffers its segment uses (the counters only grow), and an entry
// captured before any buffer of the context was freed is destroyed rather than updated.
// Capture runs on a private stream of the context (nothing another thread enqueues can fall
// into it, and a caller's stream is never put in capture mode); the graph is then launched on
// the context's stream.  Work on the side stream joins the capture through the fork event
// and rejoins the origin stream before the segment ends, so the graph keeps both branches.
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "qses_context.h"

namespace qses {

template <class K>
using SegFn = int (*)(qses_context *, const K &, SegOut &);

// QSES_TRACE=1 in the environment: one stderr line per graph action (for locating failures).
inline bool seg_trace() {
    static const bool on = getenv("QSES_TRACE") != nullptr;
    return on;
}
#define QSES_SEG_TRACE(...)                       \
    do {                                          \
        if (seg_trace()) {                        \
            fprintf(stderr, "[qses] " __VA_ARGS__); \
            fflush(stderr);                       \
        }                                         \
    } while (0)

// Ends a capture that the enqueue function left early on an error.
inline void abandon_capture(qses_context *ctx) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (ctx->side && cudaStreamIsCapturing(ctx->side, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
        cudaEventRecord(ctx->ev_join, ctx->side);
        cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0);
    }
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(ctx->stream, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
}

// Points ctx->stream at the capture stream for the enqueue function, and back.
struct CaptureStream {
    qses_context *ctx;
    cudaStream_t user;
    explicit CaptureStream(qses_context *c) : ctx(c), user(c->stream) { c->stream = c->capture; }
    ~CaptureStream() { ctx->stream = user; }
};

// Runs fn(ctx, key, out) through graph slot `slot` of the context, or directly when graphs
// are off, stage times are being recorded, or the segment is not graphable (it changes
// stream attributes).
template <class K>
int run_segment(qses_context *ctx, int slot, const K &key, SegOut &out, SegFn<K> fn, bool graphable = true) {
    static_assert(std::is_trivially_copyable<K>::value, "segment keys are compared as bytes");
    out = SegOut();
    const int l0 = ctx->launches;
    if (!ctx->use_graphs || ctx->profiling || !graphable || !ctx->capture) {
        const int rc = fn(ctx, key, out);
        out.launches = ctx->launches - l0;
        return rc;
    }
    const unsigned long long mem = ctx->memory_generation();
    GraphSeg *cache = ctx->seg[slot];
    cudaStream_t s = ctx->stream;
    cudaError_t e;
    const unsigned long long now = ++ctx->seg_clock;
    for (int i = 0; i < kSegCache; i++) {
        GraphSeg &c = cache[i];
        if (c.exec && c.key.size() == sizeof(K) && memcmp(c.key.data(), &key, sizeof(K)) == 0) {
            QSES_SEG_TRACE("slot %d replay entry %d\n", slot, i);
            e = cudaGraphLaunch(c.exec, s);
            if (e != cudaSuccess) return ctx->fail(QSES_ERR_CUDA, "graph launch", e);
            c.used = now;
            out = c.out;
            ctx->launches += out.launches;
            ctx->graph_stats[3]++;
            return QSES_OK;
        }
    }
    // a free entry, else the least recently used one
    int victim = 0;
    for (int i = 0; i < kSegCache; i++) {
        if (!cache[i].exec) {
            victim = i;
            break;
        }
        if (cache[i].used < cache[victim].used) victim = i;
    }
    GraphSeg &gs = cache[victim];
    gs.key.clear();
    QSES_SEG_TRACE("slot %d capture into entry %d (%s)\n", slot, victim, gs.exec ? "occupied" : "free");
    cudaGraph_t g = nullptr;
    {
        CaptureStream cs(ctx);
        e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return ctx->fail(QSES_ERR_CUDA, "graph capture", e);
        const int rc = fn(ctx, key, out);
        out.launches = ctx->launches - l0;
        if (rc != QSES_OK) {
            abandon_capture(ctx);
            return rc;
        }
        e = cudaStreamEndCapture(ctx->stream, &g);
    }
    if (e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        return ctx->fail(QSES_ERR_CUDA, "graph capture", e);
    }
    ctx->graph_stats[0]++;
    if (gs.exec && gs.mem != mem) {  // it may use freed buffers: never update it, start afresh
        QSES_SEG_TRACE("slot %d entry %d predates a freed buffer: dropped\n", slot, victim);
        cudaGraphExecDestroy(gs.exec);
        gs.exec = nullptr;
    }
    if (gs.exec) {
        cudaGraphExecUpdateResultInfo info;
        QSES_SEG_TRACE("slot %d update entry %d\n", slot, victim);
        if (cudaGraphExecUpdate(gs.exec, g, &info) == cudaSuccess) {
            ctx->graph_stats[2]++;
        } else {
            cudaGetLastError();
            cudaGraphExecDestroy(gs.exec);
            gs.exec = nullptr;
        }
    }
    if (!gs.exec) {
        QSES_SEG_TRACE("slot %d instantiate entry %d\n", slot, victim);
        e = cudaGraphInstantiate(&gs.exec, g, 0);
        if (e != cudaSuccess) {
            gs.exec = nullptr;
            gs.key.clear();
            cudaGraphDestroy(g);
            return ctx->fail(QSES_ERR_CUDA, "graph instantiate", e);
        }
        ctx->graph_stats[1]++;
    }
    cudaGraphDestroy(g);
    gs.key.assign((const unsigned char *)&key, (const unsigned char *)&key + sizeof(K));
    gs.out = out;
    gs.used = now;
    gs.mem = mem;
    QSES_SEG_TRACE("slot %d launch entry %d\n", slot, victim);
    e = cudaGraphLaunch(gs.exec, s);
    if (e != cudaSuccess) {
        gs.key.clear();
        return ctx->fail(QSES_ERR_CUDA, "graph launch", e);
    }
    return QSES_OK;
}

}  // namespace qses
