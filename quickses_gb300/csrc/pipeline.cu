// Host orchestration of the SES pipeline on one GPU (one context = one stream).
//
// Replaces computeSlicedSES / computeMarchingCubes (CudaSurf.cu:373-776).  The reference
// walks 300^3 slices serially with ~6 host syncs, cudaMalloc/cudaFree and thrust calls per
// slice, and smooths on the host; here the whole grid is one set of launches into a
// context-owned workspace that is reused across calls, with four small count read-backs.
// The mesh is the reference's single-slice result (its output for -s >= grid size).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"
#include "prims.h"
#include "qses_context.h"
#include "segment.h"

namespace qses {

// ------------------------------------------------------------------ sizing

// Field value of code n: probe - dx * sqrt(n) (distanceFieldRefine, Kernels.cu:540-541),
// evaluated in double and rounded once, so the sign is exact (float arithmetic would give
// 0.0 instead of -4.5e-8 at dx = 0.2, n = 49 and flip the marching-cubes corner).
static float code_value(float probe, float dx, int n) {
    return (float)((double)probe - (double)dx * std::sqrt((double)n));
}

int grid_from_bounds(const float mn_in[3], const float mx_in[3], float maxR_in, unsigned n, float dx, QGrid &g,
                     qses_grid_info *info, std::string *why, bool sliced) {
    if (!(dx > 0.0f) || !std::isfinite(dx)) {
        if (why) *why = "voxel size must be a positive finite number";
        return QSES_ERR_INVALID_ARG;
    }
    // getMinMax starts from +-100000 (CudaSurf.cu:154-155).
    float mn[3], mx[3];
    for (int c = 0; c < 3; c++) {
        mn[c] = std::min(100000.0f, mn_in[c]);
        mx[c] = std::max(-100000.0f, mx_in[c]);
    }
    const float maxR = std::max(0.0f, maxR_in);
    const float probe = QSES_PROBE;
    // computeMaxDist (CudaSurf.cu:250-253) and the sizing of CudaSurf.cu:548-562, 629.
    const float maxDist = std::max(mx[0] - mn[0], std::max(mx[1] - mn[1], mx[2] - mn[2])) + (2 * maxR) + (4 * probe);
    memset(&g, 0, sizeof(g));
    g.cell = probe + maxR;
    g.ox = mn[0] - maxR - probe;
    g.oy = mn[1] - maxR - probe;
    g.oz = mn[2] - maxR - probe;
    g.dx = dx;
    g.probe = probe;
    g.N = n;
    const double gnb_f = std::ceil(maxDist / g.cell), G_f = std::ceil(maxDist / dx), R_f = std::ceil(probe / dx);
    // A sliced grid is only ever held one slice box at a time, so only its neighbour cells
    // bound it.
    const double G_max = sliced ? 1048576.0 : 4096.0;
    if (!(gnb_f >= 1 && gnb_f <= 1290 && G_f >= 1 && G_f <= G_max)) {
        if (why) *why = sliced ? "grid too large (more than 1290 neighbour cells per axis)"
                               : "grid too large (more than 4096 voxels or 1290 neighbour cells per axis)";
        return QSES_ERR_UNSUPPORTED;
    }
    g.gnb = (int)gnb_f;
    g.G = (int)G_f;
    g.R = (int)R_f;
    if (g.R > QSES_RMAX) {
        if (why) *why = "voxel size below 0.156 A (refine window above 9 voxels) is not supported";
        return QSES_ERR_UNSUPPORTED;
    }
    // countVertexPerCell's single-slice cell range (MarchingCubes.cu:578-604).
    int lim = g.G - 1;
    if (g.G - g.R - 1 >= 0) lim = std::min(lim, g.G - g.R - 1);
    if (g.G - 2 * g.R - 1 >= 0) lim = std::min(lim, g.G - 2 * g.R - 1);
    g.Gc = std::max(lim, 0);
    for (int a = 0; a < 3; a++) {
        g.off[a] = 0;
        g.lim[a] = g.G - 1;  // Kernels.cu:436-441: the last layer is never computed
        g.clo[a] = 0;
        g.chi[a] = g.Gc;
    }
    g.W = (g.G + 31) / 32;
    g.Gp = 32 * g.W;
    // Code values and the first negative one (the value is non-increasing in n).
    g.negmin = 253;
    for (int c = 0; c <= 3 * g.R * g.R && c < 253; c++) {
        float v = code_value(probe, dx, c);
        if (v < 0.0f) {
            g.negmin = c;
            break;
        }
    }
    // Weld key: quantised position relative to the quantised origin, mixed radix Rq.
    const double extent = (double)g.G * (double)dx;
    if (std::fabs((double)g.ox) + extent > 16000.0 || std::fabs((double)g.oy) + extent > 16000.0 ||
        std::fabs((double)g.oz) + extent > 16000.0) {
        if (why) *why = "coordinates beyond +-16000 A are not supported (0.001 A weld quantum)";
        return QSES_ERR_UNSUPPORTED;
    }
    g.Rq = (long long)std::ceil(extent / 0.001) + 64;
    if (!sliced && g.Rq >= (1ll << 21)) {  // a slice box gets its own key base and radix
        if (why) *why = "grid extent above 2000 A is not supported by the 63-bit weld key";
        return QSES_ERR_UNSUPPORTED;
    }
    g.bx = (long long)roundf(g.ox / QSES_WELD_TOL) - 16;
    g.by = (long long)roundf(g.oy / QSES_WELD_TOL) - 16;
    g.bz = (long long)roundf(g.oz / QSES_WELD_TOL) - 16;
    if (info) {
        info->origin[0] = g.ox; info->origin[1] = g.oy; info->origin[2] = g.oz;
        info->cell = g.cell; info->dx = dx; info->probe = probe; info->max_radius = maxR;
        info->max_dist = maxDist; info->gnb = g.gnb; info->G = g.G; info->R = g.R; info->Gc = g.Gc; info->W = g.W;
    }
    return QSES_OK;
}

void fill_lut(const QGrid &g, float *lut) {
    for (int c = 0; c < 256; c++) lut[c] = -g.dx;
    for (int c = 0; c <= 3 * g.R * g.R && c < 253; c++) lut[c] = code_value(g.probe, g.dx, c);
    lut[QSES_CODE_NONE] = -g.dx;
    lut[QSES_CODE_IN] = -g.dx;
    lut[QSES_CODE_OUT] = g.probe;
}

// ------------------------------------------------------------------ tuning

// Process-wide Gauss-Seidel shapes per (mode, log2 of the vertex count), filled by the
// autotuner (qses_autotune*); absent entries use the default shape.
static std::mutex g_tune_mu;
static GsShape g_tune[2][33];
static bool g_tuned[2][33];

static int tune_bucket(unsigned nv) { return bits_for(nv); }

GsShape gs_shape(unsigned nv, bool batch) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = tune_bucket(nv);
    if (g_tuned[batch][b]) return g_tune[batch][b];
    // untuned: the shapes the tuner picks on balls of 1 000 - 50 000 atoms and on batches
    // (two vertex updates per worker warp: 14.1 -> 13.0 ms on a served batch of 23 M vertices)
    return batch ? GsShape{1024, 25000, kGsL1Positions | kGsPair, 0} : GsShape{1024, 4096, kGsL1Positions, 0};
}

void gs_shape_record(unsigned nv, bool batch, GsShape sh) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = tune_bucket(nv);
    g_tune[batch][b] = sh;
    g_tuned[batch][b] = true;
}

void gs_shape_record_all(bool batch, GsShape sh) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (int b = 0; b < 33; b++) {
        g_tune[batch][b] = sh;
        g_tuned[batch][b] = true;
    }
}

static int g_edt_tune[2][16];  // [tuned?][log2 G]

int edt_shape(int G) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = std::min(bits_for((unsigned)G), 15);
    // untuned: 16 x 16 z-rows per tile on large grids (664^3: 1.05 ms against 1.21 ms for
    // 8 x 8), 8 x 8 on small ones
    return g_edt_tune[0][b] ? g_edt_tune[1][b] : G >= 256 ? 2 : 0;
}

void edt_shape_record(int G, int shape) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = std::min(bits_for((unsigned)G), 15);
    g_edt_tune[0][b] = 1;
    g_edt_tune[1][b] = shape;
}

int gs_shape_candidates(GsShape *out, int max) {
    static const unsigned targets[] = {4096, 8192, 16384, 25000};
    // the persisting-L2 window (kGsPersistL2) is left to callers that force it: it changes
    // stream attributes (its segment then runs outside CUDA graphs) and its reset after the
    // pass costs more than the pass gains
    static const unsigned flags[] = {0,          kGsL1Positions,          kGsL1Prefetch,          kGsL1Prefetch | kGsL1Positions,
                                     kGsSmemPos, kGsSmemPos | kGsL1Positions, kGsSmemPos | kGsL1Prefetch,
                                     kGsSmemPos | kGsL1Prefetch | kGsL1Positions};
    // two vertices per worker warp with the two policies the one-vertex warps are tuned to:
    // positions through L1, with or without the slab's own in shared memory (four vertices
    // per warp, kGsQuad, measured slower than two on single molecules and batches alike)
    static const unsigned group_flags[] = {kGsPair | kGsL1Positions, kGsPair | kGsSmemPos | kGsL1Positions};
    int k = 0;
    for (int t : {512, 1024})
        for (unsigned tg : targets) {
            for (unsigned f : flags)
                if (k < max) out[k++] = GsShape{t, tg, f};
            for (unsigned f : group_flags)
                if (k < max) out[k++] = GsShape{t, tg, f};
        }
    return k;
}

// ------------------------------------------------------------------ arena

// Test hook: the next n workspace reservations fail as if the device were out of memory.
std::atomic<unsigned> g_fail_reserves{0};

int Arena::reserve(size_t bytes) {
    off = 0;
    for (unsigned f = g_fail_reserves.load(); f > 0;)
        if (g_fail_reserves.compare_exchange_weak(f, f - 1)) return QSES_ERR_OUT_OF_MEMORY;
    if (bytes <= cap) return QSES_OK;
    gen++;
    if (base) cudaFree(base);
    base = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 4 + (1 << 20);
    if (cudaMalloc(&base, want) != cudaSuccess) {
        cudaGetLastError();
        base = nullptr;
        return QSES_ERR_OUT_OF_MEMORY;
    }
    cap = want;
    return QSES_OK;
}

void *Arena::take(size_t bytes) {
    size_t o = (off + 255) & ~(size_t)255;
    if (o + bytes > cap) return nullptr;
    off = o + bytes;
    return (char *)base + o;
}

void Arena::release() {
    gen++;
    if (base) cudaFree(base);
    base = nullptr;
    cap = off = 0;
}

// ------------------------------------------------------------------ pipeline

#define QCHK(expr)                                                                      \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) return ctx->fail(QSES_ERR_CUDA, #expr, e_);              \
    } while (0)

#define QCHK_RC(expr)                                                                   \
    do {                                                                                \
        const int rc_ = (expr);                                                         \
        if (rc_ != QSES_OK) return rc_;                                                 \
    } while (0)

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

static unsigned ceil_div(unsigned long long a, unsigned long long b) { return (unsigned)((a + b - 1) / b); }

int gs_plan(int device, const GsShape &sh, unsigned nv, const unsigned *mol_off, const int *mol_depth, unsigned nm,
            GsPlan &pl) {
    // resident slab CTAs: one molecule's slabs may hold up to the largest slab; a batch's at
    // most the target, so smaller targets fit more CTAs per SM
    const bool single = mol_off == nullptr || nm <= 1;
    const unsigned cap = (sh.flags & kGsSmemPos) ? kGsSmemPosMaxVerts : kGsSlabMaxVerts;
    const unsigned smax = single && !(sh.flags & kGsSmemPos) ? cap : std::min(std::max(sh.target, 256u), cap);
    const int pmax = std::min(gs_slab_max_blocks(device, smax, sh.threads, sh.flags), 1024);
    if (pmax < 1) return QSES_ERR_NO_DEVICE;
    return gs_plan_for(pmax, sh, nv, mol_off, mol_depth, nm, pl);
}

int gs_plan_for(int pmax, const GsShape &sh, unsigned nv, const unsigned *mol_off, const int *mol_depth, unsigned nm,
                GsPlan &pl) {
    pl = GsPlan();
    if (pmax < 1 || nv == 0) return QSES_ERR_INVALID_ARG;
    // with the slab's positions in shared memory (kGsSmemPos) slabs hold at most 8192
    // vertices and a molecule may have more slabs than there are resident CTAs
    const bool spos = (sh.flags & kGsSmemPos) != 0;
    const unsigned Smax = spos ? kGsSmemPosMaxVerts : kGsSlabMaxVerts;
    const unsigned t = std::min(std::max(sh.target, 256u), Smax);
    const bool single = mol_off == nullptr || nm <= 1;
    const unsigned cap = sh.wave ? std::max(sh.wave, 1u) : nv;
    GsLaunch &L = pl.L;
    L.waves = ceil_div(nv, cap);
    L.wsize = ceil_div(nv, L.waves);  // balanced waves
    // slabs of one molecule of len vertices: spread over at most pmax CTAs, at least t per slab,
    // at most Smax per slab
    auto pieces = [&](unsigned len) {
        if (spos) return ceil_div(len, t);
        return std::max(ceil_div(len, Smax), std::min(ceil_div(len, t), (unsigned)pmax));
    };
    if (single) {
        L.qcap = pieces(L.wsize);
        L.smax = 0;
        for (unsigned w = 0; w < L.waves; w++) {
            const unsigned nw = std::min(nv, (w + 1) * L.wsize) - w * L.wsize;
            L.smax = std::max(L.smax, ceil_div(nw, pieces(nw)));
            L.qcap = std::max(L.qcap, pieces(nw));
        }
    } else {
        // split molecules: ceil(len / t) slabs of at most t each (at most len / t + 1); packed
        // runs of small molecules: at most 2 (run / t) + 1 (two neighbouring packed slabs hold
        // more than t), and at most one run more than there are split molecules
        L.qcap = 3 * ceil_div(L.wsize, t) + 2 * nm + 2;
        L.smax = t;
    }
    L.ctas = (int)std::min<unsigned>((unsigned)pmax, L.qcap);
    L.table_words = (unsigned)gs_table_words(L.qcap);
    pl.table.assign((size_t)L.waves * L.table_words, 0u);

    struct Slab {
        unsigned a, b;
        float when;  // expected start: fraction of the molecule before the slab x its depth
        int depth;
    };
    std::vector<Slab> slabs;
    std::vector<unsigned> ord;
    for (unsigned w = 0; w < L.waves; w++) {
        const unsigned v0 = w * L.wsize, v1 = std::min(nv, v0 + L.wsize);
        slabs.clear();
        auto split = [&](unsigned s0, unsigned s1, int depth) {
            const unsigned len = s1 - s0, k = single ? pieces(len) : ceil_div(len, t), S = ceil_div(len, k);
            for (unsigned a = s0; a < s1; a += S)
                slabs.push_back({a, std::min(s1, a + S), (float)((double)(a - s0) / len * depth), depth});
        };
        if (single) {
            split(v0, v1, 1);
        } else {
            unsigned pa = 0, pb = 0;  // pending packed slab [pa, pb)
            auto flush = [&]() {
                if (pb > pa) slabs.push_back({pa, pb, 0.0f, 0});
                pa = pb = 0;
            };
            for (unsigned m = 0; m < nm; m++) {
                const unsigned s0 = std::max(mol_off[m], v0), s1 = std::min(mol_off[m + 1], v1);
                if (s1 <= s0) continue;
                const unsigned len = s1 - s0;
                if (len > t) {
                    flush();
                    split(s0, s1, mol_depth ? std::max(mol_depth[m], 1) : 1);
                } else {
                    if (pb > pa && (pb - pa) + len > t) flush();
                    if (pb == pa) pa = s0;
                    pb = s1;
                }
            }
            flush();
        }
        const unsigned Q = (unsigned)slabs.size();
        if (Q == 0 || Q > L.qcap || slabs.front().a != v0 || slabs.back().b != v1) return QSES_ERR_INTERNAL;
        unsigned *tb = pl.table.data() + (size_t)w * L.table_words;
        tb[0] = Q;
        for (unsigned q = 0; q < Q; q++) {
            if (slabs[q].b - slabs[q].a > L.smax || (q && slabs[q].a != slabs[q - 1].b)) return QSES_ERR_INTERNAL;
            tb[1 + q] = slabs[q].a;
            pl.max_len = std::max(pl.max_len, slabs[q].b - slabs[q].a);
        }
        tb[1 + Q] = v1;
        // CTAs take slabs in order of expected start (ties: deeper molecule, then id).  Within a
        // molecule the expected start grows with the id, so a slab is always taken after the
        // lower slabs it waits for.
        ord.resize(Q);
        for (unsigned q = 0; q < Q; q++) ord[q] = q;
        std::sort(ord.begin(), ord.end(), [&](unsigned x, unsigned y) {
            if (slabs[x].when != slabs[y].when) return slabs[x].when < slabs[y].when;
            if (slabs[x].depth != slabs[y].depth) return slabs[x].depth > slabs[y].depth;
            return x < y;
        });
        for (unsigned q = 0; q < Q; q++) tb[2 + L.qcap + q] = ord[q];
        pl.max_slabs = std::max(pl.max_slabs, Q);
    }
    return QSES_OK;
}

int gs_buffers(qses_context *ctx, const GsPlan &pl, unsigned nv, GsBuffers &out) {
    const GsLaunch &L = pl.L;
    const size_t words = pl.table.size();
    const size_t need = align256(8ull * nv + 8) + align256(4 * words) + align256(4ull * (L.wsize + L.smax + 64)) +
                        align256(4ull * (L.qcap + 2)) + 4096;
    const void *old_ws = ctx->gs_ws.base;
    if (ctx->gs_ws.reserve(need) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "smoothing workspace");
    if (ctx->gs_ws.base != old_ws) QSES_SEG_TRACE("smoothing workspace moved (%zu bytes)\n", need);
    out.home = (uint2 *)ctx->gs_ws.take(8ull * nv + 8);
    out.table = (unsigned *)ctx->gs_ws.take(4 * words);
    out.inbox = (unsigned *)ctx->gs_ws.take(4ull * (L.wsize + L.smax + 64));
    out.inbox_tail = (unsigned *)ctx->gs_ws.take(4ull * (L.qcap + 2));  // per slab, then the slab counter
    if (!out.inbox_tail) return ctx->fail(QSES_ERR_INTERNAL, "smoothing workspace layout");
    if (4 * words > ctx->h_gs_cap) {
        QSES_SEG_TRACE("slab tables: pinned buffer grows to %zu words\n", words);
        ctx->host_gen++;
        if (ctx->h_gs) cudaFreeHost(ctx->h_gs);
        ctx->h_gs = nullptr;
        ctx->h_gs_cap = 0;
        const size_t want = 4 * words + 2 * words + 4096;
        if (cudaMallocHost((void **)&ctx->h_gs, want) != cudaSuccess) {
            cudaGetLastError();
            ctx->h_gs = nullptr;
            return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned slab tables");
        }
        ctx->h_gs_cap = want;
    }
    memcpy(ctx->h_gs, pl.table.data(), 4 * words);
    return QSES_OK;
}

int run_smoothing(qses_context *ctx, const GsShape &sh, const GsLaunch &L, int passes, float *vq, float4 *pos4,
                  unsigned nv, const uint2 *deg, const unsigned *nbr, unsigned short *cnt, int *remote, uint2 *home,
                  unsigned *table, const unsigned *h_table, unsigned *inbox, unsigned *inbox_tail, int *d_err,
                  unsigned long long *stats, cudaEvent_t before_writeback) {
    cudaStream_t s = ctx->stream;
    launch_to_float4(vq, nv, pos4, s);
    ctx->launches++;
    if (sh.flags & kGsPersistL2) gs_l2_window(ctx->device, s, pos4, 16ull * nv);
    if (stats) QCHK(cudaMemsetAsync(stats, 0, 64, s));
    QCHK(cudaMemcpyAsync(table, h_table, 4ull * L.waves * L.table_words, cudaMemcpyHostToDevice, s));
    for (int pass = 0; pass < passes; pass++) {
        for (unsigned w = 0; w < L.waves; w++) {
            const unsigned v0 = w * L.wsize, v1 = std::min(nv, v0 + L.wsize);
            const unsigned *tb = table + (size_t)w * L.table_words;
            launch_gs_setup(deg, nbr, v0, v1, tb, cnt, remote, home, s);
            ctx->launches++;
            QCHK(cudaMemsetAsync(inbox, 0xff, 4ull * (v1 - v0), s));
            QCHK(cudaMemsetAsync(inbox_tail, 0, 4ull * (L.qcap + 1), s));
            // per-update cycle counters only on profiled calls: their clock reads sit on the
            // dependency chain (1.4 % of the pass on 50 000 atoms)
            QCHK(launch_gs_slab(pos4, v0, v1, L.smax, tb, L.qcap, inbox_tail + L.qcap, home, L.ctas, sh.threads,
                                sh.flags, sh.hot, deg, nbr, cnt, remote, inbox, inbox_tail, d_err, 4000000000ll,
                                ctx->profiling ? stats : nullptr, s));
            ctx->launches++;
        }
    }
    if (sh.flags & kGsPersistL2) gs_l2_window(ctx->device, s, nullptr, 0);
    if (before_writeback) QCHK(cudaStreamWaitEvent(s, before_writeback, 0));
    launch_from_float4(pos4, nv, vq, s);
    ctx->launches++;
    return QSES_OK;
}

// ---- segment 1: atoms sorted into cells, SES field codes, marching-cubes row counts
struct FieldSeg {
    unsigned long long mem;  // free counters of the buffers it uses
    const float *xyz, *r;
    unsigned *key, *key2, *idx, *idx2;
    float4 *atoms;
    uint2 *cells;
    unsigned *in_mask, *out_mask, *sign_mask;
    unsigned char *codes, *zd;  // zd: z distances of the refine (scratch)
    float *lut;
    const unsigned char *h_lut;  // pinned; the copy node reads it when the segment runs
    uint2 *rows, *tot;
    void *tmp;
    int *err;
    unsigned char *h_out;  // pinned: [0, 8) totals, [8, 12) error word
    unsigned long long ncell, nrow;
    unsigned n;
    int atom_bits, edt, pad_;
    QGrid g;
};

static int enqueue_field(qses_context *ctx, const FieldSeg &a, SegOut &o) {
    cudaStream_t s = ctx->stream;
    QCHK(cudaMemcpyAsync(a.lut, a.h_lut, 1024, cudaMemcpyHostToDevice, s));
    launch_atom_hash(a.g, a.xyz, a.n, a.key, s);
    ctx->launches++;
    QCHK(radix_sort<unsigned>(a.key, a.key2, a.idx, a.idx2, a.n, a.atom_bits, true, a.tmp, a.err, s, &ctx->launches,
                              &o.alt));
    const unsigned *skey = o.alt ? a.key2 : a.key, *sidx = o.alt ? a.idx2 : a.idx;
    QCHK(cudaMemsetAsync(a.cells, 0, 8 * a.ncell, s));
    launch_atom_gather(a.xyz, a.r, skey, sidx, a.n, a.atoms, a.cells, s);
    ctx->launches++;
    ctx->mark("atoms");
    launch_sas(a.g, a.atoms, a.cells, a.in_mask, a.out_mask, s);
    ctx->launches++;
    ctx->mark("sas");
    launch_edt(a.g, a.in_mask, a.out_mask, a.codes, a.sign_mask, s, a.edt, a.zd);
    ctx->launches++;
    ctx->launches++;
    ctx->mark("refine");
    launch_mc_count(a.g, a.sign_mask, a.rows, s);
    ctx->launches++;
    QCHK(scan_u2(a.rows, a.rows, (unsigned)a.nrow, a.tot, a.tmp, a.err, s, &ctx->launches));
    QCHK(cudaMemcpyAsync(a.h_out, a.tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
    QCHK(cudaMemcpyAsync(a.h_out + 8, a.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    return QSES_OK;
}

// ---- segment 2: triangles and pre-weld vertex keys, weld (sort, unique, rank, remap)
struct MeshSeg {
    unsigned long long mem;  // free counters of the buffers it uses
    const unsigned *sign_mask;
    const unsigned char *codes;
    const float *lut;
    const uint2 *rows;
    unsigned *tri;
    unsigned long long *vk, *vk2;
    unsigned *vv, *vv2;
    uint2 *flags, *tot;
    unsigned *vmap;
    float *vq;
    void *tmp;
    int *err;
    unsigned char *h_out;  // pinned: [0, 8) vertex total
    unsigned long long n3;
    unsigned ne;
    int key_bits;
    QGrid g;
};

static int enqueue_mesh(qses_context *ctx, const MeshSeg &b, SegOut &o) {
    cudaStream_t s = ctx->stream;
    launch_mc_emit(b.g, b.sign_mask, b.codes, b.lut, b.rows, b.tri, b.vk, s);
    ctx->launches++;
    ctx->mark("mc_emit");
    if (b.ne > 0) {
        QCHK(radix_sort<unsigned long long>(b.vk, b.vk2, b.vv, b.vv2, b.ne, b.key_bits, true, b.tmp, b.err, s,
                                            &ctx->launches, &o.alt));
        const unsigned long long *sk = o.alt ? b.vk2 : b.vk;
        const unsigned *sv = o.alt ? b.vv2 : b.vv;
        launch_weld_flags(sk, b.ne, b.flags, s);
        ctx->launches++;
        QCHK(scan_u2(b.flags, b.flags, b.ne, b.tot, b.tmp, b.err, s, &ctx->launches));
        launch_weld_scatter(b.g, sk, sv, b.flags, b.ne, b.vmap, b.vq, s);
        ctx->launches++;
        launch_remap(b.tri, b.n3, b.vmap, s);
        ctx->launches++;
        QCHK(cudaMemcpyAsync(b.h_out, b.tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
    }
    return QSES_OK;
}

// ---- segment 3: closest atom, degenerate filter and host downloads on the side stream;
// neighbour lists and Gauss-Seidel on the main stream; final read-backs
struct FinishSeg {
    unsigned long long mem;  // free counters of the buffers it uses
    const float4 *atoms;
    const uint2 *cells;
    const unsigned *sidx;
    int *asorted, *ainput;
    float *vq;
    unsigned *tri, *tri_kept;
    uint2 *tflags;
    void *tmp2;
    uint2 *tot;
    int *err;
    unsigned char *h_out;  // pinned: [0, 8) kept triangles, [8, 12) error word, [2048, 2112) stats
    char *h_dl;            // pinned host mesh block, or null
    unsigned long long dl_vb, dl_tb, dl_ab;
    uint2 *deg;
    unsigned *okey, *nbr;  // okey: the corners scattered per vertex
    void *tmpb;
    float4 *pos4;
    unsigned short *cnt;
    int *lower;
    uint2 *home;
    unsigned *table;
    const unsigned *h_table;  // pinned slab tables; the copy node reads them when the segment runs
    unsigned *inbox, *inbox_tail;
    unsigned long long *stats;
    unsigned long long n3;
    unsigned nv, nt;
    int passes, keep_all, fork, pad_;
    GsShape sh;
    GsLaunch gl;
    QGrid g;
};

static int enqueue_finish(qses_context *ctx, const FinishSeg &c, SegOut &o) {
    cudaStream_t s = ctx->stream, sd = c.fork ? ctx->side : s;
    if (c.fork) {
        QCHK(cudaEventRecord(ctx->ev_fork, s));
        QCHK(cudaStreamWaitEvent(sd, ctx->ev_fork, 0));
    }
    // closest atom per welded vertex (before smoothing, as in the reference)
    if (c.nv > 0) {
        launch_closest(c.g, c.vq, c.nv, c.atoms, c.cells, c.sidx, c.asorted, c.ainput, sd);
        ctx->launches++;
    }
    ctx->mark("closest_atom");
    // drop degenerate triangles (API_computeSES filter)
    if (!c.keep_all && c.nt > 0) {
        launch_tri_flags(c.tri, c.nt, c.tflags, sd);
        ctx->launches++;
        QCHK(scan_u2(c.tflags, c.tflags, c.nt, c.tot, c.tmp2, c.err, sd, &ctx->launches));
        launch_tri_compact(c.tri, c.nt, c.tflags, c.tri_kept, sd);
        ctx->launches++;
        QCHK(cudaMemcpyAsync(c.h_out, c.tot, sizeof(uint2), cudaMemcpyDeviceToHost, sd));
    }
    ctx->mark("filter");
    const unsigned *tri_out = c.keep_all ? c.tri : c.tri_kept;
    // triangles and atom ids to the host: beside the smoothing when forked, else (stage
    // timing) in the download stage
    auto download_rest = [&](cudaStream_t q) -> int {
        if (c.dl_tb) QCHK(cudaMemcpyAsync(c.h_dl + c.dl_vb, tri_out, c.dl_tb, cudaMemcpyDeviceToHost, q));
        if (c.dl_ab) QCHK(cudaMemcpyAsync(c.h_dl + c.dl_vb + c.dl_tb, c.asorted, c.dl_ab, cudaMemcpyDeviceToHost, q));
        if (c.dl_ab)
            QCHK(cudaMemcpyAsync(c.h_dl + c.dl_vb + c.dl_tb + c.dl_ab, c.ainput, c.dl_ab, cudaMemcpyDeviceToHost, q));
        return QSES_OK;
    };
    if (c.h_dl && c.fork) QCHK_RC(download_rest(sd));
    if (c.fork) QCHK(cudaEventRecord(ctx->ev_join, sd));

    // Gauss-Seidel smoothing on the device
    if (c.passes > 0 && c.nv > 0 && c.nt > 0) {
        // neighbour lists: count the corners per vertex, scan, scatter them per vertex, then
        // sort each vertex's few corners back into triangle order (the order
        // getNeighboorsVertices appends in) and expand them into the lists
        QCHK(cudaMemsetAsync(c.deg, 0, 8ull * (c.nv + 1), s));
        launch_csr_count(c.tri, c.n3, c.deg, s);
        ctx->launches++;
        QCHK(scan_u2(c.deg, c.deg, c.nv + 1, nullptr, c.tmpb, c.err, s, &ctx->launches));
        launch_csr_scatter(c.tri, c.n3, c.deg, c.okey, s);
        ctx->launches++;
        launch_csr_sortfill(c.tri, c.okey, c.n3, c.nv, c.deg, c.nbr, s);
        ctx->launches++;
        ctx->mark("smooth_csr");
        // the closest-atom pass on the side stream reads the welded positions in vq
        const int rc = run_smoothing(ctx, c.sh, c.gl, c.passes, c.vq, c.pos4, c.nv, c.deg, c.nbr, c.cnt, c.lower,
                                     c.home, c.table, c.h_table, c.inbox, c.inbox_tail, c.err, c.stats,
                                     c.fork ? ctx->ev_join : nullptr);
        if (rc) return rc;
    }
    ctx->mark("smooth");
    if (c.h_dl && c.dl_vb) QCHK(cudaMemcpyAsync(c.h_dl, c.vq, c.dl_vb, cudaMemcpyDeviceToHost, s));
    if (c.h_dl && !c.fork) QCHK_RC(download_rest(s));
    if (c.fork) QCHK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
    QCHK(cudaMemcpyAsync(c.h_out + 8, c.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    QCHK(cudaMemcpyAsync(c.h_out + 2048, c.stats, 64, cudaMemcpyDeviceToHost, s));
    return QSES_OK;
}

int molecule_grid(qses_context *ctx, const qses_params &p, const float *d_xyz, const float *d_r, unsigned n, QGrid &g,
                  bool sliced) {
    cudaStream_t s = ctx->stream;
    ctx->oversize = false;
    unsigned *d_mm = (unsigned *)ctx->small;
    int *d_err = (int *)((char *)ctx->small + 64);
    QCHK(cudaMemsetAsync(d_mm, 0xff, 3 * sizeof(unsigned), s));  // min encodings start high
    QCHK(cudaMemsetAsync(d_mm + 3, 0, 5 * sizeof(unsigned), s));  // max encodings start low
    QCHK(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    launch_atom_minmax(d_xyz, d_r, n, d_mm, s);
    ctx->launches++;
    QCHK(cudaGetLastError());
    unsigned *h_mm = (unsigned *)ctx->h_small;
    QCHK(cudaMemcpyAsync(h_mm, d_mm, 8 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    QCHK(cudaStreamSynchronize(s));
    auto dec = [](unsigned e) {
        unsigned b = (e & 0x80000000u) ? (e & 0x7fffffffu) : ~e;
        float f;
        memcpy(&f, &b, 4);
        return f;
    };
    float mn[3] = {dec(h_mm[0]), dec(h_mm[1]), dec(h_mm[2])}, mx[3] = {dec(h_mm[3]), dec(h_mm[4]), dec(h_mm[5])};
    float maxR = dec(h_mm[6]);
    std::string why;
    int rc = grid_from_bounds(mn, mx, maxR, n, p.voxel, g, &ctx->info, &why, sliced);
    if (rc == QSES_ERR_UNSUPPORTED && !sliced) {
        // too large for one pass: note whether the reference's slicing could take it
        QGrid gs;
        ctx->oversize = grid_from_bounds(mn, mx, maxR, n, p.voxel, gs, nullptr, nullptr, true) == QSES_OK;
    }
    if (rc != QSES_OK) return ctx->fail(rc, why.c_str());
    ctx->grid = g;
    ctx->have_grid = true;
    return QSES_OK;
}

int run_pipeline(qses_context *ctx, const qses_params &p, const float *d_xyz, const float *d_r, unsigned n) {
    cudaStream_t s = ctx->stream;
    QSES_SEG_TRACE("molecule: %u atoms, voxel %.3f, %d passes\n", n, p.voxel, p.smooth_passes);
    memset(ctx->timeline, 0, sizeof(ctx->timeline));
    ctx->tick(-1);
    ctx->launches = 0;
    for (auto &m : ctx->marks) cudaEventDestroy(m.second);
    ctx->marks.clear();
    ctx->mesh = DeviceMesh();
    ctx->have_grid = false;
    ctx->slice_nv.clear();
    ctx->slice_nt.clear();
    memset(ctx->diag, 0, sizeof(ctx->diag));
    QCHK(cudaMemsetAsync((char *)ctx->small + 256, 0, 64, ctx->stream));
    ctx->mark("start");

    // ---- bounds (one read-back) and sizing on the host
    QGrid g;
    QCHK_RC(molecule_grid(ctx, p, d_xyz, d_r, n, g, false));
    int *d_err = (int *)((char *)ctx->small + 64);
    int rc = QSES_OK;

    // ---- field workspace
    const size_t ncell = (size_t)g.gnb * g.gnb * g.gnb;
    const size_t nmask = (size_t)g.G * g.G * g.W;
    const size_t ncode = (size_t)g.G * g.G * g.Gp;
    const size_t E = (size_t)g.Gc + 1, nrow = E * E;
    const int atom_bits = bits_for(ncell ? ncell - 1 : 0);
    size_t tmpA = std::max(radix_sort_tmp_bytes(n, atom_bits), scan_u2_tmp_bytes((unsigned)nrow));
    size_t needA = align256(4ull * n) * 4 + align256(16ull * n) + align256(8 * ncell) + 3 * align256(4 * nmask) +
                   2 * align256(ncode) + align256(1024) + 2 * align256(8 * nrow) + align256(tmpA) + 4096;
    if (ctx->field.reserve(needA) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "field workspace");
    Arena &A = ctx->field;
    FieldSeg a;
    memset(&a, 0, sizeof(a));
    a.mem = ctx->input.gen + ctx->field.gen;
    a.xyz = d_xyz;
    a.r = d_r;
    a.key = (unsigned *)A.take(4ull * n);
    a.key2 = (unsigned *)A.take(4ull * n);
    a.idx = (unsigned *)A.take(4ull * n);
    a.idx2 = (unsigned *)A.take(4ull * n);
    a.atoms = (float4 *)A.take(16ull * n);
    a.cells = (uint2 *)A.take(8 * ncell);
    a.in_mask = (unsigned *)A.take(4 * nmask);
    a.out_mask = (unsigned *)A.take(4 * nmask);
    a.sign_mask = (unsigned *)A.take(4 * nmask);
    a.codes = (unsigned char *)A.take(ncode);
    a.zd = (unsigned char *)A.take(ncode);
    a.lut = (float *)A.take(1024);
    a.rows = (uint2 *)A.take(8 * nrow);
    a.tot = (uint2 *)A.take(64);
    a.tmp = A.take(tmpA);
    a.err = d_err;
    a.h_lut = ctx->h_small + 64;
    a.h_out = ctx->h_small;
    a.ncell = ncell;
    a.nrow = nrow;
    a.n = n;
    a.atom_bits = atom_bits;
    ctx->edt_used = ctx->edt_force >= 0 ? ctx->edt_force : edt_shape(g.G);
    a.edt = ctx->edt_used;
    a.g = g;
    if (!a.tmp) return ctx->fail(QSES_ERR_INTERNAL, "field workspace layout");
    fill_lut(g, (float *)(ctx->h_small + 64));
    SegOut oa;
    ctx->tick(0);
    QCHK_RC(run_segment(ctx, kSegField, a, oa, enqueue_field));
    unsigned *skey = oa.alt ? a.key2 : a.key, *sidx = oa.alt ? a.idx2 : a.idx;
    QCHK(cudaStreamSynchronize(s));
    ctx->tick(1);
    ctx->mark("mc_count");
    uint2 tot;
    memcpy(&tot, ctx->h_small, sizeof(tot));
    int herr;
    memcpy(&herr, ctx->h_small + 8, sizeof(int));
    if (herr) return ctx->fail(herr, "device wait in the field stage");
    const unsigned T = tot.x, NE = tot.y;
    ctx->mesh.n_tri_all = T;
    ctx->mesh.n_edges = NE;

    // ---- mesh workspace
    const size_t n3 = 3ull * T;
    const int key_bits = bits_for((unsigned long long)g.Rq * g.Rq * g.Rq - 1);
    const int vbits = bits_for(NE ? NE - 1 : 0);
    size_t tmpB = std::max({radix_sort_tmp_bytes(NE, key_bits), radix_sort_tmp_bytes((unsigned)n3, vbits),
                            scan_u2_tmp_bytes(NE), scan_u2_tmp_bytes(T), scan_u2_tmp_bytes(NE + 1)});
    const size_t nflag = std::max<size_t>((size_t)NE + 1, (size_t)T) + 1;
    size_t needB = 2 * align256(4 * n3) + 2 * align256(8ull * NE) + 2 * align256(4ull * NE) + align256(8ull * nflag) +
                   align256(4ull * NE) + align256(12ull * NE) + 2 * align256(4ull * NE) + align256(4 * n3 + 4) +
                   align256(8 * n3) + 3 * align256(4ull * NE) + 4096 +
                   align256(16ull * NE + 16) +
                   align256(tmpB) + align256(8ull * T + 16) + align256(scan_u2_tmp_bytes(T + 1)) + 4096;
    if (ctx->mesh_ws.reserve(needB) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "mesh workspace");
    Arena &B = ctx->mesh_ws;
    unsigned *tri = (unsigned *)B.take(4 * n3 + 4);
    unsigned *tri_kept = (unsigned *)B.take(4 * n3 + 4);
    unsigned long long *vk = (unsigned long long *)B.take(8ull * NE + 8), *vk2 = (unsigned long long *)B.take(8ull * NE + 8);
    unsigned *vv = (unsigned *)B.take(4ull * NE + 4), *vv2 = (unsigned *)B.take(4ull * NE + 4);
    uint2 *flags = (uint2 *)B.take(8ull * nflag);
    unsigned *vmap = (unsigned *)B.take(4ull * NE + 4);
    float *vq = (float *)B.take(12ull * NE + 12);
    int *asorted = (int *)B.take(4ull * NE + 4), *ainput = (int *)B.take(4ull * NE + 4);
    unsigned *okey = (unsigned *)B.take(4 * n3 + 4);
    unsigned *nbr = (unsigned *)B.take(8 * n3 + 8);
    int *lower = (int *)B.take(4ull * NE + 4), *cnt = (int *)B.take(4ull * NE + 4);
    float4 *pos4 = (float4 *)B.take(16ull * NE + 16);
    void *tmpb = B.take(tmpB);
    uint2 *tflags = (uint2 *)B.take(8ull * T + 16);      // degenerate filter (side stream)
    void *tmp2 = B.take(scan_u2_tmp_bytes(T + 1));       // its scan's scratch
    if (!tmpb || !tflags || !tmp2) return ctx->fail(QSES_ERR_INTERNAL, "mesh workspace layout");

    // ---- triangles + pre-weld vertex keys; weld
    MeshSeg b;
    memset(&b, 0, sizeof(b));
    b.mem = ctx->field.gen + ctx->mesh_ws.gen;
    b.sign_mask = a.sign_mask;
    b.codes = a.codes;
    b.lut = a.lut;
    b.rows = a.rows;
    b.tri = tri;
    b.vk = vk;
    b.vk2 = vk2;
    b.vv = vv;
    b.vv2 = vv2;
    b.flags = flags;
    b.tot = a.tot;
    b.vmap = vmap;
    b.vq = vq;
    b.tmp = tmpb;
    b.err = d_err;
    b.h_out = ctx->h_small;
    b.n3 = n3;
    b.ne = NE;
    b.key_bits = key_bits;
    b.g = g;
    SegOut ob;
    ctx->tick(2);
    QCHK_RC(run_segment(ctx, kSegMesh, b, ob, enqueue_mesh));
    unsigned nv = 0;
    if (NE > 0) {
        QCHK(cudaStreamSynchronize(s));
        memcpy(&tot, ctx->h_small, sizeof(tot));
        nv = tot.x;
    }
    ctx->tick(3);
    ctx->mark("weld");

    // Closest atom, degenerate filter and (for host results) the triangle and atom-id
    // downloads run on the side stream while the main stream builds the neighbour lists and
    // smooths; profiled calls keep one stream so the stage times stay separable.
    const bool keep_all = (p.flags & QSES_FLAG_KEEP_DEGENERATE) != 0;
    HostDownload &dl = ctx->dl;
    if (dl.want) {  // [vertices | triangles (pre-filter count) | atom_sorted | atom_input]
        dl.vb = 12ull * nv;
        dl.tb = 12ull * T;
        dl.ab = 4ull * nv;
        dl.block = pinned_take(dl.vb + dl.tb + 2 * dl.ab + 64, &dl.bytes);
        if (!dl.block) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned host mesh");
        dl.d2h = dl.vb + dl.tb + 2 * dl.ab;
    }
    FinishSeg c;
    memset((void *)&c, 0, sizeof(c));  // padding too: the key is compared bytewise
    c.atoms = a.atoms;
    c.cells = a.cells;
    c.sidx = sidx;
    c.asorted = asorted;
    c.ainput = ainput;
    c.vq = vq;
    c.tri = tri;
    c.tri_kept = tri_kept;
    c.tflags = tflags;
    c.tmp2 = tmp2;
    c.tot = a.tot;
    c.err = d_err;
    c.h_out = ctx->h_small;
    if (dl.want) {
        c.h_dl = (char *)dl.block;
        c.dl_vb = dl.vb;
        c.dl_tb = dl.tb;
        c.dl_ab = dl.ab;
    }
    c.deg = flags;  // reuse: nv + 1 <= NE + 1 entries
    c.okey = okey;
    c.nbr = nbr;
    c.tmpb = tmpb;
    c.pos4 = pos4;
    c.cnt = (unsigned short *)cnt;
    c.lower = lower;
    c.stats = (unsigned long long *)((char *)ctx->small + 256);
    c.n3 = n3;
    c.nv = nv;
    c.nt = T;
    c.passes = p.smooth_passes;
    c.keep_all = keep_all;
    c.fork = !ctx->profiling && ctx->side != nullptr;
    const bool smoothing = p.smooth_passes > 0 && nv > 0 && T > 0;
    if (smoothing) {
        c.sh = ctx->gs_force.threads ? ctx->gs_force : gs_shape(nv, false);
        c.sh.hot = kGsHotWarpsSingle;
        ctx->gs_used = c.sh;
        GsPlan plan;
        rc = gs_plan(ctx->device, c.sh, nv, nullptr, nullptr, 1, plan);
        if (rc != QSES_OK) return ctx->fail(rc, "smoothing slab plan");
        GsBuffers gb;
        QCHK_RC(gs_buffers(ctx, plan, nv, gb));
        c.gl = plan.L;
        c.home = gb.home;
        c.table = gb.table;
        c.h_table = ctx->h_gs;
        c.inbox = gb.inbox;
        c.inbox_tail = gb.inbox_tail;
        ctx->diag[0] = plan.max_slabs;
        ctx->diag[1] = plan.max_len;
    }
    c.g = g;
    c.mem = ctx->field.gen + ctx->mesh_ws.gen + ctx->gs_ws.gen + ctx->host_gen + pinned_frees();
    SegOut oc;
    ctx->tick(4);
    // an L2 persistence window is a stream attribute, set when the launch is enqueued
    QCHK_RC(run_segment(ctx, kSegFinish, c, oc, enqueue_finish, !(smoothing && (c.sh.flags & kGsPersistL2))));
    QCHK(cudaStreamSynchronize(s));
    ctx->tick(5);
    ctx->mark("download");
    memcpy(ctx->diag + 2, ctx->h_small + 2048, 8 * sizeof(unsigned long long));
    unsigned nkept = T;
    if (!keep_all && T > 0) {
        memcpy(&tot, ctx->h_small, sizeof(tot));
        nkept = tot.x;
    }
    memcpy(&herr, ctx->h_small + 8, sizeof(int));
    if (herr) return ctx->fail(herr, "device wait in the mesh stage");

    DeviceMesh &m = ctx->mesh;
    m.valid = true;
    m.nv = nv;
    m.nt = nkept;
    m.vertices = vq;
    m.triangles = keep_all ? tri : tri_kept;
    m.atom_sorted = asorted;
    m.atom_input = ainput;
    m.codes = a.codes;
    m.sorted_to_input = sidx;
    m.sorted_keys = skey;
    m.n_atoms = n;
    if (ctx->profiling) {
        cudaEventSynchronize(ctx->marks.back().second);
        ctx->times.clear();
        for (size_t q = 1; q < ctx->marks.size(); q++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ctx->marks[q - 1].second, ctx->marks[q].second);
            ctx->times.push_back({ctx->marks[q].first, ms});
        }
    }
    return QSES_OK;
}

}  // namespace qses

int qses_context::fail(int code, const char *what, cudaError_t e) {
    char buf[512];
    if (e != cudaSuccess)
        snprintf(buf, sizeof(buf), "%s: %s (%s)", qses_status_string(code), what, cudaGetErrorString(e));
    else
        snprintf(buf, sizeof(buf), "%s: %s", qses_status_string(code), what);
    last_error = buf;
    return code;
}

unsigned long long qses_context::memory_generation() const {
    return input.gen + field.gen + mesh_ws.gen + gs_ws.gen + host_gen + qses::pinned_frees();
}

void qses_context::tick(int k) {
    const auto now = std::chrono::steady_clock::now();
    if (k >= 0 && k < 6) timeline[k] = std::chrono::duration<double, std::milli>(now - tl_last).count();
    tl_last = now;
}

void qses_context::mark(const char *name) {
    if (!profiling) return;
    cudaEvent_t ev;
    cudaEventCreate(&ev);
    cudaEventRecord(ev, stream);
    marks.push_back({name, ev});
}
