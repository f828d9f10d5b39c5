// Host orchestration of the SES pipeline on one GPU (one context = one stream).
//
// Replaces computeSlicedSES / computeMarchingCubes (CudaSurf.cu:373-776).  The reference
// walks 300^3 slices serially with ~6 host syncs, cudaMalloc/cudaFree and thrust calls per
// slice, and smooths on the host; here the whole grid is one set of launches into a
// context-owned workspace that is reused across calls, with four small count read-backs.
// The mesh is the reference's single-slice result (its output for -s >= grid size).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"
#include "prims.h"
#include "qses_context.h"

namespace qses {

// ------------------------------------------------------------------ sizing

// Field value of code n: probe - dx * sqrt(n) (distanceFieldRefine, Kernels.cu:540-541),
// evaluated in double and rounded once, so the sign is exact (float arithmetic would give
// 0.0 instead of -4.5e-8 at dx = 0.2, n = 49 and flip the marching-cubes corner).
static float code_value(float probe, float dx, int n) {
    return (float)((double)probe - (double)dx * std::sqrt((double)n));
}

int grid_from_bounds(const float mn_in[3], const float mx_in[3], float maxR_in, unsigned n, float dx, QGrid &g,
                     qses_grid_info *info, std::string *why) {
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
    if (!(gnb_f >= 1 && gnb_f <= 1290 && G_f >= 1 && G_f <= 4096)) {
        if (why) *why = "grid too large (more than 4096 voxels or 1290 neighbour cells per axis)";
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
    if (g.Rq >= (1ll << 21)) {
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
    return g_tuned[batch][b] ? g_tune[batch][b] : GsShape();
}

void gs_shape_record(unsigned nv, bool batch, GsShape sh) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = tune_bucket(nv);
    g_tune[batch][b] = sh;
    g_tuned[batch][b] = true;
}

static int g_edt_tune[2][16];  // [tuned?][log2 G]

int edt_shape(int G) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = std::min(bits_for((unsigned)G), 15);
    return g_edt_tune[0][b] ? g_edt_tune[1][b] : 0;
}

void edt_shape_record(int G, int shape) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const int b = std::min(bits_for((unsigned)G), 15);
    g_edt_tune[0][b] = 1;
    g_edt_tune[1][b] = shape;
}

int gs_shape_candidates(GsShape *out, int max) {
    static const unsigned targets[] = {4096, 16384, 25000};
    static const unsigned flags[] = {0, kGsL1Positions, kGsPersistL2, kGsPersistL2 | kGsL1Positions};
    int k = 0;
    for (int t : {512, 1024})
        for (unsigned tg : targets)
            for (unsigned f : flags)
                if (k < max) out[k++] = GsShape{t, tg, f};
    return k;
}

// ------------------------------------------------------------------ arena

int Arena::reserve(size_t bytes) {
    off = 0;
    if (bytes <= cap) return QSES_OK;
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

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

int run_smoothing(qses_context *ctx, const GsShape &sh, int passes, float *vq, float4 *pos4, unsigned nv,
                  const uint2 *deg, const unsigned *nbr, unsigned short *cnt, int *remote, unsigned *inbox,
                  unsigned *inbox_tail, int *d_err, unsigned long long *stats, bool record_slabs,
                  cudaEvent_t before_writeback) {
    cudaStream_t s = ctx->stream;
    const int pmax = std::min(gs_slab_max_blocks(ctx->device, kGsSlabMaxVerts, sh.threads), 1024);
    if (pmax < 1) return ctx->fail(QSES_ERR_NO_DEVICE, "the smoothing kernel does not fit on this device");
    unsigned long long cap = (unsigned long long)pmax * kGsSlabMaxVerts;
    if (sh.wave && sh.wave < cap) cap = sh.wave;
    const unsigned nwaves = (unsigned)((nv + cap - 1) / cap);
    const unsigned wsize = (nv + nwaves - 1) / nwaves;  // balanced waves
    launch_to_float4(vq, nv, pos4, s);
    ctx->launches++;
    if (sh.flags & kGsPersistL2) gs_l2_window(ctx->device, s, pos4, 16ull * nv);
    if (stats) QCHK(cudaMemsetAsync(stats, 0, 64, s));
    for (int pass = 0; pass < passes; pass++) {
        for (unsigned v0 = 0; v0 < nv; v0 += wsize) {
            const unsigned v1 = std::min(nv, v0 + wsize), nw = v1 - v0;
            int P = (int)std::min<unsigned>((nw + sh.target - 1) / sh.target, (unsigned)pmax);
            if (P < 1) P = 1;
            unsigned S = (nw + P - 1) / P;
            if (S > kGsSlabMaxVerts) {
                P = (int)((nw + kGsSlabMaxVerts - 1) / kGsSlabMaxVerts);
                S = (nw + P - 1) / P;
            }
            launch_gs_setup(deg, nbr, v0, v1, S, cnt, remote, s);
            ctx->launches++;
            QCHK(cudaMemsetAsync(inbox, 0xff, 4ull * P * S, s));
            QCHK(cudaMemsetAsync(inbox_tail, 0, 4ull * P, s));
            QCHK(launch_gs_slab(pos4, v0, v1, S, P, sh.threads, sh.flags, deg, nbr, cnt, remote, inbox, inbox_tail,
                                d_err, 4000000000ll, stats, s));
            ctx->launches++;
            if (record_slabs) {
                ctx->diag[0] = std::max<unsigned long long>(ctx->diag[0], (unsigned long long)P);
                ctx->diag[1] = std::max<unsigned long long>(ctx->diag[1], (unsigned long long)S);
            }
        }
    }
    if (sh.flags & kGsPersistL2) gs_l2_window(ctx->device, s, nullptr, 0);
    if (before_writeback) QCHK(cudaStreamWaitEvent(s, before_writeback, 0));
    launch_from_float4(pos4, nv, vq, s);
    ctx->launches++;
    return QSES_OK;
}

int run_pipeline(qses_context *ctx, const qses_params &p, const float *d_xyz, const float *d_r, unsigned n) {
    cudaStream_t s = ctx->stream;
    ctx->launches = 0;
    for (auto &m : ctx->marks) cudaEventDestroy(m.second);
    ctx->marks.clear();
    ctx->mesh = DeviceMesh();
    ctx->have_grid = false;
    memset(ctx->diag, 0, sizeof(ctx->diag));
    QCHK(cudaMemsetAsync((char *)ctx->small + 256, 0, 64, ctx->stream));
    ctx->mark("start");

    // ---- bounds (one read-back) and sizing on the host
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
    QGrid g;
    std::string why;
    int rc = grid_from_bounds(mn, mx, maxR, n, p.voxel, g, &ctx->info, &why);
    if (rc != QSES_OK) return ctx->fail(rc, why.c_str());
    ctx->grid = g;
    ctx->have_grid = true;

    // ---- field workspace
    const size_t ncell = (size_t)g.gnb * g.gnb * g.gnb;
    const size_t nmask = (size_t)g.G * g.G * g.W;
    const size_t ncode = (size_t)g.G * g.G * g.Gp;
    const size_t E = (size_t)g.Gc + 1, nrow = E * E;
    const int atom_bits = bits_for(ncell ? ncell - 1 : 0);
    size_t tmpA = std::max(radix_sort_tmp_bytes(n, atom_bits), scan_u2_tmp_bytes((unsigned)nrow));
    size_t needA = align256(4ull * n) * 4 + align256(16ull * n) + align256(8 * ncell) + 3 * align256(4 * nmask) +
                   align256(ncode) + align256(1024) + 2 * align256(8 * nrow) + align256(tmpA) + 4096;
    if (ctx->field.reserve(needA) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "field workspace");
    Arena &A = ctx->field;
    unsigned *key = (unsigned *)A.take(4ull * n), *key2 = (unsigned *)A.take(4ull * n);
    unsigned *idx = (unsigned *)A.take(4ull * n), *idx2 = (unsigned *)A.take(4ull * n);
    float4 *atoms = (float4 *)A.take(16ull * n);
    uint2 *cells = (uint2 *)A.take(8 * ncell);
    unsigned *inMask = (unsigned *)A.take(4 * nmask), *outMask = (unsigned *)A.take(4 * nmask);
    unsigned *signMask = (unsigned *)A.take(4 * nmask);
    unsigned char *codes = (unsigned char *)A.take(ncode);
    float *d_lut = (float *)A.take(1024);
    uint2 *rows = (uint2 *)A.take(8 * nrow);
    uint2 *d_tot = (uint2 *)A.take(64);
    void *tmp = A.take(tmpA);
    float h_lut[256];
    fill_lut(g, h_lut);
    memcpy(ctx->h_small + 64, h_lut, sizeof(h_lut));
    QCHK(cudaMemcpyAsync(d_lut, ctx->h_small + 64, sizeof(h_lut), cudaMemcpyHostToDevice, s));

    // ---- atoms: cell keys, stable radix sort, sorted xyzr + cell ranges
    launch_atom_hash(g, d_xyz, n, key, s);
    ctx->launches++;
    int alt = 0;
    QCHK(radix_sort<unsigned>(key, key2, idx, idx2, n, atom_bits, true, tmp, d_err, s, &ctx->launches, &alt));
    unsigned *skey = alt ? key2 : key, *sidx = alt ? idx2 : idx;
    QCHK(cudaMemsetAsync(cells, 0, 8 * ncell, s));
    launch_atom_gather(d_xyz, d_r, skey, sidx, n, atoms, cells, s);
    ctx->launches++;
    ctx->mark("atoms");

    // ---- SES field
    launch_sas(g, atoms, cells, inMask, outMask, s);
    ctx->launches++;
    ctx->mark("sas");
    ctx->edt_used = ctx->edt_force >= 0 ? ctx->edt_force : edt_shape(g.G);
    launch_edt(g, inMask, outMask, codes, signMask, s, ctx->edt_used);
    ctx->launches++;
    ctx->mark("refine");

    // ---- marching cubes: per-row counts, scan, totals
    launch_mc_count(g, signMask, rows, s);
    ctx->launches++;
    QCHK(scan_u2(rows, rows, (unsigned)nrow, d_tot, tmp, d_err, s, &ctx->launches));
    QCHK(cudaMemcpyAsync(ctx->h_small, d_tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
    QCHK(cudaMemcpyAsync(ctx->h_small + 8, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    QCHK(cudaStreamSynchronize(s));
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
                   align256(4ull * NE) + align256(12ull * NE) + 2 * align256(4ull * NE) + 2 * align256(4 * n3) +
                   2 * align256(4 * n3) + align256(8 * n3) + 3 * align256(4ull * NE) + align256(4ull * NE + 4096) + 4096 +
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
    unsigned *okey = (unsigned *)B.take(4 * n3 + 4), *okey2 = (unsigned *)B.take(4 * n3 + 4);
    unsigned *oval = (unsigned *)B.take(4 * n3 + 4), *oval2 = (unsigned *)B.take(4 * n3 + 4);
    unsigned *nbr = (unsigned *)B.take(8 * n3 + 8);
    int *lower = (int *)B.take(4ull * NE + 4), *cnt = (int *)B.take(4ull * NE + 4);
    unsigned *inbox = (unsigned *)B.take(4ull * NE + 4096);
    unsigned *inbox_tail = (unsigned *)B.take(4096);
    float4 *pos4 = (float4 *)B.take(16ull * NE + 16);
    void *tmpb = B.take(tmpB);
    uint2 *tflags = (uint2 *)B.take(8ull * T + 16);      // degenerate filter (side stream)
    void *tmp2 = B.take(scan_u2_tmp_bytes(T + 1));       // its scan's scratch
    if (!tmpb || !tflags || !tmp2) return ctx->fail(QSES_ERR_INTERNAL, "mesh workspace layout");

    // ---- triangles + pre-weld vertex keys
    launch_mc_emit(g, signMask, codes, d_lut, rows, tri, vk, s);
    ctx->launches++;
    ctx->mark("mc_emit");

    // ---- weld: sort keys, unique, rank, remap triangle corners
    unsigned nv = 0;
    if (NE > 0) {
        QCHK(radix_sort<unsigned long long>(vk, vk2, vv, vv2, NE, key_bits, true, tmpb, d_err, s, &ctx->launches, &alt));
        unsigned long long *sk = alt ? vk2 : vk;
        unsigned *sv = alt ? vv2 : vv;
        launch_weld_flags(sk, NE, flags, s);
        ctx->launches++;
        QCHK(scan_u2(flags, flags, NE, d_tot, tmpb, d_err, s, &ctx->launches));
        launch_weld_scatter(g, sk, sv, flags, NE, vmap, vq, s);
        ctx->launches++;
        launch_remap(tri, n3, vmap, s);
        ctx->launches++;
        QCHK(cudaMemcpyAsync(ctx->h_small, d_tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
        QCHK(cudaStreamSynchronize(s));
        memcpy(&tot, ctx->h_small, sizeof(tot));
        nv = tot.x;
    }
    ctx->mark("weld");

    // Closest atom, degenerate filter and (for host results) the triangle and atom-id
    // downloads run on the side stream while the main stream builds the neighbour lists and
    // smooths; profiled calls keep one stream so the stage times stay separable.
    const bool fork = !ctx->profiling && ctx->side != nullptr;
    cudaStream_t sd = fork ? ctx->side : s;
    const bool keep_all = (p.flags & QSES_FLAG_KEEP_DEGENERATE) != 0;
    HostDownload &dl = ctx->dl;
    if (dl.want) {  // [vertices | triangles (pre-filter count) | atom_sorted | atom_input]
        dl.vb = 12ull * nv;
        dl.tb = 12ull * T;
        dl.ab = 4ull * nv;
        dl.block = pinned_take(dl.vb + dl.tb + 2 * dl.ab + 64, &dl.bytes);
        if (!dl.block) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned host mesh");
    }
    if (fork) {
        QCHK(cudaEventRecord(ctx->ev_fork, s));
        QCHK(cudaStreamWaitEvent(sd, ctx->ev_fork, 0));
    }

    // ---- closest atom per welded vertex (before smoothing, as in the reference)
    if (nv > 0) {
        launch_closest(g, vq, nv, atoms, cells, sidx, asorted, ainput, sd);
        ctx->launches++;
    }
    ctx->mark("closest_atom");

    // ---- drop degenerate triangles (API_computeSES filter)
    if (!keep_all && T > 0) {
        launch_tri_flags(tri, T, tflags, sd);
        ctx->launches++;
        QCHK(scan_u2(tflags, tflags, T, d_tot, tmp2, d_err, sd, &ctx->launches));
        launch_tri_compact(tri, T, tflags, tri_kept, sd);
        ctx->launches++;
        QCHK(cudaMemcpyAsync(ctx->h_small, d_tot, sizeof(uint2), cudaMemcpyDeviceToHost, sd));
    }
    ctx->mark("filter");
    const unsigned *tri_out = keep_all ? tri : tri_kept;
    if (dl.want) {
        char *hb = (char *)dl.block;
        if (dl.tb) QCHK(cudaMemcpyAsync(hb + dl.vb, tri_out, dl.tb, cudaMemcpyDeviceToHost, sd));
        if (dl.ab) QCHK(cudaMemcpyAsync(hb + dl.vb + dl.tb, asorted, dl.ab, cudaMemcpyDeviceToHost, sd));
        if (dl.ab) QCHK(cudaMemcpyAsync(hb + dl.vb + dl.tb + dl.ab, ainput, dl.ab, cudaMemcpyDeviceToHost, sd));
        dl.d2h = dl.tb + 2 * dl.ab;
    }
    if (fork) QCHK(cudaEventRecord(ctx->ev_join, sd));

    // ---- Gauss-Seidel smoothing on the device
    if (p.smooth_passes > 0 && nv > 0 && T > 0) {
        uint2 *deg = flags;  // reuse: nv + 1 <= NE + 1 entries
        QCHK(cudaMemsetAsync(deg, 0, 8ull * (nv + 1), s));
        launch_degree(tri, n3, nv, deg, s);
        ctx->launches++;
        QCHK(scan_u2(deg, deg, nv + 1, nullptr, tmpb, d_err, s, &ctx->launches));
        launch_copy_keys(tri, n3, okey, s);
        ctx->launches++;
        QCHK(radix_sort<unsigned>(okey, okey2, oval, oval2, (unsigned)n3, bits_for(nv - 1), true, tmpb, d_err, s,
                                  &ctx->launches, &alt));
        unsigned *socc = alt ? oval2 : oval;
        launch_csr_fill(tri, socc, n3, nbr, s);
        ctx->launches++;
        ctx->mark("smooth_csr");
        const GsShape sh = ctx->gs_force.threads ? ctx->gs_force : gs_shape(nv, false);
        ctx->gs_used = sh;
        unsigned long long *stats = (unsigned long long *)((char *)ctx->small + 256);
        // the closest-atom pass on the side stream reads the welded positions in vq
        int rc2 = run_smoothing(ctx, sh, p.smooth_passes, vq, pos4, nv, deg, nbr, (unsigned short *)cnt, lower, inbox,
                                inbox_tail, d_err, stats, true, fork ? ctx->ev_join : nullptr);
        if (rc2) return rc2;
    }
    ctx->mark("smooth");
    if (dl.want && dl.vb) {
        QCHK(cudaMemcpyAsync(dl.block, vq, dl.vb, cudaMemcpyDeviceToHost, s));
        dl.d2h += dl.vb;
    }
    if (fork) QCHK(cudaStreamWaitEvent(s, ctx->ev_join, 0));

    QCHK(cudaMemcpyAsync(ctx->h_small + 8, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    QCHK(cudaMemcpyAsync(ctx->h_small + 2048, (char *)ctx->small + 256, 64, cudaMemcpyDeviceToHost, s));
    QCHK(cudaStreamSynchronize(s));
    ctx->mark("download");
    memcpy(ctx->diag + 2, ctx->h_small + 2048, 7 * sizeof(unsigned long long));
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
    m.codes = codes;
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

void qses_context::mark(const char *name) {
    if (!profiling) return;
    cudaEvent_t ev;
    cudaEventCreate(&ev);
    cudaEventRecord(ev, stream);
    marks.push_back({name, ev});
}
