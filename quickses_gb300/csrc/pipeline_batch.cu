// Host orchestration of a batch: many molecules (or trajectory frames) of uneven size in one
// pass through the pipeline on one stream.
//
// The reference has no batch form: a caller loops over API_computeSES, and every call
// re-runs its per-slice loop (CudaSurf.cu:653-754) with its own allocations and syncs.  Here
// the molecules' grids are sized on the host, their atoms uploaded in one copy, and every
// stage is one launch over all of them:
//   * atoms of every molecule are cell-sorted by one stable radix sort (cell keys offset by
//     each molecule's first cell), so each molecule sees exactly its own sorted order;
//   * the field runs as persistent CTAs pulling (molecule, tile) items from one device
//     work counter;
//   * marching-cubes rows are numbered molecule after molecule, so one scan gives each
//     molecule a contiguous range of triangles and edge slots;
//   * weld keys carry the molecule above the local key bits, so one sort + unique welds
//     every molecule separately and numbers its vertices contiguously in its own order;
//   * Gauss-Seidel runs as one dataflow over all molecules (no dependency crosses a
//     molecule, so each molecule is smoothed exactly as alone, and the critical path is the
//     deepest molecule, not the sum), in waves of at most 152 x 25 000 vertices.
// Per-molecule arithmetic is the single-molecule path's: the same tile bodies, the same
// row body, the same keys and the same update order.
#include <algorithm>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "prims.h"
#include "qses_context.h"
#include "segment.h"

namespace qses {

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

static size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

// Pinned host staging that grows geometrically and stays with the context.
static int stage_reserve(qses_context *ctx, size_t bytes) {
    if (bytes <= ctx->h_stage_cap) return QSES_OK;
    ctx->host_gen++;
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    ctx->h_stage_cap = 0;
    const size_t want = bytes + bytes / 2 + (1 << 20);
    if (cudaMallocHost(&ctx->h_stage, want) != cudaSuccess) {
        cudaGetLastError();
        ctx->h_stage = nullptr;
        return QSES_ERR_OUT_OF_MEMORY;
    }
    ctx->h_stage_cap = want;
    return QSES_OK;
}

// ---- segment 1: descriptors and atoms up, atoms sorted into cells, field, row counts
struct BatchFieldSeg {
    unsigned long long mem;  // free counters of the buffers it uses
    const char *h_desc;  // pinned staging; the copy nodes read it when the segment runs
    char *d_desc;
    const float *h_x;
    float *d_x;
    unsigned long long desc_bytes, atom_bytes;
    unsigned *key, *key2, *idx, *idx2;
    float4 *atoms;
    uint2 *cells;
    unsigned *in_mask, *out_mask, *sign_mask;
    unsigned char *codes, *zd;  // zd: z distances of the refine (scratch)
    uint2 *rows, *tot;
    unsigned *counters;
    void *tmp;
    int *err;
    unsigned *tri_off, *edge_off;
    unsigned char *h_out;  // pinned: [0, 8) totals, [8, 12) error word
    unsigned long long cell_tot, n_rows;
    unsigned n, tiles, units, words;
    int cell_bits, pad_;
    QBatch b;
};

static int enqueue_batch_field(qses_context *ctx, const BatchFieldSeg &a, SegOut &o) {
    cudaStream_t s = ctx->stream;
    QCHK(cudaMemcpyAsync(a.d_desc, a.h_desc, a.desc_bytes, cudaMemcpyHostToDevice, s));
    QCHK(cudaMemcpyAsync(a.d_x, a.h_x, a.atom_bytes, cudaMemcpyHostToDevice, s));
    QCHK(cudaMemsetAsync(a.err, 0, sizeof(int), s));
    QCHK(cudaMemsetAsync(a.counters, 0, 64, s));
    // atoms
    launch_atom_hash_batch(a.b, a.d_x, a.n, a.key, s);
    ctx->launches++;
    QCHK(radix_sort<unsigned>(a.key, a.key2, a.idx, a.idx2, a.n, a.cell_bits, true, a.tmp, a.err, s, &ctx->launches,
                              &o.alt));
    const unsigned *skey = o.alt ? a.key2 : a.key, *sidx = o.alt ? a.idx2 : a.idx;
    QCHK(cudaMemsetAsync(a.cells, 0, 8 * a.cell_tot, s));
    launch_atom_gather(a.d_x, a.d_x + 3ull * a.n, skey, sidx, a.n, a.atoms, a.cells, s);
    ctx->launches++;
    ctx->mark("atoms");
    // field: persistent CTAs over (molecule, tile) items
    launch_sas_batch(a.b, a.tiles, a.atoms, a.cells, a.in_mask, a.out_mask, a.counters, s);
    ctx->launches++;
    ctx->mark("sas");
    launch_edt_batch(a.b, a.tiles, a.in_mask, a.out_mask, a.codes, a.sign_mask, a.counters + 1, s, a.words, a.zd);
    ctx->launches += 2;
    ctx->mark("refine");
    // marching-cubes counts, one scan over all rows, per-molecule offsets
    launch_mc_count_batch(a.b, a.units, a.sign_mask, a.rows, s);
    ctx->launches++;
    QCHK(scan_u2(a.rows, a.rows, (unsigned)a.n_rows, a.tot, a.tmp, a.err, s, &ctx->launches));
    launch_gather_offsets(a.rows, a.b.row_off, a.b.n_mol, (unsigned)a.n_rows, a.tot, a.tri_off, a.edge_off, s);
    ctx->launches++;
    QCHK(cudaMemcpyAsync(a.h_out, a.tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
    QCHK(cudaMemcpyAsync(a.h_out + 8, a.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    return QSES_OK;
}

// ---- segment 2: triangles and molecule-tagged weld keys, one weld for all molecules
struct BatchMeshSeg {
    unsigned long long mem;  // free counters of the buffers it uses
    const unsigned *sign_mask;
    const unsigned char *codes;
    const uint2 *rows;
    unsigned *tri;
    unsigned long long *vk, *vk2;
    unsigned *vv, *vv2;
    uint2 *flags, *tot;
    unsigned *vmap;
    float *vq;
    unsigned *vmol;
    void *tmp;
    int *err;
    unsigned *edge_off, *vtx_off;
    unsigned char *h_out;  // pinned: [0, 8) vertex total
    void *h_vtx;           // pinned: per-molecule first vertex
    unsigned long long n3;
    unsigned units, ne;
    int tot_bits, pad_;
    QBatch b;
};

static int enqueue_batch_mesh(qses_context *ctx, const BatchMeshSeg &m, SegOut &o) {
    cudaStream_t s = ctx->stream;
    const unsigned nm = m.b.n_mol;
    launch_mc_emit_batch(m.b, m.units, m.sign_mask, m.codes, m.rows, m.tri, m.vk, s);
    ctx->launches++;
    ctx->mark("mc_emit");
    if (m.ne > 0) {
        QCHK(radix_sort<unsigned long long>(m.vk, m.vk2, m.vv, m.vv2, m.ne, m.tot_bits, true, m.tmp, m.err, s,
                                            &ctx->launches, &o.alt));
        const unsigned long long *sk = o.alt ? m.vk2 : m.vk;
        const unsigned *sv = o.alt ? m.vv2 : m.vv;
        launch_weld_flags(sk, m.ne, m.flags, s);
        ctx->launches++;
        QCHK(scan_u2(m.flags, m.flags, m.ne, m.tot, m.tmp, m.err, s, &ctx->launches));
        launch_weld_scatter_batch(m.b, sk, sv, m.flags, m.ne, m.vmap, m.vq, m.vmol, s);
        ctx->launches++;
        // molecule k's edges occupy sorted positions [edge_off[k], edge_off[k+1]) (its keys
        // sort between the other molecules'), so its first vertex is the rank there
        launch_gather_offsets(m.flags, m.edge_off, nm, m.ne, m.tot, m.vtx_off, nullptr, s);
        ctx->launches++;
        launch_remap(m.tri, m.n3, m.vmap, s);
        ctx->launches++;
    } else {
        QCHK(cudaMemsetAsync(m.vtx_off, 0, 4ull * (nm + 1), s));
    }
    QCHK(cudaMemcpyAsync(m.h_out, m.tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
    QCHK(cudaMemcpyAsync(m.h_vtx, m.vtx_off, 4ull * (nm + 1), cudaMemcpyDeviceToHost, s));
    return QSES_OK;
}

// ---- segment 3: closest atom, per-molecule filter and host downloads on the side stream;
// neighbour lists and one Gauss-Seidel dataflow over all molecules on the main stream
struct BatchFinishSeg {
    unsigned long long mem;  // free counters of the buffers it uses
    const float4 *atoms;
    const uint2 *cells;
    const unsigned *sidx, *vmol;
    int *asorted, *ainput;
    float *vq;
    unsigned *tri, *tri_kept;
    uint2 *tflags;
    void *tmp2;
    uint2 *tot;
    int *err;
    unsigned *tri_off, *kept_off;
    unsigned char *h_out;  // pinned: [0, 8) kept triangles, [8, 12) error word
    void *h_kept;          // pinned: per-molecule first kept triangle
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
    unsigned long long n3;
    unsigned nv, nt;
    int passes, fork;
    GsShape sh;
    GsLaunch gl;
    QBatch b;
};

static int enqueue_batch_finish(qses_context *ctx, const BatchFinishSeg &c, SegOut &o) {
    cudaStream_t s = ctx->stream, sd = c.fork ? ctx->side : s;
    const unsigned nm = c.b.n_mol;
    if (c.fork) {
        QCHK(cudaEventRecord(ctx->ev_fork, s));
        QCHK(cudaStreamWaitEvent(sd, ctx->ev_fork, 0));
    }
    if (c.nv > 0) {
        launch_closest_batch(c.b, c.vq, c.vmol, c.nv, c.atoms, c.cells, c.sidx, c.asorted, c.ainput, sd);
        ctx->launches++;
    }
    ctx->mark("closest_atom");
    // per-molecule filter and molecule-local corner ids
    if (c.nt > 0) {
        launch_tri_flags_batch(c.b, c.tri, c.nt, c.tflags, sd);
        ctx->launches++;
        QCHK(scan_u2(c.tflags, c.tflags, c.nt, c.tot, c.tmp2, c.err, sd, &ctx->launches));
        launch_tri_compact_batch(c.b, c.tri, c.nt, c.tflags, c.tri_kept, sd);
        ctx->launches++;
        launch_gather_offsets(c.tflags, c.tri_off, nm, c.nt, c.tot, c.kept_off, nullptr, sd);
        ctx->launches++;
    } else {
        QCHK(cudaMemsetAsync(c.kept_off, 0, 4ull * (nm + 1), sd));
        QCHK(cudaMemsetAsync(c.tot, 0, sizeof(uint2), sd));
    }
    QCHK(cudaMemcpyAsync(c.h_out, c.tot, sizeof(uint2), cudaMemcpyDeviceToHost, sd));
    QCHK(cudaMemcpyAsync(c.h_kept, c.kept_off, 4ull * (nm + 1), cudaMemcpyDeviceToHost, sd));
    ctx->mark("filter");
    // triangles and atom ids to the host: beside the smoothing when forked, else (stage
    // timing) in the download stage
    auto download_rest = [&](cudaStream_t q) -> int {
        if (c.dl_tb) QCHK(cudaMemcpyAsync(c.h_dl + c.dl_vb, c.tri_kept, c.dl_tb, cudaMemcpyDeviceToHost, q));
        if (c.dl_ab) QCHK(cudaMemcpyAsync(c.h_dl + c.dl_vb + c.dl_tb, c.asorted, c.dl_ab, cudaMemcpyDeviceToHost, q));
        if (c.dl_ab)
            QCHK(cudaMemcpyAsync(c.h_dl + c.dl_vb + c.dl_tb + c.dl_ab, c.ainput, c.dl_ab, cudaMemcpyDeviceToHost, q));
        return QSES_OK;
    };
    if (c.h_dl && c.fork) QCHK_RC(download_rest(sd));
    if (c.fork) QCHK(cudaEventRecord(ctx->ev_join, sd));

    // Gauss-Seidel over all molecules
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
                                     c.home, c.table, c.h_table, c.inbox, c.inbox_tail, c.err, nullptr,
                                     c.fork ? ctx->ev_join : nullptr);
        if (rc) return rc;
    }
    ctx->mark("smooth");
    if (c.h_dl && c.dl_vb) QCHK(cudaMemcpyAsync(c.h_dl, c.vq, c.dl_vb, cudaMemcpyDeviceToHost, s));
    if (c.h_dl && !c.fork) QCHK_RC(download_rest(s));
    if (c.fork) QCHK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
    QCHK(cudaMemcpyAsync(c.h_out + 8, c.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    return QSES_OK;
}

int run_batch(qses_context *ctx, const BatchItem *items, unsigned count, int passes, int key_bits) {
    cudaStream_t s = ctx->stream;
    QSES_SEG_TRACE("batch: %u molecules, %d passes\n", count, passes);
    memset(ctx->timeline, 0, sizeof(ctx->timeline));
    ctx->tick(-1);
    ctx->launches = 0;
    for (auto &m : ctx->marks) cudaEventDestroy(m.second);
    ctx->marks.clear();
    ctx->mesh = DeviceMesh();
    ctx->have_grid = false;
    ctx->slice_nv.clear();
    ctx->slice_nt.clear();
    BatchResult &R = ctx->batch;
    R = BatchResult();
    if (count == 0) return QSES_OK;
    ctx->mark("start");

    // ---- per-molecule layout on the host
    const unsigned nm = count;
    std::vector<QMol> mols(nm);
    std::vector<unsigned> tile_off(nm + 1), atom_off(nm + 1), row_off(nm + 1), unit_off(nm + 1), word_off(nm + 1);
    unsigned long long mask_tot = 0, code_tot = 0, cell_tot = 0, tiles = 0, rows = 0, atoms_tot = 0, units = 0;
    for (unsigned m = 0; m < nm; m++) {
        const QGrid &g = items[m].g;
        QMol &q = mols[m];
        memset(&q, 0, sizeof(q));
        q.g = g;
        q.mask_off = mask_tot;
        q.code_off = code_tot;
        q.atom_off = (unsigned)atoms_tot;
        q.cell_off = (unsigned)cell_tot;
        q.row_off = (unsigned)rows;
        q.flags = items[m].flags;
        tile_off[m] = (unsigned)tiles;
        atom_off[m] = (unsigned)atoms_tot;
        row_off[m] = (unsigned)rows;
        unit_off[m] = (unsigned)units;
        word_off[m] = (unsigned)mask_tot;
        mask_tot += (unsigned long long)g.G * g.G * g.W;
        code_tot += (unsigned long long)g.G * g.G * g.Gp;
        cell_tot += (unsigned long long)g.gnb * g.gnb * g.gnb;
        tiles += (unsigned long long)g.W * ((g.G + 7) / 8) * ((g.G + 7) / 8);
        const unsigned long long r = (unsigned long long)(g.Gc + 1) * (g.Gc + 1);
        const unsigned long long rpw = (unsigned long long)mc_rows_per_warp(g.Gc);
        rows += r;
        units += (r + rpw - 1) / rpw;
        atoms_tot += items[m].n;
    }
    tile_off[nm] = (unsigned)tiles;
    atom_off[nm] = (unsigned)atoms_tot;
    row_off[nm] = (unsigned)rows;
    unit_off[nm] = (unsigned)units;
    word_off[nm] = (unsigned)mask_tot;
    if (tiles >= (1ull << 31) || rows >= (1ull << 31) || cell_tot >= (1ull << 31) || atoms_tot >= (1ull << 30) ||
        mask_tot >= (1ull << 32))
        return ctx->fail(QSES_ERR_UNSUPPORTED, "batch too large for 32-bit item indices; split it");
    const unsigned N = (unsigned)atoms_tot;

    // ---- pinned staging: descriptor block then atoms, one copy each
    const size_t desc_bytes = a256(sizeof(QMol) * nm) + 9 * a256(4ull * (nm + 1)) + a256(1024ull * nm);
    const size_t atom_bytes = 16ull * N;
    if (stage_reserve(ctx, desc_bytes + atom_bytes + 256) != QSES_OK)
        return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned batch staging");
    char *hs = (char *)ctx->h_stage;
    memset(hs, 0, desc_bytes);
    size_t o = 0;
    auto hput = [&](const void *src, size_t bytes) {
        if (src) memcpy(hs + o, src, bytes);
        o += a256(bytes);
    };
    hput(mols.data(), sizeof(QMol) * nm);
    hput(tile_off.data(), 4ull * (nm + 1));
    hput(atom_off.data(), 4ull * (nm + 1));
    hput(row_off.data(), 4ull * (nm + 1));
    hput(unit_off.data(), 4ull * (nm + 1));
    hput(word_off.data(), 4ull * (nm + 1));
    hput(nullptr, 4ull * (nm + 1));  // tri_off   (device-filled)
    hput(nullptr, 4ull * (nm + 1));  // edge_off  (device-filled)
    hput(nullptr, 4ull * (nm + 1));  // vtx_off   (device-filled)
    hput(nullptr, 4ull * (nm + 1));  // kept_off  (device-filled)
    {
        float *lut = (float *)(hs + o);
        for (unsigned m = 0; m < nm; m++) fill_lut(items[m].g, lut + 256ull * m);
        o += a256(1024ull * nm);
    }
    float *hx = (float *)(hs + desc_bytes);
    float *hr = hx + 3ull * N;
    for (unsigned m = 0; m < nm; m++) {
        memcpy(hx + 3ull * atom_off[m], items[m].xyz, 12ull * items[m].n);
        memcpy(hr + atom_off[m], items[m].r, 4ull * items[m].n);
    }

    // ---- field workspace
    const int cell_bits = bits_for(cell_tot ? cell_tot - 1 : 0);
    const size_t tmpA = std::max(radix_sort_tmp_bytes(N, cell_bits), scan_u2_tmp_bytes((unsigned)rows));
    const size_t needA = desc_bytes + a256(16ull * N) + 4 * a256(4ull * N) + a256(16ull * N) + a256(8 * cell_tot) +
                         3 * a256(4 * mask_tot) + 2 * a256(code_tot) + a256(8 * rows) + 2 * a256(64) + a256(tmpA) + 8192;
    if (ctx->field.reserve(needA) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "batch field workspace");
    Arena &A = ctx->field;
    BatchFieldSeg a;
    memset(&a, 0, sizeof(a));
    a.mem = ctx->field.gen + ctx->host_gen;
    a.h_desc = hs;
    a.d_desc = (char *)A.take(desc_bytes);
    a.h_x = hx;
    a.d_x = (float *)A.take(16ull * N);
    a.desc_bytes = desc_bytes;
    a.atom_bytes = atom_bytes;
    QBatch &b = a.b;
    unsigned *d_edge_off, *d_kept_off;
    {
        size_t q = 0;
        auto at = [&](size_t bytes) {
            char *p = a.d_desc + q;
            q += a256(bytes);
            return p;
        };
        const size_t ob = 4ull * (nm + 1);
        b.mols = (const QMol *)at(sizeof(QMol) * nm);
        b.tile_off = (const unsigned *)at(ob);
        b.atom_off = (const unsigned *)at(ob);
        b.row_off = (const unsigned *)at(ob);
        b.mc_unit_off = (const unsigned *)at(ob);
        b.word_off = (const unsigned *)at(ob);
        b.tri_off = (const unsigned *)at(ob);
        d_edge_off = (unsigned *)at(ob);
        b.vtx_off = (const unsigned *)at(ob);
        d_kept_off = (unsigned *)at(ob);
        b.lut = (const float *)at(1024ull * nm);
        b.n_mol = nm;
        b.key_bits = key_bits;
    }
    unsigned *d_tri_off = (unsigned *)b.tri_off, *d_vtx_off = (unsigned *)b.vtx_off;
    a.key = (unsigned *)A.take(4ull * N);
    a.key2 = (unsigned *)A.take(4ull * N);
    a.idx = (unsigned *)A.take(4ull * N);
    a.idx2 = (unsigned *)A.take(4ull * N);
    a.atoms = (float4 *)A.take(16ull * N);
    a.cells = (uint2 *)A.take(8 * cell_tot);
    a.in_mask = (unsigned *)A.take(4 * mask_tot);
    a.out_mask = (unsigned *)A.take(4 * mask_tot);
    a.sign_mask = (unsigned *)A.take(4 * mask_tot);
    a.codes = (unsigned char *)A.take(code_tot);
    a.zd = (unsigned char *)A.take(code_tot);
    a.words = (unsigned)mask_tot;
    a.rows = (uint2 *)A.take(8 * rows);
    a.tot = (uint2 *)A.take(64);
    a.counters = (unsigned *)A.take(64);
    a.tmp = A.take(tmpA);
    if (!a.tmp) return ctx->fail(QSES_ERR_INTERNAL, "batch field workspace layout");
    int *d_err = (int *)((char *)ctx->small + 64);
    a.err = d_err;
    a.tri_off = d_tri_off;
    a.edge_off = d_edge_off;
    a.h_out = ctx->h_small;
    a.cell_tot = cell_tot;
    a.n_rows = rows;
    a.n = N;
    a.tiles = (unsigned)tiles;
    a.units = (unsigned)units;
    a.cell_bits = cell_bits;
    SegOut oa;
    ctx->tick(0);
    QCHK_RC(run_segment(ctx, kSegBatchField, a, oa, enqueue_batch_field));
    const unsigned *sidx = oa.alt ? a.idx2 : a.idx;
    unsigned *hsm = (unsigned *)ctx->h_small;  // 4 KB pinned: totals and the error word
    QCHK(cudaStreamSynchronize(s));
    ctx->tick(1);
    ctx->mark("mc_count");
    if (hsm[2]) return ctx->fail((int)hsm[2], "device wait in the batch field stage");
    const unsigned T = hsm[0], NE = hsm[1];

    // ---- mesh workspace
    const int mol_bits = bits_for(nm - 1);
    const int tot_bits = key_bits + mol_bits;
    const size_t n3 = 3ull * T;
    const int vbits = bits_for(NE ? NE - 1 : 0);
    const size_t tmpB = std::max({radix_sort_tmp_bytes(NE, tot_bits), radix_sort_tmp_bytes((unsigned)n3, vbits),
                                  scan_u2_tmp_bytes(NE), scan_u2_tmp_bytes(T), scan_u2_tmp_bytes(NE + 1)});
    const size_t nflag = std::max<size_t>((size_t)NE + 1, (size_t)T) + 1;
    const size_t needB = 2 * a256(4 * n3 + 4) + 2 * a256(8ull * NE + 8) + 2 * a256(4ull * NE + 4) +
                         a256(8ull * nflag) + a256(4ull * NE + 4) + a256(12ull * NE + 12) + 3 * a256(4ull * NE + 4) +
                         a256(4 * n3 + 4) + a256(8 * n3 + 8) + 3 * a256(4ull * NE + 4) + a256(16ull * NE + 16) + a256(tmpB) + a256(8ull * T + 16) +
                         a256(scan_u2_tmp_bytes(T + 1)) + 8192;
    if (ctx->mesh_ws.reserve(needB) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "batch mesh workspace");
    Arena &B = ctx->mesh_ws;
    unsigned *tri = (unsigned *)B.take(4 * n3 + 4);
    unsigned *tri_kept = (unsigned *)B.take(4 * n3 + 4);
    unsigned long long *vk = (unsigned long long *)B.take(8ull * NE + 8), *vk2 = (unsigned long long *)B.take(8ull * NE + 8);
    unsigned *vv = (unsigned *)B.take(4ull * NE + 4), *vv2 = (unsigned *)B.take(4ull * NE + 4);
    uint2 *flags = (uint2 *)B.take(8ull * nflag);
    unsigned *vmap = (unsigned *)B.take(4ull * NE + 4);
    float *vq = (float *)B.take(12ull * NE + 12);
    unsigned *vmol = (unsigned *)B.take(4ull * NE + 4);
    int *asorted = (int *)B.take(4ull * NE + 4), *ainput = (int *)B.take(4ull * NE + 4);
    unsigned *okey = (unsigned *)B.take(4 * n3 + 4);
    unsigned *nbr = (unsigned *)B.take(8 * n3 + 8);
    int *lower = (int *)B.take(4ull * NE + 4), *cnt = (int *)B.take(4ull * NE + 4);
    float4 *pos4 = (float4 *)B.take(16ull * NE + 16);
    void *tmpb = B.take(tmpB);
    uint2 *tflags = (uint2 *)B.take(8ull * T + 16);  // degenerate filter (side stream)
    void *tmp2 = B.take(scan_u2_tmp_bytes(T + 1));   // its scan's scratch
    if (!tmpb || !tflags || !tmp2) return ctx->fail(QSES_ERR_INTERNAL, "batch mesh workspace layout");

    // ---- triangles + molecule-tagged weld keys, then one weld for all molecules
    BatchMeshSeg mb;
    memset(&mb, 0, sizeof(mb));
    mb.mem = ctx->field.gen + ctx->mesh_ws.gen + ctx->host_gen;
    mb.sign_mask = a.sign_mask;
    mb.codes = a.codes;
    mb.rows = a.rows;
    mb.tri = tri;
    mb.vk = vk;
    mb.vk2 = vk2;
    mb.vv = vv;
    mb.vv2 = vv2;
    mb.flags = flags;
    mb.tot = a.tot;
    mb.vmap = vmap;
    mb.vq = vq;
    mb.vmol = vmol;
    mb.tmp = tmpb;
    mb.err = d_err;
    mb.edge_off = d_edge_off;
    mb.vtx_off = d_vtx_off;
    mb.h_out = ctx->h_small;
    mb.h_vtx = ctx->h_stage;
    mb.n3 = n3;
    mb.units = (unsigned)units;
    mb.ne = NE;
    mb.tot_bits = tot_bits;
    mb.b = b;
    SegOut ob;
    ctx->tick(2);
    QCHK_RC(run_segment(ctx, kSegBatchMesh, mb, ob, enqueue_batch_mesh));
    QCHK(cudaStreamSynchronize(s));
    ctx->tick(3);
    std::vector<unsigned> vtx_off(nm + 1);
    memcpy(vtx_off.data(), ctx->h_stage, 4ull * (nm + 1));
    const unsigned nv = NE > 0 ? hsm[0] : 0;
    ctx->mark("weld");

    // Closest atom, filter and (for host results) the triangle and atom-id downloads run on
    // the side stream beside the neighbour-list build and the smoothing; profiled calls keep
    // one stream so the stage times stay separable.
    HostDownload &dl = ctx->dl;
    if (dl.want) {  // [vertices | triangles (pre-filter count) | atom_sorted | atom_input]
        dl.vb = 12ull * nv;
        dl.tb = 12ull * T;
        dl.ab = 4ull * nv;
        dl.block = pinned_take(dl.vb + dl.tb + 2 * dl.ab + 256, &dl.bytes);
        if (!dl.block) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned batch meshes");
        dl.d2h = dl.vb + dl.tb + 2 * dl.ab;
    }
    BatchFinishSeg c;
    memset((void *)&c, 0, sizeof(c));  // padding too: the key is compared bytewise
    c.atoms = a.atoms;
    c.cells = a.cells;
    c.sidx = sidx;
    c.vmol = vmol;
    c.asorted = asorted;
    c.ainput = ainput;
    c.vq = vq;
    c.tri = tri;
    c.tri_kept = tri_kept;
    c.tflags = tflags;
    c.tmp2 = tmp2;
    c.tot = a.tot;
    c.err = d_err;
    c.tri_off = d_tri_off;
    c.kept_off = d_kept_off;
    c.h_out = ctx->h_small;
    c.h_kept = ctx->h_stage;
    if (dl.want) {
        c.h_dl = (char *)dl.block;
        c.dl_vb = dl.vb;
        c.dl_tb = dl.tb;
        c.dl_ab = dl.ab;
    }
    c.deg = flags;
    c.okey = okey;
    c.nbr = nbr;
    c.tmpb = tmpb;
    c.pos4 = pos4;
    c.cnt = (unsigned short *)cnt;
    c.lower = lower;
    c.n3 = n3;
    c.nv = nv;
    c.nt = T;
    c.passes = passes;
    c.fork = !ctx->profiling && ctx->side != nullptr;
    const bool smoothing = passes > 0 && nv > 0 && T > 0;
    if (smoothing) {
        c.sh = ctx->gs_force.threads ? ctx->gs_force : gs_shape(std::min<unsigned>(nv, 152u * kGsSlabMaxVerts), true);
        ctx->gs_used = c.sh;
        // molecules are never split between slabs unless larger than one; their grid sizes
        // estimate the dependency depths that order the slabs
        std::vector<int> depth(nm);
        for (unsigned m = 0; m < nm; m++) depth[m] = items[m].g.G;
        GsPlan plan;
        const int rp = gs_plan(ctx->device, c.sh, nv, vtx_off.data(), depth.data(), nm, plan);
        if (rp != QSES_OK) return ctx->fail(rp, "smoothing slab plan");
        GsBuffers gb;
        QCHK_RC(gs_buffers(ctx, plan, nv, gb));
        c.gl = plan.L;
        c.home = gb.home;
        c.table = gb.table;
        c.h_table = ctx->h_gs;
        c.inbox = gb.inbox;
        c.inbox_tail = gb.inbox_tail;
        ctx->diag[0] = std::max<unsigned long long>(ctx->diag[0], plan.max_slabs);
        ctx->diag[1] = std::max<unsigned long long>(ctx->diag[1], plan.max_len);
    }
    c.b = b;
    c.mem = ctx->field.gen + ctx->mesh_ws.gen + ctx->gs_ws.gen + ctx->host_gen + pinned_frees();
    SegOut oc;
    ctx->tick(4);
    // an L2 persistence window is a stream attribute, set when the launch is enqueued
    QCHK_RC(run_segment(ctx, kSegBatchFinish, c, oc, enqueue_batch_finish, !(smoothing && (c.sh.flags & kGsPersistL2))));
    QCHK(cudaStreamSynchronize(s));
    ctx->tick(5);
    ctx->mark("download");
    if (hsm[2]) return ctx->fail((int)hsm[2], "device wait in the batch mesh stage");
    const unsigned nkept = hsm[0];
    std::vector<unsigned> kept_off(nm + 1);
    memcpy(kept_off.data(), ctx->h_stage, 4ull * (nm + 1));

    R.n_mol = nm;
    R.nv = nv;
    R.nkept = nkept;
    R.vtx_off = vtx_off;
    R.kept_off = kept_off;
    R.vertices = vq;
    R.triangles = tri_kept;
    R.atom_sorted = asorted;
    R.atom_input = ainput;
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
