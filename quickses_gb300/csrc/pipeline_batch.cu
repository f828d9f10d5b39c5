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

namespace qses {

#define QCHK(expr)                                                                      \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) return ctx->fail(QSES_ERR_CUDA, #expr, e_);              \
    } while (0)

static size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

// Pinned host staging that grows geometrically and stays with the context.
static int stage_reserve(qses_context *ctx, size_t bytes) {
    if (bytes <= ctx->h_stage_cap) return QSES_OK;
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

int run_batch(qses_context *ctx, const BatchItem *items, unsigned count, int passes, int key_bits) {
    cudaStream_t s = ctx->stream;
    ctx->launches = 0;
    for (auto &m : ctx->marks) cudaEventDestroy(m.second);
    ctx->marks.clear();
    ctx->mesh = DeviceMesh();
    ctx->have_grid = false;
    BatchResult &R = ctx->batch;
    R = BatchResult();
    if (count == 0) return QSES_OK;
    ctx->mark("start");

    // ---- per-molecule layout on the host
    const unsigned nm = count;
    std::vector<QMol> mols(nm);
    std::vector<unsigned> tile_off(nm + 1), atom_off(nm + 1), row_off(nm + 1), unit_off(nm + 1);
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
    if (tiles >= (1ull << 31) || rows >= (1ull << 31) || cell_tot >= (1ull << 31) || atoms_tot >= (1ull << 30))
        return ctx->fail(QSES_ERR_UNSUPPORTED, "batch too large for 32-bit item indices; split it");
    const unsigned N = (unsigned)atoms_tot;

    // ---- pinned staging: descriptor block then atoms, one copy each
    const size_t desc_bytes = a256(sizeof(QMol) * nm) + 8 * a256(4ull * (nm + 1)) + a256(1024ull * nm);
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
                         3 * a256(4 * mask_tot) + a256(code_tot) + a256(8 * rows) + 2 * a256(64) + a256(tmpA) + 8192;
    if (ctx->field.reserve(needA) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "batch field workspace");
    Arena &A = ctx->field;
    char *d_desc = (char *)A.take(desc_bytes);
    float *d_x = (float *)A.take(16ull * N);
    QCHK(cudaMemcpyAsync(d_desc, hs, desc_bytes, cudaMemcpyHostToDevice, s));
    QCHK(cudaMemcpyAsync(d_x, hx, atom_bytes, cudaMemcpyHostToDevice, s));
    const float *d_r = d_x + 3ull * N;
    QBatch b;
    unsigned *d_edge_off, *d_kept_off;
    {
        size_t q = 0;
        auto at = [&](size_t bytes) {
            char *p = d_desc + q;
            q += a256(bytes);
            return p;
        };
        const size_t ob = 4ull * (nm + 1);
        b.mols = (const QMol *)at(sizeof(QMol) * nm);
        b.tile_off = (const unsigned *)at(ob);
        b.atom_off = (const unsigned *)at(ob);
        b.row_off = (const unsigned *)at(ob);
        b.mc_unit_off = (const unsigned *)at(ob);
        b.tri_off = (const unsigned *)at(ob);
        d_edge_off = (unsigned *)at(ob);
        b.vtx_off = (const unsigned *)at(ob);
        d_kept_off = (unsigned *)at(ob);
        b.lut = (const float *)at(1024ull * nm);
        b.n_mol = nm;
        b.key_bits = key_bits;
    }
    unsigned *d_tri_off = (unsigned *)b.tri_off, *d_vtx_off = (unsigned *)b.vtx_off;

    unsigned *key = (unsigned *)A.take(4ull * N), *key2 = (unsigned *)A.take(4ull * N);
    unsigned *idx = (unsigned *)A.take(4ull * N), *idx2 = (unsigned *)A.take(4ull * N);
    float4 *atoms = (float4 *)A.take(16ull * N);
    uint2 *cells = (uint2 *)A.take(8 * cell_tot);
    unsigned *inMask = (unsigned *)A.take(4 * mask_tot), *outMask = (unsigned *)A.take(4 * mask_tot);
    unsigned *signMask = (unsigned *)A.take(4 * mask_tot);
    unsigned char *codes = (unsigned char *)A.take(code_tot);
    uint2 *rowsb = (uint2 *)A.take(8 * rows);
    uint2 *d_tot = (uint2 *)A.take(64);
    unsigned *counters = (unsigned *)A.take(64);
    void *tmp = A.take(tmpA);
    if (!tmp) return ctx->fail(QSES_ERR_INTERNAL, "batch field workspace layout");
    int *d_err = (int *)((char *)ctx->small + 64);
    QCHK(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    QCHK(cudaMemsetAsync(counters, 0, 64, s));

    // ---- atoms
    launch_atom_hash_batch(b, d_x, N, key, s);
    ctx->launches++;
    int alt = 0;
    QCHK(radix_sort<unsigned>(key, key2, idx, idx2, N, cell_bits, true, tmp, d_err, s, &ctx->launches, &alt));
    unsigned *skey = alt ? key2 : key, *sidx = alt ? idx2 : idx;
    QCHK(cudaMemsetAsync(cells, 0, 8 * cell_tot, s));
    launch_atom_gather(d_x, d_r, skey, sidx, N, atoms, cells, s);
    ctx->launches++;
    ctx->mark("atoms");

    // ---- field: persistent CTAs over (molecule, tile) items
    launch_sas_batch(b, (unsigned)tiles, atoms, cells, inMask, outMask, counters, s);
    ctx->launches++;
    ctx->mark("sas");
    launch_edt_batch(b, (unsigned)tiles, inMask, outMask, codes, signMask, counters + 1, s);
    ctx->launches++;
    ctx->mark("refine");

    // ---- marching-cubes counts, one scan over all rows, per-molecule offsets
    launch_mc_count_batch(b, (unsigned)units, signMask, rowsb, s);
    ctx->launches++;
    QCHK(scan_u2(rowsb, rowsb, (unsigned)rows, d_tot, tmp, d_err, s, &ctx->launches));
    launch_gather_offsets(rowsb, b.row_off, nm, (unsigned)rows, d_tot, d_tri_off, d_edge_off, s);
    ctx->launches++;
    unsigned *hsm = (unsigned *)ctx->h_small;  // 4 KB pinned: totals and the error word
    QCHK(cudaMemcpyAsync(hsm, d_tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
    QCHK(cudaMemcpyAsync(hsm + 2, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    QCHK(cudaStreamSynchronize(s));
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
                         4 * a256(4 * n3 + 4) + a256(8 * n3 + 8) + 3 * a256(4ull * NE + 4) + a256(4ull * NE + 65536) +
                         a256(4096) + a256(16ull * NE + 16) + a256(tmpB) + a256(8ull * T + 16) +
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
    unsigned *okey = (unsigned *)B.take(4 * n3 + 4), *okey2 = (unsigned *)B.take(4 * n3 + 4);
    unsigned *oval = (unsigned *)B.take(4 * n3 + 4), *oval2 = (unsigned *)B.take(4 * n3 + 4);
    unsigned *nbr = (unsigned *)B.take(8 * n3 + 8);
    int *lower = (int *)B.take(4ull * NE + 4), *cnt = (int *)B.take(4ull * NE + 4);
    unsigned *inbox = (unsigned *)B.take(4ull * NE + 65536);
    unsigned *inbox_tail = (unsigned *)B.take(4096);
    float4 *pos4 = (float4 *)B.take(16ull * NE + 16);
    void *tmpb = B.take(tmpB);
    uint2 *tflags = (uint2 *)B.take(8ull * T + 16);  // degenerate filter (side stream)
    void *tmp2 = B.take(scan_u2_tmp_bytes(T + 1));   // its scan's scratch
    if (!tmpb || !tflags || !tmp2) return ctx->fail(QSES_ERR_INTERNAL, "batch mesh workspace layout");

    // ---- triangles + molecule-tagged weld keys, then one weld for all molecules
    launch_mc_emit_batch(b, (unsigned)units, signMask, codes, rowsb, tri, vk, s);
    ctx->launches++;
    ctx->mark("mc_emit");
    unsigned nv = 0;
    if (NE > 0) {
        QCHK(radix_sort<unsigned long long>(vk, vk2, vv, vv2, NE, tot_bits, true, tmpb, d_err, s, &ctx->launches,
                                            &alt));
        unsigned long long *sk = alt ? vk2 : vk;
        unsigned *sv = alt ? vv2 : vv;
        launch_weld_flags(sk, NE, flags, s);
        ctx->launches++;
        QCHK(scan_u2(flags, flags, NE, d_tot, tmpb, d_err, s, &ctx->launches));
        launch_weld_scatter_batch(b, sk, sv, flags, NE, vmap, vq, vmol, s);
        ctx->launches++;
        // molecule m's edges occupy sorted positions [edge_off[m], edge_off[m+1]) (its keys
        // sort between the other molecules'), so its first vertex is the rank there
        launch_gather_offsets(flags, d_edge_off, nm, NE, d_tot, d_vtx_off, nullptr, s);
        ctx->launches++;
        launch_remap(tri, n3, vmap, s);
        ctx->launches++;
    } else {
        QCHK(cudaMemsetAsync(d_vtx_off, 0, 4ull * (nm + 1), s));
    }
    std::vector<unsigned> vtx_off(nm + 1);
    QCHK(cudaMemcpyAsync(hsm, d_tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
    QCHK(cudaMemcpyAsync(ctx->h_stage, d_vtx_off, 4ull * (nm + 1), cudaMemcpyDeviceToHost, s));
    QCHK(cudaStreamSynchronize(s));
    memcpy(vtx_off.data(), ctx->h_stage, 4ull * (nm + 1));
    nv = NE > 0 ? hsm[0] : 0;
    ctx->mark("weld");

    // Closest atom, filter and (for host results) the triangle and atom-id downloads run on
    // the side stream beside the neighbour-list build and the smoothing; profiled calls keep
    // one stream so the stage times stay separable.
    const bool fork = !ctx->profiling && ctx->side != nullptr;
    cudaStream_t sd = fork ? ctx->side : s;
    HostDownload &dl = ctx->dl;
    if (dl.want) {  // [vertices | triangles (pre-filter count) | atom_sorted | atom_input]
        dl.vb = 12ull * nv;
        dl.tb = 12ull * T;
        dl.ab = 4ull * nv;
        dl.block = pinned_take(dl.vb + dl.tb + 2 * dl.ab + 256, &dl.bytes);
        if (!dl.block) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "pinned batch meshes");
    }
    if (fork) {
        QCHK(cudaEventRecord(ctx->ev_fork, s));
        QCHK(cudaStreamWaitEvent(sd, ctx->ev_fork, 0));
    }
    if (nv > 0) {
        launch_closest_batch(b, vq, vmol, nv, atoms, cells, sidx, asorted, ainput, sd);
        ctx->launches++;
    }
    ctx->mark("closest_atom");

    // ---- per-molecule filter and molecule-local corner ids
    if (T > 0) {
        launch_tri_flags_batch(b, tri, T, tflags, sd);
        ctx->launches++;
        QCHK(scan_u2(tflags, tflags, T, d_tot, tmp2, d_err, sd, &ctx->launches));
        launch_tri_compact_batch(b, tri, T, tflags, tri_kept, sd);
        ctx->launches++;
        launch_gather_offsets(tflags, d_tri_off, nm, T, d_tot, d_kept_off, nullptr, sd);
        ctx->launches++;
    } else {
        QCHK(cudaMemsetAsync(d_kept_off, 0, 4ull * (nm + 1), sd));
        QCHK(cudaMemsetAsync(d_tot, 0, sizeof(uint2), sd));
    }
    QCHK(cudaMemcpyAsync(hsm, d_tot, sizeof(uint2), cudaMemcpyDeviceToHost, sd));
    QCHK(cudaMemcpyAsync(ctx->h_stage, d_kept_off, 4ull * (nm + 1), cudaMemcpyDeviceToHost, sd));
    ctx->mark("filter");
    if (dl.want) {
        char *hb = (char *)dl.block;
        if (dl.tb) QCHK(cudaMemcpyAsync(hb + dl.vb, tri_kept, dl.tb, cudaMemcpyDeviceToHost, sd));
        if (dl.ab) QCHK(cudaMemcpyAsync(hb + dl.vb + dl.tb, asorted, dl.ab, cudaMemcpyDeviceToHost, sd));
        if (dl.ab) QCHK(cudaMemcpyAsync(hb + dl.vb + dl.tb + dl.ab, ainput, dl.ab, cudaMemcpyDeviceToHost, sd));
        dl.d2h = dl.tb + 2 * dl.ab;
    }
    if (fork) QCHK(cudaEventRecord(ctx->ev_join, sd));

    // ---- Gauss-Seidel over all molecules
    if (passes > 0 && nv > 0 && T > 0) {
        uint2 *deg = flags;
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
        const GsShape sh = ctx->gs_force.threads ? ctx->gs_force
                                                  : gs_shape(std::min<unsigned>(nv, 152u * kGsSlabMaxVerts), true);
        ctx->gs_used = sh;
        // the closest-atom pass on the side stream reads the welded positions in vq
        int rc2 = run_smoothing(ctx, sh, passes, vq, pos4, nv, deg, nbr, (unsigned short *)cnt, lower, inbox,
                                inbox_tail, d_err, nullptr, true, fork ? ctx->ev_join : nullptr);
        if (rc2) return rc2;
    }
    ctx->mark("smooth");
    if (dl.want && dl.vb) {
        QCHK(cudaMemcpyAsync(dl.block, vq, dl.vb, cudaMemcpyDeviceToHost, s));
        dl.d2h += dl.vb;
    }
    if (fork) QCHK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
    std::vector<unsigned> kept_off(nm + 1);
    QCHK(cudaMemcpyAsync(hsm + 2, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    QCHK(cudaStreamSynchronize(s));
    ctx->mark("download");
    if (hsm[2]) return ctx->fail((int)hsm[2], "device wait in the batch mesh stage");
    const unsigned nkept = hsm[0];
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
