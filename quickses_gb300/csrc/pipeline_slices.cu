// The reference's slicing mode (QSES_FLAG_REFERENCE_SLICES): QuickSES's per-slice output,
// for callers that diff against meshes the reference wrote.
//
// The reference cuts the grid into cores of S = min(slice, G) voxels and computes each
// slice in a box of D = min(slice + 2R, G) voxels starting R before its core, clamped at 0
// (CudaSurf.cu:629-682).  Within a box the field is classified at its grid positions, the
// box's last layer and everything at or past the grid's last layer stay outside, and the
// refine window is clamped to the box (Kernels.cu:394-545).  Marching cubes emits the cells
// countVertexPerCell keeps (MarchingCubes.cu:578-604; two cell layers at every seam are
// emitted by both neighbours), with vertices at box positions plus offset * dx
// (MarchingCubes.cu:841-848).  The last triangle of a slice is never written
// (MarchingCubes.cu:845 with CudaSurf.cu:421); here it is dropped with any vertex only it
// used.  Each slice is welded, given closest atoms and smoothed on its own
// (CudaSurf.cu:444-500, 746), slices without a border voxel give no mesh
// (CudaSurf.cu:691-697), and the meshes are concatenated as API_computeSES does
// (CudaSurf.cu:796-836).
//
// The stages are the single-molecule kernels on one box at a time, so device memory is
// bounded by the box, not the grid: any grid size within the neighbour-cell limit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "kernels.h"
#include "prims.h"
#include "qses_context.h"

namespace qses {

namespace {

// Border voxels (neither inside nor outside) in a box's masks.
__global__ void k_border_count(const unsigned *__restrict__ in, const unsigned *__restrict__ out, size_t words,
                               int W, int G, unsigned long long *__restrict__ count) {
    unsigned long long c = 0;
    const unsigned tail = (G & 31) ? ((1u << (G & 31)) - 1u) : 0xffffffffu;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < words; q += (size_t)gridDim.x * blockDim.x) {
        const unsigned valid = ((int)(q % (size_t)W) == W - 1) ? tail : 0xffffffffu;
        c += (unsigned)__popc(~(in[q] | out[q]) & valid);
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// used[v].x = 1 for every vertex a triangle corner names.
__global__ void k_mark_used(const unsigned *__restrict__ tri, size_t n3, uint2 *__restrict__ used) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n3) used[tri[q]].x = 1u;
}

// Keeps the used vertices in their order: excl is the exclusive scan of used.
__global__ void k_compact_vertices(const uint2 *__restrict__ used, const uint2 *__restrict__ excl, unsigned nv,
                                   const float *__restrict__ vq, float *__restrict__ vq2, unsigned *__restrict__ vmap) {
    const unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const unsigned to = excl[v].x;
    vmap[v] = to;
    if (used[v].x) {
        vq2[3ull * to] = vq[3ull * v];
        vq2[3ull * to + 1] = vq[3ull * v + 1];
        vq2[3ull * to + 2] = vq[3ull * v + 2];
    }
}

unsigned blocks(size_t n, unsigned t) { return (unsigned)std::max<size_t>(1, (n + t - 1) / t); }

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

// Cells of one box axis that countVertexPerCell keeps, its int bounds compared with the
// unsigned cell index as the kernel does them: [lo, hi), empty when lo == hi.
void box_cells(int D, int R, int off, int &lo, int &hi) {
    lo = hi = 0;
    bool any = false;
    for (int c = 0; c < D; c++) {
        const unsigned i = (unsigned)c;
        bool skip = i > (unsigned)(D - 2);
        if (off != 0 && i < (unsigned)(R - 3)) skip = true;
        if (off == 0 && i >= (unsigned)(D - 2 * R - 1)) skip = true;
        if (i >= (unsigned)(D - R - 1)) skip = true;
        if (!skip) {
            if (!any) lo = c;
            any = true;
            hi = c + 1;
        }
    }
}

}  // namespace

#define SCHK(expr)                                                                      \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) return ctx->fail(QSES_ERR_CUDA, #expr, e_);              \
    } while (0)

int run_pipeline_slices(qses_context *ctx, const qses_params &p, const float *d_xyz, const float *d_r, unsigned n,
                        SlicedMesh &out) {
    cudaStream_t s = ctx->stream;
    out = SlicedMesh();
    ctx->launches = 0;
    for (auto &m : ctx->marks) cudaEventDestroy(m.second);
    ctx->marks.clear();
    ctx->mesh = DeviceMesh();
    ctx->have_grid = false;
    ctx->slice_nv.clear();
    ctx->slice_nt.clear();
    if (p.slice < 1) return ctx->fail(QSES_ERR_INVALID_ARG, "slice must be >= 1");
    SCHK(cudaMemsetAsync((char *)ctx->small + 256, 0, 64, s));
    QGrid g;
    const int grc = molecule_grid(ctx, p, d_xyz, d_r, n, g, true);
    if (grc != QSES_OK) return grc;
    int *d_err = (int *)((char *)ctx->small + 64);
    unsigned long long *d_border = (unsigned long long *)((char *)ctx->small + 128);
    unsigned long long *stats = (unsigned long long *)((char *)ctx->small + 256);

    const int G = g.G, R = g.R;
    const int S = std::min(p.slice, G), D = (int)std::min<long long>((long long)p.slice + 2 * R, G);
    const int W = (D + 31) / 32, Gp = 32 * W;
    const size_t ncell = (size_t)g.gnb * g.gnb * g.gnb;
    const size_t nmask = (size_t)D * D * W, ncode = (size_t)D * D * Gp, nrow = (size_t)D * D;
    const int atom_bits = bits_for(ncell ? ncell - 1 : 0);
    const size_t tmpA = std::max(radix_sort_tmp_bytes(n, atom_bits), scan_u2_tmp_bytes((unsigned)nrow));
    const size_t needA = a256(4ull * n) * 4 + a256(16ull * n) + a256(8 * ncell) + 3 * a256(4 * nmask) +
                         2 * a256(ncode) + a256(1024) + a256(8 * nrow) + a256(64) + a256(tmpA) + 4096;
    if (ctx->field.reserve(needA) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "field workspace");
    Arena &A = ctx->field;
    unsigned *key = (unsigned *)A.take(4ull * n), *key2 = (unsigned *)A.take(4ull * n);
    unsigned *idx = (unsigned *)A.take(4ull * n), *idx2 = (unsigned *)A.take(4ull * n);
    float4 *atoms = (float4 *)A.take(16ull * n);
    uint2 *cells = (uint2 *)A.take(8 * ncell);
    unsigned *in_mask = (unsigned *)A.take(4 * nmask), *out_mask = (unsigned *)A.take(4 * nmask);
    unsigned *sign_mask = (unsigned *)A.take(4 * nmask);
    unsigned char *codes = (unsigned char *)A.take(ncode), *zd = (unsigned char *)A.take(ncode);
    float *lut = (float *)A.take(1024);
    uint2 *rows = (uint2 *)A.take(8 * nrow);
    uint2 *tot = (uint2 *)A.take(64);
    void *tmp = A.take(tmpA);
    if (!tmp) return ctx->fail(QSES_ERR_INTERNAL, "field workspace layout");

    // ---- atoms into the molecule's neighbour cells, once for every slice
    launch_atom_hash(g, d_xyz, n, key, s);
    ctx->launches++;
    int alt = 0;
    SCHK(radix_sort<unsigned>(key, key2, idx, idx2, n, atom_bits, true, tmp, d_err, s, &ctx->launches, &alt));
    const unsigned *skey = alt ? key2 : key, *sidx = alt ? idx2 : idx;
    SCHK(cudaMemsetAsync(cells, 0, 8 * ncell, s));
    launch_atom_gather(d_xyz, d_r, skey, sidx, n, atoms, cells, s);
    ctx->launches++;
    fill_lut(g, (float *)(ctx->h_small + 64));
    SCHK(cudaMemcpyAsync(lut, ctx->h_small + 64, 1024, cudaMemcpyHostToDevice, s));
    SCHK(cudaStreamSynchronize(s));  // the pinned table is rewritten below

    const bool keep_all = (p.flags & QSES_FLAG_KEEP_DEGENERATE) != 0;
    const int edt = ctx->edt_force >= 0 ? ctx->edt_force : edt_shape(D);
    for (int x = 0; x < G; x += S)
        for (int y = 0; y < G; y += S)
            for (int z = 0; z < G; z += S) {
                // ---- the box and its grid
                const int core[3] = {x, y, z};
                QGrid b = g;
                b.G = D;
                b.W = W;
                b.Gp = Gp;
                bool cells_any = true;
                for (int a = 0; a < 3; a++) {
                    b.off[a] = std::max(0, core[a] - R);
                    b.lim[a] = std::min(D - 1, G - 1 - b.off[a]);
                    box_cells(D, R, b.off[a], b.clo[a], b.chi[a]);
                    cells_any = cells_any && b.clo[a] < b.chi[a];
                }
                b.Gc = std::max(b.chi[0], std::max(b.chi[1], b.chi[2]));
                // weld keys relative to the box's own corner: positions lie in
                // [origin + off dx, origin + (off + D) dx]
                const float tol = QSES_WELD_TOL;
                b.bx = (long long)std::floor(((double)g.ox + (double)b.off[0] * g.dx) / tol) - 16;
                b.by = (long long)std::floor(((double)g.oy + (double)b.off[1] * g.dx) / tol) - 16;
                b.bz = (long long)std::floor(((double)g.oz + (double)b.off[2] * g.dx) / tol) - 16;
                b.Rq = (long long)std::ceil((double)D * g.dx / 0.001) + 64;
                if (b.Rq >= (1ll << 21)) return ctx->fail(QSES_ERR_UNSUPPORTED, "slice box above 2000 A");

                // ---- field of the box, its border count, marching-cubes row counts
                SCHK(cudaMemsetAsync(d_border, 0, 8, s));
                launch_sas(b, atoms, cells, in_mask, out_mask, s);
                k_border_count<<<blocks(nmask, 256 * 8), 256, 0, s>>>(in_mask, out_mask, nmask, W, D, d_border);
                launch_edt(b, in_mask, out_mask, codes, sign_mask, s, edt, zd);
                ctx->launches += 4;
                uint2 *h_tot = (uint2 *)ctx->h_small;
                if (cells_any) {
                    const size_t E = (size_t)b.Gc + 1;
                    launch_mc_count(b, sign_mask, rows, s);
                    ctx->launches++;
                    SCHK(scan_u2(rows, rows, (unsigned)(E * E), tot, tmp, d_err, s, &ctx->launches));
                    SCHK(cudaMemcpyAsync(h_tot, tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
                } else {
                    h_tot->x = h_tot->y = 0;
                }
                SCHK(cudaMemcpyAsync(ctx->h_small + 16, d_border, 8, cudaMemcpyDeviceToHost, s));
                SCHK(cudaMemcpyAsync(ctx->h_small + 24, d_err, 4, cudaMemcpyDeviceToHost, s));
                SCHK(cudaStreamSynchronize(s));
                int herr;
                unsigned long long border;
                memcpy(&herr, ctx->h_small + 24, 4);
                memcpy(&border, ctx->h_small + 16, 8);
                if (herr) return ctx->fail(herr, "device wait in a slice's field");
                if (border == 0) continue;  // no mesh for this slice
                const unsigned T = cells_any ? h_tot->x : 0u, NE = cells_any ? h_tot->y : 0u;
                const unsigned T1 = T > 0 ? T - 1 : 0;  // the last triangle is never written
                if (T1 == 0) {
                    out.slice_nv.push_back(0);
                    out.slice_nt.push_back(0);
                    continue;
                }

                // ---- mesh workspace of this slice
                const size_t n3 = 3ull * T, n3k = 3ull * T1;
                const int key_bits = bits_for((unsigned long long)b.Rq * b.Rq * b.Rq - 1);
                const size_t tmpB = std::max({radix_sort_tmp_bytes(NE, key_bits), scan_u2_tmp_bytes(NE + 1),
                                              scan_u2_tmp_bytes(T + 1)});
                const size_t needB = 3 * a256(4 * n3 + 4) + 2 * a256(8ull * NE + 8) + 2 * a256(4ull * NE + 4) +
                                     3 * a256(8ull * (NE + 2)) + 2 * a256(4ull * NE + 4) + 2 * a256(12ull * NE + 12) +
                                     2 * a256(4ull * NE + 4) + a256(8 * n3 + 8) + 2 * a256(4ull * NE + 4) +
                                     a256(16ull * NE + 16) + a256(8ull * T + 16) + a256(tmpB) + 4096;
                if (ctx->mesh_ws.reserve(needB) != QSES_OK) return ctx->fail(QSES_ERR_OUT_OF_MEMORY, "mesh workspace");
                Arena &B = ctx->mesh_ws;
                unsigned *tri = (unsigned *)B.take(4 * n3 + 4), *tri_kept = (unsigned *)B.take(4 * n3 + 4);
                unsigned *okey = (unsigned *)B.take(4 * n3 + 4);
                unsigned long long *vk = (unsigned long long *)B.take(8ull * NE + 8);
                unsigned long long *vk2 = (unsigned long long *)B.take(8ull * NE + 8);
                unsigned *vv = (unsigned *)B.take(4ull * NE + 4), *vv2 = (unsigned *)B.take(4ull * NE + 4);
                uint2 *flags = (uint2 *)B.take(8ull * (NE + 2)), *used = (uint2 *)B.take(8ull * (NE + 2));
                uint2 *excl = (uint2 *)B.take(8ull * (NE + 2));
                unsigned *vmap = (unsigned *)B.take(4ull * NE + 4), *vmap2 = (unsigned *)B.take(4ull * NE + 4);
                float *vq = (float *)B.take(12ull * NE + 12), *vq2 = (float *)B.take(12ull * NE + 12);
                int *asorted = (int *)B.take(4ull * NE + 4), *ainput = (int *)B.take(4ull * NE + 4);
                unsigned *nbr = (unsigned *)B.take(8 * n3 + 8);
                int *lower = (int *)B.take(4ull * NE + 4), *cnt = (int *)B.take(4ull * NE + 4);
                float4 *pos4 = (float4 *)B.take(16ull * NE + 16);
                uint2 *tflags = (uint2 *)B.take(8ull * T + 16);
                void *tmpb = B.take(tmpB);
                if (!tmpb) return ctx->fail(QSES_ERR_INTERNAL, "mesh workspace layout");

                // ---- triangles and edge keys; weld; the last triangle's own vertices out
                launch_mc_emit(b, sign_mask, codes, lut, rows, tri, vk, s);
                int walt = 0;
                SCHK(radix_sort<unsigned long long>(vk, vk2, vv, vv2, NE, key_bits, true, tmpb, d_err, s,
                                                    &ctx->launches, &walt));
                const unsigned long long *sk = walt ? vk2 : vk;
                const unsigned *sv = walt ? vv2 : vv;
                launch_weld_flags(sk, NE, flags, s);
                SCHK(scan_u2(flags, flags, NE, tot, tmpb, d_err, s, &ctx->launches));
                launch_weld_scatter(b, sk, sv, flags, NE, vmap, vq, s);
                launch_remap(tri, n3k, vmap, s);
                ctx->launches += 4;
                SCHK(cudaMemcpyAsync(h_tot, tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
                SCHK(cudaStreamSynchronize(s));
                const unsigned V = h_tot->x;
                SCHK(cudaMemsetAsync(used, 0, 8ull * (V + 1), s));
                k_mark_used<<<blocks(n3k, 256), 256, 0, s>>>(tri, n3k, used);
                SCHK(scan_u2(used, excl, V, tot, tmpb, d_err, s, &ctx->launches));
                k_compact_vertices<<<blocks(V, 256), 256, 0, s>>>(used, excl, V, vq, vq2, vmap2);
                launch_remap(tri, n3k, vmap2, s);
                ctx->launches += 3;
                SCHK(cudaMemcpyAsync(h_tot, tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
                SCHK(cudaStreamSynchronize(s));
                const unsigned nv = h_tot->x;

                // ---- closest atom (the molecule's cells), smoothing, degenerate filter
                launch_closest(g, vq2, nv, atoms, cells, sidx, asorted, ainput, s);
                ctx->launches++;
                if (p.smooth_passes > 0 && nv > 0) {
                    uint2 *deg = flags;  // nv + 1 <= NE + 1 entries
                    SCHK(cudaMemsetAsync(deg, 0, 8ull * (nv + 1), s));
                    launch_csr_count(tri, n3k, deg, s);
                    SCHK(scan_u2(deg, deg, nv + 1, nullptr, tmpb, d_err, s, &ctx->launches));
                    launch_csr_scatter(tri, n3k, deg, okey, s);
                    launch_csr_sortfill(tri, okey, n3k, nv, deg, nbr, s);
                    ctx->launches += 3;
                    GsShape sh = ctx->gs_force.threads ? ctx->gs_force : gs_shape(nv, false);
                    sh.hot = kGsHotWarpsSingle;
                    ctx->gs_used = sh;
                    GsPlan plan;
                    const int prc = gs_plan(ctx->device, sh, nv, nullptr, nullptr, 1, plan);
                    if (prc != QSES_OK) return ctx->fail(prc, "smoothing slab plan");
                    GsBuffers gb;
                    const int brc = gs_buffers(ctx, plan, nv, gb);
                    if (brc != QSES_OK) return brc;
                    const int src = run_smoothing(ctx, sh, plan.L, p.smooth_passes, vq2, pos4, nv, deg, nbr,
                                                  (unsigned short *)cnt, lower, gb.home, gb.table, ctx->h_gs, gb.inbox,
                                                  gb.inbox_tail, d_err, stats);
                    if (src != QSES_OK) return src;
                }
                const unsigned *tri_out = tri;
                unsigned nt = T1;
                if (!keep_all) {
                    launch_tri_flags(tri, T1, tflags, s);
                    SCHK(scan_u2(tflags, tflags, T1, tot, tmpb, d_err, s, &ctx->launches));
                    launch_tri_compact(tri, T1, tflags, tri_kept, s);
                    ctx->launches += 2;
                    SCHK(cudaMemcpyAsync(h_tot, tot, sizeof(uint2), cudaMemcpyDeviceToHost, s));
                    SCHK(cudaStreamSynchronize(s));
                    nt = h_tot->x;
                    tri_out = tri_kept;
                }

                // ---- download, appended to the concatenated mesh
                const size_t v0 = out.vertices.size() / 3, t0 = out.triangles.size();
                out.vertices.resize(3 * (v0 + nv));
                out.triangles.resize(t0 + 3ull * nt);
                out.atom_sorted.resize(v0 + nv);
                out.atom_input.resize(v0 + nv);
                if (nv) {
                    SCHK(cudaMemcpyAsync(out.vertices.data() + 3 * v0, vq2, 12ull * nv, cudaMemcpyDeviceToHost, s));
                    SCHK(cudaMemcpyAsync(out.atom_sorted.data() + v0, asorted, 4ull * nv, cudaMemcpyDeviceToHost, s));
                    SCHK(cudaMemcpyAsync(out.atom_input.data() + v0, ainput, 4ull * nv, cudaMemcpyDeviceToHost, s));
                }
                if (nt)
                    SCHK(cudaMemcpyAsync(out.triangles.data() + t0, tri_out, 12ull * nt, cudaMemcpyDeviceToHost, s));
                SCHK(cudaMemcpyAsync(ctx->h_small + 24, d_err, 4, cudaMemcpyDeviceToHost, s));
                SCHK(cudaStreamSynchronize(s));
                memcpy(&herr, ctx->h_small + 24, 4);
                if (herr) return ctx->fail(herr, "device wait in a slice's mesh");
                for (size_t q = t0; q < out.triangles.size(); q++) out.triangles[q] += (int)v0;
                out.slice_nv.push_back(nv);
                out.slice_nt.push_back(nt);
            }
    ctx->slice_nv = out.slice_nv;
    ctx->slice_nt = out.slice_nt;
    return QSES_OK;
}

}  // namespace qses
