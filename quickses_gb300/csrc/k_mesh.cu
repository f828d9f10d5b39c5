// Marching cubes, vertex weld, closest atom, degenerate filter and Laplacian smoothing.
//
//  k_mc<false>    per (x, y) row of cells: triangle count and active-edge count
//                 (countVertexPerCell, MarchingCubes.cu:571-658, single-slice cell range)
//  k_mc<true>     the same rows again: triangles in cell linear order x*G^2 + y*G + z and
//                 one quantised key per active edge (generateTriangleVerticesSMEM +
//                 groupVertices, MarchingCubes.cu:736-862).  One warp per row; the sign of
//                 32 voxels is one word, so cube indices and edge activity are bit ops.
//  k_weld_*       unique quantised positions in lexicographic order (CudaSurf.cu:444-457)
//  k_closest      closest atom per welded vertex (closestAtomPerVertex, Kernels.cu:547-604)
//  k_tri_*        drop triangles with a repeated index (CudaSurf.cu:820-829)
//  k_csr_* / k_gs_setup  neighbour lists in triangle order (getNeighboorsVertices,
//                 SmoothMesh.cpp:45-123) and the per-vertex dependency counts and slab homes
//                 of the Gauss-Seidel dataflow (k_smooth.cu)
#include <cfloat>
#include <cstdlib>
#include <cstring>

#include "device_common.cuh"

#include "kernels.h"
#include "mc_tables.h"

namespace qses {

__constant__ unsigned long long c_mc[256] = QSES_MC_TABLE_INIT;

// Owner of each cube edge relative to the cell: bit0 di, bit1 dj, bit2 dk, bits3-4 axis.
// Edges follow MarchingCubes.cu:814-825 with corners as in :625-632.
constexpr unsigned long long kEdgeOwner =
    (0ull << 0) | (9ull << 5) | (2ull << 10) | (8ull << 15) | (4ull << 20) | (13ull << 25) | (6ull << 30) |
    (12ull << 35) | (16ull << 40) | (17ull << 45) | (19ull << 50) | (18ull << 55);

__device__ __forceinline__ unsigned ld_sign(const unsigned *__restrict__ sign, const QGrid &g, int i, int j, int w) {
    if (i >= g.G || j >= g.G || w >= g.W) return 0u;
    return __ldg(&sign[((size_t)i * g.G + j) * g.W + w]);
}

__device__ __forceinline__ unsigned cube_index(unsigned b, unsigned c0, unsigned c1, unsigned c2, unsigned c3,
                                               unsigned c4, unsigned c5, unsigned c6, unsigned c7) {
    return ((c0 >> b) & 1u) | (((c1 >> b) & 1u) << 1) | (((c2 >> b) & 1u) << 2) | (((c3 >> b) & 1u) << 3) |
           (((c4 >> b) & 1u) << 4) | (((c5 >> b) & 1u) << 5) | (((c6 >> b) & 1u) << 6) | (((c7 >> b) & 1u) << 7);
}

__device__ __forceinline__ unsigned warp_sum(unsigned v) { return __reduce_add_sync(0xffffffffu, v); }

// Quantised key of the vertex on edge (i, j, k) -> (i, j, k) + e_axis.
__device__ unsigned long long edge_key(const QGrid &g, const unsigned char *__restrict__ codes, const float *lut,
                                       int i, int j, int k, int ax) {
    const size_t base = ((size_t)i * g.G + j) * g.Gp + k;
    const size_t step = ax == 0 ? (size_t)g.G * g.Gp : (ax == 1 ? (size_t)g.Gp : (size_t)1);
    const float fa = lut[__ldg(codes + base)], fb = lut[__ldg(codes + base + step)];
    const float t = __fdiv_rn(-fa, __fsub_rn(fb, fa));  // vertexInterp (MarchingCubes.cu:731-734)
    float p[3] = {vox(i, g.dx, g.ox), vox(j, g.dx, g.oy), vox(k, g.dx, g.oz)};
    const float o[3] = {g.ox, g.oy, g.oz};
    const int idx[3] = {i, j, k};
#pragma unroll
    for (int c = 0; c < 3; c++)
        if (c == ax) p[c] = __fmaf_rn(t, __fsub_rn(vox(idx[c] + 1, g.dx, o[c]), p[c]), p[c]);
    if (g.off[0] | g.off[1] | g.off[2]) {  // a slice box: + offset * dx (MarchingCubes.cu:841-848)
#pragma unroll
        for (int c = 0; c < 3; c++) p[c] = __fadd_rn(p[c], __fmul_rn((float)g.off[c], g.dx));
    }
    // groupVertices: round(v / 0.001) (MarchingCubes.cu:859)
    long long mx = (long long)roundf(__fdiv_rn(p[0], QSES_WELD_TOL));
    long long my = (long long)roundf(__fdiv_rn(p[1], QSES_WELD_TOL));
    long long mz = (long long)roundf(__fdiv_rn(p[2], QSES_WELD_TOL));
    return ((unsigned long long)(mx - g.bx) * (unsigned long long)g.Rq + (unsigned long long)(my - g.by)) *
               (unsigned long long)g.Rq +
           (unsigned long long)(mz - g.bz);
}

__device__ __forceinline__ unsigned sel4(int o, unsigned a, unsigned b, unsigned c, unsigned d) {
    return o == 0 ? a : (o == 1 ? b : (o == 2 ? c : d));
}

// Lanes per owner row: the row's words (voxels 0..Gc) rounded up to a power of two, at
// most 32, so a warp covers 32 / lanes rows of a small grid at once.
__host__ __device__ __forceinline__ int mc_lanes(int Gc) {
    const int Wc = (Gc + 32) / 32;
    int L = 1;
    while (L < Wc && L < 32) L <<= 1;
    return L;
}

// Sum / inclusive scan over aligned groups of Lg lanes (Lg a power of two, warp-uniform).
__device__ __forceinline__ unsigned grp_sum(unsigned v, int Lg) {
    if (Lg == 32) return __reduce_add_sync(0xffffffffu, v);
    for (int o = Lg >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, Lg);
    return v;
}
__device__ __forceinline__ unsigned grp_incl_scan(unsigned v, int sub, int Lg) {
    for (int o = 1; o < Lg; o <<= 1) {
        const unsigned a = __shfl_up_sync(0xffffffffu, v, o, Lg);
        if (sub >= o) v += a;
    }
    return v;
}

// One owner row (i, j) of a molecule's grid per group of Lg lanes; every lane of the warp
// calls this (groups whose row is past the end pass valid = false and write nothing).
// Edge keys get `keyhi` added (the molecule's slot above the local key bits in a batch, 0
// for a single molecule).
// Bits [a, b) of a 32-bit word, the bounds clamped to [0, 32].
__device__ __forceinline__ unsigned bits_in(int a, int b) {
    a = max(a, 0);
    b = min(b, 32);
    if (a >= b) return 0u;
    const unsigned below_b = b == 32 ? 0xffffffffu : ((1u << b) - 1u);
    return below_b & ~((1u << a) - 1u);
}

// Words per lane record of the triangle pass (34 used; an odd stride spreads the lanes'
// writes over the shared-memory banks).
constexpr int kRecW = 35;

template <bool EMIT, bool FULL>
__device__ __forceinline__ void mc_row(const QGrid &g, long long row, bool valid, int Lg,
                                       const unsigned *__restrict__ sign, const unsigned char *__restrict__ codes,
                                       const float *lut, const unsigned long long *s_tab,
                                       uint2 *__restrict__ rowCount, const uint2 *__restrict__ rowBase,
                                       unsigned *__restrict__ tri, unsigned long long *__restrict__ vkey,
                                       unsigned long long keyhi, unsigned *s_rec) {
    // FULL: one row per warp (Lg = 32, every group valid), known at compile time.
    if (FULL) {
        Lg = 32;
        valid = true;
    }
    const int sub = (int)(threadIdx.x & 31) & (Lg - 1);
    const int Gc = g.Gc, E = Gc + 1;
    if (!valid) row = 0;
    const int i = (int)(row / E), j = (int)(row % E);
    // Emitted cells: [clo, chi) per axis (the whole grid: [0, Gc)).  A row's +x edges are
    // used when a cell of the range has them (x in [clo, chi), y in [clo, chi]), likewise +y;
    // its +z edges when x and y are in [clo, chi].
    const int lox = g.clo[0], hix = g.chi[0], loy = g.clo[1], hiy = g.chi[1], loz = g.clo[2], hiz = g.chi[2];
    auto xr = [&](int a, int b) { return a >= lox && a < hix && b >= loy && b <= hiy; };
    auto yr = [&](int a, int b) { return a >= lox && a <= hix && b >= loy && b < hiy; };
    auto zr = [&](int a, int b) { return a >= lox && a <= hix && b >= loy && b <= hiy; };
    const bool cellsRow = valid && i >= lox && i < hix && j >= loy && j < hiy;
    const int Wc = (Gc + 32) / 32;  // words holding voxels 0..Gc

    unsigned triBase = 0, eb0 = 0, eb1 = 0, eb2 = 0, eb3 = 0;  // owners (0,0) (0,1) (1,0) (1,1)
    if (EMIT && valid) {
        triBase = rowBase[row].x;
        eb0 = rowBase[row].y;
        if (j + 1 <= Gc) eb1 = rowBase[(size_t)i * E + j + 1].y;
        if (i + 1 <= Gc) eb2 = rowBase[(size_t)(i + 1) * E + j].y;
        if (i + 1 <= Gc && j + 1 <= Gc) eb3 = rowBase[(size_t)(i + 1) * E + j + 1].y;
    }
    unsigned triCarry = 0, ec0 = 0, ec1 = 0, ec2 = 0, ec3 = 0;
    for (int w0 = 0; w0 < Wc; w0 += Lg) {
        const int w = w0 + sub;
        const bool act = valid && w < Wc;
        const int kb = w * 32;
        unsigned kv = 0u, kc = 0u;
        if (act) {
            kv = bits_in(loz - kb, hiz - kb + 1);  // voxels in [loz, hiz]
            kc = bits_in(loz - kb, hiz - kb);      // cells / z-edges in [loz, hiz)
        }
        const bool nxt = act && (kb + 32 <= hiz) && (kb + 32 >= loz);
        auto L = [&](int a, int b, int ww) { return act ? ld_sign(sign, g, i + a, j + b, ww) : 0u; };
        const unsigned S00 = L(0, 0, w), S10 = L(1, 0, w), S01 = L(0, 1, w), S11 = L(1, 1, w);
        const unsigned N00 = L(0, 0, w + 1), N10 = L(1, 0, w + 1), N01 = L(0, 1, w + 1), N11 = L(1, 1, w + 1);
        const unsigned P00 = (S00 >> 1) | (N00 << 31), P10 = (S10 >> 1) | (N10 << 31);
        const unsigned P01 = (S01 >> 1) | (N01 << 31), P11 = (S11 >> 1) | (N11 << 31);
        const unsigned X00 = xr(i, j) ? (S00 ^ S10) & kv : 0u;
        const unsigned Y00 = yr(i, j) ? (S00 ^ S01) & kv : 0u;
        const unsigned Z00 = zr(i, j) ? (S00 ^ P00) & kc : 0u;
        const unsigned c00 = __popc(X00) + __popc(Y00) + __popc(Z00);
        unsigned cellm = 0u, ntri = 0u, nt0 = 0u, nt1 = 0u, nt2 = 0u;  // nt bit k of each active cell
        if (cellsRow) {
            cellm = ((S00 ^ S10) | (S00 ^ S11) | (S00 ^ S01) | (S00 ^ P00) | (S00 ^ P10) | (S00 ^ P11) |
                     (S00 ^ P01)) & kc;
            for (unsigned m = cellm; m; m &= m - 1u) {
                unsigned b = __ffs(m) - 1;
                const unsigned nt = (unsigned)(s_tab[cube_index(b, S00, S10, S11, S01, P00, P10, P11, P01)] >> 60);
                ntri += nt;
                if (EMIT) {
                    nt0 |= (nt & 1u) << b;
                    nt1 |= ((nt >> 1) & 1u) << b;
                    nt2 |= ((nt >> 2) & 1u) << b;
                }
            }
        }
        if (!EMIT) {
            triCarry += grp_sum(ntri, Lg);
            ec0 += grp_sum(c00, Lg);
            continue;
        }
        // Edges owned by the three neighbouring rows, for triangle corners.
        const unsigned S20 = L(2, 0, w), S21 = L(2, 1, w), S02 = L(0, 2, w), S12 = L(1, 2, w);
        const unsigned N20 = L(2, 0, w + 1), N21 = L(2, 1, w + 1), N02 = L(0, 2, w + 1), N12 = L(1, 2, w + 1);
        const unsigned X01 = xr(i, j + 1) ? (S01 ^ S11) & kv : 0u;
        const unsigned Y01 = yr(i, j + 1) ? (S01 ^ S02) & kv : 0u;
        const unsigned Z01 = zr(i, j + 1) ? (S01 ^ P01) & kc : 0u;
        const unsigned X10 = xr(i + 1, j) ? (S10 ^ S20) & kv : 0u;
        const unsigned Y10 = yr(i + 1, j) ? (S10 ^ S11) & kv : 0u;
        const unsigned Z10 = zr(i + 1, j) ? (S10 ^ P10) & kc : 0u;
        const unsigned X11 = xr(i + 1, j + 1) ? (S11 ^ S21) & kv : 0u;
        const unsigned Y11 = yr(i + 1, j + 1) ? (S11 ^ S12) & kv : 0u;
        const unsigned Z11 = zr(i + 1, j + 1) ? (S11 ^ P11) & kc : 0u;
        const unsigned c01 = __popc(X01) + __popc(Y01) + __popc(Z01);
        const unsigned c10 = __popc(X10) + __popc(Y10) + __popc(Z10);
        const unsigned c11 = __popc(X11) + __popc(Y11) + __popc(Z11);
        // Activity of the x/y edges of voxel kb+32 (bit 0 of the next word).
        const unsigned xn0 = (nxt && xr(i, j)) ? ((N00 ^ N10) & 1u) : 0u, yn0 = (nxt && yr(i, j)) ? ((N00 ^ N01) & 1u) : 0u;
        const unsigned xn1 = (nxt && xr(i, j + 1)) ? ((N01 ^ N11) & 1u) : 0u, yn1 = (nxt && yr(i, j + 1)) ? ((N01 ^ N02) & 1u) : 0u;
        const unsigned xn2 = (nxt && xr(i + 1, j)) ? ((N10 ^ N20) & 1u) : 0u, yn2 = (nxt && yr(i + 1, j)) ? ((N10 ^ N11) & 1u) : 0u;
        const unsigned xn3 = (nxt && xr(i + 1, j + 1)) ? ((N11 ^ N21) & 1u) : 0u, yn3 = (nxt && yr(i + 1, j + 1)) ? ((N11 ^ N12) & 1u) : 0u;

        const unsigned p0 = grp_incl_scan(c00, sub, Lg) - c00, p1 = grp_incl_scan(c01, sub, Lg) - c01;
        const unsigned p2 = grp_incl_scan(c10, sub, Lg) - c10, p3 = grp_incl_scan(c11, sub, Lg) - c11;
        const unsigned tp = grp_incl_scan(ntri, sub, Lg) - ntri;

        // Vertices owned by this row, in voxel order, x then y then z within a voxel: edge e of
        // the group's words goes to slot eb0 + ec0 + e.  The few words a surface crosses hold
        // all of a row's edges, so the edges are dealt out over the group's lanes: lane `sub`
        // takes e = sub, sub + Lg, ..., finds the owning lane (largest L with p0[L] <= e) and
        // the voxel and axis of the edge inside that lane's word.
        {
            const unsigned etot = grp_sum(c00, Lg);
            const unsigned emax = FULL ? etot : __reduce_max_sync(0xffffffffu, etot);  // warp-uniform
            const int gbase = (int)(threadIdx.x & 31) & ~(Lg - 1);
            for (unsigned eb = 0; eb < emax; eb += (unsigned)Lg) {
                const unsigned e = eb + (unsigned)sub;
                int lo = 0;
                for (int step = Lg >> 1; step > 0; step >>= 1) {
                    const unsigned pl = __shfl_sync(0xffffffffu, p0, gbase + lo + step);
                    if (pl <= e) lo += step;
                }
                const unsigned Xo = __shfl_sync(0xffffffffu, X00, gbase + lo);
                const unsigned Yo = __shfl_sync(0xffffffffu, Y00, gbase + lo);
                const unsigned Zo = __shfl_sync(0xffffffffu, Z00, gbase + lo);
                const unsigned po = __shfl_sync(0xffffffffu, p0, gbase + lo);
                if (e < etot) {
                    const unsigned r = e - po;  // rank of the edge inside the owner's word
                    int b = 0;                  // its voxel: the largest b with fewer than r+1 edges below
                    for (int step = 16; step > 0; step >>= 1) {
                        const unsigned lt = (1u << (b + step)) - 1u;
                        if ((unsigned)(__popc(Xo & lt) + __popc(Yo & lt) + __popc(Zo & lt)) <= r) b += step;
                    }
                    const unsigned lt = (1u << b) - 1u;
                    unsigned qa = r - (unsigned)(__popc(Xo & lt) + __popc(Yo & lt) + __popc(Zo & lt));
                    int ax = 2;
                    if ((Xo >> b) & 1u) {
                        if (qa == 0) ax = 0;
                        else qa--;
                    }
                    if (ax == 2 && ((Yo >> b) & 1u) && qa == 0) ax = 1;
                    const int k = (w0 + lo) * 32 + b;
                    vkey[eb0 + ec0 + e] = keyhi + edge_key(g, codes, lut, i, j, k, ax);
                }
            }
        }
        // Triangles in cell order, corners as pre-weld vertex slots.  The few words a surface
        // crosses hold all of a row's cells, so the row's active cells are dealt out over the
        // group's lanes: every lane publishes its word's sign words, edge masks, slot bases and
        // per-cell triangle counts, and lane `sub` takes the row's active cells sub, sub + Lg,
        // ...; a cell's first triangle is its word's first plus the counts of the cells below.
        {
            unsigned *my = s_rec + (threadIdx.x & 31) * kRecW;
            my[0] = S00; my[1] = S10; my[2] = S11; my[3] = S01;
            my[4] = P00; my[5] = P10; my[6] = P11; my[7] = P01;
            my[8] = X00; my[9] = Y00; my[10] = Z00; my[11] = X01; my[12] = Y01; my[13] = Z01;
            my[14] = X10; my[15] = Y10; my[16] = Z10; my[17] = X11; my[18] = Y11; my[19] = Z11;
            my[20] = eb0 + ec0 + p0; my[21] = eb1 + ec1 + p1; my[22] = eb2 + ec2 + p2; my[23] = eb3 + ec3 + p3;
            my[24] = c00; my[25] = c01; my[26] = c10; my[27] = c11;
            my[28] = xn0 | (yn0 << 1) | (xn1 << 2) | (yn1 << 3) | (xn2 << 4) | (yn2 << 5) | (xn3 << 6) | (yn3 << 7);
            my[29] = nt0; my[30] = nt1; my[31] = nt2; my[32] = cellm; my[33] = triBase + triCarry + tp;
            __syncwarp();
            const unsigned nc = __popc(cellm);
            const unsigned cp = grp_incl_scan(nc, sub, Lg) - nc;
            const unsigned ctot = grp_sum(nc, Lg);
            const unsigned cmax = FULL ? ctot : __reduce_max_sync(0xffffffffu, ctot);  // warp-uniform
            const int gbase = (int)(threadIdx.x & 31) & ~(Lg - 1);
            for (unsigned cb = 0; cb < cmax; cb += (unsigned)Lg) {
                const unsigned ci = cb + (unsigned)sub;
                int lo = 0;
                for (int step = Lg >> 1; step > 0; step >>= 1) {
                    const unsigned pl = __shfl_sync(0xffffffffu, cp, gbase + lo + step);
                    if (pl <= ci) lo += step;
                }
                const unsigned po = __shfl_sync(0xffffffffu, cp, gbase + lo);
                if (ci < ctot) {
                    const unsigned *R = s_rec + (gbase + lo) * kRecW;
                    const unsigned cm = R[32], r = ci - po;
                    int b = 0;  // the r-th active cell of the owner's word: the largest b with r cells below
                    for (int step = 16; step > 0; step >>= 1)
                        if ((unsigned)__popc(cm & ((1u << (b + step)) - 1u)) <= r) b += step;
                    const unsigned lt = (1u << b) - 1u;
                    const unsigned ts = R[33] + __popc(R[29] & lt) + 2u * __popc(R[30] & lt) + 4u * __popc(R[31] & lt);
                    const unsigned long long e = s_tab[cube_index(b, R[0], R[1], R[2], R[3], R[4], R[5], R[6], R[7])];
                    const unsigned nt = (unsigned)(e >> 60);
                    for (unsigned q = 0; q < 3 * nt; q++) {
                        const unsigned edge = (unsigned)(e >> (4 * q)) & 15u;
                        const unsigned own = (unsigned)(kEdgeOwner >> (5 * edge)) & 31u;
                        const int o = (int)((own & 1u) * 2 + ((own >> 1) & 1u));  // (di, dj) -> owner index
                        const unsigned dk = (own >> 2) & 1u, ax = own >> 3;
                        const unsigned Xo = R[8 + 3 * o], Yo = R[9 + 3 * o], Zo = R[10 + 3 * o];
                        unsigned slot = R[20 + o];
                        const unsigned vb = (unsigned)b + dk;
                        if (vb < 32) {
                            const unsigned lt2 = (1u << vb) - 1u;
                            slot += __popc(Xo & lt2) + __popc(Yo & lt2) + __popc(Zo & lt2);
                            if (ax >= 1) slot += (Xo >> vb) & 1u;
                            if (ax >= 2) slot += (Yo >> vb) & 1u;
                        } else {
                            slot += R[24 + o];
                            if (ax >= 1) slot += (R[28] >> (2 * o)) & 1u;
                            if (ax >= 2) slot += (R[28] >> (2 * o + 1)) & 1u;
                        }
                        tri[3ull * ts + q] = slot;
                    }
                }
            }
            __syncwarp();  // the records are read before the next words' are written
        }
        triCarry += grp_sum(ntri, Lg);
        ec0 += grp_sum(c00, Lg);
        ec1 += grp_sum(c01, Lg);
        ec2 += grp_sum(c10, Lg);
        ec3 += grp_sum(c11, Lg);
    }
    if (!EMIT && valid && sub == 0) rowCount[row] = make_uint2(triCarry, ec0);
}

// Resident CTAs per SM: the emit is latency-bound, so four CTAs (64 registers, a few spilled)
// beat three: whole-warp rows 0.89 -> 0.82 ms on a 664^3 grid, 4-lane rows 0.780 -> 0.750 ms.
template <bool EMIT, bool FULL>
__global__ void __launch_bounds__(256, 4) k_mc(QGrid g, const unsigned *__restrict__ sign,
                                            const unsigned char *__restrict__ codes, const float *__restrict__ lut,
                                            uint2 *__restrict__ rowCount, const uint2 *__restrict__ rowBase,
                                            unsigned *__restrict__ tri, unsigned long long *__restrict__ vkey,
                                            int lanes) {
    __shared__ unsigned long long s_tab[256];
    __shared__ float s_lut[256];
    __shared__ unsigned s_rec[EMIT ? 8 * 32 * kRecW : 1];  // per warp: one record per lane
    s_tab[threadIdx.x] = c_mc[threadIdx.x];
    if (EMIT) s_lut[threadIdx.x] = lut[threadIdx.x];
    __syncthreads();
    const int E = g.Gc + 1, Lg = FULL ? 32 : lanes;
    const long long first = ((long long)blockIdx.x * 8 + (threadIdx.x >> 5)) * (32 / Lg), nrow = (long long)E * E;
    if (first >= nrow) return;  // the whole warp
    const long long row = first + (threadIdx.x & 31) / Lg;
    mc_row<EMIT, FULL>(g, row, row < nrow, Lg, sign, codes, s_lut, s_tab, rowCount, rowBase, tri, vkey, 0ull,
                       s_rec + (EMIT ? (threadIdx.x >> 5) * 32 * kRecW : 0));
}

// Batch form: rows are numbered molecule after molecule, so one scan over all rows gives
// every molecule's triangles and edge slots contiguous ranges in molecule order.  Each warp
// takes one unit of 32 / Lg rows of one molecule (units numbered by mc_unit_off).
// Four resident CTAs per SM (7.17 -> 5.68 ms for the emit of 256 molecules against two).
template <bool EMIT>
__global__ void __launch_bounds__(256, 4) k_mc_batch(QBatch b, const unsigned *__restrict__ sign,
                                                  const unsigned char *__restrict__ codes, uint2 *__restrict__ rowCount,
                                                  const uint2 *__restrict__ rowBase, unsigned *__restrict__ tri,
                                                  unsigned long long *__restrict__ vkey) {
    __shared__ unsigned long long s_tab[256];
    __shared__ unsigned s_rec[EMIT ? 8 * 32 * kRecW : 1];  // per warp: one record per lane
    s_tab[threadIdx.x] = c_mc[threadIdx.x];
    __syncthreads();
    unsigned *rec = s_rec + (EMIT ? (threadIdx.x >> 5) * 32 * kRecW : 0);
    const unsigned unit = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (unit >= __ldg(b.mc_unit_off + b.n_mol)) return;  // the whole warp
    const unsigned m = qses_find(b.mc_unit_off, b.n_mol, unit);
    const QMol &mol = b.mols[m];
    const QGrid g = mol.g;
    // the batch keeps the words-per-row width (narrow groups, as the single-molecule
    // launches use, measured slower here: emit 5.68 -> 6.12 ms on a 256-molecule batch)
    const int Lg = mc_lanes(g.Gc);
    const unsigned r0 = mol.row_off, nrow = (unsigned)(g.Gc + 1) * (unsigned)(g.Gc + 1);
    const unsigned row = (unit - __ldg(b.mc_unit_off + m)) * (32u / Lg) + (threadIdx.x & 31) / Lg;
    if (Lg == 32)  // warp-uniform
        mc_row<EMIT, true>(g, (long long)row, true, 32, sign + mol.mask_off, codes + mol.code_off,
                           b.lut + 256ull * m, s_tab, rowCount + r0, rowBase + r0, tri, vkey,
                           (unsigned long long)m << b.key_bits, rec);
    else
        mc_row<EMIT, false>(g, (long long)row, row < nrow, Lg, sign + mol.mask_off, codes + mol.code_off,
                            b.lut + 256ull * m, s_tab, rowCount + r0, rowBase + r0, tri, vkey,
                            (unsigned long long)m << b.key_bits, rec);
}

// ------------------------------------------------------------------ weld

__global__ void k_weld_flags(const unsigned long long *__restrict__ skey, unsigned n, uint2 *__restrict__ flags) {
    unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    flags[p] = make_uint2((p == 0 || skey[p] != skey[p - 1]) ? 1u : 0u, 0u);
}

__global__ void k_weld_scatter(QGrid g, const unsigned long long *__restrict__ skey,
                               const unsigned *__restrict__ sval, const uint2 *__restrict__ excl, unsigned n,
                               unsigned *__restrict__ vmap, float *__restrict__ vq) {
    unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const bool first = (p == 0 || skey[p] != skey[p - 1]);
    const unsigned rank = excl[p].x + (first ? 1u : 0u) - 1u;
    vmap[sval[p]] = rank;
    if (first) {
        const unsigned long long key = skey[p], R = (unsigned long long)g.Rq;
        const long long mz = (long long)(key % R) + g.bz;
        const long long my = (long long)((key / R) % R) + g.by;
        const long long mx = (long long)(key / (R * R)) + g.bx;
        vq[3ull * rank] = __fmul_rn((float)mx, QSES_WELD_TOL);
        vq[3ull * rank + 1] = __fmul_rn((float)my, QSES_WELD_TOL);
        vq[3ull * rank + 2] = __fmul_rn((float)mz, QSES_WELD_TOL);
    }
}

// Batch form: the key's high bits name the molecule whose grid decodes the low bits.
__global__ void k_weld_scatter_batch(QBatch b, const unsigned long long *__restrict__ skey,
                                     const unsigned *__restrict__ sval, const uint2 *__restrict__ excl, unsigned n,
                                     unsigned *__restrict__ vmap, float *__restrict__ vq, unsigned *__restrict__ vmol) {
    unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const bool first = (p == 0 || skey[p] != skey[p - 1]);
    const unsigned rank = excl[p].x + (first ? 1u : 0u) - 1u;
    vmap[sval[p]] = rank;
    if (first) {
        const unsigned m = (unsigned)(skey[p] >> b.key_bits);
        const unsigned long long key = skey[p] & ((1ull << b.key_bits) - 1ull);
        const QGrid &g = b.mols[m].g;
        const unsigned long long R = (unsigned long long)g.Rq;
        const long long mz = (long long)(key % R) + g.bz;
        const long long my = (long long)((key / R) % R) + g.by;
        const long long mx = (long long)(key / (R * R)) + g.bx;
        vq[3ull * rank] = __fmul_rn((float)mx, QSES_WELD_TOL);
        vq[3ull * rank + 1] = __fmul_rn((float)my, QSES_WELD_TOL);
        vq[3ull * rank + 2] = __fmul_rn((float)mz, QSES_WELD_TOL);
        vmol[rank] = m;
    }
}

// out[m] = excl[at[m]] for at[m] < n, else the scan total: the first scanned element of
// each molecule's range gives that molecule's offset in the compacted output.
__global__ void k_gather_offsets(const uint2 *__restrict__ excl, const unsigned *__restrict__ at, unsigned n_mol,
                                 unsigned n, const uint2 *__restrict__ total, unsigned *__restrict__ outx,
                                 unsigned *__restrict__ outy) {
    unsigned m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m > n_mol) return;
    const unsigned a = at[m];
    const uint2 v = a < n ? excl[a] : *total;
    if (outx) outx[m] = v.x;
    if (outy) outy[m] = v.y;
}

__global__ void k_remap(unsigned *__restrict__ tri, size_t n3, const unsigned *__restrict__ vmap) {
    size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n3) tri[q] = vmap[tri[q]];
}

// ------------------------------------------------------------ closest atom

__global__ void k_closest(QGrid g, const float *__restrict__ vq, unsigned nv, const float4 *__restrict__ atoms,
                          const uint2 *__restrict__ cells, const unsigned *__restrict__ sorted_to_input,
                          int *__restrict__ asorted, int *__restrict__ ainput) {
    unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const float qx = vq[3ull * v], qy = vq[3ull * v + 1], qz = vq[3ull * v + 2];
    const int cx = __float2int_rz(__fdiv_rn(__fsub_rn(qx, g.ox), g.cell));
    const int cy = __float2int_rz(__fdiv_rn(__fsub_rn(qy, g.oy), g.cell));
    const int cz = __float2int_rz(__fdiv_rn(__fsub_rn(qz, g.oz), g.cell));
    int best = -1;
    float bestd = FLT_MAX;
    for (int a = -1; a <= 1; a++) {
        const int xx = min(max(cx + a, 0), g.gnb - 1);
        for (int b = -1; b <= 1; b++) {
            const int yy = min(max(cy + b, 0), g.gnb - 1);
            for (int d = -1; d <= 1; d++) {
                const int zz = min(max(cz + d, 0), g.gnb - 1);
                const uint2 rg = cells[((size_t)xx * g.gnb + yy) * g.gnb + zz];
                for (unsigned s = rg.x; s < rg.y; s++) {
                    const float4 at = atoms[s];
                    const float ex = __fsub_rn(at.x, qx), ey = __fsub_rn(at.y, qy), ez = __fsub_rn(at.z, qz);
                    const float d2 = __fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex)));
                    if (d2 < bestd) {
                        bestd = d2;
                        best = (int)s;
                    }
                }
            }
        }
    }
    asorted[v] = best;
    ainput[v] = best >= 0 ? (int)sorted_to_input[best] : -1;
}

// Batch form: molecule from the vertex, atom ids local to the molecule.
__global__ void k_closest_batch(QBatch b, const float *__restrict__ vq, const unsigned *__restrict__ vmol,
                                unsigned nv, const float4 *__restrict__ atoms, const uint2 *__restrict__ cells,
                                const unsigned *__restrict__ sorted_to_input, int *__restrict__ asorted,
                                int *__restrict__ ainput) {
    unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const QMol &mol = b.mols[vmol[v]];
    const QGrid g = mol.g;
    const uint2 *mcells = cells + mol.cell_off;
    const float qx = vq[3ull * v], qy = vq[3ull * v + 1], qz = vq[3ull * v + 2];
    const int cx = __float2int_rz(__fdiv_rn(__fsub_rn(qx, g.ox), g.cell));
    const int cy = __float2int_rz(__fdiv_rn(__fsub_rn(qy, g.oy), g.cell));
    const int cz = __float2int_rz(__fdiv_rn(__fsub_rn(qz, g.oz), g.cell));
    int best = -1;
    float bestd = FLT_MAX;
    for (int a = -1; a <= 1; a++) {
        const int xx = min(max(cx + a, 0), g.gnb - 1);
        for (int bb = -1; bb <= 1; bb++) {
            const int yy = min(max(cy + bb, 0), g.gnb - 1);
            for (int d = -1; d <= 1; d++) {
                const int zz = min(max(cz + d, 0), g.gnb - 1);
                const uint2 rg = mcells[((size_t)xx * g.gnb + yy) * g.gnb + zz];
                for (unsigned s = rg.x; s < rg.y; s++) {
                    const float4 at = atoms[s];
                    const float ex = __fsub_rn(at.x, qx), ey = __fsub_rn(at.y, qy), ez = __fsub_rn(at.z, qz);
                    const float d2 = __fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex)));
                    if (d2 < bestd) {
                        bestd = d2;
                        best = (int)s;
                    }
                }
            }
        }
    }
    asorted[v] = best >= 0 ? best - (int)mol.atom_off : -1;
    ainput[v] = best >= 0 ? (int)sorted_to_input[best] - (int)mol.atom_off : -1;
}

// ------------------------------------------------------ degenerate filter

__global__ void k_tri_flags(const unsigned *__restrict__ tri, unsigned nt, uint2 *__restrict__ flags) {
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const unsigned a = tri[3ull * t], b = tri[3ull * t + 1], c = tri[3ull * t + 2];
    flags[t] = make_uint2((a != b && b != c && a != c) ? 1u : 0u, 0u);
}

__global__ void k_tri_compact(const unsigned *__restrict__ tri, unsigned nt, const uint2 *__restrict__ excl,
                              unsigned *__restrict__ out) {
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const unsigned a = tri[3ull * t], b = tri[3ull * t + 1], c = tri[3ull * t + 2];
    if (a != b && b != c && a != c) {
        const size_t o = 3ull * excl[t].x;
        out[o] = a; out[o + 1] = b; out[o + 2] = c;
    }
}

// Batch form: molecules flagged QSES_FLAG_KEEP_DEGENERATE keep every triangle; corners are
// rewritten as molecule-local vertex ids.
__global__ void k_tri_flags_batch(QBatch b, const unsigned *__restrict__ tri, unsigned nt, uint2 *__restrict__ flags) {
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const unsigned m = qses_find(b.tri_off, b.n_mol, t);
    const unsigned a = tri[3ull * t], c1 = tri[3ull * t + 1], c2 = tri[3ull * t + 2];
    const bool keep = (b.mols[m].flags & QSES_FLAG_KEEP_DEGENERATE) || (a != c1 && c1 != c2 && a != c2);
    flags[t] = make_uint2(keep ? 1u : 0u, 0u);
}

__global__ void k_tri_compact_batch(QBatch b, const unsigned *__restrict__ tri, unsigned nt,
                                    const uint2 *__restrict__ excl, unsigned *__restrict__ out) {
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const unsigned m = qses_find(b.tri_off, b.n_mol, t);
    const unsigned a = tri[3ull * t], c1 = tri[3ull * t + 1], c2 = tri[3ull * t + 2];
    const bool keep = (b.mols[m].flags & QSES_FLAG_KEEP_DEGENERATE) || (a != c1 && c1 != c2 && a != c2);
    if (keep) {
        const unsigned v0 = __ldg(b.vtx_off + m);
        const size_t o = 3ull * excl[t].x;
        out[o] = a - v0; out[o + 1] = c1 - v0; out[o + 2] = c2 - v0;
    }
}

// --------------------------------------------------------------- smoothing

// Neighbour lists without a sort.  count: occurrences of each vertex among the 3T triangle
// corners (start[v].x, later scanned); scatter: each corner q is written into its vertex's
// range at a position taken with an atomic (start[v].y, zero after the scan), so the order
// within a range is arbitrary; sortfill: one thread per vertex sorts its range by corner
// index, which restores triangle order exactly (the order getNeighboorsVertices appends
// in, SmoothMesh.cpp:45-66), writes the two other corners of each triangle to the list, and
// doubles the offset (two entries per occurrence).
__global__ void k_csr_count(const unsigned *__restrict__ tri, size_t n3, uint2 *__restrict__ start) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n3) atomicAdd(&start[tri[q]].x, 1u);
}

__global__ void k_csr_scatter(const unsigned *__restrict__ tri, size_t n3, uint2 *__restrict__ start,
                              unsigned *__restrict__ occ) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n3) return;
    const unsigned v = tri[q];
    const unsigned k = atomicAdd(&start[v].y, 1u);
    occ[start[v].x + k] = (unsigned)q;
}

// 12 resident CTAs per SM (at most 42 registers) instead of 9: the kernel waits on scattered
// triangle reads, so more warps in flight hide them
__global__ void __launch_bounds__(128, 12) k_csr_sortfill(const unsigned *__restrict__ tri, unsigned *__restrict__ occ, size_t n3, unsigned nv,
                               uint2 *__restrict__ start, unsigned *__restrict__ nbr) {
    const unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v > nv) return;
    if (v == nv) {
        start[nv] = make_uint2(2u * (unsigned)n3, 0u);
        return;
    }
    const uint2 st = start[v];
    const unsigned o = st.x, n = st.y;  // offset, occurrences
    constexpr unsigned kReg = 16;
    if (n <= kReg) {
        unsigned r[kReg];
#pragma unroll
        for (unsigned i = 0; i < kReg; i++) r[i] = i < n ? occ[o + i] : 0xffffffffu;
        // insertion sort in registers (n is small: ~6 incident triangles per vertex)
#pragma unroll
        for (unsigned i = 1; i < kReg; i++) {
#pragma unroll
            for (unsigned j = i; j > 0; j--) {
                const unsigned a = r[j - 1], b = r[j];
                r[j - 1] = min(a, b);
                r[j] = max(a, b);
            }
        }
#pragma unroll
        for (unsigned i = 0; i < kReg; i++) {
            if (i < n) {
                const unsigned q = r[i], t = q / 3u, c = q - 3u * t;
                const unsigned a = tri[3ull * t], b = tri[3ull * t + 1], d = tri[3ull * t + 2];
                nbr[2ull * (o + i)] = c == 0 ? b : a;
                nbr[2ull * (o + i) + 1] = c == 2 ? b : d;
            }
        }
    } else {
        // rare high-degree vertex: insertion sort in place in global memory
        for (unsigned i = 1; i < n; i++) {
            const unsigned x = occ[o + i];
            unsigned j = i;
            while (j > 0 && occ[o + j - 1] > x) {
                occ[o + j] = occ[o + j - 1];
                j--;
            }
            occ[o + j] = x;
        }
        for (unsigned i = 0; i < n; i++) {
            const unsigned q = occ[o + i], t = q / 3u, c = q - 3u * t;
            const unsigned a = tri[3ull * t], b = tri[3ull * t + 1], d = tri[3ull * t + 2];
            nbr[2ull * (o + i)] = c == 0 ? b : a;
            nbr[2ull * (o + i) + 1] = c == 2 ? b : d;
        }
    }
    start[v] = make_uint2(2u * o, 0u);
}

// Per vertex: lower-id neighbour entries inside its slab (+1 if any lie in lower slabs),
// the count of entries in lower slabs, and its home: slab id and the slab's first vertex.
// Vertices [v0, v1) form the slabs of the table (Q, then Q + 1 bounds in id order).
// Neighbours below v0 belong to waves that finished before this one (final values);
// neighbours at or above v1 are read before their update.
__global__ void k_gs_setup(const uint2 *__restrict__ start, const unsigned *__restrict__ nbr, unsigned v0,
                           unsigned v1, const unsigned *__restrict__ table, unsigned short *__restrict__ cnt_local,
                           int *__restrict__ remote, uint2 *__restrict__ home) {
    unsigned v = v0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= v1) return;
    const unsigned Q = __ldg(table);
    const unsigned *bnd = table + 1;
    unsigned lo = 0, hi = Q;  // bnd[lo] <= v < bnd[hi]
    while (hi - lo > 1) {
        const unsigned mid = (lo + hi) >> 1;
        if (__ldg(bnd + mid) <= v) lo = mid; else hi = mid;
    }
    const unsigned a = __ldg(bnd + lo);
    unsigned loc = 0, rem = 0;
    for (unsigned e = start[v].x; e < start[v + 1].x; e++) {
        const unsigned u = nbr[e];
        if (u < v && u >= v0) {  // below v0: an earlier wave, already final
            if (u >= a) loc++; else rem++;
        }
    }
    cnt_local[v] = (unsigned short)min(loc + (rem ? 1u : 0u), 65535u);
    remote[v] = (int)rem;
    home[v] = make_uint2(lo, a);
}

__global__ void k_to_float4(const float *__restrict__ v3, unsigned nv, float4 *__restrict__ v4) {
    unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nv) v4[v] = make_float4(v3[3ull * v], v3[3ull * v + 1], v3[3ull * v + 2], 0.0f);
}
__global__ void k_from_float4(const float4 *__restrict__ v4, unsigned nv, float *__restrict__ v3) {
    unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nv) {
        const float4 q = v4[v];
        v3[3ull * v] = q.x; v3[3ull * v + 1] = q.y; v3[3ull * v + 2] = q.z;
    }
}

// ------------------------------------------------------------ launchers

static inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

int mc_rows_per_warp(int Gc) { return 32 / mc_lanes(Gc); }
// Lanes per row of the single-molecule count and emit (the per-row totals do not depend on
// it, so the two may differ).  Narrow groups put more rows in flight per warp; measured on
// GB300 (count / emit ms): 664^3 grid 0.248 / 0.821 with whole-warp rows, 0.127 / 0.780
// with 2 / 4 lanes; 502^3 0.105 / 0.404 -> 0.074 / 0.370; 85^3 emit 0.029 -> 0.023 with 8.
static int mc_lanes_for(int Gc, bool emit) {
    const int Wc = (Gc + 32) / 32;
    if (Wc >= 8) return emit ? 4 : 2;
    return emit ? 8 : mc_lanes(Gc);
}
void launch_mc_count(const QGrid &g, const unsigned *sign, uint2 *rowCount, cudaStream_t s) {
    size_t rows = (size_t)(g.Gc + 1) * (g.Gc + 1);
    const int L = mc_lanes_for(g.Gc, false);
    if (L == 32)
        k_mc<false, true><<<nblk(rows, 8), 256, 0, s>>>(g, sign, nullptr, nullptr, rowCount, nullptr, nullptr,
                                                         nullptr, 32);
    else
        k_mc<false, false><<<nblk(rows, 8 * (32 / L)), 256, 0, s>>>(g, sign, nullptr, nullptr,
                                                                    rowCount, nullptr, nullptr, nullptr, L);
}
void launch_mc_emit(const QGrid &g, const unsigned *sign, const unsigned char *codes, const float *lut,
                    const uint2 *rowBase, unsigned *tri, unsigned long long *vkey, cudaStream_t s) {
    size_t rows = (size_t)(g.Gc + 1) * (g.Gc + 1);
    const int L = mc_lanes_for(g.Gc, true);
    if (L == 32)
        k_mc<true, true><<<nblk(rows, 8), 256, 0, s>>>(g, sign, codes, lut, nullptr, rowBase, tri, vkey, 32);
    else
        k_mc<true, false><<<nblk(rows, 8 * (32 / L)), 256, 0, s>>>(g, sign, codes, lut, nullptr,
                                                                   rowBase, tri, vkey, L);
}
void launch_mc_count_batch(const QBatch &b, unsigned units, const unsigned *sign, uint2 *rowCount, cudaStream_t s) {
    k_mc_batch<false><<<nblk(units, 8), 256, 0, s>>>(b, sign, nullptr, rowCount, nullptr, nullptr, nullptr);
}
void launch_mc_emit_batch(const QBatch &b, unsigned units, const unsigned *sign, const unsigned char *codes,
                          const uint2 *rowBase, unsigned *tri, unsigned long long *vkey, cudaStream_t s) {
    k_mc_batch<true><<<nblk(units, 8), 256, 0, s>>>(b, sign, codes, nullptr, rowBase, tri, vkey);
}
void launch_weld_scatter_batch(const QBatch &b, const unsigned long long *skey, const unsigned *sval,
                               const uint2 *excl, unsigned n, unsigned *vmap, float *vq, unsigned *vmol,
                               cudaStream_t s) {
    k_weld_scatter_batch<<<nblk(n, 256), 256, 0, s>>>(b, skey, sval, excl, n, vmap, vq, vmol);
}
void launch_gather_offsets(const uint2 *excl, const unsigned *at, unsigned n_mol, unsigned n, const uint2 *total,
                           unsigned *outx, unsigned *outy, cudaStream_t s) {
    k_gather_offsets<<<nblk(n_mol + 1, 256), 256, 0, s>>>(excl, at, n_mol, n, total, outx, outy);
}
void launch_closest_batch(const QBatch &b, const float *vq, const unsigned *vmol, unsigned nv, const float4 *atoms,
                          const uint2 *cells, const unsigned *sorted_to_input, int *asorted, int *ainput,
                          cudaStream_t s) {
    k_closest_batch<<<nblk(nv, 128), 128, 0, s>>>(b, vq, vmol, nv, atoms, cells, sorted_to_input, asorted, ainput);
}
void launch_tri_flags_batch(const QBatch &b, const unsigned *tri, unsigned nt, uint2 *flags, cudaStream_t s) {
    k_tri_flags_batch<<<nblk(nt, 256), 256, 0, s>>>(b, tri, nt, flags);
}
void launch_tri_compact_batch(const QBatch &b, const unsigned *tri, unsigned nt, const uint2 *excl, unsigned *out,
                              cudaStream_t s) {
    k_tri_compact_batch<<<nblk(nt, 256), 256, 0, s>>>(b, tri, nt, excl, out);
}
void launch_weld_flags(const unsigned long long *skey, unsigned n, uint2 *flags, cudaStream_t s) {
    k_weld_flags<<<nblk(n, 256), 256, 0, s>>>(skey, n, flags);
}
void launch_weld_scatter(const QGrid &g, const unsigned long long *skey, const unsigned *sval, const uint2 *excl,
                         unsigned n, unsigned *vmap, float *vq, cudaStream_t s) {
    k_weld_scatter<<<nblk(n, 256), 256, 0, s>>>(g, skey, sval, excl, n, vmap, vq);
}
void launch_remap(unsigned *tri, size_t n3, const unsigned *vmap, cudaStream_t s) {
    k_remap<<<nblk(n3, 256), 256, 0, s>>>(tri, n3, vmap);
}
void launch_closest(const QGrid &g, const float *vq, unsigned nv, const float4 *atoms, const uint2 *cells,
                    const unsigned *sorted_to_input, int *asorted, int *ainput, cudaStream_t s) {
    k_closest<<<nblk(nv, 128), 128, 0, s>>>(g, vq, nv, atoms, cells, sorted_to_input, asorted, ainput);
}
void launch_tri_flags(const unsigned *tri, unsigned nt, uint2 *flags, cudaStream_t s) {
    k_tri_flags<<<nblk(nt, 256), 256, 0, s>>>(tri, nt, flags);
}
void launch_tri_compact(const unsigned *tri, unsigned nt, const uint2 *excl, unsigned *out, cudaStream_t s) {
    k_tri_compact<<<nblk(nt, 256), 256, 0, s>>>(tri, nt, excl, out);
}
void launch_csr_count(const unsigned *tri, size_t n3, uint2 *start, cudaStream_t s) {
    k_csr_count<<<nblk(n3, 256), 256, 0, s>>>(tri, n3, start);
}
void launch_csr_scatter(const unsigned *tri, size_t n3, uint2 *start, unsigned *occ, cudaStream_t s) {
    k_csr_scatter<<<nblk(n3, 256), 256, 0, s>>>(tri, n3, start, occ);
}
void launch_csr_sortfill(const unsigned *tri, unsigned *occ, size_t n3, unsigned nv, uint2 *start, unsigned *nbr,
                         cudaStream_t s) {
    k_csr_sortfill<<<nblk((size_t)nv + 1, 128), 128, 0, s>>>(tri, occ, n3, nv, start, nbr);
}
void launch_gs_setup(const uint2 *start, const unsigned *nbr, unsigned v0, unsigned v1, const unsigned *table,
                     unsigned short *cnt_local, int *remote, uint2 *home, cudaStream_t s) {
    k_gs_setup<<<nblk(v1 - v0, 256), 256, 0, s>>>(start, nbr, v0, v1, table, cnt_local, remote, home);
}
void launch_to_float4(const float *v3, unsigned nv, float4 *v4, cudaStream_t s) {
    k_to_float4<<<nblk(nv, 256), 256, 0, s>>>(v3, nv, v4);
}
void launch_from_float4(const float4 *v4, unsigned nv, float *v3, cudaStream_t s) {
    k_from_float4<<<nblk(nv, 256), 256, 0, s>>>(v4, nv, v3);
}
}  // namespace qses
