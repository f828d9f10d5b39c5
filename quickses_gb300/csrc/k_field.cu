// Atom grid and SES distance field.
//
//  k_atom_minmax  bbox + largest radius for the grid sizing (getMinMax, CudaSurf.cu:149-174)
//  k_atom_hash    (k_hash.cu) neighbour-cell key per atom
//  k_atom_gather  cell-sorted xyzr + cell start/end (sortCell, Kernels.cu:306-341)
//  k_sas          SAS classification, 8x8 rows x 32 voxels per CTA, atoms staged in shared
//                 memory, row intervals found analytically and verified with the exact
//                 per-voxel predicate (computeInOrOut / probeIntersection, Kernels.cu:344-475)
//  k_edt          probe refine as an exact windowed squared distance transform over the
//                 outside bitmask (distanceFieldRefine, Kernels.cu:478-545)
//
// Field values are stored as one byte per voxel: n in [0, 3R^2] is the squared voxel
// distance to the nearest outside voxel (value probe - dx*sqrt(n)), 253 = border voxel
// with no outside voxel in its window (-dx), 254 = inside (-dx), 255 = outside (probe).
#include "device_common.cuh"
#include "kernels.h"

namespace qses {

// ---------------------------------------------------------------- atoms

__device__ __forceinline__ unsigned enc_f(float f) {
    unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__global__ void k_atom_minmax(const float *__restrict__ xyz, const float *__restrict__ r, unsigned n,
                              unsigned *mm /* 7: min xyz, max xyz, max r (order-preserving encodings) */) {
    unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[4] = {0u, 0u, 0u, 0u};
    for (size_t a = (size_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            unsigned e = enc_f(xyz[3 * a + c]);
            lo[c] = min(lo[c], e);
            hi[c] = max(hi[c], e);
        }
        hi[3] = max(hi[3], enc_f(r[a]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            lo[c] = min(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
            hi[c] = max(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
        }
        hi[3] = max(hi[3], __shfl_xor_sync(0xffffffffu, hi[3], o));
    }
    if ((threadIdx.x & 31) == 0) {
        for (int c = 0; c < 3; c++) {
            atomicMin(&mm[c], lo[c]);
            atomicMax(&mm[3 + c], hi[c]);
        }
        atomicMax(&mm[6], hi[3]);
    }
}

__global__ void k_atom_gather(const float *__restrict__ xyz, const float *__restrict__ r,
                              const unsigned *__restrict__ skey, const unsigned *__restrict__ sidx, unsigned n,
                              float4 *__restrict__ atoms, uint2 *__restrict__ cells) {
    unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    unsigned a = sidx[s];
    atoms[s] = make_float4(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2], r[a]);
    unsigned k = skey[s];
    if (s == 0 || skey[s - 1] != k) cells[k].x = s;
    if (s == n - 1 || skey[s + 1] != k) cells[k].y = s + 1;
}

// ------------------------------------------------------------------ SAS

constexpr int kSasTX = 8, kSasTY = 8, kSasNT = kSasTX * kSasTY, kSasCap = 768;

// Exact per-voxel test along a z row: fma(ez, ez, sxy) < t with ez = z(k) - az.
__device__ __forceinline__ bool zpred(int k, float az, float sxy, float t, float dx, float oz) {
    float ez = __fsub_rn(vox(k, dx, oz), az);
    return __fmaf_rn(ez, ez, sxy) < t;
}

__device__ __forceinline__ unsigned span_bits(int a, int b) {  // bits a..b inclusive, 0 <= a <= b <= 31
    unsigned m = (b - a == 31) ? 0xffffffffu : ((1u << (b - a + 1)) - 1u);
    return m << a;
}

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Voxels k in [k0, klim] of one z row whose squared distance to the atom is below t.
// The set is an interval (the predicate is monotone in |k - k_atom|); its ends are
// estimated in closed form and verified with the exact predicate, with a brute-force
// fallback if the estimate does not verify (so the estimate's square root need not be
// correctly rounded: one approximate instruction).
__device__ __forceinline__ unsigned zmask(float az, float sxy, float t, int k0, int klim, float dx, float oz,
                                          float inv_dx) {
    float kcf = fminf(fmaxf((az - oz) * inv_dx, -1.0e6f), 1.0e6f);
    float h = sqrt_approx(fmaxf(t - sxy, 0.0f)) * inv_dx;
    int lo = max(k0, (int)ceilf(kcf - h));
    int hi = min(klim, (int)floorf(kcf + h));
    if (lo <= hi) {
        if (zpred(lo, az, sxy, t, dx, oz) && zpred(hi, az, sxy, t, dx, oz) &&
            (lo == k0 || !zpred(lo - 1, az, sxy, t, dx, oz)) && (hi == klim || !zpred(hi + 1, az, sxy, t, dx, oz)))
            return span_bits(lo - k0, hi - k0);
    } else {
        int c = min(max(__float2int_rn(kcf), k0), klim);
        if (!zpred(c, az, sxy, t, dx, oz) && (c == k0 || !zpred(c - 1, az, sxy, t, dx, oz)) &&
            (c == klim || !zpred(c + 1, az, sxy, t, dx, oz)))
            return 0u;
    }
    unsigned m = 0;
    for (int k = k0; k <= klim; k++)
        if (zpred(k, az, sxy, t, dx, oz)) m |= 1u << (k - k0);
    return m;
}

// Row-interval classification of one z row against one atom.
__device__ __forceinline__ void sas_row_atom(float px, float py, float ax, float ay, float az, float tin, float tsas,
                                             int k0, int klim, const QGrid &g, float inv_dx, unsigned &sasw,
                                             unsigned &inw) {
    float ex = __fsub_rn(px, ax), ey = __fsub_rn(py, ay);
    float sxy = __fmaf_rn(ey, ey, __fmul_rn(ex, ex));
    if (sxy < tsas) {
        sasw |= zmask(az, sxy, tsas, k0, klim, g.dx, g.oz, inv_dx);
        if (sxy < tin) inw |= zmask(az, sxy, tin, k0, klim, g.dx, g.oz, inv_dx);
    }
}

__device__ __forceinline__ void atom_thresholds(float r, const QGrid &g, float &tin, float &tsas) {
    float rin = __fsub_rn(r, g.dx);                        // d < r - dx  (Kernels.cu:377)
    tin = rin > 0.0f ? __fmul_rn(rin, rin) : -1.0f;
    float rs = __fadd_rn(g.probe, r);                      // d < probe + r  (Kernels.cu:380)
    tsas = __fmul_rn(rs, rs);
}

// One SAS tile: z-word w of the 8 x 8 rows starting at (i0, j0) = (8 ib, 8 jb).
__device__ __forceinline__ void sas_tile(const QGrid &g, int w, int jb, int ib, const float4 *__restrict__ atoms,
                                         const uint2 *__restrict__ cells, unsigned *__restrict__ inMask,
                                         unsigned *__restrict__ outMask) {
    __shared__ float s_x[kSasCap], s_y[kSasCap], s_z[kSasCap], s_tin[kSasCap], s_ts[kSasCap];
    __shared__ int s_n, s_over;
    const int j0 = jb * kSasTY, i0 = ib * kSasTX;
    const int t = threadIdx.x, i = i0 + t / kSasTY, j = j0 + t % kSasTY, k0 = w * 32;
    // Voxels with an index >= lim on an axis are never computed and stay outside: the last
    // layer G-1 (Kernels.cu:436-441) and, for a slice box, its own last layer and whatever
    // lies at or past the molecule grid's last layer.  Positions use the grid index
    // box index + off (gridToSpace of ijkOffset, Kernels.cu:427-446).
    const int G = g.G, lastx = g.lim[0] - 1, lasty = g.lim[1] - 1, lastz = g.lim[2] - 1;
    const int oi = g.off[0], oj = g.off[1], ok = g.off[2];
    const unsigned valid = (k0 + 32 <= G) ? 0xffffffffu : ((1u << (G - k0)) - 1u);
    const int fz = max(g.lim[2] - k0, 0);  // first forced-outside bit of this word
    const unsigned forced = fz >= 32 ? 0u : (valid & ~((1u << fz) - 1u));
    const int klim = min(k0 + 31, lastz);
    const float inv_dx = 1.0f / g.dx;
    unsigned sasw = 0, inw = 0;

    if (i0 <= lastx && j0 <= lasty && k0 <= lastz) {
        const float bx0 = vox(i0 + oi, g.dx, g.ox), bx1 = vox(min(i0 + kSasTX - 1, lastx) + oi, g.dx, g.ox);
        const float by0 = vox(j0 + oj, g.dx, g.oy), by1 = vox(min(j0 + kSasTY - 1, lasty) + oj, g.dx, g.oy);
        const float bz0 = vox(k0 + ok, g.dx, g.oz), bz1 = vox(klim + ok, g.dx, g.oz);
        const float ext = g.cell * 1.01f + g.dx;
        auto crange = [&](float lo, float hi, float o, int &c0, int &c1) {
            c0 = min(max((int)floorf((lo - ext - o) / g.cell), 0), g.gnb - 1);
            c1 = min(max((int)floorf((hi + ext - o) / g.cell), 0), g.gnb - 1);
        };
        int cx0, cx1, cy0, cy1, cz0, cz1;
        crange(bx0, bx1, g.ox, cx0, cx1);
        crange(by0, by1, g.oy, cy0, cy1);
        crange(bz0, bz1, g.oz, cz0, cz1);
        const int ncy = cy1 - cy0 + 1, ncz = cz1 - cz0 + 1, ncell = (cx1 - cx0 + 1) * ncy * ncz;
        if (t == 0) { s_n = 0; s_over = 0; }
        __syncthreads();
        // Stage every atom whose probe-inflated sphere can reach the tile (conservative box test).
        for (int c = t; c < ncell; c += kSasNT) {
            int cz = c % ncz, cy = (c / ncz) % ncy, cx = c / (ncz * ncy);
            uint2 rg = cells[((size_t)(cx0 + cx) * g.gnb + (cy0 + cy)) * g.gnb + (cz0 + cz)];
            for (unsigned s = rg.x; s < rg.y; s++) {
                float4 a = atoms[s];
                float ddx = fmaxf(fmaxf(bx0 - a.x, a.x - bx1), 0.0f);
                float ddy = fmaxf(fmaxf(by0 - a.y, a.y - by1), 0.0f);
                float ddz = fmaxf(fmaxf(bz0 - a.z, a.z - bz1), 0.0f);
                float rs = g.probe + a.w;
                if (ddx * ddx + ddy * ddy + ddz * ddz <= rs * rs * 1.001f + 1e-3f) {
                    int q = atomicAdd(&s_n, 1);
                    if (q < kSasCap) {
                        float tin, tsas;
                        atom_thresholds(a.w, g, tin, tsas);
                        s_x[q] = a.x; s_y[q] = a.y; s_z[q] = a.z; s_tin[q] = tin; s_ts[q] = tsas;
                    } else {
                        s_over = 1;
                    }
                }
            }
        }
        __syncthreads();
        if (i <= lastx && j <= lasty) {
            const float px = vox(i + oi, g.dx, g.ox), py = vox(j + oj, g.dx, g.oy);
            const int kg0 = k0 + ok, kglim = klim + ok;  // z range as grid indices (bits from kg0)
            if (!s_over) {
                const int na = s_n;
                for (int q = 0; q < na; q++)
                    sas_row_atom(px, py, s_x[q], s_y[q], s_z[q], s_tin[q], s_ts[q], kg0, kglim, g, inv_dx, sasw,
                                 inw);
            } else {
                // Too many candidates for shared memory: walk the cells directly.
                for (int c = 0; c < ncell; c++) {
                    int cz = c % ncz, cy = (c / ncz) % ncy, cx = c / (ncz * ncy);
                    uint2 rg = cells[((size_t)(cx0 + cx) * g.gnb + (cy0 + cy)) * g.gnb + (cz0 + cz)];
                    for (unsigned s = rg.x; s < rg.y; s++) {
                        float4 a = atoms[s];
                        float tin, tsas;
                        atom_thresholds(a.w, g, tin, tsas);
                        sas_row_atom(px, py, a.x, a.y, a.z, tin, tsas, kg0, kglim, g, inv_dx, sasw, inw);
                    }
                }
            }
        }
    }
    if (i < G && j < G) {
        unsigned outw, inw2;
        if (i > lastx || j > lasty) {
            outw = valid;
            inw2 = 0u;
        } else {
            outw = (~sasw & valid) | forced;
            inw2 = inw & ~forced;
        }
        size_t idx = ((size_t)i * G + j) * g.W + w;
        inMask[idx] = inw2;
        outMask[idx] = outw;
    }
}

__global__ void __launch_bounds__(kSasNT) k_sas(QGrid g, const float4 *__restrict__ atoms,
                                                const uint2 *__restrict__ cells, unsigned *__restrict__ inMask,
                                                unsigned *__restrict__ outMask) {
    sas_tile(g, blockIdx.x, blockIdx.y, blockIdx.z, atoms, cells, inMask, outMask);
}

// ------------------------------------------------------------------ refine

constexpr int kEdtNT = 256;

// One refine tile: z-word w of the TX x TY rows starting at (TX ib, TY jb), with an R halo.
// Larger tiles re-read less halo per row (the z pass runs on (TX+2R)(TY+2R) rows for TX TY
// output rows) at the cost of shared memory (dynamic, edt_smem_bytes); the shape is chosen
// by the autotuner.

// Min-plus on four byte distances of a word (255 = none) without the byte-SIMD add and
// min, which this GPU runs as several instructions each: the bytes are spread over two
// words of 16-bit halves (one byte permute each), where adding a square <= 81 cannot carry
// (255 + 81 < 2^16) and the 16-bit min is one instruction; packing back clamps at 255.
// Real distances stay below 255 (y <= 2 R^2 = 162, x <= 3 R^2 = 243) and "none" at or above
// it, so the results equal the saturating byte arithmetic's.
__device__ __forceinline__ unsigned spread_lo(unsigned w) { return __byte_perm(w, 0u, 0x4140); }  // bytes 0, 1
__device__ __forceinline__ unsigned spread_hi(unsigned w) { return __byte_perm(w, 0u, 0x4342); }  // bytes 2, 3
__device__ __forceinline__ unsigned pack_bytes(unsigned lo, unsigned hi) {
    return __byte_perm(__vminu2(lo, 0x00ff00ffu), __vminu2(hi, 0x00ff00ffu), 0x6420);
}

// Squared z distances of one 32-voxel word c (bit = outside voxel) with its neighbouring
// words a (below) and d (above), one byte per voxel (<= R^2, 255 = none), four per output
// word.  Bit-parallel: the outside set grows by one voxel per step (two funnel shifts over
// the neighbouring words), and the voxels first covered at step k are at distance k.
__device__ __forceinline__ unsigned nibble_bytes(unsigned nib) {  // 4 bits -> 0xff in each set bit's byte
    return ((nib * 0x00204081u) & 0x01010101u) * 0xffu;           // copies at bits 0, 7, 14, 21: no carries
}
__device__ __forceinline__ void z_word(unsigned a, unsigned c, unsigned d, int R, unsigned out[8]) {
    if ((a | c | d) == 0u || c == 0xffffffffu) {  // no outside voxel within 32, or all outside
#pragma unroll
        for (int k = 0; k < 8; k++) out[k] = c ? 0u : 0xffffffffu;
        return;
    }
#pragma unroll
    for (int j = 0; j < 8; j++) out[j] = ~nibble_bytes((c >> (4 * j)) & 0xfu);  // outside: 0, else none
    unsigned cov = c;  // voxels with an outside voxel within k
    for (int k = 1; k <= R; k++) {
        // bit b of the right funnel shift is voxel b + k, of the left one voxel b - k
        const unsigned nc = cov | __funnelshift_r(c, d, k) | __funnelshift_l(a, c, k);
        const unsigned nw = nc & ~cov;  // nearest outside voxel at distance k
        cov = nc;
        if (nw == 0u) continue;
        const unsigned v = (unsigned)(k * k) * 0x01010101u;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const unsigned m = nibble_bytes((nw >> (4 * j)) & 0xfu);
            out[j] = (out[j] & ~m) | (v & m);
        }
    }
}

// Shared-memory layout of one refine tile for a window of R voxels: the halo rows' outside
// words (only without precomputed z distances), their z distances, the y-pass rows, and the
// tile's in/out words.  Sized per launch, so a smaller window (a larger voxel) fits more CTAs
// per SM; the largest layout (R = QSES_RMAX, no z distances) bounds every other.
struct EdtLayout {
    size_t g_off, h_off, in_off, ot_off, bytes;
};
__host__ __device__ __forceinline__ EdtLayout edt_layout(int TX, int TY, int R, bool have_zd) {
    const size_t HX = (size_t)TX + 2 * R, HY = (size_t)TY + 2 * R;
    EdtLayout L;
    L.g_off = have_zd ? 0 : ((12 * HX * HY + 15) & ~(size_t)15);  // [HX HY][3] outside words first
    L.h_off = L.g_off + 32 * HX * HY;                                 // [HX HY][32] z distances
    L.in_off = L.h_off + 32 * HX * (size_t)TY;                         // [HX][TY][32] y-pass rows
    L.ot_off = L.in_off + 4 * (size_t)TX * TY;
    L.bytes = L.ot_off + 4 * (size_t)TX * TY;
    return L;
}

template <int TX, int TY>
__device__ __forceinline__ void edt_tile(const QGrid &g, int w, int jb, int ib, const unsigned *__restrict__ inMask,
                                         const unsigned *__restrict__ outMask, unsigned char *__restrict__ codes,
                                         unsigned *__restrict__ signMask,
                                         const unsigned char *__restrict__ zd = nullptr) {
    const EdtLayout L = edt_layout(TX, TY, g.R, zd != nullptr);
    extern __shared__ __align__(16) unsigned char edt_smem[];
    unsigned (*s_out)[3] = reinterpret_cast<unsigned (*)[3]>(edt_smem);  // without zd only
    // Squared distances, one byte per voxel (255 = none); the y and x passes work on four
    // voxels per 32-bit word with saturating byte adds, so 255 stays "none".
    unsigned char (*s_g)[32] = reinterpret_cast<unsigned char (*)[32]>(edt_smem + L.g_off);
    unsigned char (*s_h)[TY][32] = reinterpret_cast<unsigned char (*)[TY][32]>(edt_smem + L.h_off);
    unsigned *s_in = reinterpret_cast<unsigned *>(edt_smem + L.in_off);
    unsigned *s_ot = reinterpret_cast<unsigned *>(edt_smem + L.ot_off);
    const int j0 = jb * TY, i0 = ib * TX;
    const int R = g.R, G = g.G, W = g.W, t = threadIdx.x;
    const int HX = TX + 2 * R, HY = TY + 2 * R, k0 = w * 32;
    const unsigned valid = (k0 + 32 <= G) ? 0xffffffffu : ((1u << (G - k0)) - 1u);

    int anyb = 0;
    for (int q = t; q < TX * TY; q += kEdtNT) {
        int i = i0 + q / TY, j = j0 + q % TY;
        unsigned iw = 0u, ow = 0xffffffffu;
        if (i < G && j < G) {
            size_t idx = ((size_t)i * G + j) * W + w;
            iw = inMask[idx];
            ow = outMask[idx];
            anyb |= (valid & ~iw & ~ow) != 0u;
        }
        s_in[q] = iw;
        s_ot[q] = ow;
    }
    const int has_border = __syncthreads_or(anyb);
    int has_out = 0;
    if (has_border && zd) {
        // z distances computed once per voxel by k_edt_z: load the halo rows' bytes
        int any = 0;
        for (int q = t; q < HX * HY * 2; q += kEdtNT) {
            const int row = q >> 1, half = q & 1;
            const int i = i0 - R + row / HY, j = j0 - R + row % HY;
            uint4 v = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
            if (i >= 0 && i < G && j >= 0 && j < G)
                v = __ldg(reinterpret_cast<const uint4 *>(zd + ((size_t)i * G + j) * g.Gp + (size_t)k0) + half);
            reinterpret_cast<uint4 *>(s_g[row])[half] = v;
            any |= (v.x & v.y & v.z & v.w) != 0xffffffffu;
        }
        has_out = __syncthreads_or(any);
        if (has_out) {
            // y: min over dj of dj^2 + g^2 (<= 2 R^2 = 162 < 255), four voxels per word.
            for (int q = t; q < HX * TY * 8; q += kEdtNT) {
                const int w4 = q & 7, y = (q >> 3) % TY, hx = (q >> 3) / TY;
                unsigned lo = 0xffffffffu, hi = 0xffffffffu;
                for (int dj = -R; dj <= R; dj++) {
                    const unsigned gw = reinterpret_cast<const unsigned *>(s_g[hx * HY + y + R + dj])[w4];
                    const unsigned d2 = (unsigned)(dj * dj) * 0x00010001u;
                    lo = __vminu2(lo, spread_lo(gw) + d2);
                    hi = __vminu2(hi, spread_hi(gw) + d2);
                }
                reinterpret_cast<unsigned *>(s_h[hx][y])[w4] = pack_bytes(lo, hi);
            }
            __syncthreads();
        }
    } else if (has_border) {
        int any = 0;
        for (int q = t; q < HX * HY; q += kEdtNT) {
            int i = i0 - R + q / HY, j = j0 - R + q % HY;
            unsigned a = 0u, b = 0u, c = 0u;
            if (i >= 0 && i < G && j >= 0 && j < G) {
                size_t base = ((size_t)i * G + j) * W;
                if (w > 0) a = outMask[base + w - 1];
                b = outMask[base + w];
                if (w + 1 < W) c = outMask[base + w + 1];
            }
            s_out[q][0] = a; s_out[q][1] = b; s_out[q][2] = c;
            any |= (a | b | c) != 0u;
        }
        has_out = __syncthreads_or(any);
    }
    if (has_border && has_out && !zd) {
        // z: squared distance (in voxels, <= R^2) to the nearest outside voxel along the row,
        // one row of 32 voxels per thread
        for (int q = t; q < HX * HY; q += kEdtNT) {
            unsigned out[8];
            z_word(s_out[q][0], s_out[q][1], s_out[q][2], R, out);
            uint4 *dst = reinterpret_cast<uint4 *>(s_g[q]);
            dst[0] = make_uint4(out[0], out[1], out[2], out[3]);
            dst[1] = make_uint4(out[4], out[5], out[6], out[7]);
        }
        __syncthreads();
        // y: min over dj of dj^2 + g^2 (<= 2 R^2 = 162 < 255), four voxels per word.
        for (int q = t; q < HX * TY * 8; q += kEdtNT) {
            const int w4 = q & 7, y = (q >> 3) % TY, hx = (q >> 3) / TY;
            unsigned lo = 0xffffffffu, hi = 0xffffffffu;
            for (int dj = -R; dj <= R; dj++) {
                const unsigned gw = reinterpret_cast<const unsigned *>(s_g[hx * HY + y + R + dj])[w4];
                const unsigned d2 = (unsigned)(dj * dj) * 0x00010001u;
                lo = __vminu2(lo, spread_lo(gw) + d2);
                hi = __vminu2(hi, spread_hi(gw) + d2);
            }
            reinterpret_cast<unsigned *>(s_h[hx][y])[w4] = pack_bytes(lo, hi);
        }
        __syncthreads();
    }
    // x: min over di of di^2 + h, then codes and sign bits; 4 threads per row, 8 voxels each
    // (TX TY / 64 rows per thread: the same trip count in every warp).
    for (int row = t >> 2; row < TX * TY; row += kEdtNT / 4) {
    const int part = t & 3, x = row / TY, y = row % TY, i = i0 + x, j = j0 + y;
    unsigned sgn = 0u;
    if (i < G && j < G) {
        const unsigned iw = s_in[row], ow = s_ot[row];
        // min over di of di^2 + h (<= 3 R^2 = 243 < 255) for this thread's 8 voxels
        unsigned bw0 = 0xffffffffu, bw1 = 0xffffffffu;
        if (has_out) {
            unsigned l0 = 0xffffffffu, h0 = 0xffffffffu, l1 = 0xffffffffu, h1 = 0xffffffffu;
            for (int di = -R; di <= R; di++) {
                const uint2 hw = reinterpret_cast<const uint2 *>(s_h[x + R + di][y])[part];
                const unsigned d2 = (unsigned)(di * di) * 0x00010001u;
                l0 = __vminu2(l0, spread_lo(hw.x) + d2);
                h0 = __vminu2(h0, spread_hi(hw.x) + d2);
                l1 = __vminu2(l1, spread_lo(hw.y) + d2);
                h1 = __vminu2(h1, spread_hi(hw.y) + d2);
            }
            bw0 = pack_bytes(l0, h0);
            bw1 = pack_bytes(l1, h1);
        }
        unsigned long long packed = 0ull;
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int b = part * 8 + e;
            const unsigned bit = 1u << b;
            unsigned code;
            if (!(valid & bit)) code = QSES_CODE_OUT;  // row padding, never read
            else if (ow & bit) code = QSES_CODE_OUT;
            else if (iw & bit) code = QSES_CODE_IN;
            else {
                const unsigned best = ((e < 4 ? bw0 : bw1) >> (8 * (e & 3))) & 0xffu;
                code = best != 255u ? best : QSES_CODE_NONE;
            }
            packed |= (unsigned long long)code << (8 * e);
            if ((valid & bit) && code != QSES_CODE_OUT && (int)code >= g.negmin) sgn |= bit;
        }
        *(unsigned long long *)(codes + ((size_t)i * G + j) * g.Gp + k0 + part * 8) = packed;
    }
    sgn |= __shfl_xor_sync(0xffffffffu, sgn, 1);
    sgn |= __shfl_xor_sync(0xffffffffu, sgn, 2);
    if (part == 0 && i < G && j < G) signMask[((size_t)i * G + j) * W + w] = sgn;
    }
}

// z pass of the refine, once per voxel: squared distance (in voxels, <= R^2, 255 = none) to
// the nearest outside voxel along the z row within the R window, one thread per 32-voxel
// word.  zd has the codes' layout.
__device__ __forceinline__ void edt_z_word(const QGrid &g, size_t q, const unsigned *__restrict__ outMask,
                                           unsigned char *__restrict__ zd) {
    const size_t row = q / g.W;
    const int w = (int)(q - row * g.W), W = g.W;
    const size_t base = row * W;
    const unsigned a = w > 0 ? __ldg(outMask + base + w - 1) : 0u, c = __ldg(outMask + base + w),
                   d = w + 1 < W ? __ldg(outMask + base + w + 1) : 0u;
    unsigned out[8];
    z_word(a, c, d, g.R, out);
    uint4 *dst = reinterpret_cast<uint4 *>(zd + row * g.Gp + (size_t)w * 32);
    dst[0] = make_uint4(out[0], out[1], out[2], out[3]);
    dst[1] = make_uint4(out[4], out[5], out[6], out[7]);
}

__global__ void __launch_bounds__(256) k_edt_z(QGrid g, const unsigned *__restrict__ outMask,
                                               unsigned char *__restrict__ zd) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < (size_t)g.G * g.G * g.W) edt_z_word(g, q, outMask, zd);
}

// Batch form: one thread per mask word of every molecule.
__global__ void __launch_bounds__(256) k_edt_z_batch(QBatch b, unsigned words, const unsigned *__restrict__ outMask,
                                                     unsigned char *__restrict__ zd) {
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= words) return;
    const unsigned m = qses_find(b.word_off, b.n_mol, q);
    const QMol &mol = b.mols[m];
    edt_z_word(mol.g, q - __ldg(b.word_off + m), outMask + mol.mask_off, zd + mol.code_off);
}

template <int TX, int TY>
__global__ void __launch_bounds__(kEdtNT) k_edt(QGrid g, const unsigned *__restrict__ inMask,
                                                const unsigned *__restrict__ outMask,
                                                unsigned char *__restrict__ codes, unsigned *__restrict__ signMask,
                                                const unsigned char *__restrict__ zd) {
    edt_tile<TX, TY>(g, blockIdx.x, blockIdx.y, blockIdx.z, inMask, outMask, codes, signMask, zd);
}

// ------------------------------------------------------------ batched field

// Persistent CTAs take field tiles of every molecule of a batch from one work counter.
// A tile is decoded within its molecule exactly as the single-molecule grid would index it.
__device__ __forceinline__ bool next_tile(const QBatch &b, unsigned *counter, unsigned &m, int &w, int &jb, int &ib) {
    __shared__ unsigned s_item, s_m;
    __syncthreads();  // the previous tile's shared memory is no longer in use
    if (threadIdx.x == 0) {
        const unsigned it = atomicAdd(counter, 1u);
        s_item = it;
        s_m = it < __ldg(b.tile_off + b.n_mol) ? qses_find(b.tile_off, b.n_mol, it) : 0xffffffffu;
    }
    __syncthreads();
    m = s_m;
    if (m == 0xffffffffu) return false;
    const QGrid &g = b.mols[m].g;
    const unsigned loc = s_item - __ldg(b.tile_off + m), ny = (unsigned)(g.G + 7) / 8u;
    w = (int)(loc % (unsigned)g.W);
    jb = (int)((loc / (unsigned)g.W) % ny);
    ib = (int)(loc / ((unsigned)g.W * ny));
    return true;
}

__global__ void __launch_bounds__(kSasNT) k_sas_batch(QBatch b, const float4 *__restrict__ atoms,
                                                      const uint2 *__restrict__ cells, unsigned *__restrict__ inMask,
                                                      unsigned *__restrict__ outMask, unsigned *counter) {
    unsigned m;
    int w, jb, ib;
    while (next_tile(b, counter, m, w, jb, ib)) {
        const QMol mol = b.mols[m];
        sas_tile(mol.g, w, jb, ib, atoms, cells + mol.cell_off, inMask + mol.mask_off, outMask + mol.mask_off);
    }
}

__global__ void __launch_bounds__(kEdtNT) k_edt_batch(QBatch b, const unsigned *__restrict__ inMask,
                                                      const unsigned *__restrict__ outMask,
                                                      unsigned char *__restrict__ codes,
                                                      unsigned *__restrict__ signMask, unsigned *counter,
                                                      const unsigned char *__restrict__ zd) {
    unsigned m;
    int w, jb, ib;
    while (next_tile(b, counter, m, w, jb, ib)) {
        const QMol mol = b.mols[m];
        edt_tile<8, 8>(mol.g, w, jb, ib, inMask + mol.mask_off, outMask + mol.mask_off, codes + mol.code_off,
                       signMask + mol.mask_off, zd ? zd + mol.code_off : nullptr);
    }
}

// ------------------------------------------------------------ launchers

void launch_atom_minmax(const float *xyz, const float *r, unsigned n, unsigned *mm, cudaStream_t s) {
    unsigned blocks = (n + 255) / 256;
    if (blocks > 608) blocks = 608;
    if (blocks == 0) blocks = 1;
    k_atom_minmax<<<blocks, 256, 0, s>>>(xyz, r, n, mm);
}
void launch_atom_gather(const float *xyz, const float *r, const unsigned *skey, const unsigned *sidx, unsigned n,
                        float4 *atoms, uint2 *cells, cudaStream_t s) {
    k_atom_gather<<<(n + 255) / 256, 256, 0, s>>>(xyz, r, skey, sidx, n, atoms, cells);
}
void launch_sas(const QGrid &g, const float4 *atoms, const uint2 *cells, unsigned *inMask, unsigned *outMask,
                cudaStream_t s) {
    dim3 grid(g.W, (g.G + kSasTY - 1) / kSasTY, (g.G + kSasTX - 1) / kSasTX);
    k_sas<<<grid, kSasNT, 0, s>>>(g, atoms, cells, inMask, outMask);
}
template <int TX, int TY>
static void launch_edt_shape(const QGrid &g, const unsigned *inMask, const unsigned *outMask, unsigned char *codes,
                             unsigned *signMask, cudaStream_t s, const unsigned char *zd) {
    static const bool attr = [] {
        return cudaFuncSetAttribute((const void *)k_edt<TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)edt_layout(TX, TY, QSES_RMAX, false).bytes) == cudaSuccess;
    }();
    (void)attr;
    const size_t smem = edt_layout(TX, TY, g.R, zd != nullptr).bytes;
    dim3 grid(g.W, (g.G + TY - 1) / TY, (g.G + TX - 1) / TX);
    k_edt<TX, TY><<<grid, kEdtNT, smem, s>>>(g, inMask, outMask, codes, signMask, zd);
}

void launch_edt(const QGrid &g, const unsigned *inMask, const unsigned *outMask, unsigned char *codes,
                unsigned *signMask, cudaStream_t s, int shape, unsigned char *zd) {
    // zd (G G Gp bytes, optional): the z pass once per voxel, then tiles load it.  Without
    // it each tile computes its halo rows' z distances itself (the allocation-free entry
    // point); with the bit-parallel z pass that measured the same or slower (0.846 against
    // 0.836 ms on the 664^3 grid), so the pipeline keeps the separate pass.
    if (zd) {
        const size_t words = (size_t)g.G * g.G * g.W;
        k_edt_z<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(g, outMask, zd);
    }
    // shape 0: 8 x 8 rows, 1: 16 x 8, 2: 16 x 16, 3: 32 x 16 (shared memory per CTA at R = 7
    // with z distances: 21, 29, 45 and 70 KB)
    switch (shape) {
        case 3: launch_edt_shape<32, 16>(g, inMask, outMask, codes, signMask, s, zd); break;
        case 2: launch_edt_shape<16, 16>(g, inMask, outMask, codes, signMask, s, zd); break;
        case 1: launch_edt_shape<16, 8>(g, inMask, outMask, codes, signMask, s, zd); break;
        default: launch_edt_shape<8, 8>(g, inMask, outMask, codes, signMask, s, zd); break;
    }
}
static unsigned persistent_blocks(const void *fn, int threads, unsigned items, size_t smem = 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    unsigned blocks = (unsigned)(sms * (per_sm > 0 ? per_sm : 1));
    return items < blocks ? (items ? items : 1u) : blocks;
}
void launch_sas_batch(const QBatch &b, unsigned tiles, const float4 *atoms, const uint2 *cells, unsigned *inMask,
                      unsigned *outMask, unsigned *counter, cudaStream_t s) {
    k_sas_batch<<<persistent_blocks((const void *)k_sas_batch, kSasNT, tiles), kSasNT, 0, s>>>(
        b, atoms, cells, inMask, outMask, counter);
}
void launch_edt_batch(const QBatch &b, unsigned tiles, const unsigned *inMask, const unsigned *outMask,
                      unsigned char *codes, unsigned *signMask, unsigned *counter, cudaStream_t s, unsigned words,
                      unsigned char *zd) {
    if (zd) k_edt_z_batch<<<(words + 255) / 256, 256, 0, s>>>(b, words, outMask, zd);
    const size_t smem = edt_layout(8, 8, QSES_RMAX, false).bytes;  // molecules of any window
    k_edt_batch<<<persistent_blocks((const void *)k_edt_batch, kEdtNT, tiles, smem), kEdtNT, smem, s>>>(
        b, inMask, outMask, codes, signMask, counter, zd);
}

}  // namespace qses
