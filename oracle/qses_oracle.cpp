/*
 * CPU oracle for the QuickSES atoms+radii -> SES mesh path (see qses_oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY - the checker for the CUDA path, never part of it.
 * Compiled with -ffp-contract=off so that FP32 arithmetic is plain IEEE single precision
 * except where fmaf() is written out; the CUDA kernels use the same operation order with
 * explicit __f*_rn intrinsics, so fp32 mode agrees with them bit for bit.
 *
 * Reference semantics restated here (file:line into nezix/QuickSES):
 *   grid sizing ................ CudaSurf.cu:149-174, 250-253, 546-574, 629-635
 *   atom hashing + sort ........ Kernels.cu:119-131, 185-216; CudaSurf.cu:605-618
 *   cell start/end ............. Kernels.cu:306-341
 *   SAS classification ......... Kernels.cu:344-475
 *   probe refine ............... Kernels.cu:478-545
 *   marching cubes ............. MarchingCubes.cu:571-851 (single-slice cell range)
 *   vertex weld ................ MarchingCubes.cu:853-862; CudaSurf.cu:425-500
 *   closest atom per vertex .... Kernels.cu:547-604
 *   Laplacian smoothing ........ SmoothMesh.cpp:26-123
 *   concatenation + filter ..... CudaSurf.cu:787-841
 *   reference slicing mode ..... CudaSurf.cu:629-754 (per-slice boxes, seam cell ranges,
 *                                the unwritten last triangle, per-slice weld and smoothing)
 */
#include "qses_oracle.h"
#include "mc_table.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const float kProbe = 1.4f;     /* PROBERADIUS, Kernels.cu:26 */
const float kWeldTol = 0.001f; /* EPSILON, Kernels.cu:27 */

/* Corner offsets in QuickSES order (MarchingCubes.cu:625-632, 774-780). */
const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                           {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
/* Edge e joins corners kEdge[e][0] -> kEdge[e][1] (MarchingCubes.cu:814-825). */
const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                          {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* ---------------- arithmetic policies ---------------- */

struct F32 {
    typedef float T;
    static float vox(int i, float dx, float o) { return fmaf((float)i, dx, o); }
    static float sq(float ex, float ey, float ez) { return fmaf(ez, ez, fmaf(ey, ey, ex * ex)); }
    /* inside: d < r - dx and near: d < probe + r (Kernels.cu:377-381), compared on
       squared distances against thresholds rounded to float. */
    static void thresholds(float r, float dx, float &tin, float &tsas) {
        float rin = r - dx;
        tin = rin > 0.0f ? rin * rin : -1.0f;
        float rs = kProbe + r;
        tsas = rs * rs;
    }
    static bool inside(float s, float tin, float, float) { return s < tin; }
    static bool near_(float s, float tsas, float, float) { return s < tsas; }
};

struct F64 {
    typedef double T;
    static double vox(int i, float dx, float o) { return (double)o + (double)i * (double)dx; }
    static double sq(double ex, double ey, double ez) { return ex * ex + ey * ey + ez * ez; }
    static void thresholds(float, float, float &tin, float &tsas) { tin = 0; tsas = 0; }
    static bool inside(double s, float, float r, float dx) {
        return std::sqrt(s) < (double)r - (double)dx;
    }
    static bool near_(double s, float, float r, float) {
        return std::sqrt(s) < (double)kProbe + (double)r;
    }
};

struct Atoms {
    std::vector<float> x, y, z, r;   /* cell-sorted */
    std::vector<uint32_t> sorted_to_input;
    std::vector<uint32_t> cell_start; /* gnb^3 + 1 */
};

int hash_of(float px, float py, float pz, const oracle_grid *g) {
    /* spaceToGrid + flatten3DTo1D (Kernels.cu:119-131): truncating float division. */
    int cx = (int)((px - g->ox) / g->cell);
    int cy = (int)((py - g->oy) / g->cell);
    int cz = (int)((pz - g->oz) / g->cell);
    return g->gnb * g->gnb * cx + g->gnb * cy + cz;
}

void build_atoms(const float *xyz, const float *rad, unsigned N, const oracle_grid *g, Atoms &A) {
    std::vector<int32_t> h(N);
    std::vector<uint32_t> idx(N);
    for (unsigned a = 0; a < N; a++) {
        h[a] = hash_of(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2], g);
        idx[a] = a;
    }
    /* thrust::sort with compare_int2 is CUB's merge sort, which is stable
       (CudaSurf.cu:610-612): equal cells keep input order. */
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return h[a] < h[b]; });
    size_t ncell = (size_t)g->gnb * g->gnb * g->gnb;
    A.cell_start.assign(ncell + 1, 0);
    A.x.resize(N); A.y.resize(N); A.z.resize(N); A.r.resize(N);
    A.sorted_to_input = idx;
    for (unsigned s = 0; s < N; s++) {
        unsigned a = idx[s];
        A.x[s] = xyz[3 * a]; A.y[s] = xyz[3 * a + 1]; A.z[s] = xyz[3 * a + 2]; A.r[s] = rad[a];
        A.cell_start[(size_t)h[a] + 1]++;
    }
    for (size_t c = 0; c < ncell; c++) A.cell_start[c + 1] += A.cell_start[c];
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Neighbour-cell range covering [p - ext, p + ext] (monotone in p, so it contains the
   cells of all atoms within ext of p). */
inline void cell_range(double p, double o, double cell, double ext, int gnb, int &lo, int &hi) {
    lo = clampi((int)std::floor((p - ext - o) / cell), 0, gnb - 1);
    hi = clampi((int)std::floor((p + ext - o) / cell), 0, gnb - 1);
}

/* SAS classification of one voxel (computeInOrOut, Kernels.cu:344-392): 2 = inside
   (value -dx), 1 = border (value 0), 0 = outside (value probe).  Every atom within reach
   is tested; the result does not depend on visiting order. */
template <class P>
int sas_class(int i, int j, int k, const oracle_grid *g, const Atoms &A,
              const std::vector<float> &tin, const std::vector<float> &tsas) {
    if (i >= g->G - 1 || j >= g->G - 1 || k >= g->G - 1) return 0; /* Kernels.cu:436-441 */
    typename P::T px = P::vox(i, g->dx, g->ox), py = P::vox(j, g->dx, g->oy),
                  pz = P::vox(k, g->dx, g->oz);
    double ext = 1.01 * (double)g->cell + (double)g->dx;
    int x0, x1, y0, y1, z0, z1;
    cell_range((double)px, g->ox, g->cell, ext, g->gnb, x0, x1);
    cell_range((double)py, g->oy, g->cell, ext, g->gnb, y0, y1);
    cell_range((double)pz, g->oz, g->cell, ext, g->gnb, z0, z1);
    bool nearp = false;
    for (int cx = x0; cx <= x1; cx++)
        for (int cy = y0; cy <= y1; cy++) {
            size_t base = ((size_t)cx * g->gnb + cy) * g->gnb;
            for (unsigned s = A.cell_start[base + z0]; s < A.cell_start[base + z1 + 1]; s++) {
                typename P::T ex = px - (typename P::T)A.x[s];
                typename P::T ey = py - (typename P::T)A.y[s];
                typename P::T ez = pz - (typename P::T)A.z[s];
                typename P::T d2 = P::sq(ex, ey, ez);
                if (P::inside(d2, tin[s], A.r[s], g->dx)) return 2;
                if (P::near_(d2, tsas[s], A.r[s], g->dx)) nearp = true;
            }
        }
    return nearp ? 1 : 0;
}

template <class P>
void field_codes(const oracle_grid *g, const Atoms &A, int x0, int x1, uint8_t *codes) {
    const int G = g->G, R = g->R;
    const unsigned N = (unsigned)A.x.size();
    std::vector<float> tin(N), tsas(N);
    for (unsigned s = 0; s < N; s++) P::thresholds(A.r[s], g->dx, tin[s], tsas[s]);

    /* SAS classes for planes [ax0, ax1): the slab plus the refine halo. */
    int ax0 = std::max(0, x0 - R), ax1 = std::min(G, x1 + R);
    int nx = ax1 - ax0;
    std::vector<uint8_t> cls((size_t)nx * G * G);
#pragma omp parallel for schedule(dynamic, 1)
    for (int ii = 0; ii < nx; ii++)
        for (int j = 0; j < G; j++)
            for (int k = 0; k < G; k++)
                cls[((size_t)ii * G + j) * G + k] = (uint8_t)sas_class<P>(ax0 + ii, j, k, g, A, tin, tsas);

    /* Summed-area table of "outside" for O(1) empty-window tests. */
    const size_t Gp = (size_t)G + 1;
    std::vector<int32_t> sat((size_t)(nx + 1) * Gp * Gp, 0);
    for (int ii = 0; ii < nx; ii++)
        for (int j = 0; j < G; j++)
            for (int k = 0; k < G; k++) {
                int o = cls[((size_t)ii * G + j) * G + k] == 0;
                size_t a = ((size_t)(ii + 1) * Gp + (j + 1)) * Gp + (k + 1);
                sat[a] = o + sat[a - 1] + sat[a - Gp] + sat[a - Gp * Gp] - sat[a - Gp - 1] -
                         sat[a - Gp * Gp - 1] - sat[a - Gp * Gp - Gp] + sat[a - Gp * Gp - Gp - 1];
            }
    auto box = [&](int i0, int i1, int j0, int j1, int k0, int k1) -> int32_t {
        /* inclusive bounds in slab-local i */
        auto S = [&](int a, int b, int c) { return sat[((size_t)a * Gp + b) * Gp + c]; };
        i1++; j1++; k1++;
        return S(i1, j1, k1) - S(i0, j1, k1) - S(i1, j0, k1) - S(i1, j1, k0) + S(i0, j0, k1) +
               S(i0, j1, k0) + S(i1, j0, k0) - S(i0, j0, k0);
    };

    /* Window offsets ordered by squared length: the first outside voxel found is the
       nearest one (distanceFieldRefine, Kernels.cu:513-539, window clamped to the grid). */
    struct Off { int di, dj, dk, n; };
    std::vector<Off> offs;
    for (int a = -R; a <= R; a++)
        for (int b = -R; b <= R; b++)
            for (int c = -R; c <= R; c++) offs.push_back({a, b, c, a * a + b * b + c * c});
    std::stable_sort(offs.begin(), offs.end(), [](const Off &p, const Off &q) { return p.n < q.n; });

#pragma omp parallel for schedule(dynamic, 1)
    for (int i = x0; i < x1; i++) {
        int ii = i - ax0;
        for (int j = 0; j < G; j++)
            for (int k = 0; k < G; k++) {
                uint8_t c = cls[((size_t)ii * G + j) * G + k];
                uint8_t code;
                if (c == 0) code = ORACLE_CODE_OUT;
                else if (c == 2) code = ORACLE_CODE_IN;
                else {
                    int wi0 = std::max(i - R, 0) - ax0, wi1 = std::min(i + R, G - 1) - ax0;
                    int wj0 = std::max(j - R, 0), wj1 = std::min(j + R, G - 1);
                    int wk0 = std::max(k - R, 0), wk1 = std::min(k + R, G - 1);
                    code = ORACLE_CODE_NONE;
                    if (box(wi0, wi1, wj0, wj1, wk0, wk1) > 0) {
                        for (const Off &o : offs) {
                            int a = i + o.di, b = j + o.dj, d = k + o.dk;
                            if (a < 0 || b < 0 || d < 0 || a >= G || b >= G || d >= G) continue;
                            if (cls[((size_t)(a - ax0) * G + b) * G + d] == 0) {
                                code = (uint8_t)o.n;
                                break;
                            }
                        }
                    }
                }
                codes[((size_t)(i - x0) * G + j) * G + k] = code;
            }
    }
}

/* ---------------- marching cubes, weld, closest atom, smoothing ---------------- */

template <class P> struct Lut;
template <> struct Lut<F32> {
    float v[256];
    explicit Lut(const oracle_grid *g) { oracle_code_lut_f32(g, v); }
};
template <> struct Lut<F64> {
    double v[256];
    explicit Lut(const oracle_grid *g) { oracle_code_lut_f64(g, v); }
};

template <class P> struct Quant;
template <> struct Quant<F32> {
    static int64_t q(float v) { return (int64_t)roundf(v / kWeldTol); }  /* MarchingCubes.cu:859 */
    static double back(int64_t m) { return (double)((float)m * kWeldTol); }
    static float interp(float pa, float pb, float fa, float fb) {
        float t = (-fa) / (fb - fa);                       /* MarchingCubes.cu:731-734 */
        return fmaf(t, pb - pa, pa);
    }
    static float offset(int o, float dx) { return (float)o * dx; }
};
template <> struct Quant<F64> {
    static int64_t q(double v) { return (int64_t)std::llround(v / (double)kWeldTol); }
    static double back(int64_t m) { return (double)m * (double)kWeldTol; }
    static double interp(double pa, double pb, double fa, double fb) {
        double t = (-fa) / (fb - fa);
        return pa + t * (pb - pa);
    }
    static double offset(int o, float dx) { return (double)o * (double)dx; }
};

/* One box of the reference's slicing (CudaSurf.cu:629-682): D^3 voxels whose index
   (i, j, k) is voxel (i, j, k) + off of the grid; cells [clo, chi) per axis are emitted
   (countVertexPerCell's rules, MarchingCubes.cu:578-604).  Without a box the whole grid is
   one box: D = G, off = 0, cells [0, Gc). */
struct BoxView {
    int D;
    int off[3];
    int clo[3], chi[3];
};

template <class P>
oracle_mesh *mesh_from_codes(const uint8_t *codes, const oracle_grid *g, const Atoms &A,
                             const BoxView *bv = nullptr) {
    typedef typename P::T T;
    BoxView whole = {g->G, {0, 0, 0}, {0, 0, 0}, {g->Gc, g->Gc, g->Gc}};
    const BoxView &box = bv ? *bv : whole;
    const int G = box.D;
    const int lox = box.clo[0], hix = box.chi[0], loy = box.clo[1], hiy = box.chi[1], loz = box.clo[2], hiz = box.chi[2];
    const int Gc = std::max(hix, std::max(hiy, hiz));
    const bool shifted = (box.off[0] | box.off[1] | box.off[2]) != 0;
    Lut<P> lut(g);
    auto code = [&](int i, int j, int k) { return codes[((size_t)i * G + j) * G + k]; };
    auto neg = [&](int i, int j, int k) { return lut.v[code(i, j, k)] < (T)0; };

    oracle_mesh *m = (oracle_mesh *)calloc(1, sizeof(oracle_mesh));
    if (Gc <= 0 || lox >= hix || loy >= hiy || loz >= hiz) return m;
    const int64_t E = Gc + 1;
    /* Active edges in owner-voxel linear order; voxel (i,j,k) owns its +x, +y, +z edges.
       An edge counts when an emitted cell has it. */
    std::vector<int64_t> eid;
    for (int i = lox; i <= hix; i++)
        for (int j = loy; j <= hiy; j++)
            for (int k = loz; k <= hiz; k++) {
                bool s = neg(i, j, k);
                int64_t base = ((i * E + j) * E + k) * 3;
                if (i < hix && s != neg(i + 1, j, k)) eid.push_back(base + 0);
                if (j < hiy && s != neg(i, j + 1, k)) eid.push_back(base + 1);
                if (k < hiz && s != neg(i, j, k + 1)) eid.push_back(base + 2);
            }
    const size_t ne = eid.size();
    auto slot_of = [&](int i, int j, int k, int axis) -> int32_t {
        int64_t id = ((i * E + j) * E + k) * 3 + axis;
        auto it = std::lower_bound(eid.begin(), eid.end(), id);
        return (int32_t)(it - eid.begin());
    };

    /* Triangles in cell linear order x*G^2 + y*G + z (MarchingCubes.cu:397-399, 830-850). */
    static const int owner[12][4] = {{0, 0, 0, 0}, {1, 0, 0, 1}, {0, 1, 0, 0}, {0, 0, 0, 1},
                                     {0, 0, 1, 0}, {1, 0, 1, 1}, {0, 1, 1, 0}, {0, 0, 1, 1},
                                     {0, 0, 0, 2}, {1, 0, 0, 2}, {1, 1, 0, 2}, {0, 1, 0, 2}};
    std::vector<int32_t> tri;
    for (int i = lox; i < hix; i++)
        for (int j = loy; j < hiy; j++)
            for (int k = loz; k < hiz; k++) {
                int ci = 0;
                for (int c = 0; c < 8; c++)
                    if (neg(i + kCorner[c][0], j + kCorner[c][1], k + kCorner[c][2])) ci |= 1 << c;
                const int *row = ORACLE_TRI_TABLE[ci];
                for (int v = 0; v < 15 && row[v] != -1; v++) {
                    const int *o = owner[row[v]];
                    tri.push_back(slot_of(i + o[0], j + o[1], k + o[2], o[3]));
                }
            }

    /* Edge vertices (vertexInterp, MarchingCubes.cu:731-734) quantised to 0.001 A
       (groupVertices, MarchingCubes.cu:853-862). */
    std::vector<int64_t> mq(ne * 3);
    for (size_t s = 0; s < ne; s++) {
        int64_t id = eid[s];
        int axis = (int)(id % 3);
        int64_t vox = id / 3;
        int k = (int)(vox % E), j = (int)((vox / E) % E), i = (int)(vox / (E * E));
        int ijk[3] = {i, j, k};
        float org[3] = {g->ox, g->oy, g->oz};
        int b[3] = {i, j, k};
        b[axis]++;
        T fa = lut.v[code(i, j, k)], fb = lut.v[code(b[0], b[1], b[2])];
        for (int c = 0; c < 3; c++) {
            T pa = P::vox(ijk[c], g->dx, org[c]);
            T v = pa;
            if (c == axis) v = Quant<P>::interp(pa, P::vox(ijk[c] + 1, g->dx, org[c]), fa, fb);
            if (shifted) v = v + Quant<P>::offset(box.off[c], g->dx); /* MarchingCubes.cu:841-848 */
            mq[s * 3 + c] = Quant<P>::q(v);
        }
    }
    /* Weld: unique quantised positions in lexicographic (x, y, z) order; each edge takes
       the rank of its position (CudaSurf.cu:444-457: sort, unique, lower_bound). */
    std::vector<uint32_t> order(ne);
    for (size_t s = 0; s < ne; s++) order[s] = (uint32_t)s;
    auto lexless = [&](uint32_t a, uint32_t b) {
        for (int c = 0; c < 3; c++)
            if (mq[a * 3 + c] != mq[b * 3 + c]) return mq[a * 3 + c] < mq[b * 3 + c];
        return false;
    };
    std::sort(order.begin(), order.end(), lexless);
    std::vector<int32_t> rank(ne);
    std::vector<int64_t> uq;
    for (size_t p = 0; p < ne; p++) {
        if (p == 0 || lexless(order[p - 1], order[p])) {
            for (int c = 0; c < 3; c++) uq.push_back(mq[order[p] * 3 + c]);
        }
        rank[order[p]] = (int32_t)(uq.size() / 3 - 1);
    }
    const unsigned nv = (unsigned)(uq.size() / 3);
    const unsigned nt = (unsigned)(tri.size() / 3);

    m->nv = nv; m->nt = nt; m->ne = (unsigned)ne;
    m->v = (double *)malloc(sizeof(double) * 3 * (nv ? nv : 1));
    m->vq = (double *)malloc(sizeof(double) * 3 * (nv ? nv : 1));
    m->tri = (int32_t *)malloc(sizeof(int32_t) * 3 * (nt ? nt : 1));
    m->atom_sorted = (int32_t *)malloc(sizeof(int32_t) * (nv ? nv : 1));
    m->atom_input = (int32_t *)malloc(sizeof(int32_t) * (nv ? nv : 1));
    m->edge_vertex = (int32_t *)malloc(sizeof(int32_t) * (ne ? ne : 1));
    for (size_t s = 0; s < ne; s++) m->edge_vertex[s] = rank[s];
    for (size_t t = 0; t < tri.size(); t++) m->tri[t] = rank[tri[t]];
    for (size_t q = 0; q < uq.size(); q++) m->vq[q] = Quant<P>::back(uq[q]);

    /* Closest atom per welded vertex (closestAtomPerVertex, Kernels.cu:547-604): 27
       clamped neighbour cells, first strict minimum, index into the sorted atom array. */
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t)nv; v++) {
        T q[3] = {(T)m->vq[v * 3], (T)m->vq[v * 3 + 1], (T)m->vq[v * 3 + 2]};
        int c0[3];
        float org[3] = {g->ox, g->oy, g->oz};
        for (int c = 0; c < 3; c++) c0[c] = (int)((float)((float)q[c] - org[c]) / g->cell);
        int best = -1;
        T bestd = std::numeric_limits<T>::max();
        for (int a = -1; a <= 1; a++)
            for (int b = -1; b <= 1; b++)
                for (int d = -1; d <= 1; d++) {
                    int cx = clampi(c0[0] + a, 0, g->gnb - 1), cy = clampi(c0[1] + b, 0, g->gnb - 1),
                        cz = clampi(c0[2] + d, 0, g->gnb - 1);
                    size_t cid = ((size_t)cx * g->gnb + cy) * g->gnb + cz;
                    for (unsigned s = A.cell_start[cid]; s < A.cell_start[cid + 1]; s++) {
                        T ex = (T)A.x[s] - q[0], ey = (T)A.y[s] - q[1], ez = (T)A.z[s] - q[2];
                        T d2 = P::sq(ex, ey, ez);
                        if (d2 < bestd) { bestd = d2; best = (int)s; }
                    }
                }
        m->atom_sorted[v] = best;
        m->atom_input[v] = best >= 0 ? (int32_t)A.sorted_to_input[best] : -1;
    }
    memcpy(m->v, m->vq, sizeof(double) * 3 * nv);
    return m;
}

/* Neighbour lists with multiplicity in triangle order (getNeighboorsVertices,
   SmoothMesh.cpp:45-66) as CSR. */
void neighbour_csr(const int32_t *tri, unsigned nt, unsigned nv, std::vector<uint32_t> &start,
                   std::vector<int32_t> &nbr) {
    start.assign(nv + 1, 0);
    for (size_t t = 0; t < (size_t)nt * 3; t++) start[tri[t] + 1] += 2;
    for (unsigned v = 0; v < nv; v++) start[v + 1] += start[v];
    nbr.resize(start[nv]);
    std::vector<uint32_t> fill(start.begin(), start.end() - 1);
    for (unsigned t = 0; t < nt; t++) {
        int32_t a = tri[3 * t], b = tri[3 * t + 1], c = tri[3 * t + 2];
        nbr[fill[a]++] = b; nbr[fill[a]++] = c;
        nbr[fill[b]++] = a; nbr[fill[b]++] = c;
        nbr[fill[c]++] = a; nbr[fill[c]++] = b;
    }
}

/* Gauss-Seidel Laplacian in vertex-id order, in place (smoothMeshLaplacian,
   SmoothMesh.cpp:96-123). */
template <typename T>
void smooth_gs(T *v, unsigned nv, const int32_t *tri, unsigned nt, int passes) {
    if (passes <= 0) return;
    std::vector<uint32_t> start;
    std::vector<int32_t> nbr;
    neighbour_csr(tri, nt, nv, start, nbr);
    for (int p = 0; p < passes; p++)
        for (unsigned i = 0; i < nv; i++) {
            T sx = 0, sy = 0, sz = 0;
            for (uint32_t e = start[i]; e < start[i + 1]; e++) {
                sx = sx + v[3 * nbr[e]];
                sy = sy + v[3 * nbr[e] + 1];
                sz = sz + v[3 * nbr[e] + 2];
            }
            T n = (T)(int)(start[i + 1] - start[i]);
            v[3 * i] = sx / n;
            v[3 * i + 1] = sy / n;
            v[3 * i + 2] = sz / n;
        }
}

void finish_mesh(oracle_mesh *m, int smooth, int fp64) {
    if (smooth > 0 && m->nv) {
        if (fp64) {
            smooth_gs<double>(m->v, m->nv, m->tri, m->nt, smooth);
        } else {
            std::vector<float> f(m->nv * 3);
            for (size_t q = 0; q < f.size(); q++) f[q] = (float)m->v[q];
            smooth_gs<float>(f.data(), m->nv, m->tri, m->nt, smooth);
            for (size_t q = 0; q < f.size(); q++) m->v[q] = f[q];
        }
    }
    /* API_computeSES drops triangles with a repeated index (CudaSurf.cu:820-829). */
    std::vector<int32_t> kept;
    for (unsigned t = 0; t < m->nt; t++) {
        int32_t a = m->tri[3 * t], b = m->tri[3 * t + 1], c = m->tri[3 * t + 2];
        if (a != b && b != c && a != c) { kept.push_back(a); kept.push_back(b); kept.push_back(c); }
    }
    m->nt_kept = (unsigned)(kept.size() / 3);
    m->tri_kept = (int32_t *)malloc(sizeof(int32_t) * (kept.size() ? kept.size() : 1));
    if (!kept.empty()) memcpy(m->tri_kept, kept.data(), sizeof(int32_t) * kept.size());
}

/* ---------------- the reference's slicing (CudaSurf.cu:629-754) ---------------- */

/* Voxel codes of one slice box, as probeIntersection and distanceFieldRefine compute them
   on a slice (Kernels.cu:394-545, launched by CudaSurf.cu:653-729): box voxels at or past
   lim on an axis keep the memset value probe (outside); the others are classified at their
   grid index off + (i, j, k) (sas_class applies the grid's own last layer); a border
   voxel's refine window is clamped to the box (Kernels.cu:517-523).  Returns the number of
   border voxels (notEmptyCells, CudaSurf.cu:688-691). */
template <class P>
size_t box_codes(const oracle_grid *g, const Atoms &A, int D, const int off[3], const int lim[3], uint8_t *codes) {
    const int R = g->R;
    const unsigned N = (unsigned)A.x.size();
    std::vector<float> tin(N), tsas(N);
    for (unsigned s = 0; s < N; s++) P::thresholds(A.r[s], g->dx, tin[s], tsas[s]);
    const size_t D2 = (size_t)D * D;
    std::vector<uint8_t> cls(D2 * D);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < D; i++)
        for (int j = 0; j < D; j++)
            for (int k = 0; k < D; k++) {
                const bool kept = i >= lim[0] || j >= lim[1] || k >= lim[2];
                cls[i * D2 + (size_t)j * D + k] =
                    kept ? 0 : (uint8_t)sas_class<P>(off[0] + i, off[1] + j, off[2] + k, g, A, tin, tsas);
            }
    /* Summed-area table of "outside" for O(1) empty-window tests. */
    const size_t P1 = (size_t)D + 1;
    std::vector<int32_t> sat(P1 * P1 * P1, 0);
    for (int i = 0; i < D; i++)
        for (int j = 0; j < D; j++)
            for (int k = 0; k < D; k++) {
                const int o = cls[i * D2 + (size_t)j * D + k] == 0;
                const size_t a = ((size_t)(i + 1) * P1 + (j + 1)) * P1 + (k + 1);
                sat[a] = o + sat[a - 1] + sat[a - P1] + sat[a - P1 * P1] - sat[a - P1 - 1] - sat[a - P1 * P1 - 1] -
                         sat[a - P1 * P1 - P1] + sat[a - P1 * P1 - P1 - 1];
            }
    auto outside_in = [&](int i0, int i1, int j0, int j1, int k0, int k1) {  // inclusive bounds
        auto S_ = [&](int a, int b, int c) { return sat[((size_t)a * P1 + b) * P1 + c]; };
        i1++; j1++; k1++;
        return S_(i1, j1, k1) - S_(i0, j1, k1) - S_(i1, j0, k1) - S_(i1, j1, k0) + S_(i0, j0, k1) + S_(i0, j1, k0) +
               S_(i1, j0, k0) - S_(i0, j0, k0);
    };
    struct Off { int di, dj, dk, n; };
    std::vector<Off> offs;
    for (int a = -R; a <= R; a++)
        for (int b = -R; b <= R; b++)
            for (int c = -R; c <= R; c++) offs.push_back({a, b, c, a * a + b * b + c * c});
    std::stable_sort(offs.begin(), offs.end(), [](const Off &p, const Off &q) { return p.n < q.n; });
    size_t border = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : border)
    for (int i = 0; i < D; i++)
        for (int j = 0; j < D; j++)
            for (int k = 0; k < D; k++) {
                const uint8_t c = cls[i * D2 + (size_t)j * D + k];
                uint8_t code = c == 0 ? ORACLE_CODE_OUT : ORACLE_CODE_IN;
                if (c == 1) {
                    border++;
                    code = ORACLE_CODE_NONE;
                    if (outside_in(std::max(i - R, 0), std::min(i + R, D - 1), std::max(j - R, 0),
                                   std::min(j + R, D - 1), std::max(k - R, 0), std::min(k + R, D - 1)) == 0) {
                        codes[i * D2 + (size_t)j * D + k] = code;
                        continue;
                    }
                    for (const Off &o : offs) {
                        const int a = i + o.di, b = j + o.dj, d = k + o.dk;
                        if (a < 0 || b < 0 || d < 0 || a >= D || b >= D || d >= D) continue;
                        if (cls[a * D2 + (size_t)b * D + d] == 0) {
                            code = (uint8_t)o.n;
                            break;
                        }
                    }
                }
                codes[i * D2 + (size_t)j * D + k] = code;
            }
    return border;
}

/* Cells of one box axis that countVertexPerCell emits (MarchingCubes.cu:578-604), its
   int bounds compared with the unsigned cell index as the kernel does: [lo, hi), empty as
   lo == hi. */
void box_cells(int D, int R, int off, int &lo, int &hi) {
    lo = hi = 0;
    bool any = false;
    for (int c = 0; c < D; c++) {
        const unsigned i = (unsigned)c;
        bool skip = i > (unsigned)(D - 2);
        if (off != 0 && i < (unsigned)(R - 3)) skip = true;
        if (off == 0 && i >= (unsigned)(D - R * 2 - 1)) skip = true;
        if (i >= (unsigned)(D - R - 1)) skip = true;
        if (!skip) {
            if (!any) lo = c;
            any = true;
            hi = c + 1;
        }
    }
}

/* generateTriangleVerticesSMEM writes indices below totalVerts - 3 only (MarchingCubes.cu:845
   with CudaSurf.cu:421): a slice's last triangle is never written.  It is dropped here, with
   every vertex that only it used; the other vertices keep their order. */
void drop_last_triangle(oracle_mesh *m) {
    if (m->nt == 0) return;
    m->nt--;
    std::vector<char> used(m->nv, 0);
    for (size_t q = 0; q < (size_t)m->nt * 3; q++) used[m->tri[q]] = 1;
    std::vector<int32_t> id(m->nv, -1);
    unsigned nv = 0;
    for (unsigned v = 0; v < m->nv; v++)
        if (used[v]) {
            id[v] = (int32_t)nv;
            for (int c = 0; c < 3; c++) {
                m->vq[3 * nv + c] = m->vq[3 * v + c];
                m->v[3 * nv + c] = m->v[3 * v + c];
            }
            m->atom_sorted[nv] = m->atom_sorted[v];
            m->atom_input[nv] = m->atom_input[v];
            nv++;
        }
    m->nv = nv;
    for (size_t q = 0; q < (size_t)m->nt * 3; q++) m->tri[q] = id[m->tri[q]];
    for (unsigned e = 0; e < m->ne; e++) m->edge_vertex[e] = id[m->edge_vertex[e]];
}

/* computeSlicedSES's slice loop (CudaSurf.cu:629-754) and API_computeSES's concatenation
   (CudaSurf.cu:796-836): cores of S = min(slice, G) voxels, boxes of D = min(slice + 2R, G)
   voxels starting R before each core (clamped at 0), x outermost; a slice without border
   voxels gives no mesh; each slice's mesh is welded and smoothed alone; vertex ids of later
   slices are offset by the vertices before them. */
template <class P>
oracle_mesh *sliced_ses(const float *xyz, const float *rad, unsigned N, const oracle_grid *g, int slice, int smooth,
                        int fp64) {
    Atoms A;
    build_atoms(xyz, rad, N, g, A);
    const int G = g->G, R = g->R;
    const int S = std::min(slice, G), D = std::min(slice + 2 * R, G);
    std::vector<oracle_mesh *> parts;
    std::vector<uint8_t> codes((size_t)D * D * D);
    for (int x = 0; x < G; x += S)
        for (int y = 0; y < G; y += S)
            for (int z = 0; z < G; z += S) {
                const int core[3] = {x, y, z};
                int off[3], lim[3];
                BoxView bv;
                bv.D = D;
                for (int a = 0; a < 3; a++) {
                    off[a] = std::max(0, core[a] - R);
                    lim[a] = std::min(D - 1, G - 1 - off[a]);
                    bv.off[a] = off[a];
                    box_cells(D, R, off[a], bv.clo[a], bv.chi[a]);
                }
                if (box_codes<P>(g, A, D, off, lim, codes.data()) == 0) continue;
                oracle_mesh *m = mesh_from_codes<P>(codes.data(), g, A, &bv);
                drop_last_triangle(m);
                finish_mesh(m, smooth, fp64);
                parts.push_back(m);
            }
    oracle_mesh *out = (oracle_mesh *)calloc(1, sizeof(oracle_mesh));
    const unsigned ns = (unsigned)parts.size();
    out->nslices = ns;
    out->slice_v = (uint32_t *)calloc(ns + 1, sizeof(uint32_t));
    out->slice_t = (uint32_t *)calloc(ns + 1, sizeof(uint32_t));
    out->slice_tk = (uint32_t *)calloc(ns + 1, sizeof(uint32_t));
    for (unsigned q = 0; q < ns; q++) {
        out->slice_v[q + 1] = out->slice_v[q] + parts[q]->nv;
        out->slice_t[q + 1] = out->slice_t[q] + parts[q]->nt;
        out->slice_tk[q + 1] = out->slice_tk[q] + parts[q]->nt_kept;
    }
    const unsigned nv = out->slice_v[ns], nt = out->slice_t[ns], ntk = out->slice_tk[ns];
    out->nv = nv; out->nt = nt; out->nt_kept = ntk;
    out->v = (double *)malloc(sizeof(double) * 3 * (nv ? nv : 1));
    out->vq = (double *)malloc(sizeof(double) * 3 * (nv ? nv : 1));
    out->tri = (int32_t *)malloc(sizeof(int32_t) * 3 * (nt ? nt : 1));
    out->tri_kept = (int32_t *)malloc(sizeof(int32_t) * 3 * (ntk ? ntk : 1));
    out->atom_sorted = (int32_t *)malloc(sizeof(int32_t) * (nv ? nv : 1));
    out->atom_input = (int32_t *)malloc(sizeof(int32_t) * (nv ? nv : 1));
    for (unsigned q = 0; q < ns; q++) {
        const oracle_mesh *m = parts[q];
        const unsigned v0 = out->slice_v[q], t0 = out->slice_t[q], k0 = out->slice_tk[q];
        memcpy(out->v + 3ull * v0, m->v, sizeof(double) * 3 * m->nv);
        memcpy(out->vq + 3ull * v0, m->vq, sizeof(double) * 3 * m->nv);
        memcpy(out->atom_sorted + v0, m->atom_sorted, sizeof(int32_t) * m->nv);
        memcpy(out->atom_input + v0, m->atom_input, sizeof(int32_t) * m->nv);
        for (size_t e = 0; e < 3ull * m->nt; e++) out->tri[3ull * t0 + e] = m->tri[e] + (int32_t)v0;
        for (size_t e = 0; e < 3ull * m->nt_kept; e++) out->tri_kept[3ull * k0 + e] = m->tri_kept[e] + (int32_t)v0;
        oracle_mesh_free(parts[q]);
    }
    return out;
}

/* ---------------- point-to-triangle distance for Hausdorff ---------------- */

struct V3 { double x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 madd(V3 a, V3 b, double s) { return {a.x + b.x * s, a.y + b.y * s, a.z + b.z * s}; }

/* Closest point on triangle (Ericson, Real-Time Collision Detection, 5.1.5). */
double pt_tri_d2(V3 p, V3 a, V3 b, V3 c) {
    V3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    double d1 = dot(ab, ap), d2 = dot(ac, ap);
    V3 q;
    if (d1 <= 0 && d2 <= 0) q = a;
    else {
        V3 bp = sub(p, b);
        double d3 = dot(ab, bp), d4 = dot(ac, bp);
        if (d3 >= 0 && d4 <= d3) q = b;
        else {
            double vc = d1 * d4 - d3 * d2;
            if (vc <= 0 && d1 >= 0 && d3 <= 0) q = madd(a, ab, d1 / (d1 - d3));
            else {
                V3 cp = sub(p, c);
                double d5 = dot(ab, cp), d6 = dot(ac, cp);
                if (d6 >= 0 && d5 <= d6) q = c;
                else {
                    double vb = d5 * d2 - d1 * d6;
                    if (vb <= 0 && d2 >= 0 && d6 <= 0) q = madd(a, ac, d2 / (d2 - d6));
                    else {
                        double va = d3 * d6 - d5 * d4;
                        if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0)
                            q = madd(b, sub(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6)));
                        else {
                            double den = 1.0 / (va + vb + vc);
                            q = madd(madd(a, ab, vb * den), ac, vc * den);
                        }
                    }
                }
            }
        }
    }
    V3 d = sub(p, q);
    return dot(d, d);
}

/* max over vertices of A (those with only[v] set, when only is given) of the distance to
   surface B */
double one_sided(const double *va, unsigned nva, const double *vb, unsigned nvb, const int32_t *tb,
                 unsigned ntb, double *per_vertex = nullptr, const uint8_t *only = nullptr) {
    if (nva == 0 || ntb == 0) return nva == 0 ? 0.0 : std::numeric_limits<double>::infinity();
    double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
    double elen = 0;
    for (unsigned t = 0; t < ntb; t++)
        for (int c = 0; c < 3; c++) {
            const double *p = vb + 3 * tb[3 * t + c];
            const double *q = vb + 3 * tb[3 * t + (c + 1) % 3];
            elen = std::max(elen, std::sqrt((p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) +
                                            (p[2] - q[2]) * (p[2] - q[2])));
        }
    for (unsigned v = 0; v < nvb; v++)
        for (int c = 0; c < 3; c++) { lo[c] = std::min(lo[c], vb[3 * v + c]); hi[c] = std::max(hi[c], vb[3 * v + c]); }
    double h = std::max(elen, 1e-3) * 2.0;
    int n[3];
    for (int c = 0; c < 3; c++) n[c] = std::max(1, (int)std::ceil((hi[c] - lo[c]) / h) + 1);
    std::vector<std::vector<uint32_t>> bins((size_t)n[0] * n[1] * n[2]);
    auto binof = [&](double x, int c) { return clampi((int)std::floor((x - lo[c]) / h), 0, n[c] - 1); };
    for (unsigned t = 0; t < ntb; t++) {
        double tl[3] = {1e30, 1e30, 1e30}, th[3] = {-1e30, -1e30, -1e30};
        for (int c = 0; c < 3; c++)
            for (int d = 0; d < 3; d++) {
                double x = vb[3 * tb[3 * t + c] + d];
                tl[d] = std::min(tl[d], x); th[d] = std::max(th[d], x);
            }
        for (int a = binof(tl[0], 0); a <= binof(th[0], 0); a++)
            for (int b = binof(tl[1], 1); b <= binof(th[1], 1); b++)
                for (int c = binof(tl[2], 2); c <= binof(th[2], 2); c++)
                    bins[((size_t)a * n[1] + b) * n[2] + c].push_back(t);
    }
    double worst = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(max : worst)
    for (int64_t v = 0; v < (int64_t)nva; v++) {
        if (only && !only[v]) continue;
        V3 p = {va[3 * v], va[3 * v + 1], va[3 * v + 2]};
        int b0[3] = {binof(p.x, 0), binof(p.y, 1), binof(p.z, 2)};
        double best = std::numeric_limits<double>::infinity();
        int maxring = std::max(n[0], std::max(n[1], n[2]));
        for (int ring = 0; ring <= maxring; ring++) {
            for (int a = b0[0] - ring; a <= b0[0] + ring; a++)
                for (int b = b0[1] - ring; b <= b0[1] + ring; b++)
                    for (int c = b0[2] - ring; c <= b0[2] + ring; c++) {
                        if (std::max(std::abs(a - b0[0]), std::max(std::abs(b - b0[1]), std::abs(c - b0[2]))) != ring) continue;
                        if (a < 0 || b < 0 || c < 0 || a >= n[0] || b >= n[1] || c >= n[2]) continue;
                        for (uint32_t t : bins[((size_t)a * n[1] + b) * n[2] + c]) {
                            V3 A = {vb[3 * tb[3 * t]], vb[3 * tb[3 * t] + 1], vb[3 * tb[3 * t] + 2]};
                            V3 B = {vb[3 * tb[3 * t + 1]], vb[3 * tb[3 * t + 1] + 1], vb[3 * tb[3 * t + 1] + 2]};
                            V3 C = {vb[3 * tb[3 * t + 2]], vb[3 * tb[3 * t + 2] + 1], vb[3 * tb[3 * t + 2] + 2]};
                            best = std::min(best, pt_tri_d2(p, A, B, C));
                        }
                    }
            /* everything outside the searched block is at least ring*h away */
            if (best < std::numeric_limits<double>::infinity() && std::sqrt(best) <= ring * h) break;
        }
        worst = std::max(worst, std::sqrt(best));
        if (per_vertex) per_vertex[v] = std::sqrt(best);
    }
    return worst;
}

} // namespace

extern "C" {

int oracle_grid_setup(const float *xyz, const float *rad, unsigned N, float dx, oracle_grid *g) {
    memset(g, 0, sizeof(*g));
    g->N = (int)N;
    g->dx = dx;
    g->probe = kProbe;
    if (N <= 1) return 1; /* CudaSurf.cu:539-543: empty result */
    /* getMinMax (CudaSurf.cu:149-174) */
    float mn[3] = {100000.0f, 100000.0f, 100000.0f}, mx[3] = {-100000.0f, -100000.0f, -100000.0f};
    float maxR = 0.0f;
    for (unsigned a = 0; a < N; a++) {
        for (int c = 0; c < 3; c++) {
            mn[c] = std::min(mn[c], xyz[3 * a + c]);
            mx[c] = std::max(mx[c], xyz[3 * a + c]);
        }
        maxR = std::max(maxR, rad[a]);
    }
    /* computeMaxDist (CudaSurf.cu:250-253) */
    float maxDist = std::max(mx[0] - mn[0], std::max(mx[1] - mn[1], mx[2] - mn[2])) + (2 * maxR) + (4 * kProbe);
    g->maxR = maxR;
    g->maxDist = maxDist;
    g->cell = kProbe + maxR;                                       /* CudaSurf.cu:548 */
    g->ox = mn[0] - maxR - kProbe;                                 /* CudaSurf.cu:551-554 */
    g->oy = mn[1] - maxR - kProbe;
    g->oz = mn[2] - maxR - kProbe;
    g->gnb = (int)std::ceil(maxDist / g->cell);                    /* CudaSurf.cu:556 */
    g->G = (int)std::ceil(maxDist / dx);                           /* CudaSurf.cu:560 */
    g->R = (int)std::ceil(kProbe / dx);                            /* CudaSurf.cu:629 */
    /* countVertexPerCell's cell range for a single slice (MarchingCubes.cu:578-604, with
       offset 0 and dim = G; the int bounds are compared as unsigned). */
    int lim = g->G - 1;
    if (g->G - g->R - 1 >= 0) lim = std::min(lim, g->G - g->R - 1);
    if (g->G - 2 * g->R - 1 >= 0) lim = std::min(lim, g->G - 2 * g->R - 1);
    g->Gc = std::max(lim, 0);
    return 0;
}

void oracle_sort_atoms(const float *xyz, unsigned N, const oracle_grid *g, uint32_t *sorted_to_input,
                       int32_t *atom_hash) {
    std::vector<float> rad(N, 1.0f);
    Atoms A;
    build_atoms(xyz, rad.data(), N, g, A);
    for (unsigned s = 0; s < N; s++) sorted_to_input[s] = A.sorted_to_input[s];
    for (unsigned a = 0; a < N; a++) atom_hash[a] = hash_of(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2], g);
}

void oracle_code_lut_f32(const oracle_grid *g, float *lut) {
    /* value = probe - min distance (Kernels.cu:540-541); -dx when nothing is found
       (Kernels.cu:505) or inside (Kernels.cu:377-378); probe outside. */
    for (int c = 0; c < 256; c++) lut[c] = -g->dx;
    int nmax = 3 * g->R * g->R;
    /* The table is evaluated in double and rounded once to float, so every entry keeps the
       sign of the exact value (at dx = 0.2, n = 49 is -4.5e-8, not the 0.0 that float
       arithmetic gives). */
    for (int n = 0; n <= nmax && n < 253; n++)
        lut[n] = (float)((double)kProbe - (double)g->dx * std::sqrt((double)n));
    lut[ORACLE_CODE_NONE] = -g->dx;
    lut[ORACLE_CODE_IN] = -g->dx;
    lut[ORACLE_CODE_OUT] = kProbe;
}

void oracle_code_lut_f64(const oracle_grid *g, double *lut) {
    for (int c = 0; c < 256; c++) lut[c] = -(double)g->dx;
    int nmax = 3 * g->R * g->R;
    for (int n = 0; n <= nmax && n < 253; n++) lut[n] = (double)kProbe - (double)g->dx * std::sqrt((double)n);
    lut[ORACLE_CODE_NONE] = -(double)g->dx;
    lut[ORACLE_CODE_IN] = -(double)g->dx;
    lut[ORACLE_CODE_OUT] = (double)kProbe;
}

int oracle_field_codes(const float *xyz, const float *rad, unsigned N, const oracle_grid *g, int fp64,
                       int x0, int x1, uint8_t *codes, int nthreads) {
    if (3 * g->R * g->R > 252) return 2;
    set_threads(nthreads);
    Atoms A;
    build_atoms(xyz, rad, N, g, A);
    if (fp64) field_codes<F64>(g, A, x0, x1, codes);
    else field_codes<F32>(g, A, x0, x1, codes);
    return 0;
}

oracle_mesh *oracle_mesh_from_codes(const uint8_t *codes, const oracle_grid *g, int fp64, const float *xyz,
                                    unsigned N, int smooth, int nthreads) {
    set_threads(nthreads);
    std::vector<float> rad(N, 1.0f);
    Atoms A;
    build_atoms(xyz, rad.data(), N, g, A);
    oracle_mesh *m = fp64 ? mesh_from_codes<F64>(codes, g, A) : mesh_from_codes<F32>(codes, g, A);
    finish_mesh(m, smooth, fp64);
    return m;
}

oracle_mesh *oracle_compute_ses(const float *xyz, const float *rad, unsigned N, float dx, int smooth,
                                int fp64, int nthreads) {
    oracle_grid g;
    if (oracle_grid_setup(xyz, rad, N, dx, &g) != 0) {
        oracle_mesh *m = (oracle_mesh *)calloc(1, sizeof(oracle_mesh));
        return m;
    }
    std::vector<uint8_t> codes((size_t)g.G * g.G * g.G);
    if (oracle_field_codes(xyz, rad, N, &g, fp64, 0, g.G, codes.data(), nthreads) != 0) return nullptr;
    return oracle_mesh_from_codes(codes.data(), &g, fp64, xyz, N, smooth, nthreads);
}

oracle_mesh *oracle_compute_ses_slices(const float *xyz, const float *rad, unsigned N, float dx, int slice,
                                       int smooth, int fp64, int nthreads) {
    oracle_grid g;
    if (slice < 1) return nullptr;
    if (oracle_grid_setup(xyz, rad, N, dx, &g) != 0) return (oracle_mesh *)calloc(1, sizeof(oracle_mesh));
    if (3 * g.R * g.R > 252) return nullptr;
    set_threads(nthreads);
    return fp64 ? sliced_ses<F64>(xyz, rad, N, &g, slice, smooth, fp64)
                : sliced_ses<F32>(xyz, rad, N, &g, slice, smooth, fp64);
}

void oracle_mesh_free(oracle_mesh *m) {
    if (!m) return;
    free(m->v); free(m->vq); free(m->tri); free(m->tri_kept);
    free(m->atom_sorted); free(m->atom_input); free(m->edge_vertex);
    free(m->slice_v); free(m->slice_t); free(m->slice_tk);
    free(m);
}

void oracle_smooth_f32(float *v, unsigned nv, const int32_t *tri, unsigned nt, int passes) {
    smooth_gs<float>(v, nv, tri, nt, passes);
}

double oracle_hausdorff(const double *va, unsigned nva, const int32_t *ta, unsigned nta, const double *vb,
                        unsigned nvb, const int32_t *tb, unsigned ntb, double *ab, double *ba, int nthreads) {
    set_threads(nthreads);
    /* Surface to surface: a vertex that no triangle names (one left only by degenerate,
       filtered triangles) is not on either surface and is not measured. */
    std::vector<uint8_t> ua(nva, 0), ub(nvb, 0);
    for (unsigned i = 0; i < 3 * nta; i++) ua[ta[i]] = 1;
    for (unsigned i = 0; i < 3 * ntb; i++) ub[tb[i]] = 1;
    double x = one_sided(va, nva, vb, nvb, tb, ntb, nullptr, ua.data());
    double y = one_sided(vb, nvb, va, nva, ta, nta, nullptr, ub.data());
    if (ab) *ab = x;
    if (ba) *ba = y;
    return std::max(x, y);
}

/* Distance from every vertex of A to surface B (for robust comparisons). */
double oracle_point_surface(const double *va, unsigned nva, const double *vb, unsigned nvb, const int32_t *tb,
                            unsigned ntb, double *dist, int nthreads) {
    set_threads(nthreads);
    return one_sided(va, nva, vb, nvb, tb, ntb, dist);
}

/* Gauss-Seidel dependency depth: level(i) = 1 + max level(j) over neighbours j < i. */
int oracle_smooth_depth(const int32_t *tri, unsigned nt, unsigned nv, int32_t *level) {
    std::vector<uint32_t> start;
    std::vector<int32_t> nbr;
    neighbour_csr(tri, nt, nv, start, nbr);
    int depth = 0;
    for (unsigned i = 0; i < nv; i++) {
        int l = 0;
        for (uint32_t e = start[i]; e < start[i + 1]; e++)
            if ((unsigned)nbr[e] < i) l = std::max(l, level[nbr[e]] + 1);
        level[i] = l;
        depth = std::max(depth, l + 1);
    }
    return depth;
}

} // extern "C"
