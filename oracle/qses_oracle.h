/*
 * CPU oracle for the QuickSES atoms+radii -> SES mesh path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke check and
 * bench.py's CPU-baseline leg may load it; the product library never does.
 *
 * Two arithmetic modes:
 *   fp64 = 0  FP32 IEEE arithmetic in exactly the operation order of the CUDA kernels
 *             (no FMA contraction except the explicit fmaf calls), so the GPU path can be
 *             checked bit for bit.
 *   fp64 = 1  the same algorithm in double precision: the accuracy reference.
 *
 * Semantics are those of QuickSES's single-slice path (slice >= grid), i.e.
 * computeSlicedSES (CudaSurf.cu:524-776) with one slice, plus API_computeSES's
 * concatenation (CudaSurf.cu:787-841).  Each function cites the reference lines it restates.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    float ox, oy, oz;   /* common grid origin = min - maxR - probe (CudaSurf.cu:551-574) */
    float cell;         /* neighbour-cell size = probe + maxR (CudaSurf.cu:548) */
    float dx;           /* SES voxel size */
    float probe;        /* 1.4 (Kernels.cu:26) */
    float maxR;         /* largest atom radius */
    float maxDist;      /* computeMaxDist (CudaSurf.cu:250-253) */
    int gnb;            /* neighbour grid dimension (CudaSurf.cu:556) */
    int G;              /* SES grid dimension (CudaSurf.cu:560) */
    int R;              /* refine window half-width ceil(probe/dx) (CudaSurf.cu:629) */
    int Gc;             /* marching-cubes cells emitted per axis (MarchingCubes.cu:578-604) */
    int N;
} oracle_grid;

/* Voxel codes: n in [0, 3R^2] = squared voxel distance to the nearest outside voxel. */
#define ORACLE_CODE_NONE 253u  /* border voxel with no outside voxel in the window */
#define ORACLE_CODE_IN   254u  /* SAS pass: inside an atom shrunk by dx */
#define ORACLE_CODE_OUT  255u  /* SAS pass: outside every probe-inflated atom */

typedef struct {
    unsigned nv;          /* welded vertices */
    unsigned nt;          /* triangles as emitted (degenerate ones included) */
    unsigned nt_kept;     /* triangles kept by API_computeSES's filter */
    unsigned ne;          /* active edges (pre-weld vertices) */
    double *v;            /* nv*3 smoothed positions (fp32 mode: exact float values) */
    double *vq;           /* nv*3 welded positions before smoothing */
    int32_t *tri;         /* nt*3 */
    int32_t *tri_kept;    /* nt_kept*3 */
    int32_t *atom_sorted; /* nv closest atom, index into the cell-sorted atom array */
    int32_t *atom_input;  /* nv closest atom, caller's input index */
    int32_t *edge_vertex; /* ne: pre-weld edge slot -> welded vertex */
    unsigned nslices;     /* reference slicing mode: slices with a mesh, in slice order */
    uint32_t *slice_v;    /* nslices+1: first vertex of each slice (then the total) */
    uint32_t *slice_t;    /* nslices+1: first triangle (all) of each slice */
    uint32_t *slice_tk;   /* nslices+1: first kept triangle of each slice */
} oracle_mesh;

int oracle_grid_setup(const float *xyz, const float *rad, unsigned N, float dx, oracle_grid *g);
void oracle_sort_atoms(const float *xyz, unsigned N, const oracle_grid *g,
                       uint32_t *sorted_to_input, int32_t *atom_hash);
void oracle_code_lut_f32(const oracle_grid *g, float *lut256);
void oracle_code_lut_f64(const oracle_grid *g, double *lut256);
int oracle_field_codes(const float *xyz, const float *rad, unsigned N, const oracle_grid *g,
                       int fp64, int x0, int x1, uint8_t *codes, int nthreads);
oracle_mesh *oracle_mesh_from_codes(const uint8_t *codes, const oracle_grid *g, int fp64,
                                    const float *xyz, unsigned N, int smooth, int nthreads);
oracle_mesh *oracle_compute_ses(const float *xyz, const float *rad, unsigned N, float dx,
                                int smooth, int fp64, int nthreads);
/* The reference's slicing (-s slice): one mesh per slice box, concatenated as
 * API_computeSES concatenates them; see qses_oracle.cpp.  NULL for slice < 1. */
oracle_mesh *oracle_compute_ses_slices(const float *xyz, const float *rad, unsigned N, float dx, int slice,
                                       int smooth, int fp64, int nthreads);
void oracle_mesh_free(oracle_mesh *m);
void oracle_smooth_f32(float *v, unsigned nv, const int32_t *tri, unsigned nt, int passes);
double oracle_hausdorff(const double *va, unsigned nva, const int32_t *ta, unsigned nta,
                        const double *vb, unsigned nvb, const int32_t *tb, unsigned ntb,
                        double *ab, double *ba, int nthreads);
double oracle_point_surface(const double *va, unsigned nva, const double *vb, unsigned nvb, const int32_t *tb,
                            unsigned ntb, double *dist, int nthreads);
int oracle_smooth_depth(const int32_t *tri, unsigned nt, unsigned nv, int32_t *level);

#ifdef __cplusplus
}
#endif
