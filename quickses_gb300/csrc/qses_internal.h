// Internal declarations shared by the host orchestration and the CUDA kernels.
#pragma once

#define QSES_API __attribute__((visibility("default")))
#include "../../include/quickses.h"

#include <stddef.h>
#include <stdint.h>

// Voxel codes (one byte per voxel): 0..3R^2 is the squared voxel distance from a border
// voxel to the nearest outside voxel of its refine window.
#define QSES_CODE_NONE 253u  // border voxel, no outside voxel in the window (value -dx)
#define QSES_CODE_IN 254u    // inside an atom shrunk by dx (value -dx)
#define QSES_CODE_OUT 255u   // outside every probe-inflated atom (value probe)
#define QSES_RMAX 9          // largest refine half-window whose 3R^2 fits below 253

#define QSES_PROBE 1.4f      // probe radius (QuickSES PROBERADIUS, Kernels.cu:26)
#define QSES_WELD_TOL 0.001f // weld quantum (QuickSES EPSILON, Kernels.cu:27)

// Grid description passed by value to every kernel.
struct QGrid {
    float ox, oy, oz;  // origin (min - maxR - probe)
    float dx;          // voxel size
    float cell;        // neighbour cell size (probe + maxR)
    float probe;
    int G;             // voxels per axis
    int gnb;           // neighbour cells per axis
    int R;             // refine half window
    int Gc;            // emitted MC cells per axis
    int W;             // 32-voxel words per z row
    int Gp;            // code row stride in bytes (32 * W)
    int negmin;        // smallest code n with value(n) < 0
    unsigned N;        // atoms
    long long bx, by, bz;  // weld key base (quantised origin - margin)
    long long Rq;          // weld key radix per axis
    // A box of the reference's slicing (else the whole grid: offsets 0, limits G - 1, cell
    // ranges [0, Gc)).  Voxel (i, j, k) of the box is voxel (i + off[0], j + off[1],
    // k + off[2]) of the molecule's grid: SAS positions use the grid index, vertex positions
    // the box index plus off * dx (CudaSurf.cu:671-682, MarchingCubes.cu:841-848).
    int off[3];
    int lim[3];        // voxels with a box index >= lim[a] on any axis a stay outside
    int clo[3], chi[3];  // marching-cubes cells emitted per axis: [clo, chi), chi <= Gc
};

// One molecule of a batch: its grid and where its pieces sit in the batch's concatenated
// device arrays.  Offsets are in elements of the array named.
struct QMol {
    QGrid g;
    unsigned long long mask_off;  // first 32-bit word of the in/out/sign masks
    unsigned long long code_off;  // first byte of the voxel codes
    unsigned atom_off;            // first atom (input order and cell-sorted order)
    unsigned cell_off;            // first neighbour cell of the cell table
    unsigned row_off;             // first marching-cubes owner row
    unsigned flags;               // QSES_FLAG_* of the request
};

// Device view of a batch.  The *_off arrays have n_mol + 1 entries (the last is the total)
// and are searched to map a global item, atom, row, triangle or vertex to its molecule.
struct QBatch {
    const QMol *mols;
    const unsigned *tile_off;  // field tiles (8 x 8 z-rows of 32 voxels) per molecule
    const unsigned *atom_off;
    const unsigned *row_off;
    const unsigned *mc_unit_off; // marching-cubes warp units (32 / lanes rows each)
    const unsigned *word_off;  // 32-bit mask words (G G W) per molecule
    const unsigned *tri_off;   // pre-filter triangles (valid after the row scan)
    const unsigned *vtx_off;   // welded vertices (valid after the weld)
    const float *lut;          // 256 field values per molecule
    unsigned n_mol;
    int key_bits;              // bits of a molecule-local weld key; the molecule sits above
};

// Largest m with off[m] <= x, for off[0] = 0 <= x < off[n].
#ifdef __CUDACC__
__device__ __forceinline__ unsigned qses_find(const unsigned *off, unsigned n, unsigned x) {
    unsigned lo = 0, hi = n;  // off[lo] <= x < off[hi]
    while (hi - lo > 1) {
        const unsigned mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= x) lo = mid; else hi = mid;
    }
    return lo;
}
#endif
