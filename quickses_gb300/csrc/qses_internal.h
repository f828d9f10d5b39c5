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
};
