// Host entry points into the reference's own code, for pinning the oracle.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py from the reference checkout
// (Kernels.cu is #included from the -I path, SmoothMesh.cpp is compiled beside this file)
// into oracle/_ref/, which never enters version control.  The wrappers only call the
// reference's __host__ __device__ helpers on the CPU; no device code runs.
#include <climits>
#include <cstdint>
#include "Kernels.cu"
#include "SmoothMesh.h"

extern "C" {

// computeInOrOut (Kernels.cu:344-392) for one voxel, with the same position and
// neighbour-cell computation as probeIntersection (Kernels.cu:444-458).
float ref_compute_in_or_out(int i, int j, int k, float ox, float oy, float oz, float cellSize, int gnb,
                            float dxSES, const int2 *cellStartEnd, const float4 *sorted_xyzr) {
    float3 origin = make_float3(ox, oy, oz);
    float3 p = gridToSpace(make_int3(i, j, k), origin, dxSES);
    int3 c = spaceToGrid(p, origin, cellSize);
    return computeInOrOut(c, (int2 *)cellStartEnd, (float4 *)sorted_xyzr, p, dxSES, make_int3(gnb, gnb, gnb));
}

// computeClosestAtom (Kernels.cu:547-585) as closestAtomPerVertex calls it (:596-603).
int ref_closest_atom(float vx, float vy, float vz, float ox, float oy, float oz, float cellSize, int gnb,
                     const int2 *cellStartEnd, const float4 *sorted_xyzr) {
    float3 v = make_float3(vx, vy, vz);
    int3 c = spaceToGrid(v, make_float3(ox, oy, oz), cellSize);
    return computeClosestAtom(v, c, (int2 *)cellStartEnd, (float4 *)sorted_xyzr, make_int3(gnb, gnb, gnb));
}

// spaceToGrid + flatten3DTo1D (Kernels.cu:119-131), as hashAtoms uses them (:204-211).
int ref_hash(float px, float py, float pz, float ox, float oy, float oz, float cellSize, int gnb) {
    int3 c = spaceToGrid(make_float3(px, py, pz), make_float3(ox, oy, oz), cellSize);
    return flatten3DTo1D(c, make_int3(gnb, gnb, gnb));
}

// smoothMeshLaplacian (SmoothMesh.cpp:45-94 variant taking raw arrays).
void ref_smooth(int times, float *vertices, int *triangles, unsigned nv, unsigned nt) {
    float3 *v = (float3 *)vertices;
    int3 *t = (int3 *)triangles;
    smoothMeshLaplacian(times, v, t, nv, nt);
}

}  // extern "C"
