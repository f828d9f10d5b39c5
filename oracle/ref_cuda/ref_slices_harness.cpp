// Calls QuickSES's own computeSlicedSES (CudaSurf.cu:524-776) through its shared library
// and hands back each slice's mesh as the reference leaves it, before API_computeSES
// concatenates them (CudaSurf.cu:796-836).
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref_cuda/Makefile against the reference's
// libQuickSES.so; MeshData comes from the reference's SmoothMesh.h (-I its sources).  The
// slice size is the reference's global SLICE (CudaSurf.cu:63), which its executable sets
// from -s (CudaSurf.cu:926-929).
#include <cstdlib>
#include <vector>

#include "SmoothMesh.h"

extern int SLICE;
std::vector<MeshData> computeSlicedSES(float3 positions[], float radii[], unsigned int N, float resoSES,
                                       int doSmoothing);

static std::vector<MeshData> g_meshes;

static void release() {
    for (MeshData &m : g_meshes)
        if (m.NVertices > 0 || m.NTriangles > 0) {  // empty slices leave the pointers unset
            free(m.vertices);
            free(m.triangles);
            free(m.atomIdPerVert);
        }
    g_meshes.clear();
}

// Runs the reference on N atoms with slices of `slice` voxels; returns the slice count.
extern "C" int ref_slices_run(const float *xyz, const float *rad, unsigned N, float reso, int slice, int smooth) {
    release();
    std::vector<float3> pos(N);
    std::vector<float> r(rad, rad + N);
    for (unsigned a = 0; a < N; a++) pos[a] = make_float3(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]);
    SLICE = slice;
    g_meshes = computeSlicedSES(pos.data(), r.data(), N, reso, smooth);
    return (int)g_meshes.size();
}

// Counts of slice s: vertices and triangles (its unwritten last triangle included).
extern "C" void ref_slices_counts(int s, int *nv, int *nt) {
    *nv = g_meshes[s].NVertices;
    *nt = g_meshes[s].NTriangles;
}

// Slice s's arrays: 3 nv floats, 3 nt ints, nv atom ids (the cell-sorted order).
extern "C" void ref_slices_copy(int s, float *v, int *t, int *atom) {
    const MeshData &m = g_meshes[s];
    for (int q = 0; q < m.NVertices; q++) {
        v[3 * q] = m.vertices[q].x;
        v[3 * q + 1] = m.vertices[q].y;
        v[3 * q + 2] = m.vertices[q].z;
        atom[q] = m.atomIdPerVert[q];
    }
    for (int q = 0; q < m.NTriangles; q++) {
        t[3 * q] = m.triangles[q].x;
        t[3 * q + 1] = m.triangles[q].y;
        t[3 * q + 2] = m.triangles[q].z;
    }
}
