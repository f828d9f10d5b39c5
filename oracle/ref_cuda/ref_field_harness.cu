// Drives QuickSES's own field kernels for a single slice and returns the distance field.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref_cuda/Makefile against the reference
// sources (Kernels.cu is #included from the -I path).  The launch sequence restates
// computeSlicedSES for one slice covering the whole grid (CudaSurf.cu:536-729 with
// offset 0 and slice size = grid size): hashAtoms, thrust stable merge sort, sortCell,
// probeIntersection, the fill-array sort + count_if, distanceFieldRefine.  It is compiled
// with the reference's own flags (-use_fast_math -O3), so the field carries the
// reference's arithmetic.
#include <climits>
#include <cmath>
#include <cstdio>
#include <vector>

#include <thrust/count.h>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/sort.h>

#include "Kernels.cu"

#define RCHK(x)                                     \
    do {                                            \
        if ((x) != cudaSuccess) {                   \
            fprintf(stderr, "ref_field: %s\n", #x); \
            rc = 3;                                 \
            goto done;                              \
        }                                           \
    } while (0)

extern "C" int ref_field(const float *xyz, const float *rad, unsigned N, float resoSES, float *field_out,
                         size_t cap, int *G_out) {
    int rc = 0;
    float4 *dAtoms = nullptr, *dSorted = nullptr;
    int2 *dHash = nullptr, *dCells = nullptr;
    float *dField = nullptr;
    int *dFill = nullptr;
    const float probe = PROBERADIUS;
    // getMinMax / computeMaxDist / grid sizing (CudaSurf.cu:149-174, 250-253, 546-574)
    float3 mn = make_float3(100000.0f, 100000.0f, 100000.0f), mx = make_float3(-100000.0f, -100000.0f, -100000.0f);
    float maxR = 0.0f;
    std::vector<float4> h(N);
    for (unsigned a = 0; a < N; a++) {
        float3 c = make_float3(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]);
        mn.x = std::min(mn.x, c.x); mn.y = std::min(mn.y, c.y); mn.z = std::min(mn.z, c.z);
        mx.x = std::max(mx.x, c.x); mx.y = std::max(mx.y, c.y); mx.z = std::max(mx.z, c.z);
        maxR = std::max(maxR, rad[a]);
        h[a] = make_float4(c.x, c.y, c.z, rad[a]);
    }
    float maxDist = std::max(mx.x - mn.x, std::max(mx.y - mn.y, mx.z - mn.z)) + (2 * maxR) + (4 * probe);
    float cellSize = probe + maxR;
    float4 oNb = make_float4(mn.x - maxR - probe, mn.y - maxR - probe, mn.z - maxR - probe, cellSize);
    float4 oSES = make_float4(oNb.x, oNb.y, oNb.z, resoSES);
    int gnb = (int)ceil(maxDist / cellSize);
    int G = (int)ceil(maxDist / resoSES);
    int3 gnbDim = make_int3(gnb, gnb, gnb), gDim = make_int3(G, G, G);
    unsigned ncell = gnb * gnb * gnb;
    int S = G;  // one slice covering the grid
    int nvox = S * S * S;
    *G_out = G;
    if (cap < (size_t)nvox) return 1;

    RCHK(cudaMalloc(&dAtoms, sizeof(float4) * N));
    RCHK(cudaMalloc(&dSorted, sizeof(float4) * N));
    RCHK(cudaMalloc(&dHash, sizeof(int2) * N));
    RCHK(cudaMalloc(&dCells, sizeof(int2) * ncell));
    RCHK(cudaMalloc(&dField, sizeof(float) * nvox));
    RCHK(cudaMalloc(&dFill, sizeof(int) * nvox));
    RCHK(cudaMemcpy(dAtoms, h.data(), sizeof(float4) * N, cudaMemcpyHostToDevice));
    {
        // CudaSurf.cu:605-618
        hashAtoms<<<N, NBTHREADS>>>(N, dAtoms, gnbDim, oNb, dHash, N);
        compare_int2 cmp;
        thrust::device_ptr<int2> hb = thrust::device_pointer_cast(dHash);
        thrust::sort(hb, hb + N, cmp);
        memsetCudaInt2<<<(ncell + NBTHREADS - 1) / NBTHREADS, NBTHREADS>>>(dCells, make_int2(EMPTYCELL, EMPTYCELL), ncell);
        sortCell<<<N, NBTHREADS>>>(N, dAtoms, dHash, dSorted, dCells);
        RCHK(cudaGetLastError());
        // CudaSurf.cu:664-685 with offset 0
        memsetCudaFloat<<<(nvox + NBTHREADS - 1) / NBTHREADS, NBTHREADS>>>(dField, probe, nvox);
        memsetCudaInt<<<(nvox + NBTHREADS - 1) / NBTHREADS, NBTHREADS>>>(dFill, EMPTYCELL, nvox);
        const int cut = 8;
        dim3 lws(cut, cut, cut), gws((S + cut - 1) / cut, (S + cut - 1) / cut, (S + cut - 1) / cut);
        int3 sliceDim = make_int3(S, S, S), off = make_int3(0, 0, 0);
        probeIntersection<<<gws, lws>>>(dFill, dHash, gnbDim, oNb, gDim, sliceDim, oSES, dCells, dSorted, dField, off,
                                        N, nvox);
        RCHK(cudaGetLastError());
        RCHK(cudaDeviceSynchronize());
        // CudaSurf.cu:688-729
        thrust::device_ptr<int> fb(dFill);
        thrust::sort(fb, fb + nvox);
        unsigned border = thrust::count_if(thrust::device, fb, fb + nvox, is_notempty());
        if (border > 0) {
            int tranche = std::min(border, 65536u / 8 * NBTHREADS);
            for (unsigned o = 0; o < border; o += tranche) {
                dim3 g1((tranche + NBTHREADS - 1) / NBTHREADS, 1, 1);
                distanceFieldRefine<<<g1, NBTHREADS>>>(dFill, dHash, gnbDim, oNb, gDim, sliceDim, oSES, dCells, dSorted,
                                                       dField, N, border, off, o);
            }
            RCHK(cudaGetLastError());
            RCHK(cudaDeviceSynchronize());
        }
        RCHK(cudaMemcpy(field_out, dField, sizeof(float) * nvox, cudaMemcpyDeviceToHost));
    }
done:
    cudaFree(dAtoms); cudaFree(dSorted); cudaFree(dHash); cudaFree(dCells); cudaFree(dField); cudaFree(dFill);
    return rc;
}
