// Kernel launchers (host side).  Every launcher enqueues on the given stream only.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "qses_internal.h"

namespace qses {

void launch_atom_minmax(const float *xyz, const float *r, unsigned n, unsigned *mm, cudaStream_t s);
void launch_atom_hash(const QGrid &g, const float *xyz, unsigned n, unsigned *key, cudaStream_t s);
void launch_atom_gather(const float *xyz, const float *r, const unsigned *skey, const unsigned *sidx, unsigned n,
                        float4 *atoms, uint2 *cells, cudaStream_t s);
void launch_sas(const QGrid &g, const float4 *atoms, const uint2 *cells, unsigned *inMask, unsigned *outMask,
                cudaStream_t s);
// shape: refine tile of 8 x 8 (0), 16 x 8 (1), 16 x 16 (2) or 32 x 16 (3) z-rows; the same
// codes for all.
// zd (optional, the codes' size): scratch for the z distances, computed once per voxel
// instead of once per tile halo row.
void launch_edt(const QGrid &g, const unsigned *inMask, const unsigned *outMask, unsigned char *codes,
                unsigned *signMask, cudaStream_t s, int shape = 0, unsigned char *zd = nullptr);

void launch_mc_count(const QGrid &g, const unsigned *sign, uint2 *rowCount, cudaStream_t s);
void launch_mc_emit(const QGrid &g, const unsigned *sign, const unsigned char *codes, const float *lut,
                    const uint2 *rowBase, unsigned *tri, unsigned long long *vkey, cudaStream_t s);
void launch_weld_flags(const unsigned long long *skey, unsigned n, uint2 *flags, cudaStream_t s);
void launch_weld_scatter(const QGrid &g, const unsigned long long *skey, const unsigned *sval, const uint2 *excl,
                         unsigned n, unsigned *vmap, float *vq, cudaStream_t s);
void launch_remap(unsigned *tri, size_t n3, const unsigned *vmap, cudaStream_t s);
void launch_closest(const QGrid &g, const float *vq, unsigned nv, const float4 *atoms, const uint2 *cells,
                    const unsigned *sorted_to_input, int *asorted, int *ainput, cudaStream_t s);
void launch_tri_flags(const unsigned *tri, unsigned nt, uint2 *flags, cudaStream_t s);
void launch_tri_compact(const unsigned *tri, unsigned nt, const uint2 *excl, unsigned *out, cudaStream_t s);
// Neighbour lists by counting: start (nv + 1 entries, zeroed) -> counts -> (scan) -> corner
// occurrences scattered per vertex into occ (n3) -> sorted per vertex and expanded into nbr
// (2 n3), start[v].x = list offset.
void launch_csr_count(const unsigned *tri, size_t n3, uint2 *start, cudaStream_t s);
void launch_csr_scatter(const unsigned *tri, size_t n3, uint2 *start, unsigned *occ, cudaStream_t s);
void launch_csr_sortfill(const unsigned *tri, unsigned *occ, size_t n3, unsigned nv, uint2 *start, unsigned *nbr,
                         cudaStream_t s);
// Slab table of one Gauss-Seidel wave (device words): [0] Q slabs, [1, Q + 2) their bounds in
// id order (qcap + 1 slots), [qcap + 2, qcap + 2 + Q) the slab ids in the order CTAs take them.
inline size_t gs_table_words(unsigned qcap) { return 2ull * qcap + 2; }
void launch_gs_setup(const uint2 *start, const unsigned *nbr, unsigned v0, unsigned v1, const unsigned *table,
                     unsigned short *cnt_local, int *remote, uint2 *home, cudaStream_t s);
size_t gs_slab_smem(unsigned S, unsigned flags);
void launch_to_float4(const float *v3, unsigned nv, float4 *v4, cudaStream_t s);
void launch_from_float4(const float4 *v4, unsigned nv, float *v3, cudaStream_t s);
// One Gauss-Seidel pass over vertices [v0, nv) in the table's slabs (each at most smax
// vertices), taken by P persistent CTAs from *next_slab (zeroed, like inbox_tail's qcap
// counters).  threads: 512 or 1024 per slab CTA.
cudaError_t launch_gs_slab(float4 *pos, unsigned v0, unsigned nv, unsigned smax, const unsigned *table,
                           unsigned qcap, unsigned *next_slab, const uint2 *home, int P, int threads, unsigned flags,
                           unsigned hot_warps, const uint2 *start, const unsigned *nbr,
                           const unsigned short *cnt_local, int *remote,
                           unsigned *inbox, unsigned *inbox_tail, int *err, long long spin_cycles,
                           unsigned long long *stats, cudaStream_t s);
int gs_slab_max_blocks(int device, unsigned S, int threads, unsigned flags);

// Gauss-Seidel launch shape: threads per slab CTA and the slab size aimed at (vertices);
// the result does not depend on it, only the time does.
struct GsShape {
    int threads = 512;
    unsigned target = 16384;
    unsigned flags = 0;  // kGsL1Prefetch | kGsL1Positions | kGsPersistL2 | kGsSmemPos | kGsPair / kGsQuad
    unsigned wave = 0;   // most vertices per slab-kernel launch (0: all that fit on the GPU)
    unsigned hot = 0;    // worker warps per CTA whose idle sleeps stay short (same results)
};
// Hot worker warps of single-molecule passes: 12 of 30 polling the ready ring every 64 ns
// at most took the 50 000-atom pass from 10.42-10.44 to 10.27-10.29 ms (0: 15.72-15.74 ms
// per call, 12: 15.51); all 30 hot was slower (16.0 ms); batches are faster with none.
constexpr unsigned kGsHotWarpsSingle = 12;
// Cache policies of the smoothing kernel (same results, different memory paths):
constexpr unsigned kGsL1Prefetch = 1;   // prefetch a successor's neighbour list into L1, not L2
constexpr unsigned kGsL1Positions = 2;  // neighbour positions through L1 (default: L2 only)
constexpr unsigned kGsPersistL2 = 4;    // host side: keep the positions in persisting L2 lines
constexpr unsigned kGsSmemPos = 8;      // the slab's own positions in shared memory (slabs <= 8192)
constexpr unsigned kGsSmemPosMaxVerts = 8192;
// Lanes per vertex update (same results): 32 by default; 16 with kGsPair (two ready vertices
// per worker warp), 8 with kGsQuad (four).
constexpr unsigned kGsPair = 16;
constexpr unsigned kGsQuad = 32;
inline bool gs_flags_valid(unsigned f) { return f < 64 && (f & (kGsPair | kGsQuad)) != (kGsPair | kGsQuad); }
// Sets (bytes > 0) or clears the stream's L2 persistence window over [p, p + bytes); the
// set-aside is this process's context limit, restored when the window is cleared.
void gs_l2_window(int device, cudaStream_t s, const void *p, size_t bytes);
// Tuned shape for a mesh of nv vertices (batch = waves of many molecules), or the default.
GsShape gs_shape(unsigned nv, bool batch);
void gs_shape_record(unsigned nv, bool batch, GsShape s);
void gs_shape_record_all(bool batch, GsShape s);  // every mesh-size class
int gs_shape_candidates(GsShape *out, int max);
// Tuned refine tile shape (launch_edt `shape`) for grids of G voxels per axis, or 0.
int edt_shape(int G);
void edt_shape_record(int G, int shape);
constexpr int kEdtShapes = 4;
constexpr unsigned kGsSlabMaxVerts = 25000;

// ---- batch forms (QBatch: per-molecule grids and offsets in device memory)
void launch_atom_hash_batch(const QBatch &b, const float *xyz, unsigned n, unsigned *key, cudaStream_t s);
void launch_sas_batch(const QBatch &b, unsigned tiles, const float4 *atoms, const uint2 *cells, unsigned *inMask,
                      unsigned *outMask, unsigned *counter, cudaStream_t s);
// words: mask words of all molecules; zd (optional, code bytes of all molecules): z distances
void launch_edt_batch(const QBatch &b, unsigned tiles, const unsigned *inMask, const unsigned *outMask,
                      unsigned char *codes, unsigned *signMask, unsigned *counter, cudaStream_t s, unsigned words = 0,
                      unsigned char *zd = nullptr);
// Owner rows a marching-cubes warp covers for a grid with Gc emitted cells per axis.
int mc_rows_per_warp(int Gc);
void launch_mc_count_batch(const QBatch &b, unsigned units, const unsigned *sign, uint2 *rowCount, cudaStream_t s);
void launch_mc_emit_batch(const QBatch &b, unsigned units, const unsigned *sign, const unsigned char *codes,
                          const uint2 *rowBase, unsigned *tri, unsigned long long *vkey, cudaStream_t s);
void launch_weld_scatter_batch(const QBatch &b, const unsigned long long *skey, const unsigned *sval,
                               const uint2 *excl, unsigned n, unsigned *vmap, float *vq, unsigned *vmol,
                               cudaStream_t s);
void launch_gather_offsets(const uint2 *excl, const unsigned *at, unsigned n_mol, unsigned n, const uint2 *total,
                           unsigned *outx, unsigned *outy, cudaStream_t s);
void launch_closest_batch(const QBatch &b, const float *vq, const unsigned *vmol, unsigned nv, const float4 *atoms,
                          const uint2 *cells, const unsigned *sorted_to_input, int *asorted, int *ainput,
                          cudaStream_t s);
void launch_tri_flags_batch(const QBatch &b, const unsigned *tri, unsigned nt, uint2 *flags, cudaStream_t s);
void launch_tri_compact_batch(const QBatch &b, const unsigned *tri, unsigned nt, const uint2 *excl, unsigned *out,
                              cudaStream_t s);  // 8 B of shared memory per vertex, 16-bit slab offsets

}  // namespace qses
