// Decoupled look-back scan and onesweep radix sort (Merrill & Garland 2016;
// Adinets & Merrill 2022), written for this project.
//
// The radix sort replaces QuickSES's thrust::sort calls (CudaSurf.cu:610-612 for the atom
// cell keys, :444-447 for the weld): one histogram kernel computes every digit's counts,
// then one kernel per 8-bit digit ranks a tile of keys in shared memory (warp match +
// per-warp digit counters, so equal digits keep input order), obtains the tile's global
// digit offsets through a decoupled look-back and scatters.  The look-back waits are
// bounded (QSES_ERR_TIMEOUT) and every scatter is bounds-checked.
#include "device_common.cuh"
#include "prims.h"

namespace qses {

// ------------------------------------------------------------------ scan
// 16 items per thread: half the tiles of 8, so a shorter look-back chain (neighbour-list
// build 0.75 -> 0.71 ms on the 50 000-atom mesh, together with the sortfill's register cap)
constexpr int kScanT = 256, kScanI = 16, kScanTile = kScanT * kScanI;

__device__ __forceinline__ unsigned long long pack31(uint2 v) {
    return (unsigned long long)(v.x & 0x7fffffffu) | ((unsigned long long)(v.y & 0x7fffffffu) << 31);
}
__device__ __forceinline__ uint2 unpack31(unsigned long long s) {
    return make_uint2((unsigned)(s & 0x7fffffffull), (unsigned)((s >> 31) & 0x7fffffffull));
}

__global__ void __launch_bounds__(kScanT) k_scan_u2(const uint2 *in, uint2 *out, unsigned n,
                                                    unsigned long long *status, unsigned *ticket,
                                                    uint2 *total, int *err) {
    __shared__ uint2 s_warp[kScanT / 32];
    __shared__ unsigned s_tile;
    __shared__ uint2 s_excl;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const unsigned tile = s_tile;
    const size_t base = (size_t)tile * kScanTile + (size_t)threadIdx.x * kScanI;
    uint2 v[kScanI];
    uint2 sum = make_uint2(0, 0);
#pragma unroll
    for (int q = 0; q < kScanI; q++) {
        v[q] = base + q < n ? in[base + q] : make_uint2(0, 0);
        sum = add2(sum, v[q]);
    }
    uint2 tot;
    uint2 texcl = block_excl_scan2<kScanT>(sum, tot, s_warp);
    if (threadIdx.x == 0) {
        uint2 excl = make_uint2(0, 0);
        if (tile == 0) {
            st_release(&status[0], kFlagPre | pack31(tot));
        } else {
            st_release(&status[tile], kFlagAgg | pack31(tot));
            for (int j = (int)tile - 1; j >= 0; j--) {
                unsigned long long s = wait_status(&status[j], err);
                excl = add2(excl, unpack31(s));
                if ((s >> 62) != 1) break;  // inclusive prefix found (or timed out)
            }
            st_release(&status[tile], kFlagPre | pack31(add2(excl, tot)));
        }
        s_excl = excl;
        if (tile == gridDim.x - 1 && total) *total = add2(excl, tot);
    }
    __syncthreads();
    uint2 run = add2(s_excl, texcl);
#pragma unroll
    for (int q = 0; q < kScanI; q++) {
        if (base + q < n) out[base + q] = run;
        run = add2(run, v[q]);
    }
}

size_t scan_u2_tmp_bytes(unsigned n) {
    size_t tiles = (n + kScanTile - 1) / kScanTile;
    return 256 + tiles * sizeof(unsigned long long);
}

cudaError_t scan_u2(const uint2 *in, uint2 *out, unsigned n, uint2 *d_total, void *tmp, int *d_err,
                    cudaStream_t s, int *launches) {
    unsigned tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 0) {
        if (d_total) return cudaMemsetAsync(d_total, 0, sizeof(uint2), s);
        return cudaSuccess;
    }
    unsigned *ticket = (unsigned *)tmp;
    unsigned long long *status = (unsigned long long *)((char *)tmp + 256);
    cudaError_t e = cudaMemsetAsync(tmp, 0, scan_u2_tmp_bytes(n), s);
    if (e != cudaSuccess) return e;
    k_scan_u2<<<tiles, kScanT, 0, s>>>(in, out, n, status, ticket, d_total, d_err);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

// ------------------------------------------------------------ radix sort
constexpr int kRsT = 256, kRsW = kRsT / 32;
// Items per thread: the tile is staged in shared memory before it is written out, so 64-bit
// keys take fewer per thread (static shared memory stays under 48 KB).
template <typename K> struct RsTile { static constexpr int kItems = sizeof(K) == 8 ? 12 : 16; };

template <typename K>
__global__ void __launch_bounds__(256) k_rs_hist(const K *keys, unsigned n, int npass, unsigned *hist) {
    __shared__ unsigned sh[8 * 256];
    for (int q = threadIdx.x; q < npass * 256; q += 256) sh[q] = 0;
    __syncthreads();
    for (size_t idx = (size_t)blockIdx.x * 256 + threadIdx.x; idx < n; idx += (size_t)gridDim.x * 256) {
        K k = keys[idx];
        for (int p = 0; p < npass; p++) atomicAdd(&sh[p * 256 + (unsigned)((k >> (8 * p)) & 255)], 1u);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < npass * 256; q += 256)
        if (sh[q]) atomicAdd(&hist[q], sh[q]);
}

// One onesweep pass over a tile of kRsT x kItems keys: stable ranks by warp-level digit
// matching, the tile's offset per digit by decoupled look-back over tiles, then the tile is
// reordered by digit in shared memory so each digit's run is written out contiguously.
template <typename K>
__global__ void __launch_bounds__(kRsT) k_rs_pass(const K *__restrict__ kin, K *__restrict__ kout,
                                                  const unsigned *__restrict__ vin, unsigned *__restrict__ vout,
                                                  unsigned n, int shift, const unsigned *__restrict__ hist,
                                                  unsigned long long *status, unsigned *ticket, int *err) {
    constexpr int I = RsTile<K>::kItems, TILE = kRsT * I;
    __shared__ unsigned s_wc[kRsW][256];
    __shared__ unsigned s_base[256], s_lstart[256];
    __shared__ unsigned s_tmp[kRsT / 32];
    __shared__ unsigned s_tile;
    __shared__ K s_key[TILE];
    __shared__ unsigned s_val[TILE];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(ticket, 1u);
    for (int q = tid; q < kRsW * 256; q += kRsT) (&s_wc[0][0])[q] = 0;
    __syncthreads();
    const unsigned tile = s_tile;
    const size_t tbase = (size_t)tile * TILE;
    const size_t wbase = tbase + (size_t)warp * (32 * I);

    K key[I];
    unsigned val[I], dig[I], rank[I];
#pragma unroll
    for (int it = 0; it < I; it++) {
        size_t idx = wbase + (size_t)it * 32 + lane;
        if (idx < n) {
            key[it] = kin[idx];
            val[it] = vin ? vin[idx] : (unsigned)idx;
            dig[it] = (unsigned)((key[it] >> shift) & 255);
        } else {
            key[it] = 0;
            val[it] = 0;
            dig[it] = 256;
        }
    }
    // Stable rank within the warp's contiguous segment, item by item in input order.
#pragma unroll
    for (int it = 0; it < I; it++) {
        const unsigned d = dig[it];
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned lower = peers & ((1u << lane) - 1u);
        const unsigned before = d < 256 ? s_wc[warp][d] : 0u;
        rank[it] = before + __popc(lower);
        __syncwarp();
        if (d < 256 && lower == 0) s_wc[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // Thread `tid` owns digit `tid`: exclusive prefix over warps, then the tile count.
    const unsigned d = tid;
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < kRsW; w++) {
        unsigned c = s_wc[w][d];
        s_wc[w][d] = run;
        run += c;
    }
    unsigned excl = 0;
    unsigned long long *st = status + (size_t)tile * 256 + d;
    if (tile == 0) {
        st_release(st, kFlagPre | run);
    } else {
        st_release(st, kFlagAgg | run);
        for (int j = (int)tile - 1; j >= 0; j--) {
            unsigned long long s = wait_status(status + (size_t)j * 256 + d, err);
            excl += (unsigned)(s & 0xffffffffull);
            if ((s >> 62) != 1) break;
        }
        st_release(st, kFlagPre | (unsigned long long)(excl + run));
    }
    unsigned htot, ltot;
    const unsigned dstart = block_excl_scan<kRsT>(hist[d], htot, s_tmp);
    const unsigned lstart = block_excl_scan<kRsT>(run, ltot, s_tmp);
    s_base[d] = dstart + excl;  // global position of this tile's first key of digit d
    s_lstart[d] = lstart;       // its position within the digit-sorted tile
    __syncthreads();
#pragma unroll
    for (int it = 0; it < I; it++) {
        const unsigned dd = dig[it];
        if (dd < 256) {
            const unsigned lp = s_lstart[dd] + s_wc[warp][dd] + rank[it];
            s_key[lp] = key[it];
            s_val[lp] = val[it];
        }
    }
    __syncthreads();
    // ltot keys of this tile, digit-sorted: consecutive threads write consecutive addresses.
    for (unsigned q = tid; q < ltot; q += kRsT) {
        const K k = s_key[q];
        const unsigned dd = (unsigned)((k >> shift) & 255);
        const unsigned pos = s_base[dd] + (q - s_lstart[dd]);
        if (pos < n) {
            kout[pos] = k;
            vout[pos] = s_val[q];
        }
    }
}

size_t radix_sort_tmp_bytes(unsigned n, int bits) {
    int npass = (bits + 7) / 8;
    size_t tiles = (n + kRsT * 12 - 1) / (kRsT * 12);  // the smaller (64-bit key) tile bounds both
    return 256 + (size_t)npass * 256 * sizeof(unsigned) + tiles * 256 * sizeof(unsigned long long);
}

template <typename K>
cudaError_t radix_sort(K *keys, K *keys_alt, unsigned *vals, unsigned *vals_alt, unsigned n, int bits,
                       bool identity, void *tmp, int *d_err, cudaStream_t s, int *launches, int *in_alt,
                       const K *keys_in) {
    *in_alt = 0;
    int npass = (bits + 7) / 8;
    if (npass > (int)sizeof(K)) npass = (int)sizeof(K);
    if (n == 0) return cudaSuccess;
    if (npass == 0) npass = 1;  // still materialise the values (identity case)
    constexpr unsigned kTile = kRsT * RsTile<K>::kItems;
    unsigned tiles = (n + kTile - 1) / kTile;
    unsigned *ticket = (unsigned *)tmp;
    unsigned *hist = (unsigned *)((char *)tmp + 256);
    unsigned long long *status = (unsigned long long *)((char *)hist + (size_t)npass * 256 * sizeof(unsigned));
    cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)npass * 256 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    unsigned hblocks = (n + 255) / 256;
    if (hblocks > 1216) hblocks = 1216;
    const K *first = keys_in ? keys_in : keys;
    k_rs_hist<K><<<hblocks, 256, 0, s>>>(first, n, npass, hist);
    if (launches) (*launches)++;
    const K *src = first;
    K *dst = keys_alt, *other = keys;  // passes after the first ping-pong between keys_alt and keys
    unsigned *vsrc = identity ? nullptr : vals, *vdst = vals_alt;
    for (int p = 0; p < npass; p++) {
        e = cudaMemsetAsync(ticket, 0, 256, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, (size_t)tiles * 256 * sizeof(unsigned long long), s);
        if (e != cudaSuccess) return e;
        k_rs_pass<K><<<tiles, kRsT, 0, s>>>(src, dst, vsrc, vdst, n, 8 * p, hist + p * 256, status, ticket, d_err);
        if (launches) (*launches)++;
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        src = dst;
        K *tk = other; other = dst; dst = tk;
        unsigned *written = vdst;
        vdst = (written == vals_alt) ? vals : vals_alt;
        vsrc = written;
    }
    *in_alt = (npass & 1);
    return cudaSuccess;
}

template cudaError_t radix_sort<unsigned>(unsigned *, unsigned *, unsigned *, unsigned *, unsigned, int, bool,
                                          void *, int *, cudaStream_t, int *, int *, const unsigned *);
template cudaError_t radix_sort<unsigned long long>(unsigned long long *, unsigned long long *, unsigned *,
                                                    unsigned *, unsigned, int, bool, void *, int *, cudaStream_t,
                                                    int *, int *, const unsigned long long *);

}  // namespace qses
