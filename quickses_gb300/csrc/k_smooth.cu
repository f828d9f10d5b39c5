// Exact Gauss-Seidel Laplacian smoothing (SmoothMesh.cpp:45-123) as a dataflow over slabs of
// vertex ids: a vertex is updated once every lower-id neighbour has been, exactly as the
// sequential loop would see them.  Persistent CTAs take the slabs from a device work queue.
#include <cstdlib>
#include <cstring>

#include "device_common.cuh"

#include "kernels.h"

namespace qses {

__device__ __forceinline__ int atom_sub_acq_rel(int *p, int v) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(-v) : "memory");
    return old;
}

// Slab-partitioned Gauss-Seidel pass.  Vertex ids are split into P contiguous slabs, one
// persistent CTA each.  Every dependency edge goes from a lower to a higher id, so a chain
// of updates crosses each slab boundary at most once: readiness inside a slab is tracked
// with shared-memory counters and a ring of ready vertices, and only boundary edges go
// through global memory (an acquire/release counter per vertex and a per-slab inbox).
// Each vertex is still computed exactly as the sequential loop would.
constexpr int kGsSlabMaxSmem = 200 * 1024;  // dynamic part: offsets, packed counters, ring: 8 B/vertex
                                            // (+ 16 B/vertex of positions with kGsSmemPos)
__host__ __device__ constexpr size_t gs_spos_offset(unsigned smax) {
    return ((4ull * (smax + 1) + 4ull * ((smax + 1) / 2) + 2ull * smax) + 15) & ~(size_t)15;
}

// Two 16-bit readiness counters per shared word; returns the counter value before the
// decrement.  Counters never go below zero, so no borrow crosses into the other half.
__device__ __forceinline__ unsigned dec16(unsigned *w, unsigned k) {
    const unsigned sh = 16u * (k & 1u);
    return (atomicSub(&w[k >> 1], 1u << sh) >> sh) & 0xffffu;
}

__device__ __forceinline__ void ring_push16(volatile unsigned short *ring, unsigned *tail, unsigned off) {
    const unsigned k = atomicAdd(tail, 1u);
    ring[k] = (unsigned short)off;  // each vertex enters the ring once: no wrap-around
}

constexpr unsigned kGsOutbox = 1024;  // shared-memory queue of cross-slab releases

__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ void prefetch_l1(const void *p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// Persistent CTAs take the wave's slabs from a counter, in the table's order (a slab only
// waits for slabs taken before it, by CTAs that were running when they took them, so every
// wait ends without a co-residency guarantee).  Per slab,
// warp 0 takes boundary arrivals from lower slabs, warp 1 sends this slab's cross-slab
// releases (GPU-scope atomics, off the workers' critical path), the other warps update
// vertices.  Table: Q, the Q + 1 slab bounds in id order (qcap + 1 slots), then the Q slab ids
// in the order they are taken.
template <int kGsT, unsigned kFlags>
__global__ void __launch_bounds__(kGsT, kGsT <= 512 ? 2 : 1) k_gs_flow(float4 *pos4, unsigned v0, unsigned nv, unsigned smax,
                                                  const unsigned *__restrict__ table, unsigned qcap,
                                                  unsigned *next_slab, const uint2 *__restrict__ home,
                                                  const uint2 *__restrict__ start, const unsigned *__restrict__ nbr,
                                                  const unsigned short *__restrict__ cnt_local, int *remote,
                                                  unsigned *inbox, unsigned *inbox_tail, int *err,
                                                  long long spin_cycles, unsigned long long *stats,
                                                  unsigned idle_ns_max, unsigned hot_warps) {
    extern __shared__ unsigned s_dyn[];
    __shared__ unsigned s_head, s_tail, s_done, s_stop, s_ob_head, s_ob_tail, s_slab;
    __shared__ unsigned s_ob[kGsOutbox];
    // Per worker warp: one row of neighbour positions, summed in list order by lane 0 (of
    // each lane group): one shared-memory round trip, then a chain of adds in registers,
    // instead of a shuffle per entry.
    __shared__ float4 s_stage[kGsT / 32][32];
    unsigned *st = s_dyn;                                        // len + 1 CSR offsets of the slab
    unsigned *cnt = s_dyn + (smax + 1);                          // (len + 1) / 2 words: packed counters
    volatile unsigned short *ring = (volatile unsigned short *)(cnt + (smax + 1) / 2);  // slab offsets
    // kGsSmemPos: the slab's positions (old until a vertex updates, then new), so neighbours
    // inside the slab are read from shared memory; others from global memory as before
    constexpr bool kSP = (kFlags & kGsSmemPos) != 0;
    // lanes per vertex update: 32 (one vertex per worker warp), or 16 / 8 with kGsPair /
    // kGsQuad (2 / 4 ready vertices per worker warp, one lane group each)
    constexpr unsigned kLanes = (kFlags & kGsQuad) ? 8u : (kFlags & kGsPair) ? 16u : 32u;
    float4 *spos = (float4 *)((char *)s_dyn + gs_spos_offset(smax));
    volatile unsigned *ob = s_ob;
    const unsigned Q = min(__ldg(table), qcap);
    const unsigned *bnd = table + 1, *order = table + 2 + qcap;
    const unsigned lane = threadIdx.x & 31;
    // longest sleep of this warp when idle: the first hot_warps worker warps poll the ring
    // every 64 ns at most, so a vertex pushed there is picked up without waiting for a
    // warp that backed off to idle_ns_max
    const unsigned idle_cap = (threadIdx.x >> 5) < 2u + hot_warps ? min(64u, idle_ns_max) : idle_ns_max;
    unsigned long long cyc_update = 0, cyc_release = 0, nproc = 0, polls = 0, cyc_ids = 0, cyc_pos = 0, cyc_fence = 0;
    if (threadIdx.x == 0) s_stop = 0;
    for (;;) {
    if (threadIdx.x == 0) {
        const unsigned k = atomicAdd(next_slab, 1u);
        s_slab = (k < Q && !s_stop) ? __ldg(order + k) : 0xffffffffu;
        s_head = 0; s_tail = 0; s_done = 0; s_ob_head = 0; s_ob_tail = 0;
    }
    __syncthreads();
    const unsigned p = s_slab;
    if (p >= Q) break;  // uniform per CTA: no slab left (or an error stopped this CTA)
    const unsigned a = __ldg(bnd + p), b = __ldg(bnd + p + 1), len = b - a;
    if (a < v0 || b > nv || b <= a || len > smax) {  // uniform: a malformed table entry
        if (threadIdx.x == 0) raise_error(err, QSES_ERR_INTERNAL);
        break;
    }
    unsigned *box = inbox + (a - v0);                            // boundary arrivals from lower slabs
    for (unsigned k = threadIdx.x; k < kGsOutbox; k += kGsT) s_ob[k] = 0xffffffffu;
    for (unsigned k = threadIdx.x; k <= len; k += kGsT) st[k] = start[a + k].x;
    for (unsigned k = threadIdx.x; k < len; k += kGsT) ring[k] = 0xffffu;
    if (kSP)
        for (unsigned k = threadIdx.x; k < len; k += kGsT) spos[k] = __ldcg(pos4 + a + k);
    for (unsigned k = threadIdx.x; 2 * k < len; k += kGsT) {
        const unsigned lo = cnt_local[a + 2 * k], hi = 2 * k + 1 < len ? cnt_local[a + 2 * k + 1] : 0u;
        cnt[k] = lo | (hi << 16);
    }
    __syncthreads();
    for (unsigned k = threadIdx.x; k < len; k += kGsT)
        if (cnt_local[a + k] == 0) ring_push16(ring, &s_tail, k);
    __syncthreads();

    if (threadIdx.x < 32) {
        // Warp 0 only takes boundary arrivals (the last lower-slab dependency of a vertex
        // finished); it never updates vertices, so arrivals are never stuck behind a chain.
        if (lane == 0) {
            unsigned seen = 0, done_seen = 0;
            long long last = clock64();
            for (;;) {
                if (*(volatile unsigned *)&s_done >= len || *(volatile unsigned *)&s_stop) break;
                const unsigned tail = min(ld_acquire_u32(inbox_tail + p), len);
                polls++;
                for (unsigned k = seen; k < tail; k++) {
                    unsigned u = 0xffffffffu;
                    for (unsigned it = 0; it < (1u << 20) && u == 0xffffffffu; it++) u = ld_acquire_u32(box + k);
                    if (u < a || u >= b) {
                        raise_error(err, u == 0xffffffffu ? QSES_ERR_TIMEOUT : QSES_ERR_INTERNAL);
                        s_stop = 1;
                        break;
                    }
                    __threadfence_block();
                    if (dec16(cnt, u - a) == 1u) ring_push16(ring, &s_tail, u - a);
                }
                const long long now = clock64();
                const unsigned d = *(volatile unsigned *)&s_done;
                if (tail != seen || d != done_seen) last = now;
                seen = tail;
                done_seen = d;
                if (now - last > spin_cycles) {
                    raise_error(err, QSES_ERR_TIMEOUT);
                    s_stop = 1;
                }
                if (tail == seen) __nanosleep(20);
            }
        }
    } else if (threadIdx.x < 64) {
        // Warp 1 sends cross-slab releases queued by the workers, up to 32 at a time.  A
        // worker queues an entry after its position store and a CTA-scope fence; the fence
        // here plus the GPU-scope acq_rel atomic carry that store to the receiving slab.
        unsigned head = 0;
        for (;;) {
            const unsigned tail = *(volatile unsigned *)&s_ob_tail;
            const unsigned count = min(tail - head, 32u);
            if (count == 0) {
                if (*(volatile unsigned *)&s_stop) break;
                if (*(volatile unsigned *)&s_done >= len) {
                    __threadfence_block();
                    if (*(volatile unsigned *)&s_ob_tail == head) break;  // every worker is done
                    continue;
                }
                __nanosleep(20);
                continue;
            }
            if (lane < count) {
                volatile unsigned *slot = ob + (head + lane) % kGsOutbox;
                unsigned u = 0xffffffffu;
                for (unsigned it = 0; it < (1u << 20) && u == 0xffffffffu; it++) u = *slot;  // reserved slot
                if (u == 0xffffffffu || u < b || u >= nv) {
                    raise_error(err, u == 0xffffffffu ? QSES_ERR_TIMEOUT : QSES_ERR_INTERNAL);
                    s_stop = 1;
                } else {
                    *slot = 0xffffffffu;
                    __threadfence_block();
                    const uint2 h = __ldg(home + u);  // u's slab and its first vertex (constant)
                    if (atom_sub_acq_rel(remote + u, 1) == 1) {
                        // last lower-slab dependency of u: hand u to its slab
                        const unsigned k = atomicAdd(inbox_tail + h.x, 1u);
                        if (k < smax && h.x < Q) st_release_u32(inbox + (h.y - v0) + k, u);
                    }
                }
            }
            head += count;
            __syncwarp();
            if (lane == 0) {
                __threadfence_block();
                *(volatile unsigned *)&s_ob_head = head;  // slots before head are free again
            }
        }
    } else if constexpr (kLanes == 32) {
        // Worker warps: one vertex per warp; lanes fetch neighbours in parallel.  An idle
        // worker backs off (32 ns doubling up to idle_ns_max, 1 us by default): a hot polling loop of up to
        // 30 warps would take issue slots and shared-memory bandwidth from the warps on the
        // critical path.
        unsigned idle_ns = 0;
        for (;;) {
            unsigned v = 0xffffffffu, quit = 0;
            if (lane == 0) {
                const unsigned h = *(volatile unsigned *)&s_head, t = *(volatile unsigned *)&s_tail;
                if (h < t && atomicCAS(&s_head, h, h + 1) == h) {
                    unsigned off = 0xffffu;
                    for (unsigned it = 0; it < (1u << 20) && off == 0xffffu; it++) off = ring[h];  // reserved slot
                    if (off == 0xffffu) {
                        raise_error(err, QSES_ERR_TIMEOUT);
                        s_stop = 1;
                    } else {
                        v = a + off;
                    }
                } else if (h >= t) {
                    quit = (*(volatile unsigned *)&s_done >= len) || *(volatile unsigned *)&s_stop;
                }
            }
            v = __shfl_sync(0xffffffffu, v, 0);
            quit = __shfl_sync(0xffffffffu, quit, 0);
            if (quit) break;
            if (v == 0xffffffffu) {
                idle_ns = idle_ns ? min(2 * idle_ns, idle_cap) : 32u;
                __nanosleep(idle_ns);
                continue;
            }
            idle_ns = 0;
            // Neighbour ids of the vertex this warp continues with, loaded as soon as the
            // release picked it (the lists are constant, so the early load is always valid).
            unsigned pre_v = 0xffffffffu, pre_id = 0u;
            while (v != 0xffffffffu) {  // follow the chain of vertices this warp releases
                __threadfence_block();
                const long long c0 = clock64();
                const unsigned e0 = st[v - a], e1 = st[v - a + 1];
                float sx = 0.0f, sy = 0.0f, sz = 0.0f;
                unsigned first_id = v;
                for (unsigned base = e0; base < e1; base += 32) {
                    const unsigned m = min(32u, e1 - base);
                    const unsigned id = (base == e0 && pre_v == v) ? pre_id
                                                                  : (lane < m ? __ldg(nbr + base + lane) : v);
                    if (base == e0) first_id = id;
                    long long ca = 0;
                    if (stats && base == e0) {  // diagnostics: when the ids have arrived (the mov waits for them)
                        unsigned t;
                        asm volatile("mov.b32 %0, %1;" : "=r"(t) : "r"(id));
                        ca = clock64();
                        cyc_ids += ca - c0 + (t & 0u);
                    }
                    // Weak loads either way: the CTA- and GPU-scope acquires above order them.
                    float4 q;
                    if (kSP && id - a < len) q = spos[id - a];
                    else q = (kFlags & kGsL1Positions) ? pos4[id] : __ldcg(pos4 + id);
                    if (stats && base == e0) {  // ... and their positions
                        float t;
                        asm volatile("mov.b32 %0, %1;" : "=f"(t) : "f"(q.x));
                        cyc_pos += clock64() - ca + (t != t ? 1 : 0);
                    }
                    // strictly in neighbour-list order, by lane 0 from the warp's row
                    float4 *row = s_stage[threadIdx.x >> 5];
                    if (lane < m) row[lane] = q;
                    __syncwarp();
                    if (lane == 0) {
#pragma unroll 4
                        for (unsigned k = 0; k < m; k++) {
                            const float4 p = row[k];
                            sx = __fadd_rn(sx, p.x);
                            sy = __fadd_rn(sy, p.y);
                            sz = __fadd_rn(sz, p.z);
                        }
                    }
                    __syncwarp();  // the row is rewritten by the next chunk or vertex
                }
                const float n = (float)(int)(e1 - e0);
                if (lane == 0) {
                    const float4 np = make_float4(__fdiv_rn(sx, n), __fdiv_rn(sy, n), __fdiv_rn(sz, n), 0.0f);
                    long long cs = 0;
                    if (stats) {  // diagnostics: the store and its fence (the movs wait for the sums)
                        float t0, t1, t2;
                        asm volatile("mov.b32 %0, %3; mov.b32 %1, %4; mov.b32 %2, %5;"
                                     : "=f"(t0), "=f"(t1), "=f"(t2) : "f"(np.x), "f"(np.y), "f"(np.z));
                        cs = clock64() + (t0 != t0 || t1 != t1 || t2 != t2 ? 1 : 0);
                    }
                    if (kSP) spos[v - a] = np;
                    __stcg(pos4 + v, np);
                    // Successors in this slab read the new position after a CTA-scope
                    // acquire; successors in higher slabs get it through the sender warp.
                    __threadfence_block();
                    if (stats) cyc_fence += clock64() - cs;
                }
                const long long c1 = clock64();
                __syncwarp();
                // Release: one lane per neighbour entry.
                unsigned next = 0xffffffffu;
                for (unsigned base = e0; base < e1; base += 32) {
                    const unsigned m = min(32u, e1 - base);
                    const unsigned u = lane < m ? (base == e0 ? first_id : __ldg(nbr + base + lane)) : 0u;
                    // successors at or above nv (the wave's end) belong to a later wave, which
                    // starts after this one has finished: nothing to release for them
                    const bool higher = lane < m && u > v && u < nv;
                    const bool remote_edge = higher && u >= b;
                    bool ready = false;
                    if (higher) {
                        if (!remote_edge) {
                            // u's list, needed when u runs
                            if (kFlags & kGsL1Prefetch) prefetch_l1(nbr + st[u - a]);
                            else prefetch_l2(nbr + st[u - a]);
                            ready = dec16(cnt, u - a) == 1u;
                        } else {
                            const unsigned k = atomicAdd(&s_ob_tail, 1u);
                            unsigned it = 0;
                            for (; it < (1u << 22) && k - *(volatile unsigned *)&s_ob_head >= kGsOutbox; it++)
                                __nanosleep(32);
                            if (k - *(volatile unsigned *)&s_ob_head >= kGsOutbox) {
                                raise_error(err, QSES_ERR_TIMEOUT);
                                s_stop = 1;
                            } else {
                                __threadfence_block();  // release: the position store before the entry
                                ob[k % kGsOutbox] = u;
                            }
                        }
                    }
                    unsigned mask = __ballot_sync(0xffffffffu, ready);
                    if (mask && next == 0xffffffffu) {
                        const unsigned f = __ffs(mask) - 1;
                        next = __shfl_sync(0xffffffffu, u, f);  // continue with it directly
                        mask &= ~(1u << f);
                        const unsigned ne0 = st[next - a], nm = min(32u, st[next - a + 1] - ne0);
                        pre_id = lane < nm ? __ldg(nbr + ne0 + lane) : next;
                        pre_v = next;
                    }
                    if ((mask >> lane) & 1u) ring_push16(ring, &s_tail, u - a);
                }
                __syncwarp();  // queued releases precede the done count the sender checks
                if (lane == 0) atomicAdd(&s_done, 1u);
                v = next;
                const long long c2 = clock64();
                cyc_update += c1 - c0;
                cyc_release += c2 - c1;
                nproc++;
            }
        }
    } else {
        // Worker warps of 32 / kLanes lane groups.  Ready vertices never depend on one another
        // (a vertex is ready only once every lower-id neighbour has been updated), so the
        // groups of a warp update different ready vertices in the same instructions; each
        // group keeps its vertex's in-order sum (shuffles of width kLanes) and follows the
        // chain of vertices it releases, and a group without a vertex takes one from the
        // ring at the top of each step.
        constexpr unsigned kGroups = 32u / kLanes;
        constexpr unsigned kLow = (1u << kLanes) - 1u;
        constexpr unsigned kLeaders = kGroups == 2 ? 0x00010001u : 0x01010101u;  // lane 0 of each group
        const unsigned gl = lane % kLanes, g0 = lane - gl;  // lane in the group, the group's lane 0
        unsigned idle_ns = 0;
        unsigned v = 0xffffffffu;  // this group's vertex
        unsigned pre_v = 0xffffffffu, pre_id[2] = {0u, 0u};
        for (;;) {
            const unsigned empty = __ballot_sync(0xffffffffu, gl == 0 && v == 0xffffffffu);
            if (empty) {
                unsigned got = 0, h0 = 0, quit = 0;
                if (lane == 0) {
                    const unsigned h = *(volatile unsigned *)&s_head, t = *(volatile unsigned *)&s_tail;
                    if (h < t) {
                        const unsigned k = min((unsigned)__popc(empty), t - h);
                        if (atomicCAS(&s_head, h, h + k) == h) {
                            got = k;
                            h0 = h;
                        }
                    } else if (empty == kLeaders) {  // no group has a vertex
                        quit = (*(volatile unsigned *)&s_done >= len) || *(volatile unsigned *)&s_stop;
                    }
                }
                got = __shfl_sync(0xffffffffu, got, 0);
                h0 = __shfl_sync(0xffffffffu, h0, 0);
                if (__shfl_sync(0xffffffffu, quit, 0)) break;
                if (gl == 0 && v == 0xffffffffu) {
                    const unsigned r = __popc(empty & ((1u << lane) - 1u));  // empty groups before this one
                    if (r < got) {
                        unsigned off = 0xffffu;
                        for (unsigned it = 0; it < (1u << 20) && off == 0xffffu; it++) off = ring[h0 + r];  // reserved slot
                        if (off == 0xffffu) {
                            raise_error(err, QSES_ERR_TIMEOUT);
                            s_stop = 1;
                        } else {
                            v = a + off;
                        }
                    }
                }
                v = __shfl_sync(0xffffffffu, v, g0);
            }
            const unsigned busy = __ballot_sync(0xffffffffu, gl == 0 && v != 0xffffffffu);
            if (!busy) {
                idle_ns = idle_ns ? min(2 * idle_ns, idle_cap) : 32u;
                __nanosleep(idle_ns);
                continue;
            }
            idle_ns = 0;
            __threadfence_block();
            const long long c0 = clock64();
            const bool act = v != 0xffffffffu;
            const unsigned e0 = act ? st[v - a] : 0u, nlen = act ? st[v - a + 1] - e0 : 0u;
            const unsigned maxlen = __reduce_max_sync(0xffffffffu, nlen);
            // Rounds of two chunks of kLanes entries: both chunks' ids, then both chunks'
            // positions are in flight before the in-order sum (lists of up to 2 kLanes
            // entries take one round trip for each, as a whole warp's 32 lanes do).
            float sx = 0.0f, sy = 0.0f, sz = 0.0f;
            unsigned first_id[2] = {0u, 0u};
            for (unsigned r0 = 0; r0 < maxlen; r0 += 2 * kLanes) {
                unsigned id[2];
                float4 q[2];
#pragma unroll
                for (unsigned j = 0; j < 2; j++) {
                    const unsigned o = r0 + j * kLanes + gl;
                    id[j] = o >= nlen ? 0u : (r0 == 0 && pre_v == v) ? pre_id[j] : __ldg(nbr + e0 + o);
                }
#pragma unroll
                for (unsigned j = 0; j < 2; j++) {
                    // weak loads: the CTA- and GPU-scope acquires order them; lanes past the
                    // list load nothing (their slots are not summed)
                    q[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (r0 + j * kLanes + gl < nlen) {
                        if (kSP && id[j] - a < len) q[j] = spos[id[j] - a];
                        else q[j] = (kFlags & kGsL1Positions) ? pos4[id[j]] : __ldcg(pos4 + id[j]);
                    }
                }
                if (r0 == 0) {
                    first_id[0] = id[0];
                    first_id[1] = id[1];
                }
                // strictly in neighbour-list order, by each group's lane 0 from the warp's row
                // (a group's entries sit in its own kLanes slots)
                float4 *row = s_stage[threadIdx.x >> 5];
#pragma unroll
                for (unsigned j = 0; j < 2; j++) {
                    if (r0 + j * kLanes >= maxlen) break;  // uniform: no group has entries here
                    row[lane] = q[j];
                    __syncwarp();
                    const unsigned o0 = r0 + j * kLanes;
                    if (gl == 0 && o0 < nlen) {
                        const unsigned cj = min(kLanes, nlen - o0);
#pragma unroll 4
                        for (unsigned k = 0; k < cj; k++) {
                            const float4 p = row[g0 + k];
                            sx = __fadd_rn(sx, p.x);
                            sy = __fadd_rn(sy, p.y);
                            sz = __fadd_rn(sz, p.z);
                        }
                    }
                    __syncwarp();  // the row is rewritten by the next chunk or vertex
                }
            }
            if (act && gl == 0) {
                const float n = (float)(int)nlen;
                const float4 np = make_float4(__fdiv_rn(sx, n), __fdiv_rn(sy, n), __fdiv_rn(sz, n), 0.0f);
                if (kSP) spos[v - a] = np;
                __stcg(pos4 + v, np);
                __threadfence_block();
            }
            const long long c1 = clock64();
            __syncwarp();
            // Release: one lane per neighbour entry of the group's vertex.
            unsigned next = 0xffffffffu;
            for (unsigned r0 = 0; r0 < maxlen; r0 += 2 * kLanes) {
#pragma unroll
                for (unsigned j = 0; j < 2; j++) {
                    if (r0 + j * kLanes >= maxlen) break;  // uniform
                    const unsigned o = r0 + j * kLanes + gl;
                    const unsigned u = o < nlen ? (r0 == 0 ? first_id[j] : __ldg(nbr + e0 + o)) : 0u;
                    const bool higher = o < nlen && u > v && u < nv;
                    const bool remote_edge = higher && u >= b;
                    bool ready = false;
                    if (higher) {
                        if (!remote_edge) {
                            if (kFlags & kGsL1Prefetch) prefetch_l1(nbr + st[u - a]);
                            else prefetch_l2(nbr + st[u - a]);
                            ready = dec16(cnt, u - a) == 1u;
                        } else {
                            const unsigned k = atomicAdd(&s_ob_tail, 1u);
                            unsigned it = 0;
                            for (; it < (1u << 22) && k - *(volatile unsigned *)&s_ob_head >= kGsOutbox; it++)
                                __nanosleep(32);
                            if (k - *(volatile unsigned *)&s_ob_head >= kGsOutbox) {
                                raise_error(err, QSES_ERR_TIMEOUT);
                                s_stop = 1;
                            } else {
                                __threadfence_block();  // release: the position store before the entry
                                ob[k % kGsOutbox] = u;
                            }
                        }
                    }
                    unsigned gm = (__ballot_sync(0xffffffffu, ready) >> g0) & kLow;  // this group's ready lanes
                    const bool take = gm != 0 && next == 0xffffffffu;
                    const unsigned f = take ? __ffs(gm) - 1 : 0u;
                    const unsigned cand = __shfl_sync(0xffffffffu, u, g0 + f);
                    if (take) {  // continue with it directly; its first two chunks of ids load now
                        next = cand;
                        gm &= ~(1u << f);
                        const unsigned ne0 = st[next - a], nn = st[next - a + 1] - ne0;
                        pre_id[0] = gl < nn ? __ldg(nbr + ne0 + gl) : 0u;
                        pre_id[1] = kLanes + gl < nn ? __ldg(nbr + ne0 + kLanes + gl) : 0u;
                        pre_v = next;
                    }
                    if ((gm >> gl) & 1u) ring_push16(ring, &s_tail, u - a);
                }
            }
            __syncwarp();  // queued releases precede the done count the sender checks
            if (lane == 0) atomicAdd(&s_done, (unsigned)__popc(busy));
            v = next;
            const long long c2 = clock64();
            cyc_update += c1 - c0;
            cyc_release += c2 - c1;
            nproc += __popc(busy);
        }
    }
    __syncthreads();
    if (stats && threadIdx.x == 0 && s_done < len) atomicAdd(stats + 1, 1ull);  // unfinished slabs
    }  // next slab
    if (stats) {  // diagnostics: polls (max), update cycles, release cycles, vertices
        if (threadIdx.x == 0) atomicMax(stats, polls);
        if (lane == 0 && nproc) {
            atomicAdd(stats + 2, cyc_update);
            atomicAdd(stats + 3, cyc_release);
            atomicAdd(stats + 4, nproc);
            atomicAdd(stats + 5, cyc_ids);
            atomicAdd(stats + 6, cyc_pos);
            atomicAdd(stats + 7, cyc_fence);
        }
    }
}

// ------------------------------------------------------------ launchers

size_t gs_slab_smem(unsigned S, unsigned flags) {
    return (flags & kGsSmemPos) ? gs_spos_offset(S) + 16ull * S + 16 : 4ull * (S + 1) + 4ull * ((S + 1) / 2) + 2ull * S + 16;
}
template <int T, unsigned M>
static constexpr const void *gs_fn(unsigned c) {
    return c == 0 ? (const void *)k_gs_flow<T, M | 0> : c == 1 ? (const void *)k_gs_flow<T, M | 1>
         : c == 2 ? (const void *)k_gs_flow<T, M | 2> : c == 3 ? (const void *)k_gs_flow<T, M | 3>
         : c == 4 ? (const void *)k_gs_flow<T, M | 8> : c == 5 ? (const void *)k_gs_flow<T, M | 9>
         : c == 6 ? (const void *)k_gs_flow<T, M | 10> : (const void *)k_gs_flow<T, M | 11>;
}
// The kernel instance for a launch shape: threads, lanes per vertex and the cache flags
// (bits 0, 1, 3; bit 2 is host-side only).
static const void *gs_flow_fn(int threads, unsigned flags) {
    const unsigned c = (flags & 3u) | ((flags & kGsSmemPos) ? 4u : 0u);
    const unsigned mode = (flags & kGsQuad) ? 2u : (flags & kGsPair) ? 1u : 0u;
    if (threads >= 1024)
        return mode == 2 ? gs_fn<1024, kGsQuad>(c) : mode == 1 ? gs_fn<1024, kGsPair>(c) : gs_fn<1024, 0>(c);
    return mode == 2 ? gs_fn<512, kGsQuad>(c) : mode == 1 ? gs_fn<512, kGsPair>(c) : gs_fn<512, 0>(c);
}
cudaError_t launch_gs_slab(float4 *pos, unsigned v0, unsigned nv, unsigned smax, const unsigned *table,
                           unsigned qcap, unsigned *next_slab, const uint2 *home, int P, int threads, unsigned flags,
                           unsigned hot_warps, const uint2 *start, const unsigned *nbr,
                           const unsigned short *cnt_local, int *remote,
                           unsigned *inbox, unsigned *inbox_tail, int *err, long long spin_cycles,
                           unsigned long long *stats, cudaStream_t s) {
    if (smax == 0 || smax > kGsSlabMaxVerts || ((flags & kGsSmemPos) && smax > kGsSmemPosMaxVerts) ||
        !gs_flags_valid(flags))
        return cudaErrorInvalidValue;
    size_t smem = gs_slab_smem(smax, flags);
    if (smem > (size_t)kGsSlabMaxSmem) return cudaErrorInvalidValue;
    const void *fn = gs_flow_fn(threads, flags);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kGsSlabMaxSmem);
    // longest sleep of an idle worker warp (ns); QSES_GS_IDLE_NS overrides it
    static const unsigned idle_ns_max = [] {
        const char *e = getenv("QSES_GS_IDLE_NS");
        const long v = e ? strtol(e, nullptr, 10) : 0;
        return v >= 32 && v <= 100000 ? (unsigned)v : 1024u;
    }();
    // worker warps that stay hot; QSES_GS_HOT_WARPS (0-30) overrides the caller's count
    static const int hot_env = [] {
        const char *e = getenv("QSES_GS_HOT_WARPS");
        const long v = e ? strtol(e, nullptr, 10) : -1;
        return v >= 0 && v <= 30 ? (int)v : -1;
    }();
    unsigned idle = idle_ns_max, hot = hot_env >= 0 ? (unsigned)hot_env : hot_warps;
    void *args[] = {&pos,    &v0,    &nv,          &smax,  (void *)&table, &qcap,         &next_slab,
                    (void *)&home, (void *)&start, (void *)&nbr, (void *)&cnt_local, &remote, &inbox,
                    &inbox_tail, &err, &spin_cycles, &stats, &idle, &hot};
    // A cooperative launch: every CTA resident from the start.  (A plain launch would also be
    // safe - a CTA only waits for slabs taken before its own, by CTAs that were running when
    // they took them - but its CTAs can then take the SMs the side stream's kernels wait for.)
    return cudaLaunchCooperativeKernel(fn, dim3(P), dim3(threads >= 1024 ? 1024 : 512), args, smem, s);
}
void gs_l2_window(int device, cudaStream_t s, const void *p, size_t bytes) {
    int max_persist = 0, max_window = 0;
    cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, device);
    cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, device);
    cudaStreamAttrValue attr;
    memset(&attr, 0, sizeof(attr));
    if (bytes > 0 && max_persist > 0 && max_window > 0) {
        const size_t window = bytes < (size_t)max_window ? bytes : (size_t)max_window;
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)max_persist);
        attr.accessPolicyWindow.base_ptr = const_cast<void *>(p);
        attr.accessPolicyWindow.num_bytes = window;
        attr.accessPolicyWindow.hitRatio = window <= (size_t)max_persist ? 1.0f : (float)max_persist / (float)window;
        attr.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &attr);
    } else {
        attr.accessPolicyWindow.num_bytes = 0;
        cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &attr);
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    }
    cudaGetLastError();  // the window is a hint: a refusal leaves the results unchanged
}

int gs_slab_max_blocks(int device, unsigned S, int threads, unsigned flags) {
    const void *fn = gs_flow_fn(threads, flags);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kGsSlabMaxSmem);
    int per_sm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads >= 1024 ? 1024 : 512, gs_slab_smem(S, flags));
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    return per_sm * sms;
}

}  // namespace qses
