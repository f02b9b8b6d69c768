// bt_device.cuh -- device building blocks shared by the peeling (msp) and
// h-index (hidx) kernels: the bounded grid barrier, the shared-memory row hash
// and the flattened butterfly walk of one edge.
#pragma once

#include <cub/block/block_scan.cuh>

#include <cstdint>

namespace bt {

constexpr int kThreads = 512;
constexpr int kHashSlots = 4096;            // shared-memory hash capacity (slots)
constexpr uint32_t kHashMaxDeg = kHashSlots / 2;
constexpr uint32_t kSliceMids = kThreads;   // mids per slice (one block scan)
constexpr uint32_t kPerThread = 4;          // consecutive probes per thread per round
constexpr uint32_t kRound = kThreads * kPerThread;
constexpr uint32_t kHitCap = kRound;        // a round finds at most kRound butterflies
constexpr uint32_t kEmpty = 0xffffffffu;

// ---------------------------------------------------------------------------
// memory-model helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct Barrier {
    unsigned count, gen, abort, error;
};

enum : unsigned { ERR_NONE = 0, ERR_TIMEOUT = 1, ERR_OVERFLOW = 2 };

// All `nblocks` CTAs of a cooperative grid meet here.  The wait is bounded by
// `wait_ns` of wall time; when it expires the CTA records ERR_TIMEOUT, raises
// `abort` and returns false, and every other waiting CTA returns false too.
__device__ inline bool grid_barrier(Barrier *b, unsigned nblocks, unsigned long long wait_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned gen = ld_acquire(&b->gen);
        __threadfence();
        unsigned arrived = atomicAdd(&b->count, 1u) + 1;
        if (arrived == nblocks) {
            b->count = 0;
            __threadfence();
            st_release(&b->gen, gen + 1);
        } else {
            unsigned long long t0 = global_ns();
            unsigned sleep = 32;
            while (ld_acquire(&b->gen) == gen) {
                if (ld_acquire(&b->abort)) { ok = 0; break; }
                if (global_ns() - t0 > wait_ns) {
                    atomicCAS(&b->error, 0u, (unsigned)ERR_TIMEOUT);
                    atomicExch(&b->abort, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(sleep);
                if (sleep < 256) sleep <<= 1;
            }
        }
        __threadfence();
        if (ld_acquire(&b->abort)) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// ---------------------------------------------------------------------------
// rows
// ---------------------------------------------------------------------------

struct Rows {
    const uint32_t *off;  // n+1 row starts
    const uint32_t *deg;  // live degree
    const uint32_t *nbr;  // neighbour ranks, ascending per row
    const uint32_t *eid;  // reference edge id of each slot
    const uint32_t *hub_base, *hub_mask;  // hub index of the original rows
    const uint2 *hub_pool;                // (neighbour rank, edge id); key kEmpty = free
};

// ---------------------------------------------------------------------------
// shared-memory state of one CTA
// ---------------------------------------------------------------------------

struct Walk {
    // anchor row staged as a hash: vertex -> edge id, plus a pending
    // decrement count per entry (peeling)
    uint32_t hkey[kHashSlots];
    uint32_t hval[kHashSlots];
    uint32_t hdec[kHashSlots];
    // one slice of at most kSliceMids pivot slots
    uint32_t mid_eid[kSliceMids];
    uint32_t mid_base[kSliceMids];
    uint32_t pre[kSliceMids + 1];
    uint32_t slot_dec[kSliceMids];
    uint8_t ok[kSliceMids];
    uint8_t pm_curr[kSliceMids];
    // butterflies found in the current round
    uint16_t hit_k[kHitCap];
    uint32_t hit_pos[kHitCap];
    uint32_t hit_a[kHitCap];
    uint32_t hit_n[2];
    uint32_t cached_anc, cached_size;  // staged anchor; size 0: use its hub table
    uint32_t gbase, gmask;             // hub table of the staged anchor
    uint32_t s_lo, s_hi;
    typename cub::BlockScan<uint32_t, kThreads>::TempStorage scan;
};

__device__ __forceinline__ uint32_t hash_slot(uint32_t y, uint32_t mask) {
    return (y * 0x9E3779B1u) & mask;
}

__device__ inline void walk_init(Walk &w) {
    for (uint32_t t = threadIdx.x; t < kHashSlots; t += blockDim.x) {
        w.hkey[t] = kEmpty;
        w.hdec[t] = 0;
    }
    for (uint32_t t = threadIdx.x; t < kSliceMids; t += blockDim.x) w.slot_dec[t] = 0;
    if (threadIdx.x == 0) {
        w.cached_anc = kEmpty;
        w.cached_size = 0;
        w.hit_n[0] = w.hit_n[1] = 0;
    }
    __syncthreads();
}

// Stage anc's live row as a shared-memory hash vertex -> edge id (rows
// longer than kHashMaxDeg use their global hub table instead).  Rows only ever
// lose processed edges, so a table built earlier for the same vertex stays a
// valid superset (callers check every edge's state).  Block-uniform; the
// caller has synchronised since the last lookup.
__device__ inline void walk_stage(const Rows &r, Walk &w, uint32_t anc) {
    if (w.cached_anc == anc) {
        __syncthreads();
        return;
    }
    const uint32_t d = r.deg[anc];
    for (uint32_t t = threadIdx.x; t < w.cached_size; t += blockDim.x) w.hkey[t] = kEmpty;
    __syncthreads();
    uint32_t size = 0;
    if (d <= kHashMaxDeg) {
        size = 64;
        while (size < 2 * d) size <<= 1;
        const uint32_t mask = size - 1, b = r.off[anc];
        for (uint32_t j = threadIdx.x; j < d; j += blockDim.x) {
            const uint32_t y = r.nbr[b + j], e = r.eid[b + j];
            uint32_t h = hash_slot(y, mask);
            for (uint32_t probe = 0; probe < size; probe++) {
                const uint32_t prev = atomicCAS(&w.hkey[h], kEmpty, y);
                if (prev == kEmpty || prev == y) {
                    w.hval[h] = e;
                    break;
                }
                h = (h + 1) & mask;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        w.cached_anc = anc;
        w.cached_size = size;
        w.gbase = size ? 0 : r.hub_base[anc];
        w.gmask = size ? 0 : r.hub_mask[anc];
    }
    __syncthreads();
}

// Where y sits in the staged anchor: its shared hash slot when the anchor is
// staged in shared memory (the edge id is hval[slot]), else the edge id
// (anc, y) from the anchor's hub table; kEmpty when y is not a neighbour.
__device__ __forceinline__ uint32_t walk_lookup(const Rows &r, const Walk &w, uint32_t y) {
    const uint32_t size = w.cached_size;
    if (size) {
        const uint32_t mask = size - 1;
        uint32_t h = hash_slot(y, mask);
        for (uint32_t probe = 0; probe < size; probe++) {
            const uint32_t k = w.hkey[h];
            if (k == y) return h;
            if (k == kEmpty) return kEmpty;
            h = (h + 1) & mask;
        }
        return kEmpty;
    }
    const uint32_t mask = w.gmask;
    const uint2 *tab = r.hub_pool + w.gbase;
    uint32_t h = hash_slot(y, mask);
    for (uint32_t probe = 0; probe <= mask; probe++) {
        const uint2 kv = tab[h];
        if (kv.x == y) return kv.y;
        if (kv.x == kEmpty) return kEmpty;
        h = (h + 1) & mask;
    }
    return kEmpty;
}

__device__ __forceinline__ uint32_t walk_anchor_edge(const Walk &w, uint32_t a) {
    return w.cached_size ? w.hval[a] : a;
}

// Build the hub tables (one CTA per row longer than kHashMaxDeg).
__device__ inline void hub_build(const Rows &r, uint32_t n, uint2 *pool) {
    for (uint32_t x = blockIdx.x; x < n; x += gridDim.x) {
        const uint32_t mask = r.hub_mask[x];
        if (!mask) continue;
        const uint32_t b = r.off[x], d = r.deg[x], base = r.hub_base[x];
        for (uint32_t j = threadIdx.x; j < d; j += blockDim.x) {
            const uint32_t y = r.nbr[b + j], e = r.eid[b + j];
            uint32_t h = hash_slot(y, mask);
            for (uint32_t probe = 0; probe <= mask; probe++) {
                const uint32_t prev = atomicCAS(&pool[base + h].x, kEmpty, y);
                if (prev == kEmpty || prev == y) {
                    pool[base + h].y = e;
                    break;
                }
                h = (h + 1) & mask;
            }
        }
    }
}

// Last slot s in [0, d) with pre[s] <= f (pre ascending, pre[0] <= f),
// by one warp with a 32-way search: log32(d) coalesced steps.
__device__ inline uint32_t warp_find_slot(const uint32_t *pre, uint32_t d, uint32_t f) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t lo = 0, hi = d;
    while (hi - lo > 32) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t idx = lo + lane * step;
        const bool ok = idx < hi && pre[idx] <= f;
        const uint32_t bal = __ballot_sync(0xffffffffu, ok);
        const uint32_t k = 31 - __clz(bal);
        lo = lo + k * step;
        hi = min(lo + step, hi);
    }
    const bool ok = lo + lane < hi && pre[lo + lane] <= f;
    const uint32_t bal = __ballot_sync(0xffffffffu, ok);
    return lo + 31 - __clz(bal);
}

// Walk the butterflies of one edge between pivot `piv` and anchor `anc`
// over the probe range [f0, f1) of piv's row (anc is staged here).  The probe
// space of a row is its mids' rows laid end to end: rowpre[pb + s] is the
// exclusive prefix of the degrees of the row's mids (as of the last row
// compaction) and `total` the row sum, so probe f is slot s (last with
// rowpre <= f) at position f - rowpre[pb + s] of mid's row.
//
// Slices of at most kSliceMids pivot slots are loaded into shared memory;
// prep_slot(k, e_pm) runs once per slot and says whether to probe its mid
// (the walk itself skips mid == anc).  Each round then probes kRound slots
// (kPerThread consecutive ones per thread) and queues the hits -- mids'
// neighbours y != piv that are also in anc's row -- in shared memory, and a
// second pass calls on_hit(k, pos, a) once per hit with all threads busy:
// k = slice slot of mid, pos = index of (mid, y) in the row arrays,
// a = walk_lookup's answer for y.  slice_done(cl) runs (block-uniform) after
// each slice's last hit.
template <class PrepSlot, class OnHit, class SliceDone>
__device__ inline void walk_range(const Rows &r, const uint32_t *rowpre, Walk &w, uint32_t piv,
                                  uint32_t anc, uint32_t total, uint32_t f0, uint32_t f1,
                                  PrepSlot prep_slot, OnHit on_hit, SliceDone slice_done) {
    if (f0 >= f1) return;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t pb = r.off[piv], pd = r.deg[piv];
    const uint32_t *pre = rowpre + pb;
    if (warp == 0) {
        const uint32_t t = warp_find_slot(pre, pd, f0);
        if (lane == 0) w.s_lo = t;
    } else if (warp == 1) {
        const uint32_t t = warp_find_slot(pre, pd, f1 - 1);
        if (lane == 0) w.s_hi = t;
    }
    walk_stage(r, w, anc);  // synchronises the block
    const uint32_t s_lo = w.s_lo, s_hi = w.s_hi;
    uint32_t par = 0;
    for (uint32_t c0 = s_lo; c0 <= s_hi; c0 += kSliceMids) {
        const uint32_t cl = min(kSliceMids, s_hi + 1 - c0);
        if (threadIdx.x < cl) {
            const uint32_t slot = c0 + threadIdx.x;
            const uint32_t mid = r.nbr[pb + slot];
            const uint32_t e_pm = r.eid[pb + slot];
            w.mid_eid[threadIdx.x] = e_pm;
            w.mid_base[threadIdx.x] = r.off[mid];
            w.pre[threadIdx.x] = pre[slot];
            w.ok[threadIdx.x] = (mid != anc && prep_slot(threadIdx.x, e_pm)) ? 1 : 0;
        }
        if (threadIdx.x == 0) w.pre[cl] = c0 + cl < pd ? pre[c0 + cl] : total;
        __syncthreads();
        const uint32_t g0 = max(f0, w.pre[0]), g1 = min(f1, w.pre[cl]);
        for (uint32_t rb = g0; rb < g1; rb += kRound) {
            // pass 1: probe, queue hits
            uint32_t hk[kPerThread], hp[kPerThread], ha[kPerThread];
            uint32_t mask = 0;
            const uint32_t f = rb + threadIdx.x * kPerThread;
            if (f < g1) {
                uint32_t lo = 0, hi = cl;
                while (hi - lo > 1) {
                    const uint32_t md = (lo + hi) >> 1;
                    if (w.pre[md] <= f) lo = md;
                    else hi = md;
                }
                uint32_t k = lo;
#pragma unroll
                for (uint32_t p = 0; p < kPerThread; p++) {
                    const uint32_t ff = f + p;
                    hk[p] = hp[p] = ha[p] = 0;
                    if (ff < g1) {
                        while (w.pre[k + 1] <= ff) k++;
                        if (w.ok[k]) {
                            const uint32_t pos = w.mid_base[k] + (ff - w.pre[k]);
                            const uint32_t y = r.nbr[pos];
                            if (y != piv) {
                                const uint32_t a = walk_lookup(r, w, y);
                                if (a != kEmpty) {
                                    hk[p] = k;
                                    hp[p] = pos;
                                    ha[p] = a;
                                    mask |= 1u << p;
                                }
                            }
                        }
                    }
                }
            }
            const uint32_t nh = __popc(mask);
            uint32_t incl = nh;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += t;
            }
            uint32_t base = 0;
            if (lane == 31 && incl) base = atomicAdd(&w.hit_n[par], incl);
            base = __shfl_sync(0xffffffffu, base, 31) + incl - nh;
#pragma unroll
            for (uint32_t p = 0; p < kPerThread; p++) {
                if (mask & (1u << p)) {
                    w.hit_k[base] = (uint16_t)hk[p];
                    w.hit_pos[base] = hp[p];
                    w.hit_a[base] = ha[p];
                    base++;
                }
            }
            __syncthreads();
            // pass 2: one hit per thread
            const uint32_t n = w.hit_n[par];
            for (uint32_t i = threadIdx.x; i < n; i += kThreads) on_hit(w.hit_k[i], w.hit_pos[i], w.hit_a[i]);
            if (threadIdx.x == 0) w.hit_n[par ^ 1] = 0;
            par ^= 1;
            __syncthreads();
        }
        slice_done(cl);
        __syncthreads();
    }
    if (threadIdx.x == 0) w.hit_n[0] = w.hit_n[1] = 0;
    __syncthreads();
}

// Row prefix of neighbour degrees (one warp per vertex): rowpre[off + s] =
// sum of deg[nbr[off + k]] for k < s, total[x] = the row sum (saturated).
__device__ inline void row_prefix(const Rows &r, uint32_t n, uint32_t *rowpre, uint32_t *total) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t x = warp; x < n; x += nw) {
        const uint32_t b = r.off[x], d = r.deg[x];
        unsigned long long run = 0;
        for (uint32_t j0 = 0; j0 < d; j0 += 32) {
            const uint32_t j = j0 + lane;
            const uint32_t v = j < d ? r.deg[r.nbr[b + j]] : 0;
            uint32_t inc = v;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= (uint32_t)o) inc += t;
            }
            if (j < d) rowpre[b + j] = (uint32_t)(run + inc - v);
            run += __shfl_sync(0xffffffffu, inc, 31);
        }
        if (lane == 0) total[x] = run > 0xffffffffull ? 0xffffffffu : (uint32_t)run;
    }
}

}  // namespace bt
