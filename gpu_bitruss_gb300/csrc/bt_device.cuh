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
constexpr uint32_t kHubMinDeg = 256;        // rows longer than this get a global hub table
constexpr uint32_t kSliceMids = kThreads;   // mids per slice (one block scan)
constexpr uint32_t kPerThread = 4;          // consecutive probes per thread per round
constexpr uint32_t kRound = kThreads * kPerThread;
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

// gen and abort share one 8-byte word, so a waiting CTA reads both with one load.
struct __align__(8) Barrier {
    unsigned gen, abort, count, error;
};

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

enum : unsigned { ERR_NONE = 0, ERR_TIMEOUT = 1, ERR_OVERFLOW = 2 };

// All `nblocks` CTAs of a cooperative grid meet here.  The wait is bounded by
// `wait_ns` of wall time; when it expires the CTA records ERR_TIMEOUT, raises
// `abort` and returns false, and every other waiting CTA returns false too.
// Thread 0 reads the generation before the block has synchronised: it cannot
// advance until this CTA has arrived, so the read overlaps the CTA's last work.
__device__ inline bool grid_barrier(Barrier *b, unsigned nblocks, unsigned long long wait_ns) {
    __shared__ int s_ok;
    const unsigned long long *word = reinterpret_cast<const unsigned long long *>(&b->gen);
    unsigned gen = 0;
    if (threadIdx.x == 0) gen = ld_acquire(&b->gen);
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        unsigned arrived = atomicAdd(&b->count, 1u) + 1;
        if (arrived == nblocks) {
            b->count = 0;
            __threadfence();
            st_release(&b->gen, gen + 1);
            if (ld_acquire(&b->abort)) ok = 0;
        } else {
            unsigned long long t0 = 0;
            unsigned sleep = 32;
            for (;;) {
                const unsigned long long w = ld_acquire64(word);  // (abort << 32) | gen
                if ((unsigned)(w >> 32)) { ok = 0; break; }
                if ((unsigned)w != gen) break;
                const unsigned long long t = global_ns();
                if (!t0) t0 = t;
                else if (t - t0 > wait_ns) {
                    atomicCAS(&b->error, 0u, (unsigned)ERR_TIMEOUT);
                    atomicExch(&b->abort, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(sleep);
                if (sleep < 128) sleep <<= 1;
            }
        }
        __threadfence();
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
    // decrement count per entry (peeling); arow / aslot list the row in order
    // with each entry's hash slot
    uint32_t hkey[kHashSlots];
    uint32_t hval[kHashSlots];
    uint32_t hdec[kHashSlots];
    uint32_t arow[kHashMaxDeg];
    uint16_t aslot[kHashMaxDeg];
    // one slice of at most kSliceMids pivot slots
    uint32_t mid_eid[kSliceMids];
    uint32_t mid_base[kSliceMids];   // forward: mid's row start; reverse: its hub table
    uint32_t mid_mask[kSliceMids];   // 0: forward (walk mid's row); else reverse (hub mask)
    uint32_t mid_j0[kSliceMids];     // first position walked in the row
    uint32_t pre[kSliceMids + 1];    // prefix of the positions walked per slot
    uint32_t slot_dec[kSliceMids];
    uint8_t pm_curr[kSliceMids];
    uint32_t cached_anc, cached_size;  // staged anchor; size 0: use its hub table
    uint32_t cached_deg;               // length of arow
    uint32_t cached_epoch;             // row-compaction epoch the anchor was staged in
    uint32_t gbase, gmask;             // hub table of the staged anchor
    uint32_t s_lo, s_hi;
    // cycle counters of this CTA's thread 0 (see prof_mark)
    unsigned long long prof_t, prof[8];
    unsigned long long walked;         // row positions walked (forward + reverse)
    typename cub::BlockScan<uint32_t, kThreads>::TempStorage scan;
};

constexpr uint16_t kRevHit = 0x8000;

// Per-CTA time accounting: thread 0 charges the SM cycles since the previous
// mark to counter k.  Marks sit right after block-wide synchronisation, so
// the counters split the CTA's time between the steps of the walk.
enum { PF_TASK = 0, PF_STAGE = 1, PF_SLICE = 2, PF_PROBE = 3, PF_HITS = 4, PF_FLUSH = 5,
       PF_BARRIER = 6, PF_OTHER = 7 };
__device__ __forceinline__ void prof_mark(Walk &w, int k) {
    if (threadIdx.x == 0) {
        const unsigned long long t = clock64();
        w.prof[k] += t - w.prof_t;
        w.prof_t = t;
    }
}

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
        w.cached_epoch = 0;
        for (int k = 0; k < 8; k++) w.prof[k] = 0;
        w.walked = 0;
        w.prof_t = clock64();
    }
    __syncthreads();
}

// Stage anc's live row as a shared-memory hash vertex -> edge id (rows
// longer than kHashMaxDeg use their global hub table instead).  `epoch`
// counts row compactions: a staged row is reused only within one epoch, so
// every CTA walks the same anchor row (the split of a slot's work between
// tasks depends on its length).  Block-uniform; the caller has synchronised
// since the last lookup.
__device__ inline void walk_stage(const Rows &r, Walk &w, uint32_t anc, uint32_t epoch) {
    if (w.cached_anc == anc && w.cached_epoch == epoch) {
        __syncthreads();
        return;
    }
    const uint32_t d = r.deg[anc], b = r.off[anc];
    for (uint32_t t = threadIdx.x; t < w.cached_size; t += blockDim.x) w.hkey[t] = kEmpty;
    __syncthreads();
    uint32_t size = 0;
    if (d <= kHashMaxDeg) {
        size = 64;
        while (size < 2 * d) size <<= 1;
        const uint32_t mask = size - 1;
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
            w.arow[j] = y;
            w.aslot[j] = (uint16_t)h;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        w.cached_anc = anc;
        w.cached_epoch = epoch;
        w.cached_size = size;
        w.gbase = size ? 0 : r.hub_base[anc];
        w.gmask = size ? 0 : r.hub_mask[anc];
        w.cached_deg = d;
    }
    __syncthreads();
}

// Edge id (x, y) from x's hub table (base, mask), or kEmpty.
__device__ __forceinline__ uint32_t hub_lookup(const uint2 *pool, uint32_t base, uint32_t mask, uint32_t y) {
    // buckets of 4 (key, edge id) pairs, 32 bytes: one sector per probe
    const uint4 *tab = reinterpret_cast<const uint4 *>(pool + base);
    uint32_t b = hash_slot(y, mask) >> 2;
    const uint32_t bmask = mask >> 2;
    for (uint32_t probe = 0; probe <= bmask; probe++) {
        const uint4 q0 = tab[2 * b], q1 = tab[2 * b + 1];
        if (q0.x == y) return q0.y;
        if (q0.z == y) return q0.w;
        if (q1.x == y) return q1.y;
        if (q1.z == y) return q1.w;
        if (q0.x == kEmpty || q0.z == kEmpty || q1.x == kEmpty || q1.z == kEmpty) return kEmpty;
        b = (b + 1) & bmask;
    }
    return kEmpty;
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
    return hub_lookup(r.hub_pool, w.gbase, w.gmask, y);
}

__device__ __forceinline__ uint32_t walk_anchor_edge(const Walk &w, uint32_t a) {
    return w.cached_size ? w.hval[a] : a;
}

// Build the hub tables (one CTA per row longer than kHubMinDeg).
__device__ inline void hub_build(const Rows &r, uint32_t n, uint2 *pool) {
    for (uint32_t x = blockIdx.x; x < n; x += gridDim.x) {
        const uint32_t mask = r.hub_mask[x];
        if (!mask) continue;
        const uint32_t b = r.off[x], d = r.deg[x], base = r.hub_base[x];
        for (uint32_t j = threadIdx.x; j < d; j += blockDim.x) {
            const uint32_t y = r.nbr[b + j], e = r.eid[b + j];
            // linear probing from the start of the key's 4-slot bucket (see hub_lookup)
            uint32_t h = hash_slot(y, mask) & ~3u;
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
// over the share [f0, f1) of piv's row (anc is staged here).  The shares are
// cut in the plain probe space of the row -- its mids' rows laid end to end:
// rowpre[pb + s] is the exclusive prefix of the degrees of the row's mids (as
// of the last row compaction) and `total` the row sum -- so slot s owns
// [rowpre[pb+s], rowpre[pb+s+1]) and a share covers parts of whole slots.
//
// Each (mid, anc) pair is intersected from the shorter side: forward, mid's
// row is walked and each y looked up in anc's staged hash (or hub table);
// reverse (mid has a hub table and a longer row than anc), anc's row is
// walked and each y looked up in mid's hub table.  A slot's part of the share
// maps onto the walked row proportionally, so the shares of a slot partition
// that row exactly.
//
// Slices of at most kSliceMids pivot slots are loaded into shared memory;
// prep_slot(k, e_pm) runs once per slot and says whether to walk its mid
// (the walk itself skips mid == anc).  Each warp then walks stretches of
// 32 * kPerThread positions (kPerThread consecutive ones per lane) on its own
// and hands every hit -- y != piv adjacent to both mid and anc -- to on_hit
// right away, in two steps so that the memory traffic of a lane's hits
// overlaps: on_hit.load(state, k, e_my, a) (loads only) for all of them,
// on_hit.apply(state) for each, then on_hit.settle(state) for each; after
// each stretch the whole warp calls on_hit.stretch_done(), and on_hit.stop()
// (the same answer across a warp, and across the block between slices) ends
// the walk early when it returns true.  k =
// slice slot of mid (| kRevHit for a reverse hit), e_my = the edge id
// (mid, y), a = the anchor's answer for y (walk_lookup's convention: a hash
// slot when anc is staged, else the edge id).  settle acts on the results of
// atomics that apply issued.  slice_done(cl, last) runs
// (block-uniform) after each slice's last hit; last marks the final slice.
template <class PrepSlot, class OnHit, class SliceDone>
__device__ __forceinline__ void walk_range(const Rows &r, const uint32_t *rowpre, Walk &w, uint32_t piv,
                                           uint32_t anc, uint32_t epoch, uint32_t total, uint32_t f0,
                                           uint32_t f1, PrepSlot prep_slot, OnHit &on_hit,
                                           SliceDone slice_done) {
    if (f0 >= f1) return;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t pb = r.off[piv], pd = r.deg[piv];
    const uint32_t *pre = rowpre + pb;
    uint32_t s_lo = 0, s_hi = 0;
    if (warp == 0) s_lo = warp_find_slot(pre, pd, f0);
    else if (warp == 1) s_hi = warp_find_slot(pre, pd, f1 - 1);
    walk_stage(r, w, anc, epoch);  // synchronises the block
    prof_mark(w, PF_STAGE);
    if (warp == 0 && lane == 0) w.s_lo = s_lo;
    if (warp == 1 && lane == 0) w.s_hi = s_hi;
    __syncthreads();
    s_lo = w.s_lo;
    s_hi = w.s_hi;
    const bool staged = w.cached_size != 0;
    // the anchor row walked in reverse: the live row (staged in this epoch)
    const uint32_t ab = r.off[anc], ad = r.deg[anc];
    for (uint32_t c0 = s_lo; c0 <= s_hi; c0 += kSliceMids) {
        const uint32_t cl = min(kSliceMids, s_hi + 1 - c0);
        uint32_t cnt = 0;
        if (threadIdx.x < cl) {
            const uint32_t slot = c0 + threadIdx.x;
            const uint32_t mid = r.nbr[pb + slot];
            const uint32_t e_pm = r.eid[pb + slot];
            const uint32_t p0 = pre[slot];
            const uint32_t p1 = slot + 1 < pd ? pre[slot + 1] : total;
            const uint32_t lo = max(f0, p0), hi = min(f1, p1);
            const uint32_t dk = p1 - p0;
            // mid's hub index and row start travel with the slot's own loads
            // (mid < n always): one round trip instead of three
            const uint32_t hm = r.hub_mask[mid], hb = r.hub_base[mid], mo = r.off[mid];
            bool ok = lo < hi && mid != anc;
            ok = ok && prep_slot(threadIdx.x, e_pm);
            uint32_t mask = 0, base = 0, j0 = 0;
            if (ok) {
                if (hm && ad < dk) {  // reverse: walk anc's row, look up in mid's table
                    mask = hm;
                    base = hb;
                    j0 = (uint32_t)((unsigned long long)(lo - p0) * ad / dk);
                    const uint32_t j1 = (uint32_t)((unsigned long long)(hi - p0) * ad / dk);
                    cnt = j1 - j0;
                } else {
                    base = mo;
                    j0 = lo - p0;
                    cnt = hi - lo;
                }
            }
            w.mid_eid[threadIdx.x] = e_pm;
            w.mid_base[threadIdx.x] = base;
            w.mid_mask[threadIdx.x] = mask;
            w.mid_j0[threadIdx.x] = j0;
        }
        uint32_t excl, tot;
        cub::BlockScan<uint32_t, kThreads>(w.scan).ExclusiveSum(cnt, excl, tot);
        if (threadIdx.x < cl) w.pre[threadIdx.x] = excl;
        if (threadIdx.x == 0) {
            w.pre[cl] = tot;
            w.walked += tot;
        }
        __syncthreads();
        prof_mark(w, PF_SLICE);
        // Warps walk independent stretches of 32 * kPerThread positions
        // (kPerThread consecutive ones per lane) and act on their own hits
        // at once: no block-wide synchronisation until the slice is done.
        for (uint32_t wb = warp * (32 * kPerThread); wb < tot; wb += kRound) {
            if (on_hit.stop()) break;  // warp-uniform
            uint32_t hk[kPerThread], hp[kPerThread], ha[kPerThread];
            uint32_t hitmask = 0, act = 0, rev = 0;
            uint32_t jp[kPerThread], yv[kPerThread], ev[kPerThread];
            const uint32_t f = wb + lane * kPerThread;
            if (f < tot) {
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
                    hk[p] = jp[p] = 0;
                    if (ff < tot) {
                        while (w.pre[k + 1] <= ff) k++;
                        hk[p] = k;
                        jp[p] = w.mid_j0[k] + (ff - w.pre[k]);
                        act |= 1u << p;
                        if (w.mid_mask[k]) rev |= 1u << p;
                    }
                }
            }
#pragma unroll
            for (uint32_t p = 0; p < kPerThread; p++) {
                yv[p] = piv;
                ev[p] = 0;
                if (act & (1u << p)) {
                    const uint32_t j = jp[p];
                    if (!(rev & (1u << p))) {
                        const uint32_t pos = w.mid_base[hk[p]] + j;
                        yv[p] = r.nbr[pos];
                        ev[p] = r.eid[pos];  // loaded with y: no round trip later
                    } else if (staged) {
                        yv[p] = w.arow[j];
                        ev[p] = w.aslot[j];
                    } else {
                        yv[p] = r.nbr[ab + j];
                        ev[p] = r.eid[ab + j];
                    }
                }
            }
#pragma unroll
            for (uint32_t p = 0; p < kPerThread; p++) {
                hp[p] = ha[p] = 0;
                if (yv[p] == piv) continue;  // inactive positions carry piv
                if (!(rev & (1u << p))) {
                    // forward: y in mid's row, looked up in the anchor
                    const uint32_t a = walk_lookup(r, w, yv[p]);
                    if (a != kEmpty) {
                        hp[p] = ev[p];
                        ha[p] = a;
                        hitmask |= 1u << p;
                    }
                } else {
                    // reverse: y in the anchor's row, looked up in mid's hub table
                    const uint32_t e_my = hub_lookup(r.hub_pool, w.mid_base[hk[p]], w.mid_mask[hk[p]], yv[p]);
                    if (e_my != kEmpty) {
                        hk[p] |= kRevHit;
                        hp[p] = e_my;
                        ha[p] = ev[p];
                        hitmask |= 1u << p;
                    }
                }
            }
            // this lane's hits: all loads first, then the actions
            typename OnHit::State hs[kPerThread];
#pragma unroll
            for (uint32_t p = 0; p < kPerThread; p++)
                if (hitmask & (1u << p)) on_hit.load(hs[p], hk[p], hp[p], ha[p]);
#pragma unroll
            for (uint32_t p = 0; p < kPerThread; p++)
                if (hitmask & (1u << p)) on_hit.apply(hs[p]);
#pragma unroll
            for (uint32_t p = 0; p < kPerThread; p++)
                if (hitmask & (1u << p)) on_hit.settle(hs[p]);
            on_hit.stretch_done();  // the whole warp
        }
        __syncthreads();
        prof_mark(w, PF_PROBE);
        slice_done(cl, c0 + kSliceMids > s_hi);
        __syncthreads();
        prof_mark(w, PF_FLUSH);
        if (on_hit.stop()) break;  // block-uniform: nothing changes it after the syncs
    }
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
