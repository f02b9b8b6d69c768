// bt_device.cuh -- device building blocks shared by the peeling (msp) and
// h-index (hidx) kernels: the bounded grid barrier, the shared-memory row hash
// and the flattened butterfly walk of one edge.
#pragma once

#include <cub/block/block_scan.cuh>

#include <cstdint>

namespace bt {

constexpr int kThreads = 512;
constexpr int kHashSlots = 8192;            // shared-memory hash capacity (slots)
constexpr uint32_t kHashMaxDeg = kHashSlots / 2;
constexpr uint32_t kSliceMids = kThreads;   // mids per slice (one block scan)
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
};

// ---------------------------------------------------------------------------
// shared-memory state of one CTA
// ---------------------------------------------------------------------------

struct Walk {
    uint32_t hkey[kHashSlots];
    uint32_t hval[kHashSlots];
    uint32_t mid_eid[kSliceMids];
    uint32_t mid_base[kSliceMids];
    uint32_t pre[kSliceMids + 1];
    uint32_t cached_anc, cached_size;
    typename cub::BlockScan<uint32_t, kThreads>::TempStorage scan;
};

__device__ __forceinline__ uint32_t hash_slot(uint32_t y, uint32_t mask) {
    return (y * 0x9E3779B1u) & mask;
}

__device__ inline void walk_init(Walk &w) {
    for (uint32_t t = threadIdx.x; t < kHashSlots; t += blockDim.x) w.hkey[t] = kEmpty;
    if (threadIdx.x == 0) {
        w.cached_anc = kEmpty;
        w.cached_size = 0;
    }
    __syncthreads();
}

// Stage anc's live row as a hash vertex -> edge id.  Rows only ever lose
// processed edges, so a table built earlier for the same vertex stays a valid
// superset (callers check every edge's state).  Rows longer than kHashMaxDeg
// are not staged; lookups then binary-search the row (rows are sorted).
__device__ inline void walk_stage(const Rows &r, Walk &w, uint32_t anc) {
    if (w.cached_anc == anc) return;
    const uint32_t d = r.deg[anc];
    __syncthreads();
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
    }
    __syncthreads();
}

// edge id of (anc, y) if y is a neighbour of the staged vertex, else kEmpty
__device__ __forceinline__ uint32_t walk_lookup(const Rows &r, const Walk &w, uint32_t anc_b,
                                                uint32_t anc_d, uint32_t y) {
    const uint32_t size = w.cached_size;
    if (size) {
        const uint32_t mask = size - 1;
        uint32_t h = hash_slot(y, mask);
        for (uint32_t probe = 0; probe < size; probe++) {
            const uint32_t k = w.hkey[h];
            if (k == y) return w.hval[h];
            if (k == kEmpty) return kEmpty;
            h = (h + 1) & mask;
        }
        return kEmpty;
    }
    uint32_t lo = 0, hi = anc_d;
    const uint32_t *row = r.nbr + anc_b;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t v = row[mid];
        if (v == y) return r.eid[anc_b + mid];
        if (v < y) lo = mid + 1;
        else hi = mid;
    }
    return kEmpty;
}

// Walk the butterflies of one edge between pivot `piv` and anchor `anc`
// (anc already staged): for every mid in piv's row slots [s0, s1) other than
// anc, and every y in mid's row other than piv that is also in anc's row.
// `skip_mid(e_pm)` filters mids by the (piv, mid) edge.  `visit` is called by
// every lane of every warp in a loop of uniform trip count with
// (active, valid, e_pm, e_my, e_ay): active = the lane probed a slot, valid =
// y is a common neighbour; the edges are (piv,mid), (mid,y), (anc,y).
template <class SkipMid, class Visit>
__device__ inline void walk_edge(const Rows &r, Walk &w, uint32_t piv, uint32_t anc, uint32_t s0,
                                 uint32_t s1, SkipMid skip_mid, Visit visit) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t anc_b = r.off[anc], anc_d = r.deg[anc];
    const uint32_t pb = r.off[piv];
    for (uint32_t c0 = s0; c0 < s1; c0 += kSliceMids) {
        const uint32_t cl = min(kSliceMids, s1 - c0);
        uint32_t dm = 0;
        if (threadIdx.x < cl) {
            const uint32_t mid = r.nbr[pb + c0 + threadIdx.x];
            const uint32_t e_pm = r.eid[pb + c0 + threadIdx.x];
            if (mid != anc && !skip_mid(e_pm)) dm = r.deg[mid];
            w.mid_eid[threadIdx.x] = e_pm;
            w.mid_base[threadIdx.x] = r.off[mid];
        }
        uint32_t excl, tot;
        cub::BlockScan<uint32_t, kThreads>(w.scan).ExclusiveSum(dm, excl, tot);
        if (threadIdx.x < cl) w.pre[threadIdx.x] = excl;
        if (threadIdx.x == 0) w.pre[cl] = tot;
        __syncthreads();
        const uint32_t wbase = (threadIdx.x >> 5) * 32;
        for (uint32_t f0 = wbase; f0 < tot; f0 += kThreads) {
            const uint32_t f = f0 + lane;
            const bool active = f < tot;
            bool valid = false;
            uint32_t e_pm = 0, e_my = 0, e_ay = kEmpty;
            if (f < tot) {
                uint32_t lo = 0, hi = cl;
                while (hi - lo > 1) {
                    const uint32_t md = (lo + hi) >> 1;
                    if (w.pre[md] <= f) lo = md;
                    else hi = md;
                }
                const uint32_t mb = w.mid_base[lo];
                const uint32_t j = f - w.pre[lo];
                const uint32_t y = r.nbr[mb + j];
                if (y != piv) {
                    e_ay = walk_lookup(r, w, anc_b, anc_d, y);
                    if (e_ay != kEmpty) {
                        valid = true;
                        e_pm = w.mid_eid[lo];
                        e_my = r.eid[mb + j];
                    }
                }
            }
            visit(active, valid, e_pm, e_my, e_ay);
        }
        __syncthreads();
    }
}

}  // namespace bt
