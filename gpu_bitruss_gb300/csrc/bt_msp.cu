// bt_msp.cu -- multi-stage bitruss peeling (GBiD, the reference's "msp").
//
// Semantics (bit-exact with the reference, src/bitruss/bitruss_msp.cu:440-583
// and src/bitruss/cpu_bitruss.cpp:563-624):
//  * edges with support 0 are processed first (count_es_zero, :38-65);
//  * level L: the frontier is every unprocessed edge with support == L
//    (scan_sub_kernel, :77-93); levels with an empty frontier change nothing
//    and are skipped here;
//  * a sub-round peels the whole frontier: for each frontier edge uv and each
//    butterfly (u,v,w,x) whose three other edges wv, wx, ux are unprocessed,
//    the peel rule (peel_one/two/three_edge, :126-184) decides which of them
//    lose one support; a decrement that takes an edge from L+1 to L puts it
//    in the next frontier and supports are clamped at L (update_edge_support,
//    :110-123);
//  * the frontier is then marked processed and the next frontier becomes the
//    frontier of a new sub-round at the same level (:516-534);
//  * the result is each edge's support when it was processed.
// The order of decrements inside a sub-round does not change the result
// (clamping makes the final value max(L, s - d)), so the GPU may apply them in
// any order and aggregate them.
//
// GB300 design: one cooperative persistent kernel runs the whole level /
// sub-round loop on the device (no host round trip per sub-round; the
// reference pays 3 syncs and ~9m bytes of copies per sub-round, :527-533).
// Phases are separated by a grid barrier whose waits are bounded by a time
// limit (an expired wait sets an error and the kernel returns).
//  * Frontier discovery uses two support buckets: "near" holds the unprocessed
//    edges with support < hi, "far" the rest.  A level scans only the near
//    list; when it runs dry the far list is split again.  A decrement that
//    crosses hi appends the edge to near.
//  * A peeled edge is walked from the endpoint whose two-hop neighbourhood is
//    smaller (both directions visit the same butterflies and name the four
//    edges the same way).  Its work is split into CTA tasks over slices of the
//    walked row; a task stages the other endpoint's row in a shared-memory
//    hash (vertex -> edge id) and probes every neighbour list of the slice
//    against it, with the slice's rows flattened so all threads stay busy.
//  * Processed edges are dropped from the rows (device-side compaction) with
//    the reference's trigger (:537-549), which only changes work, not results.
#include <cstdlib>

#include "bt_device.cuh"
#include "bt_internal.h"

namespace {

using bt::kEmpty;
using bt::kSliceMids;
using bt::kThreads;
constexpr uint32_t kMinGrain = 512;         // probes per task, at least
constexpr uint32_t kTasksPerCta = 2;        // target tasks per CTA per sub-round

enum : uint8_t { ST_LIVE = 0, ST_CURR = 1, ST_DONE = 2 };

struct MspState {
    bt::Barrier bar;
    // control
    unsigned long long level, hi, delta;
    unsigned long long min_sup, far_min;
    long long edge_num;            // unprocessed edges
    unsigned long long live_at_compress;
    unsigned long long last_level; // last level with a non-empty frontier
    uint32_t len[2];               // frontier lists: len[par] = current, len[par^1] = next
    uint32_t near_len, near2_len, far_len, far2_len;
    uint32_t task_total, task_next, done;
    unsigned long long ph_ns[4];   // CTA 0's time in: level transitions, peel, finalize
    // statistics
    unsigned long long subrounds, compressions, tasks, levels_seen, rebuilds;
    // work counters (algorithmic bytes): pivot slots walked, neighbour slots
    // probed, anchor slots of the peeled edges, butterflies found, decrements
    unsigned long long w_mids, w_probes, w_anchor, w_hits, w_decs;
};

struct Work {
    unsigned long long mids = 0, probes = 0, hits = 0, decs = 0;
};

struct MspArgs {
    MspState *s;
    uint32_t n, nblocks, exact;
    uint64_t m;
    unsigned long long wait_ns;
    const uint32_t *off;
    const uint2 *ends;
    uint32_t *deg, *nbr, *eid;      // live rows (compacted in place)
    uint32_t *two_hop;              // per vertex: sum of live neighbour degrees (row probe total)
    uint32_t *rowpre;               // per slot: prefix of the row's neighbour degrees
    unsigned long long *sup;        // working supports
    uint8_t *st;
    uint32_t *list_a, *list_b;      // curr / next (swap by parity)
    uint32_t *near_a, *near_b, *far_a, *far_b;
    uint32_t *pl_piv, *pl_anc, *pl_grain, *task_start;  // plan of the frontier
    const uint32_t *hub_base, *hub_mask;
    const uint2 *hub_pool;
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool barrier(const MspArgs &a) {
    return bt::grid_barrier(&a.s->bar, a.nblocks, a.wait_ns);
}

__device__ __forceinline__ unsigned long long warp_min(unsigned long long v) {
    for (int o = 16; o; o >>= 1) {
        unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t < v ? t : v;
    }
    return v;
}

// subtract k from sup[e]; push to the next frontier when it crosses L+1 -> L
// and to the near bucket when it crosses hi
__device__ __forceinline__ void dec_edge(const MspArgs &a, uint32_t *next, uint32_t *next_len,
                                         uint32_t *near_list, unsigned long long L,
                                         unsigned long long hi, uint32_t e, uint32_t k) {
    unsigned long long old = atomicAdd(a.sup + e, (unsigned long long)(-(long long)k));
    unsigned long long nw = old - k;
    if (old > L && nw <= L) next[atomicAdd(next_len, 1u)] = e;
    if (old >= hi && nw < hi) near_list[atomicAdd(&a.s->near_len, 1u)] = e;
}

// the peel rule for one butterfly seen from frontier edge uv; returns a 3-bit
// mask of the edges to decrement: bit0 wv, bit1 wx, bit2 ux
__device__ __forceinline__ uint32_t peel_rule(uint32_t uv, uint32_t wv, uint32_t wx, uint32_t ux,
                                              bool cwv, bool cwx, bool cux, uint32_t exact) {
    const bool pwv = !cwv, pwx = !cwx, pux = !cux;
    const int cnt = (int)pwv + (int)pwx + (int)pux;
    uint32_t d = 0;
    if (cnt == 3) {
        d = 7;  // peel_three_edge, bitruss_msp.cu:178-184
    } else if (cnt == 2) {  // peel_two_edge, :148-175
        if (pwv && pwx && uv < ux) d = 3;
        if (pwv && pux && uv < wx) d = 5;
        if (pwx && pux && uv < wv) d = 6;
    } else if (cnt == 1) {  // peel_one_edge, :126-145
        if (!exact) {
            if (pwx && uv < ux && ux < wv) d = 2;
            if (pwv && uv < ux && ux < wx) d = 1;
            if (pux && uv < wv && wv < wx) d = 4;
        } else {  // decrement the survivor once: by the smallest frontier edge
            if (pwx && uv < ux && uv < wv) d = 2;
            if (pwv && uv < ux && uv < wx) d = 1;
            if (pux && uv < wv && uv < wx) d = 4;
        }
    }
    return d;
}

// ---------------------------------------------------------------------------
// phases
// ---------------------------------------------------------------------------

struct Smem {
    bt::Walk walk;
    uint32_t task, idx, k;
    uint32_t running;
    unsigned long long total;
};

// Plan the frontier (one CTA): orientation of every edge, then tasks of equal
// probe counts.  The grain adapts to the sub-round's total work so that all
// CTAs get tasks; an edge's grain is at least twice its anchor row (each task
// stages that row).
__device__ void plan_frontier(const MspArgs &a, Smem &sm, const uint32_t *curr, uint32_t len) {
    if (threadIdx.x == 0) {
        sm.running = 0;
        sm.total = 0;
    }
    __syncthreads();
    unsigned long long mine = 0;
    for (uint32_t i = threadIdx.x; i < len; i += kThreads) {
        const uint32_t e = curr[i];
        const uint2 uv = a.ends[e];
        const uint32_t cu = a.two_hop[uv.x], cv = a.two_hop[uv.y];
        const uint32_t piv = cv <= cu ? uv.y : uv.x, anc = cv <= cu ? uv.x : uv.y;
        a.pl_piv[i] = piv;
        a.pl_anc[i] = anc;
        mine += cv <= cu ? cv : cu;
    }
    for (int o = 16; o; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&sm.total, mine);
    __syncthreads();
    unsigned long long g = sm.total / ((unsigned long long)kTasksPerCta * a.nblocks);
    if (g < kMinGrain) g = kMinGrain;
    if (g > (1u << 30)) g = 1u << 30;
    unsigned long long anchor = 0;
    for (uint32_t base = 0; base < len; base += kThreads) {
        const uint32_t i = base + threadIdx.x;
        uint32_t nt = 0;
        if (i < len) {
            const uint32_t piv = a.pl_piv[i], anc = a.pl_anc[i];
            const uint32_t work = a.two_hop[piv];
            const uint32_t da = a.deg[anc];
            unsigned long long gi = g > 2ull * da ? g : 2ull * da;
            if (gi > (1u << 30)) gi = 1u << 30;
            nt = (uint32_t)((work + gi - 1) / gi);
            a.pl_grain[i] = (uint32_t)gi;
            anchor += da;
        }
        uint32_t excl, tot;
        cub::BlockScan<uint32_t, kThreads>(sm.walk.scan).ExclusiveSum(nt, excl, tot);
        if (i < len) a.task_start[i] = sm.running + excl;
        __syncthreads();
        if (threadIdx.x == 0) sm.running += tot;
        __syncthreads();
    }
    for (int o = 16; o; o >>= 1) anchor += __shfl_xor_sync(0xffffffffu, anchor, o);
    if ((threadIdx.x & 31) == 0 && anchor) atomicAdd(&a.s->w_anchor, anchor);
    if (threadIdx.x == 0) {
        a.task_start[len] = sm.running;
        a.s->task_total = sm.running;
        a.s->task_next = 0;
    }
}

// Peel all tasks of the current sub-round.
__device__ void peel_tasks(const MspArgs &a, Smem &sm, const uint32_t *curr, uint32_t curr_len,
                           uint32_t *next, uint32_t *next_len, uint32_t *near_list,
                           unsigned long long L, unsigned long long hi, Work &wk) {
    const bt::Rows rows{a.off, a.deg, a.nbr, a.eid, a.hub_base, a.hub_mask, a.hub_pool};
    const uint8_t *st = a.st;
    const uint32_t ntasks = a.s->task_total;
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        // frontier edge of task t: last i with task_start[i] <= t
        if (threadIdx.x < 32) {
            const uint32_t i = bt::warp_find_slot(a.task_start, curr_len, t);
            if (threadIdx.x == 0) {
                sm.idx = i;
                sm.k = t - a.task_start[i];
            }
        }
        __syncthreads();
        const uint32_t i = sm.idx, k = sm.k;
        const uint32_t uv = curr[i];
        const uint32_t piv = a.pl_piv[i], anc = a.pl_anc[i], gi = a.pl_grain[i];
        const bool piv_is_v = (piv == a.ends[uv].y);
        const uint32_t total = a.two_hop[piv];
        const uint32_t f0 = k * gi;
        const uint32_t f1 = total - f0 < gi ? total : f0 + gi;
        const uint32_t exact = a.exact;
        if (threadIdx.x == 0) wk.mids++;
        bt::Walk &w = sm.walk;
        bt::walk_range(
            rows, a.rowpre, w, piv, anc, total, f0, f1,
            [&](uint32_t k, uint32_t e_pm) {
                const uint8_t sp = st[e_pm];
                w.pm_curr[k] = sp == ST_CURR;
                return sp != ST_DONE;
            },
            [&](uint32_t k, uint32_t pos, uint32_t ah) {
                const uint32_t e_pm = w.mid_eid[k];
                const uint32_t e_ay = bt::walk_anchor_edge(w, ah);
                const uint32_t e_my = a.eid[pos];
                const uint8_t s_ay = st[e_ay], s_my = st[e_my];
                wk.hits++;
                if (s_ay == ST_DONE || s_my == ST_DONE) return;
                const bool c_pm = w.pm_curr[k], c_my = s_my == ST_CURR, c_ay = s_ay == ST_CURR;
                // name the edges as the reference does: w on u's side, x on v's
                uint32_t wv, ux;
                bool cwv, cux;
                if (piv_is_v) { wv = e_pm; ux = e_ay; cwv = c_pm; cux = c_ay; }
                else { wv = e_ay; ux = e_pm; cwv = c_ay; cux = c_pm; }
                const uint32_t d = peel_rule(uv, wv, e_my, ux, cwv, c_my, cux, exact);
                if (!d) return;
                const bool d_wv = d & 1, d_wx = d & 2, d_ux = d & 4;
                const bool dec_pm = piv_is_v ? d_wv : d_ux;
                const bool dec_ay = piv_is_v ? d_ux : d_wv;
                wk.decs += (uint32_t)dec_pm + (uint32_t)d_wx + (uint32_t)dec_ay;
                if (dec_pm) atomicAdd(&w.slot_dec[k], 1u);
                if (d_wx) dec_edge(a, next, next_len, near_list, L, hi, e_my, 1);
                if (dec_ay) {
                    if (w.cached_size) atomicAdd(&w.hdec[ah], 1u);
                    else dec_edge(a, next, next_len, near_list, L, hi, e_ay, 1);
                }
            },
            [&](uint32_t cl) {
                __syncthreads();
                if (threadIdx.x < cl) {
                    const uint32_t c = w.slot_dec[threadIdx.x];
                    if (c) {
                        w.slot_dec[threadIdx.x] = 0;
                        dec_edge(a, next, next_len, near_list, L, hi, w.mid_eid[threadIdx.x], c);
                    }
                }
            });
        // flush the anchor-side decrements of this task
        if (w.cached_size) {
            for (uint32_t h = threadIdx.x; h < w.cached_size; h += kThreads) {
                const uint32_t c = w.hdec[h];
                if (c) {
                    w.hdec[h] = 0;
                    dec_edge(a, next, next_len, near_list, L, hi, w.hval[h], c);
                }
            }
        }
        if (threadIdx.x == 0) wk.probes += f1 - f0;
        __syncthreads();
    }
    __syncthreads();
}

// Minimum support over the live entries of `list` (grid-wide atomicMin).
__device__ void list_min(const MspArgs &a, Smem &sm, const uint32_t *list, uint32_t len,
                         unsigned long long *out) {
    unsigned long long v = ~0ull;
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gsz = gridDim.x * blockDim.x;
    for (uint32_t i = gtid; i < len; i += gsz) {
        const uint32_t e = list[i];
        if (a.st[e] != ST_DONE) {
            const unsigned long long s = a.sup[e];
            v = s < v ? s : v;
        }
    }
    v = warp_min(v);
    if ((threadIdx.x & 31) == 0 && v != ~0ull) atomicMin(out, v);
}

// Drop processed edges from every row; one warp per vertex, in place.
__device__ void compress_rows(const MspArgs &a) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t x = warp; x < a.n; x += nw) {
        const uint32_t b = a.off[x], d = a.deg[x];
        uint32_t w = 0;
        for (uint32_t j0 = 0; j0 < d; j0 += 32) {
            const uint32_t j = j0 + lane;
            uint32_t y = 0, e = 0;
            bool keep = false;
            if (j < d) {
                y = a.nbr[b + j];
                e = a.eid[b + j];
                keep = a.st[e] != ST_DONE;
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, keep);
            __syncwarp();
            if (keep) {
                const uint32_t pos = w + __popc(bal & ((1u << lane) - 1));
                a.nbr[b + pos] = y;
                a.eid[b + pos] = e;
            }
            w += __popc(bal);
            __syncwarp();
        }
        if (lane == 0) a.deg[x] = w;
    }
}

__device__ void compute_two_hop(const MspArgs &a) {
    const bt::Rows rows{a.off, a.deg, a.nbr, a.eid, a.hub_base, a.hub_mask, a.hub_pool};
    bt::row_prefix(rows, a.n, a.rowpre, a.two_hop);
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kThreads, 2) k_msp(MspArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
    MspState *s = a.s;
    bt::walk_init(sm.walk);
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gsz = gridDim.x * blockDim.x;
    constexpr uint32_t kNearTarget = 1u << 16;
    uint32_t *lists[2] = {a.list_a, a.list_b};
    Work wk;
    uint32_t par = 0;  // lists[par] is the frontier, lists[par ^ 1] the next frontier
    if (gtid == 0) s->min_sup = ~0ull;
    if (!barrier(a)) return;
    unsigned long long t_mark = gtid == 0 ? bt::global_ns() : 0;
    auto lap = [&](int k) {
        if (gtid == 0) {
            const unsigned long long t = bt::global_ns();
            s->ph_ns[k] += t - t_mark;
            t_mark = t;
        }
    };

    for (;;) {
        // ------------------------------------------------ level transition
        if (s->len[par] == 0) {
            // T1: min over the near bucket (min_sup was reset before the barrier)
            list_min(a, sm, a.near_a, s->near_len, &s->min_sup);
            if (!barrier(a)) return;
            if (s->min_sup == ~0ull) {
                // T2: near is dry -> split the far bucket
                list_min(a, sm, a.far_a, s->far_len, &s->far_min);
                if (!barrier(a)) return;
                const unsigned long long lo = s->far_min;
                if (lo == ~0ull) break;  // nothing left
                const unsigned long long hi = lo + s->delta;
                for (uint32_t i = gtid; i < s->far_len; i += gsz) {
                    const uint32_t e = a.far_a[i];
                    if (a.st[e] == ST_DONE) continue;
                    if (a.sup[e] < hi) a.near_b[atomicAdd(&s->near2_len, 1u)] = e;
                    else a.far_b[atomicAdd(&s->far2_len, 1u)] = e;
                }
                if (!barrier(a)) return;
                {   // every CTA swaps its copies of the bucket pointers
                    uint32_t *t = a.near_a; a.near_a = a.near_b; a.near_b = t;
                    t = a.far_a; a.far_a = a.far_b; a.far_b = t;
                }
                if (gtid == 0) {
                    s->near_len = s->near2_len;
                    s->far_len = s->far2_len;
                    s->near2_len = 0;
                    s->far2_len = 0;
                    s->hi = hi;
                    s->min_sup = lo;
                    s->far_min = ~0ull;
                    s->rebuilds++;
                    if (s->near_len > 4 * kNearTarget && s->delta > 1) s->delta >>= 1;
                    else if (s->near_len < kNearTarget / 4) s->delta <<= 1;
                }
                if (!barrier(a)) return;
            }
            // T3: frontier = near edges with support == L; compact near
            const unsigned long long L = s->min_sup;
            const uint32_t near_len = s->near_len;
            for (uint32_t i = gtid; i < near_len; i += gsz) {
                const uint32_t e = a.near_a[i];
                if (a.st[e] == ST_DONE) continue;
                if (a.sup[e] == L) {
                    a.st[e] = ST_CURR;
                    lists[par][atomicAdd(&s->len[par], 1u)] = e;
                } else {
                    a.near_b[atomicAdd(&s->near2_len, 1u)] = e;
                }
            }
            // T4: compression (reference trigger, bitruss_msp.cu:537)
            const bool squeeze = (double)s->edge_num <= 0.5 * (double)s->live_at_compress &&
                                 (double)s->live_at_compress >= 0.1 * (double)a.m;
            if (!barrier(a)) return;
            {
                uint32_t *t = a.near_a; a.near_a = a.near_b; a.near_b = t;
            }
            if (squeeze) {
                compress_rows(a);
                if (!barrier(a)) return;
                compute_two_hop(a);
                if (!barrier(a)) return;
            }
            // T5: plan the frontier; publish the level
            if (blockIdx.x == 0) plan_frontier(a, sm, lists[par], s->len[par]);
            if (gtid == 0) {
                s->near_len = s->near2_len;
                s->near2_len = 0;
                s->level = L;
                s->last_level = L;
                s->levels_seen++;
                if (squeeze) {
                    s->live_at_compress = (unsigned long long)s->edge_num;
                    s->compressions++;
                }
            }
            if (!barrier(a)) return;
            lap(0);
        }
        // ------------------------------------------------ sub-round
        const unsigned long long L = s->level, hi = s->hi;
        const uint32_t curr_len = s->len[par];
        uint32_t *curr = lists[par], *next = lists[par ^ 1];
        peel_tasks(a, sm, curr, curr_len, next, &s->len[par ^ 1], a.near_a, L, hi, wk);
        if (!barrier(a)) return;
        lap(1);
        // finalize: frontier -> processed, next -> frontier (clamped at L)
        const uint32_t next_len = s->len[par ^ 1];
        for (uint32_t i = gtid; i < curr_len; i += gsz) a.st[curr[i]] = ST_DONE;
        for (uint32_t i = gtid; i < next_len; i += gsz) {
            const uint32_t e = next[i];
            a.st[e] = ST_CURR;
            a.sup[e] = L;
        }
        if (gtid == 0) {
            s->tasks += s->task_total;
            s->edge_num -= curr_len;
            s->subrounds++;
            s->len[par] = 0;      // every CTA holds curr_len in a register
            if (next_len == 0) s->min_sup = ~0ull;
        }
        __syncthreads();
        if (blockIdx.x == 0 && next_len) plan_frontier(a, sm, next, next_len);
        par ^= 1;
        if (!barrier(a)) return;
        lap(2);
    }
    if (gtid == 0) s->done = 1;
    // flush the work counters (one atomic per warp)
    for (int o = 16; o; o >>= 1) {
        wk.mids += __shfl_xor_sync(0xffffffffu, wk.mids, o);
        wk.probes += __shfl_xor_sync(0xffffffffu, wk.probes, o);
        wk.hits += __shfl_xor_sync(0xffffffffu, wk.hits, o);
        wk.decs += __shfl_xor_sync(0xffffffffu, wk.decs, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&s->w_mids, wk.mids);
        atomicAdd(&s->w_probes, wk.probes);
        atomicAdd(&s->w_hits, wk.hits);
        atomicAdd(&s->w_decs, wk.decs);
    }
}

// ---------------------------------------------------------------------------
// set-up kernels
// ---------------------------------------------------------------------------

__global__ void k_msp_init(uint64_t m, const unsigned long long *sup_in, unsigned long long *sup,
                           uint8_t *st, uint32_t *far_list, MspState *s) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long v = sup_in[e];
        sup[e] = v;
        if (v == 0) {
            st[e] = ST_DONE;  // count_es_zero, bitruss_msp.cu:38-50
        } else {
            st[e] = ST_LIVE;
            far_list[atomicAdd(&s->far_len, 1u)] = (uint32_t)e;
        }
    }
}

__global__ void k_two_hop(MspArgs a) { compute_two_hop(a); }

__global__ void k_msp_result(uint64_t m, const unsigned long long *sup, uint32_t *out, MspState *s) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long v = sup[e];
        if (v > 0xffffffffull) atomicCAS(&s->bar.error, 0u, (unsigned)bt::ERR_OVERFLOW);
        out[e] = (uint32_t)v;
    }
}

}  // namespace

static unsigned long long wait_limit_ns() {
    const char *v = getenv("BT_WAIT_LIMIT_MS");
    unsigned long long ms = v ? strtoull(v, nullptr, 10) : 120000ull;
    if (ms == 0) ms = 120000ull;
    return ms * 1000000ull;
}

bt_status dev_msp(bt_ctx *ctx, bool exact, uint32_t *levels) {
    uint64_t dummy = 0;
    BT_TRY(dev_ebfc(ctx, true, &dummy));
    DevGraph &g = ctx->g;
    cudaStream_t st = ctx->stream;
    const uint64_t m = g.m, n = g.n;
    cudaEvent_t e0 = ctx->ev[2], e1 = ctx->ev[3];
    cudaEventRecord(e0, st);

    // working buffers
    struct Buf { void *p = nullptr; };
    std::vector<void *> owned;
    auto alloc = [&](void **p, uint64_t bytes) -> bt_status {
        bt_status r = ctx_alloc(ctx, p, bytes);
        if (r == BT_OK) owned.push_back(*p);
        return r;
    };
    auto release = [&]() {
        for (void *p : owned) ctx_free(ctx, p);
        owned.clear();
    };
    MspArgs a{};
    MspState *s = nullptr;
    const uint64_t mm = m ? m : 1, nn = n ? n : 1;
    bt_status rc = BT_OK;
#define A(p, bytes)                                       \
    do {                                                  \
        rc = alloc((void **)&(p), (bytes));               \
        if (rc != BT_OK) { release(); return rc; }        \
    } while (0)
    A(s, sizeof(MspState));
    A(a.deg, 4 * nn);
    A(a.nbr, 8 * mm);
    A(a.eid, 8 * mm);
    A(a.two_hop, 4 * nn);
    A(a.sup, 8 * mm);
    A(a.st, mm);
    A(a.list_a, 4 * mm);
    A(a.list_b, 4 * mm);
    A(a.near_a, 4 * mm);
    A(a.near_b, 4 * mm);
    A(a.far_a, 4 * mm);
    A(a.far_b, 4 * mm);
    A(a.pl_piv, 4 * mm);
    A(a.pl_anc, 4 * mm);
    A(a.pl_grain, 4 * mm);
    A(a.rowpre, 8 * mm);
    A(a.task_start, 4 * (mm + 1));
#undef A
#define C(x)                                                                  \
    do {                                                                      \
        cudaError_t _e = (x);                                                 \
        if (_e != cudaSuccess) { release(); return bt_cuda_fail(_e, #x, __FILE__, __LINE__); } \
    } while (0)
    C(cudaMemsetAsync(s, 0, sizeof(MspState), st));
    {
        MspState init{};
        init.delta = 1;
        init.hi = 0;
        init.min_sup = ~0ull;
        init.far_min = ~0ull;
        init.live_at_compress = m;
        C(cudaMemcpyAsync(s, &init, sizeof(MspState), cudaMemcpyHostToDevice, st));
        C(cudaStreamSynchronize(st));
    }
    C(cudaMemcpyAsync(a.deg, g.deg0, 4 * n, cudaMemcpyDeviceToDevice, st));
    C(cudaMemcpyAsync(a.nbr, g.nbr0, 8 * m, cudaMemcpyDeviceToDevice, st));
    C(cudaMemcpyAsync(a.eid, g.eid0, 8 * m, cudaMemcpyDeviceToDevice, st));
    a.s = s;
    a.n = g.n;
    a.m = m;
    a.exact = exact ? 1u : 0u;
    a.wait_ns = wait_limit_ns();
    a.off = g.off;
    a.ends = g.ends;
    a.hub_base = g.hub_base;
    a.hub_mask = g.hub_mask;
    a.hub_pool = g.hub_pool;
    const unsigned blk = 256, cap = (unsigned)ctx->sm_count * 8;
    if (m) {
        k_msp_init<<<(unsigned)std::min<uint64_t>((m + blk - 1) / blk, cap), blk, 0, st>>>(
            m, (const unsigned long long *)ctx->sup, a.sup, a.st, a.far_a, s);
        C(cudaGetLastError());
    }
    // edge_num = live edges
    {
        C(cudaStreamSynchronize(st));
        MspState h;
        C(cudaMemcpy(&h, s, sizeof(MspState), cudaMemcpyDeviceToHost));
        h.edge_num = h.far_len;
        C(cudaMemcpy(s, &h, sizeof(MspState), cudaMemcpyHostToDevice));
    }
    if (n) {
        k_two_hop<<<(unsigned)std::min<uint64_t>((n * 32 + blk - 1) / blk, cap), blk, 0, st>>>(a);
        C(cudaGetLastError());
    }
    // cooperative persistent launch
    const size_t smem = sizeof(Smem);
    C(cudaFuncSetAttribute(k_msp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    C(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_msp, kThreads, smem));
    if (per_sm < 1) { release(); return bt_fail(BT_ERR_CUDA, "msp kernel does not fit on an SM"); }
    a.nblocks = (uint32_t)(ctx->sm_count * per_sm);
    if (m) {
        void *params[] = {&a};
        cudaEventRecord(ctx->ev[4], st);
        C(cudaLaunchCooperativeKernel((void *)k_msp, dim3(a.nblocks), dim3(kThreads), params, smem, st));
        C(cudaGetLastError());
        cudaEventRecord(ctx->ev[5], st);
        k_msp_result<<<(unsigned)std::min<uint64_t>((m + blk - 1) / blk, cap), blk, 0, st>>>(
            m, a.sup, ctx->result, s);
        C(cudaGetLastError());
    }
    cudaEventRecord(e1, st);
    MspState h{};
    C(cudaMemcpyAsync(&h, s, sizeof(MspState), cudaMemcpyDeviceToHost, st));
    C(cudaStreamSynchronize(st));
#undef C
    float ms = -1;
    cudaEventElapsedTime(&ms, e0, e1);
    ctx->phase_ms[PH_MSP] = ms;
    ms = -1;
    if (m) cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
    ctx->phase_ms[PH_PEEL] = ms;
    release();
    if (h.bar.error == bt::ERR_TIMEOUT)
        return bt_fail(BT_ERR_TIMEOUT, "msp: a grid barrier wait exceeded its time limit");
    if (h.bar.error == bt::ERR_OVERFLOW)
        return bt_fail(BT_ERR_OVERFLOW, "msp: a bitruss number exceeds uint32");
    if (m && !h.done) return bt_fail(BT_ERR_CUDA, "msp kernel ended without finishing");
    ctx->stats[0] = h.last_level;
    ctx->stats[1] = h.subrounds;
    ctx->stats[2] = h.compressions;
    ctx->stats[3] = h.tasks;
    ctx->stats[5] = h.levels_seen;
    ctx->stats[6] = h.rebuilds;
    ctx->work[0] = h.w_mids;
    ctx->work[1] = h.w_probes;
    ctx->work[2] = h.w_anchor;
    ctx->work[3] = h.w_hits;
    ctx->work[4] = h.w_decs;
    ctx->work[5] = m;
    ctx->work[6] = h.ph_ns[0];
    ctx->work[7] = h.ph_ns[1];
    ctx->work[8] = h.ph_ns[2];
    ctx->last_result = 2;
    if (levels) *levels = (uint32_t)h.last_level;
    return BT_OK;
}
