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
//  * the result is each edge's support when it was processed, i.e. the level
//    at which it joined a frontier.
// The order of decrements inside a sub-round does not change the result, so
// the GPU may apply them in any order and aggregate them.
//
// GB300 design: one cooperative persistent kernel runs the whole level /
// sub-round loop on the device (the reference pays 3 host syncs and ~9m bytes
// of copies per sub-round, :527-533).
//  * Edge state is one stamp per edge: enter[e] = the index of the sub-round
//    whose frontier e joined (0: not yet).  In sub-round r an edge is in the
//    frontier iff enter == r and processed iff 0 < enter < r, so "mark the
//    frontier processed, promote the next frontier" costs nothing: the thread
//    that pushes an edge to the next frontier stamps it r+1 and records its
//    result (L).  A sub-round therefore needs one grid barrier.
//  * Frontier discovery uses two support buckets: "near" holds the live
//    edges with support < hi, "far" the rest.  A level scans only the near
//    list; when it runs dry the far list is split again.  A decrement that
//    crosses hi appends the edge to near.
//  * Every CTA plans a small frontier itself in shared memory (orientation of
//    each edge, tasks of equal probe counts); a large one is planned by CTA 0
//    behind one more barrier.  Tasks are taken from a counter.
//  * A task walks its share of the pivot's mids (bt::walk_range): anchor row
//    in a shared hash or its hub table, each (mid, anchor) pair intersected
//    from the shorter side, hits queued in shared memory and ruled on in a
//    dense pass; decrements of the pivot-side and anchor-side edges are summed
//    in shared memory and flushed once.
//  * Processed edges are dropped from the rows (device-side compaction)
//    whenever the live edges have halved (the reference's trigger, :537-549,
//    without its floor at a tenth of the edges); compaction only changes
//    work, not results.
// Grid barriers are bounded by a time limit; an expired wait sets an error and
// the kernel returns.
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <mutex>
#include <type_traits>

#include "bt_device.cuh"
#include "bt_internal.h"

namespace {

using bt::kEmpty;
using bt::kThreads;
constexpr uint32_t kLocalPlan = kMspLocalPlan;  // largest frontier every CTA may plan itself

struct MspState {
    bt::Barrier bar;
    // control
    unsigned long long hi, delta;
    unsigned long long min_sup, far_min;
    long long edge_num;            // unprocessed edges
    unsigned long long live_at_compress;
    unsigned long long last_level; // last level with a non-empty frontier
    uint32_t len[3];               // frontier list lengths by sub-round index mod 3
    uint32_t task_ctr[3];          // task counters by sub-round index mod 3
    uint32_t near_ctr[2];          // near bucket lengths (selector kept by every CTA)
    uint32_t far_len, far2_len;
    uint32_t task_total, done, overflow;
    unsigned long long ph_ns[4];   // CTA 0's time in: level transitions, sub-rounds
    unsigned long long prof[8];    // SM cycles summed over CTAs, by step (bt::PF_*)
    // statistics
    unsigned long long subrounds, compressions, tasks, levels_seen, rebuilds;
    // work counters (algorithmic bytes): tasks, row positions walked, anchor
    // slots of the peeled edges, butterflies found, decrements
    unsigned long long w_mids, w_probes, w_anchor, w_hits, w_decs;
};

struct Work {
    unsigned long long mids = 0, probes = 0, hits = 0, decs = 0;
};

// Optional per-sub-round trace (BT_MSP_TRACE=<path>): what bounds a sub-round.
struct TraceRow {
    unsigned long long t_ns;        // sub-round duration seen by CTA 0 (plan to barrier exit)
    unsigned long long max_task_ns; // longest task
    unsigned long long walked;      // row positions walked
    uint32_t frontier, tasks;
};

struct MspArgs {
    MspState *s;
    uint32_t n, nblocks, exact;
    uint32_t min_grain, tasks_per_cta, local_plan;  // task schedule (results do not depend on it)
    // row compaction trigger: compact when the live edges fall to cfrac of
    // the live edges at the last compaction, while those were at least
    // cfloor * m (compaction changes work, never results)
    float cfrac, cfloor;
    uint64_t m;
    unsigned long long wait_ns;
    const uint32_t *off;
    const uint2 *ends;
    uint32_t *deg, *nbr, *eid;      // live rows (compacted in place)
    uint32_t *two_hop;              // per vertex: sum of live neighbour degrees (row probe total)
    uint32_t *rowpre;               // per slot: prefix of the row's neighbour degrees
    unsigned long long *sup;        // working supports (64-bit)
    uint32_t *sup32;                // working supports when every support fits 32 bits (else null)
    uint32_t *enter;                // sub-round index at which the edge joined a frontier
    uint32_t *result;               // bitruss number per edge
    uint32_t *list[3];              // frontier lists by sub-round index mod 3
    uint32_t *near_a, *near_b, *far_a, *far_b;
    uint32_t *pl_piv, *pl_anc, *pl_grain, *pl_total, *task_start;  // plan of a large frontier
    const uint32_t *hub_base, *hub_mask;
    const uint2 *hub_pool;
    TraceRow *trace;                // optional, trace_cap rows
    uint32_t trace_cap;
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool is_done(uint32_t en, uint32_t r) { return en != 0 && en < r; }

__device__ __forceinline__ unsigned long long warp_min(unsigned long long v) {
    for (int o = 16; o; o >>= 1) {
        unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t < v ? t : v;
    }
    return v;
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

// One sub-round's view of the state.
struct Round {
    uint32_t r;                     // sub-round index
    unsigned long long L, hi;       // level and near-bucket bound
    uint32_t *next, *next_len;      // next frontier
    uint32_t *near_list, *near_len;
};

// The kernel is compiled twice: N32 = every working support fits 32 bits
// (4-byte supports and atomics), else 64-bit supports.
template <bool N32>
using SupWord = typename std::conditional<N32, uint32_t, unsigned long long>::type;

template <bool N32>
__device__ __forceinline__ unsigned long long sup_of(const MspArgs &a, uint32_t e) {
    if constexpr (N32) return a.sup32[e];
    else return a.sup[e];
}

// Subtract k from sup[e].  The decrement that takes it from above L to L or
// below puts e in the next frontier (stamp r+1, result L): the reference's
// clamp at L (update_edge_support, bitruss_msp.cu:110-123) then only matters
// for the value it is processed with, which is L.  A decrement crossing hi
// appends e to the near bucket.
// A decrement is split in two so that a thread can have several in flight:
// dec_issue sends the atomic and returns the old support (nothing waits for
// it until the value is used), dec_settle acts on the crossings it shows.
template <bool N32>
__device__ __forceinline__ SupWord<N32> dec_issue(const MspArgs &a, uint32_t e, uint32_t k) {
    // supports never fall below 0: a decrement reaches an edge only while it is
    // above the level, and each butterfly decrements an edge at most once
    if constexpr (N32) return atomicSub(a.sup32 + e, k);
    else return atomicAdd(a.sup + e, (unsigned long long)(-(long long)k));
}

__device__ __forceinline__ void dec_settle(const MspArgs &a, const Round &rd, uint32_t e, uint32_t k,
                                           unsigned long long old) {
    const unsigned long long nw = old - k;
    if (old > rd.L && nw <= rd.L) {
        rd.next[atomicAdd(rd.next_len, 1u)] = e;
        a.enter[e] = rd.r + 1;
        a.result[e] = (uint32_t)rd.L;
    }
    if (old >= rd.hi && nw < rd.hi) rd.near_list[atomicAdd(rd.near_len, 1u)] = e;
}

// ---------------------------------------------------------------------------
// shared memory
// ---------------------------------------------------------------------------

struct Smem {
    bt::Walk walk;
    // plan of a small frontier (every CTA computes it)
    uint32_t lp_piv[kLocalPlan];
    uint32_t lp_anc[kLocalPlan];
    uint32_t lp_grain[kLocalPlan];
    uint32_t lp_total[kLocalPlan];
    uint32_t lp_start[kLocalPlan + 1];
    uint32_t task, idx;
    uint32_t running;
    unsigned long long total;
};

__device__ __forceinline__ bool barrier(const MspArgs &a, Smem &sm) {
    bt::prof_mark(sm.walk, bt::PF_OTHER);
    const bool ok = bt::grid_barrier(&a.s->bar, a.nblocks, a.wait_ns);
    bt::prof_mark(sm.walk, bt::PF_BARRIER);
    return ok;
}

// ---------------------------------------------------------------------------
// plan: orientation of every frontier edge and tasks of equal probe counts
// ---------------------------------------------------------------------------
//
// The pivot is the endpoint whose row's probe total (two_hop) is smaller.  The
// grain is the sub-round's total over tasks_per_cta tasks per CTA (tasks are
// taken dynamically, so a few per CTA even out their unequal real costs), at
// least min_grain and, for an anchor staged in shared memory, at least twice
// its row (each task stages that row).
// Writes piv/anc per edge, the grain (bit 31: the pivot is the V end), the
// pivot row's probe total and the exclusive prefix of task counts
// (start[len] = number of tasks).  Runs on one whole CTA.
constexpr uint32_t kPivIsV = 0x80000000u;
__device__ void plan(const MspArgs &a, Smem &sm, const uint32_t *curr, uint32_t len, uint32_t *piv_out,
                     uint32_t *anc_out, uint32_t *grain_out, uint32_t *total_out, uint32_t *start_out,
                     bool count_anchor) {
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
        piv_out[i] = cv <= cu ? uv.y : uv.x;
        anc_out[i] = cv <= cu ? uv.x : uv.y;
        total_out[i] = cv <= cu ? cv : cu;
        grain_out[i] = cv <= cu ? kPivIsV : 0;
        mine += cv <= cu ? cv : cu;
    }
    for (int o = 16; o; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&sm.total, mine);
    __syncthreads();
    unsigned long long g = sm.total / ((unsigned long long)a.tasks_per_cta * a.nblocks);
    if (g < a.min_grain) g = a.min_grain;
    if (g > (1u << 30)) g = 1u << 30;
    unsigned long long anchor = 0;
    for (uint32_t base = 0; base < len; base += kThreads) {
        const uint32_t i = base + threadIdx.x;
        uint32_t nt = 0;
        if (i < len) {
            const uint32_t anc = anc_out[i];
            const uint32_t work = total_out[i];
            const uint32_t da = a.deg[anc];
            // a task stages a short anchor row in shared memory: make it worth it
            unsigned long long gi = (da <= bt::kHashMaxDeg && 2ull * da > g) ? 2ull * da : g;
            if (gi > (1u << 30)) gi = 1u << 30;  // leaves bit 31 for kPivIsV
            nt = (uint32_t)((work + gi - 1) / gi);
            grain_out[i] |= (uint32_t)gi;
            anchor += da;
        }
        uint32_t excl, tot;
        cub::BlockScan<uint32_t, kThreads>(sm.walk.scan).ExclusiveSum(nt, excl, tot);
        if (i < len) start_out[i] = sm.running + excl;
        __syncthreads();
        if (threadIdx.x == 0) sm.running += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) start_out[len] = sm.running;
    if (count_anchor) {
        for (int o = 16; o; o >>= 1) anchor += __shfl_xor_sync(0xffffffffu, anchor, o);
        if ((threadIdx.x & 31) == 0 && anchor) atomicAdd(&a.s->w_anchor, anchor);
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// peel: all tasks of one sub-round
// ---------------------------------------------------------------------------

// The rule applied to the butterflies of one frontier edge uv (see
// bt::walk_range for the two-step interface).
template <bool N32>
struct MspHit {
    const MspArgs &a;
    bt::Walk &w;
    const Round &rd;
    uint32_t uv, exact;
    bool piv_is_v;
    unsigned long long decs = 0, hits = 0;
    struct State {
        uint32_t kslot, e_my, e_ay, ah;
        // After load(): the stamps of e_my and e_ay.  After apply(): the old
        // supports of the global decrements the hit has in flight, 0 for none
        // (a decremented edge's old support is at least 1: an edge loses at
        // most one support per butterfly it is in).  One pair of fields for
        // both keeps a lane's four hits within the register budget.
        SupWord<N32> x_my, x_ay;
    };
    __device__ __forceinline__ void load(State &s, uint32_t kk, uint32_t e_my, uint32_t ah) const {
        s.kslot = kk & ~(uint32_t)bt::kRevHit;
        s.e_my = e_my;
        s.ah = ah;
        s.e_ay = bt::walk_anchor_edge(w, ah);
        s.x_my = a.enter[e_my];
        s.x_ay = a.enter[s.e_ay];
    }
    // The rule for one hit.  Pivot-side and staged anchor-side decrements are
    // summed in shared memory; the others are issued here and settled by
    // settle() once every hit of the lane has issued its own.
    __device__ __forceinline__ void apply(State &s) {
        const uint32_t r = rd.r;
        hits++;  // a butterfly visited (the reference's intersection hit)
        const uint32_t en_my = (uint32_t)s.x_my, en_ay = (uint32_t)s.x_ay;
        s.x_my = s.x_ay = 0;
        if (is_done(en_ay, r) || is_done(en_my, r)) return;
        const uint32_t e_pm = w.mid_eid[s.kslot];
        const bool c_pm = w.pm_curr[s.kslot], c_my = en_my == r, c_ay = en_ay == r;
        // name the edges as the reference does: w on u's side, x on v's
        uint32_t wv, ux;
        bool cwv, cux;
        if (piv_is_v) { wv = e_pm; ux = s.e_ay; cwv = c_pm; cux = c_ay; }
        else { wv = s.e_ay; ux = e_pm; cwv = c_ay; cux = c_pm; }
        const uint32_t d = peel_rule(uv, wv, s.e_my, ux, cwv, c_my, cux, exact);
        if (!d) return;
        const bool d_wv = d & 1, d_wx = d & 2, d_ux = d & 4;
        const bool dec_pm = piv_is_v ? d_wv : d_ux;
        const bool dec_ay = piv_is_v ? d_ux : d_wv;
        decs += (uint32_t)dec_pm + (uint32_t)d_wx + (uint32_t)dec_ay;
        if (dec_pm) atomicAdd(&w.slot_dec[s.kslot], 1u);
        if (d_wx) s.x_my = dec_issue<N32>(a, s.e_my, 1);
        if (dec_ay) {
            if (w.cached_size) atomicAdd(&w.hdec[s.ah], 1u);
            else s.x_ay = dec_issue<N32>(a, s.e_ay, 1);
        }
    }
    __device__ __forceinline__ void settle(const State &s) const {
        if (s.x_my) dec_settle(a, rd, s.e_my, 1, s.x_my);
        if (s.x_ay) dec_settle(a, rd, s.e_ay, 1, s.x_ay);
    }
    __device__ __forceinline__ void stretch_done() const {}
    __device__ __forceinline__ bool stop() const { return false; }  // a peel walks every butterfly
};

template <bool N32>
__device__ void peel_tasks(const MspArgs &a, Smem &sm, const uint32_t *curr, uint32_t curr_len,
                           const uint32_t *pl_piv, const uint32_t *pl_anc, const uint32_t *pl_grain,
                           const uint32_t *pl_total, const uint32_t *start, uint32_t ntasks, uint32_t *ctr,
                           const Round &rd, uint32_t epoch, Work &wk) {
    const bt::Rows rows{a.off, a.deg, a.nbr, a.eid, a.hub_base, a.hub_mask, a.hub_pool};
    const uint32_t *enter = a.enter;
    const uint32_t r = rd.r;
    const uint32_t lane = threadIdx.x & 31;
    bt::Walk &w = sm.walk;
    bool first = true;
    for (;;) {
        if (threadIdx.x < 32) {
            // the first task of every CTA is its block index; the rest come
            // from the counter, which starts at the number of CTAs
            uint32_t t = blockIdx.x;
            if (!first && lane == 0) t = gridDim.x + atomicAdd(ctr, 1u);
            t = __shfl_sync(0xffffffffu, t, 0);
            uint32_t i = 0;
            if (t < ntasks) i = bt::warp_find_slot(start, curr_len, t);  // last i: start[i] <= t
            if (lane == 0) {
                sm.task = t;
                sm.idx = i;
            }
        }
        __syncthreads();
        first = false;
        const uint32_t t = sm.task;
        if (t >= ntasks) break;
        const unsigned long long task_t0 = (a.trace && threadIdx.x == 0) ? bt::global_ns() : 0;
        const unsigned long long walked0 = w.walked;
        const uint32_t i = sm.idx, k = t - start[i];
        const uint32_t uv = curr[i];
        const uint32_t piv = pl_piv[i], anc = pl_anc[i], gword = pl_grain[i];
        const uint32_t gi = gword & ~kPivIsV, total = pl_total[i];
        const bool piv_is_v = (gword & kPivIsV) != 0;
        const uint32_t f0 = k * gi;
        const uint32_t f1 = total - f0 < gi ? total : f0 + gi;
        const uint32_t exact = a.exact;
        if (threadIdx.x == 0) wk.mids++;
        bt::prof_mark(w, bt::PF_TASK);
        MspHit<N32> hit{a, w, rd, uv, exact, piv_is_v};
        bt::walk_range(
            rows, a.rowpre, w, piv, anc, epoch, total, f0, f1,
            [&](uint32_t kk, uint32_t e_pm) {
                const uint32_t en = enter[e_pm];
                w.pm_curr[kk] = en == r;
                return !is_done(en, r);
            },
            hit,
            [&](uint32_t cl, bool last) {
                // flush the pivot-side decrements of the slice and, after the
                // last slice, the anchor-side decrements of the task
                // (every decrement of a thread is issued before any is settled)
                __syncthreads();
                uint32_t c = 0;
                SupWord<N32> old = 0;
                if (threadIdx.x < cl) {
                    c = w.slot_dec[threadIdx.x];
                    if (c) {
                        w.slot_dec[threadIdx.x] = 0;
                        old = dec_issue<N32>(a, w.mid_eid[threadIdx.x], c);
                    }
                }
                constexpr uint32_t kPer = bt::kHashSlots / kThreads;
                uint32_t hc[kPer];
                SupWord<N32> hold[kPer];
                const uint32_t hsize = last ? w.cached_size : 0;
#pragma unroll
                for (uint32_t q = 0; q < kPer; q++) {
                    const uint32_t h = threadIdx.x + q * kThreads;
                    hc[q] = 0;
                    hold[q] = 0;
                    if (h < hsize) {
                        hc[q] = w.hdec[h];
                        if (hc[q]) {
                            w.hdec[h] = 0;
                            hold[q] = dec_issue<N32>(a, w.hval[h], hc[q]);
                        }
                    }
                }
                if (c) dec_settle(a, rd, w.mid_eid[threadIdx.x], c, old);
#pragma unroll
                for (uint32_t q = 0; q < kPer; q++)
                    if (hc[q]) dec_settle(a, rd, w.hval[threadIdx.x + q * kThreads], hc[q], hold[q]);
            });
        wk.decs += hit.decs;
        wk.hits += hit.hits;
        bt::prof_mark(w, bt::PF_FLUSH);
        if (a.trace && threadIdx.x == 0 && r < a.trace_cap) {
            atomicMax(&a.trace[r].max_task_ns, bt::global_ns() - task_t0);
            atomicAdd(&a.trace[r].walked, w.walked - walked0);
        }
    }
}

// ---------------------------------------------------------------------------
// level transition helpers
// ---------------------------------------------------------------------------

// Minimum support over the live entries of `list` (grid-wide atomicMin).
template <bool N32>
__device__ void list_min(const MspArgs &a, const uint32_t *list, uint32_t len, unsigned long long *out) {
    unsigned long long v = ~0ull;
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gsz = gridDim.x * blockDim.x;
    for (uint32_t i = gtid; i < len; i += gsz) {
        const uint32_t e = list[i];
        if (a.enter[e] == 0) {
            const unsigned long long s = sup_of<N32>(a, e);
            v = s < v ? s : v;
        }
    }
    v = warp_min(v);
    if ((threadIdx.x & 31) == 0 && v != ~0ull) atomicMin(out, v);
}

// Drop processed edges (enter in (0, r)) from every row; one warp per vertex,
// in place.
__device__ void compress_rows(const MspArgs &a, uint32_t r) {
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
                keep = !is_done(a.enter[e], r);
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

template <bool N32>
__global__ void __launch_bounds__(kThreads, 1) k_msp(MspArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
    MspState *s = a.s;
    bt::walk_init(sm.walk);
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gsz = gridDim.x * blockDim.x;
    constexpr uint32_t kNearTarget = 1u << 16;
    Work wk;
    uint32_t r = 2;            // sub-round index (1 marks the zero-support edges)
    uint32_t epoch = 0;        // row compactions so far (same in every CTA)
    unsigned long long L = 0;  // current level (same in every CTA)
    unsigned long long t_mark = gtid == 0 ? bt::global_ns() : 0;
    auto lap = [&](int k) {
        if (gtid == 0) {
            const unsigned long long t = bt::global_ns();
            s->ph_ns[k] += t - t_mark;
            t_mark = t;
        }
    };
    if (!barrier(a, sm)) return;

    uint32_t nsel = 0;         // near bucket: list near_a, length near_ctr[nsel]
    for (;;) {
        // ------------------------------------------------ level transition
        if (s->len[r % 3] == 0) {
            // T1: min over the near bucket (min_sup was reset in the last sub-round)
            list_min<N32>(a, a.near_a, s->near_ctr[nsel], &s->min_sup);
            if (!barrier(a, sm)) return;
            if (s->min_sup == ~0ull) {
                // T2: near is dry -> split the far bucket
                list_min<N32>(a, a.far_a, s->far_len, &s->far_min);
                if (!barrier(a, sm)) return;
                const unsigned long long lo = s->far_min;
                if (lo == ~0ull) break;  // nothing left
                const unsigned long long hi = lo + s->delta;
                for (uint32_t i = gtid; i < s->far_len; i += gsz) {
                    const uint32_t e = a.far_a[i];
                    if (a.enter[e] != 0) continue;
                    if (sup_of<N32>(a, e) < hi) a.near_b[atomicAdd(&s->near_ctr[nsel ^ 1], 1u)] = e;
                    else a.far_b[atomicAdd(&s->far2_len, 1u)] = e;
                }
                if (!barrier(a, sm)) return;
                {   // every CTA swaps its copies of the bucket pointers
                    uint32_t *t = a.near_a; a.near_a = a.near_b; a.near_b = t;
                    t = a.far_a; a.far_a = a.far_b; a.far_b = t;
                }
                nsel ^= 1;
                if (gtid == 0) {
                    s->near_ctr[nsel ^ 1] = 0;
                    s->far_len = s->far2_len;
                    s->far2_len = 0;
                    s->hi = hi;
                    s->min_sup = lo;
                    s->far_min = ~0ull;
                    s->rebuilds++;
                    if (s->near_ctr[nsel] > 4 * kNearTarget && s->delta > 1) s->delta >>= 1;
                    else if (s->near_ctr[nsel] < kNearTarget / 4) s->delta <<= 1;
                }
                if (!barrier(a, sm)) return;
            }
            // T3: frontier of sub-round r = near edges with support == L; the
            // rest of the live near edges are compacted into the other list
            L = s->min_sup;
            const uint32_t near_len = s->near_ctr[nsel];
            uint32_t *front = a.list[r % 3];
            for (uint32_t i = gtid; i < near_len; i += gsz) {
                const uint32_t e = a.near_a[i];
                if (a.enter[e] != 0) continue;
                if (sup_of<N32>(a, e) == L) {
                    a.enter[e] = r;
                    a.result[e] = (uint32_t)L;
                    front[atomicAdd(&s->len[r % 3], 1u)] = e;
                } else {
                    a.near_b[atomicAdd(&s->near_ctr[nsel ^ 1], 1u)] = e;
                }
            }
            // T4: compression (the reference's trigger, bitruss_msp.cu:537, see cfrac)
            const bool squeeze = (double)s->edge_num <= (double)a.cfrac * (double)s->live_at_compress &&
                                 (double)s->live_at_compress >= (double)a.cfloor * (double)a.m;
            if (!barrier(a, sm)) return;
            {
                uint32_t *t = a.near_a; a.near_a = a.near_b; a.near_b = t;
            }
            nsel ^= 1;
            if (gtid == 0) {
                s->last_level = L;
                s->levels_seen++;
                if (L > 0xffffffffull) s->overflow = 1;
                if (squeeze) {
                    s->live_at_compress = (unsigned long long)s->edge_num;
                    s->compressions++;
                }
            }
            if (squeeze) {
                compress_rows(a, r);
                if (!barrier(a, sm)) return;
                compute_two_hop(a);
                epoch++;
                if (!barrier(a, sm)) return;
            }
            lap(0);
        }
        // ------------------------------------------------ sub-round r
        const unsigned long long sr_t0 = (a.trace && gtid == 0) ? bt::global_ns() : 0;
        const uint32_t curr_len = s->len[r % 3];
        const uint32_t *curr = a.list[r % 3];
        Round rd;
        rd.r = r;
        rd.L = L;
        rd.hi = s->hi;
        rd.next = a.list[(r + 1) % 3];
        rd.next_len = &s->len[(r + 1) % 3];
        rd.near_list = a.near_a;
        rd.near_len = &s->near_ctr[nsel];
        uint32_t ntasks;
        if (curr_len <= a.local_plan) {
            plan(a, sm, curr, curr_len, sm.lp_piv, sm.lp_anc, sm.lp_grain, sm.lp_total, sm.lp_start,
                 blockIdx.x == 0);
            ntasks = sm.lp_start[curr_len];
            if (gtid == 0) s->tasks += ntasks;
        } else {
            if (blockIdx.x == 0) {
                plan(a, sm, curr, curr_len, a.pl_piv, a.pl_anc, a.pl_grain, a.pl_total, a.task_start, true);
                if (threadIdx.x == 0) {
                    s->task_total = a.task_start[curr_len];
                    s->tasks += s->task_total;
                }
            }
            if (!barrier(a, sm)) return;
            ntasks = s->task_total;
        }
        if (gtid == 0) {
            // slots used two sub-rounds from now; every CTA is past their last use
            s->len[(r + 2) % 3] = 0;
            s->task_ctr[(r + 2) % 3] = 0;
            s->near_ctr[nsel ^ 1] = 0;  // the compaction target of the next transition
            s->min_sup = ~0ull;
            s->edge_num -= curr_len;
            s->subrounds++;
        }
        if (curr_len <= a.local_plan)
            peel_tasks<N32>(a, sm, curr, curr_len, sm.lp_piv, sm.lp_anc, sm.lp_grain, sm.lp_total, sm.lp_start,
                       ntasks, &s->task_ctr[r % 3], rd, epoch, wk);
        else
            peel_tasks<N32>(a, sm, curr, curr_len, a.pl_piv, a.pl_anc, a.pl_grain, a.pl_total, a.task_start,
                       ntasks, &s->task_ctr[r % 3], rd, epoch, wk);
        if (!barrier(a, sm)) return;
        if (a.trace && gtid == 0 && r < a.trace_cap) {
            a.trace[r].t_ns = bt::global_ns() - sr_t0;
            a.trace[r].frontier = curr_len;
            a.trace[r].tasks = ntasks;
        }
        lap(1);
        r++;
    }
    if (gtid == 0) s->done = 1;
    // flush the counters
    if (threadIdx.x == 0) {
        for (int q = 0; q < 8; q++) atomicAdd(&s->prof[q], sm.walk.prof[q]);
        wk.probes += sm.walk.walked;
    }
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
                           uint32_t *sup32, uint32_t *enter, uint32_t *result, uint32_t *far_list, MspState *s) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long v = sup_in[e];
        if (sup32) sup32[e] = (uint32_t)v;  // every support fits (checked on the host)
        else sup[e] = v;
        result[e] = 0;
        if (v == 0) {
            enter[e] = 1;  // processed first (count_es_zero, bitruss_msp.cu:38-50)
        } else {
            enter[e] = 0;
            far_list[atomicAdd(&s->far_len, 1u)] = (uint32_t)e;
        }
    }
}

__global__ void k_two_hop(MspArgs a) { compute_two_hop(a); }

}  // namespace

// SM slots of the peeling kernel, per device.  A cooperative peel of nblocks
// CTAs (per_sm resident per SM) holds ceil(nblocks / per_sm) slots from its
// launch until it has finished; a device has one slot per SM, so the peels
// that run together -- contexts with a share of the SMs each, such as serving
// slots -- always fit side by side and never wait at a grid barrier for CTAs
// that cannot be placed.  A peel that wants every SM waits for the others to
// finish.
namespace {
constexpr int kMaxPoolDevices = 64;
std::mutex g_pool_mu;
std::condition_variable g_pool_cv;
int g_pool_free[kMaxPoolDevices];
bool g_pool_init[kMaxPoolDevices];

struct CtaSlots {
    int dev = -1, n = 0;
    void acquire(int device, int capacity, int want) {
        std::unique_lock<std::mutex> lk(g_pool_mu);
        if (!g_pool_init[device]) {
            g_pool_free[device] = capacity;
            g_pool_init[device] = true;
        }
        g_pool_cv.wait(lk, [&] { return g_pool_free[device] >= want; });
        g_pool_free[device] -= want;
        dev = device;
        n = want;
    }
    void release() {
        if (n == 0) return;
        {
            std::lock_guard<std::mutex> lk(g_pool_mu);
            g_pool_free[dev] += n;
            n = 0;
        }
        g_pool_cv.notify_all();
    }
    ~CtaSlots() { release(); }
};
}  // namespace

static unsigned long long wait_limit_ns() {
    const char *us = getenv("BT_WAIT_LIMIT_US");
    if (us && strtoull(us, nullptr, 10) > 0) return strtoull(us, nullptr, 10) * 1000ull;
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
    // 32-bit working supports when they all fit: half the footprint and
    // 4-byte atomics for the decrements
    // (BT_MSP_WIDE=1 keeps 64-bit supports: the path graphs with a support
    // above 2^32 take, testable on small graphs)
    const char *wide = getenv("BT_MSP_WIDE");
    if (ctx->last_sup_max <= 0xffffffffull && !(wide && *wide == '1')) A(a.sup32, 4 * mm);
    else A(a.sup, 8 * mm);
    A(a.enter, 4 * mm);
    A(a.list[0], 4 * mm);
    A(a.list[1], 4 * mm);
    A(a.list[2], 4 * mm);
    A(a.near_a, 4 * mm);
    A(a.near_b, 4 * mm);
    A(a.far_a, 4 * mm);
    A(a.far_b, 4 * mm);
    A(a.pl_piv, 4 * mm);
    A(a.pl_anc, 4 * mm);
    A(a.pl_grain, 4 * mm);
    A(a.pl_total, 4 * mm);
    A(a.rowpre, 8 * mm);
    A(a.task_start, 4 * (mm + 1));
    const char *trace_path = getenv("BT_MSP_TRACE");
    if (trace_path && *trace_path) {
        a.trace_cap = 4u << 20;
        A(a.trace, sizeof(TraceRow) * a.trace_cap);
    }
#undef A
    a.result = ctx->result;
#define C(x)                                                                  \
    do {                                                                      \
        cudaError_t _e = (x);                                                 \
        if (_e != cudaSuccess) { release(); return bt_cuda_fail(_e, #x, __FILE__, __LINE__); } \
    } while (0)
    {
        MspState init{};
        init.delta = 1;
        init.hi = 0;
        init.min_sup = ~0ull;
        init.far_min = ~0ull;
        init.live_at_compress = m;
        C(cudaMemcpyAsync(s, &init, sizeof(MspState), cudaMemcpyHostToDevice, st));
        C(cudaStreamSynchronize(st));  // `init` lives on the host stack
    }
    if (a.trace) C(cudaMemsetAsync(a.trace, 0, sizeof(TraceRow) * a.trace_cap, st));
    C(cudaMemcpyAsync(a.deg, g.deg0, 4 * n, cudaMemcpyDeviceToDevice, st));
    C(cudaMemcpyAsync(a.nbr, g.nbr0, 8 * m, cudaMemcpyDeviceToDevice, st));
    C(cudaMemcpyAsync(a.eid, g.eid0, 8 * m, cudaMemcpyDeviceToDevice, st));
    a.s = s;
    a.n = g.n;
    a.m = m;
    a.exact = exact ? 1u : 0u;
    a.min_grain = ctx->msp_schedule[0] ? ctx->msp_schedule[0] : kMspMinGrain;
    a.tasks_per_cta = ctx->msp_schedule[1] ? ctx->msp_schedule[1] : kMspTasksPerCta;
    a.local_plan = ctx->msp_schedule[2] ? std::min(ctx->msp_schedule[2], kLocalPlan) : kLocalPlan;
    a.wait_ns = wait_limit_ns();
    // Row compaction: whenever the live edges have halved since the last
    // compaction.  The reference also stops compacting once fewer than a tenth
    // of all edges are live (bitruss_msp.cu:537), which leaves the long tail
    // of the peel walking rows full of processed edges; dropping that floor
    // cut the row positions walked on the 20M-edge Chung-Lu graph by 11%.
    // Compaction changes which rows are walked, never a result.
    // BT_MSP_COMPACT="frac,floor" sets the trigger (the reference's is 0.5,0.1).
    a.cfrac = 0.5f;
    a.cfloor = 0.0f;
    if (const char *cv = getenv("BT_MSP_COMPACT")) {
        float f = 0, fl = 0;
        if (sscanf(cv, "%f,%f", &f, &fl) == 2 && f > 0 && f < 1 && fl >= 0 && fl <= 1) {
            a.cfrac = f;
            a.cfloor = fl;
        }
    }
    a.off = g.off;
    a.ends = g.ends;
    a.hub_base = g.hub_base;
    a.hub_mask = g.hub_mask;
    a.hub_pool = g.hub_pool;
    const unsigned blk = 256, cap = (unsigned)ctx->sm_count * 8;
    if (m) {
        k_msp_init<<<(unsigned)std::min<uint64_t>((m + blk - 1) / blk, cap), blk, 0, st>>>(
            m, (const unsigned long long *)ctx->sup, a.sup, a.sup32, a.enter, a.result, a.far_a, s); bt_note_launches(1);
        C(cudaGetLastError());
    }
    // edge_num = live edges
    MspState h0;
    {
        C(cudaMemcpyAsync(&h0, s, sizeof(MspState), cudaMemcpyDeviceToHost, st));
        C(cudaStreamSynchronize(st));
        h0.edge_num = h0.far_len;
        C(cudaMemcpyAsync(s, &h0, sizeof(MspState), cudaMemcpyHostToDevice, st));
    }
    if (n) {
        k_two_hop<<<(unsigned)std::min<uint64_t>((n * 32 + blk - 1) / blk, cap), blk, 0, st>>>(a); bt_note_launches(1);
        C(cudaGetLastError());
    }
    // cooperative persistent launch
    const size_t smem = sizeof(Smem);
    const void *kfn = a.sup32 ? (const void *)k_msp<true> : (const void *)k_msp<false>;
    C(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    C(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, kThreads, smem));
    if (per_sm < 1) { release(); return bt_fail(BT_ERR_CUDA, "msp kernel does not fit on an SM"); }
    const uint32_t capacity = (uint32_t)(ctx->sm_count * per_sm);
    a.nblocks = ctx->peel_ctas && ctx->peel_ctas < capacity ? ctx->peel_ctas : capacity;
    if (ctx->device < 0 || ctx->device >= kMaxPoolDevices) {
        release();
        return bt_fail(BT_ERR_INVALID, "device index out of range");
    }
    // SM slots (see CtaSlots): concurrent peels of this process fit side by side
    CtaSlots slots;
    NvtxRange range("k_msp");
    if (m) {
        slots.acquire(ctx->device, ctx->sm_count, (int)((a.nblocks + per_sm - 1) / per_sm));
        void *params[] = {&a};
        cudaEventRecord(ctx->ev[4], st);
        cudaError_t le = cudaLaunchCooperativeKernel(kfn, dim3(a.nblocks), dim3(kThreads), params, smem, st);
        if (le == cudaSuccess) le = cudaGetLastError();
        if (le != cudaSuccess) {
            slots.release();
            release();
            return bt_cuda_fail(le, "cudaLaunchCooperativeKernel(k_msp)", __FILE__, __LINE__);
        }
        cudaEventRecord(ctx->ev[5], st);
        bt_note_launches(1);
    }
    cudaEventRecord(e1, st);
    MspState h{};
    {
        cudaError_t ce = cudaMemcpyAsync(&h, s, sizeof(MspState), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        slots.release();
        if (ce != cudaSuccess) {
            release();
            return bt_cuda_fail(ce, "msp state readback", __FILE__, __LINE__);
        }
    }
    if (a.trace) {
        // rows 2 .. subrounds+1 are sub-rounds; written as raw TraceRow records
        const uint64_t rows = std::min<uint64_t>(h.subrounds + 2, a.trace_cap);
        std::vector<TraceRow> tr(rows);
        C(cudaMemcpyAsync(tr.data(), a.trace, sizeof(TraceRow) * rows, cudaMemcpyDeviceToHost, st));
        C(cudaStreamSynchronize(st));
        if (FILE *f = fopen(trace_path, "wb")) {
            fwrite(tr.data(), sizeof(TraceRow), rows, f);
            fclose(f);
        }
    }
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
    if (h.overflow) return bt_fail(BT_ERR_OVERFLOW, "msp: a bitruss number exceeds uint32");
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
    ctx->work[8] = 0;
    ctx->work[9] = a.sup32 ? 4 : 8;  // bytes per working support (and per decrement)
    for (int q = 0; q < 8; q++) ctx->prof[q] = h.prof[q] / (a.nblocks ? a.nblocks : 1);
    ctx->last_result = 2;
    if (levels) *levels = (uint32_t)h.last_level;
    return BT_OK;
}
