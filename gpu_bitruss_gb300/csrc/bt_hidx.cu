// bt_hidx.cu -- h-index bitruss iteration (the reference's "hidx").
//
// Same iteration as the reference (src/bitruss/bitruss_hidx.cu:51-168,
// 179-256; CPU src/bitruss/cpu_bitruss.cpp:152-266): starting from the
// butterfly supports, every round sets
//   h(uv) = h-index of { min(prev[ux], prev[wx], prev[wv]) : butterflies
//                        (u,v,w,x) of uv whose three other edges have prev > 0 }
// (0 when prev[uv] == 0), synchronously for all edges, until a round changes
// nothing.  The fixpoint is each edge's bitruss number.
//
// GB300 design: the reference gathers every min value of an edge into a
// per-block buffer of support_max entries and quicksorts it with one thread
// (bitruss_hidx.cu:111-157, with a 32-entry explicit stack).  Here no value
// list is stored: the h-index only needs counts.  Since h never rises above
// prev[uv], a first pass counts the values >= prev[uv]; when there are at
// least prev[uv] of them the edge is unchanged.  Otherwise the answer lies in
// [0, min(prev, K)] and is found by histogram refinement: each pass
// re-walks the edge's butterflies, bins the values of the current window into
// 4096 shared-memory buckets and narrows the window to one bucket, so a window
// of 2^36 values needs three passes.  Butterflies are walked as in the
// peeling kernel (anchor row staged in a shared-memory hash, pivot rows
// flattened over the block).
//
// Active edges: a round only recomputes the edges that can change.  Values
// only fall, and h_k(e) = min(h_{k-1}(e), hindex(butterfly values of round
// k-1)), where a butterfly's value is the minimum of its three other edges.
// An edge keeps h = h_{k-1}(e) as long as at least h butterflies have a
// value >= h, so it can only change if some butterfly edge f fell, in round
// k-1, from a value >= h to one below h.  A butterfly of uv = (u, v) has edges
// ux, wv and wx with x a neighbour of u and w a neighbour of v, so f has an
// end in N[u] or N[v].  After each round every vertex z holds the lowest new
// value (lo) and the highest old value (hi) of the changed edges with an end
// in N[z]; edge (u, v) with value h is recomputed iff lo < h <= hi at u or at
// v.  The test never skips an edge that could change, so values, and the
// number of rounds, are those of the full synchronous iteration.
//
// Starting values.  The reference starts from the butterfly supports.  The
// iteration is monotone: started from any values s with b <= s <= supports,
// where b are the bitruss numbers (the largest fixpoint below the supports),
// every round keeps the values at or above b and they converge to the
// largest fixpoint below s, which is b.  So the result does not depend on
// the start, only the number of rounds does.  Graphs of up to 2^20 edges
// start from the supports (the reference's rounds); larger graphs start from
// the exact peel's values (bt_msp_exact, the bitruss numbers themselves),
// and the rounds then verify that those values are the fixpoint: one round
// that changes nothing.  BT_HIDX_START=support or =peel picks the start.
#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "bt_device.cuh"
#include "bt_internal.h"

namespace {

using bt::kThreads;
constexpr uint32_t kBuckets = 4096;
constexpr uint32_t kEdgeChunk = 8;  // consecutive edge ids per grab (they share the U end)

struct HidxArgs {
    bt::Rows rows;
    const uint2 *ends;
    const uint32_t *two_hop;   // per vertex: row probe total
    const uint32_t *rowpre;    // per slot: prefix of the row's neighbour degrees
    const unsigned long long *prev;  // values of the last round, by edge id
    unsigned long long *curr;        // this round's value of active edge k, by list index
    const uint32_t *active;          // edge ids recomputed this round (ascending)
    uint64_t m;                      // active edges
    unsigned long long *next_edge;   // work counter
    unsigned *changed;
};

// pass 1 of an edge: K = list length, cge = values >= H.  The walk stops once
// the block has counted H values >= H (the edge keeps H whatever the rest);
// K is then partial, which is fine: it is only used when cge < H.
struct CountHits {
    const unsigned long long *prev;
    const bt::Walk &w;
    unsigned long long H;
    unsigned long long *live;  // shared: values >= H counted by the block so far
    unsigned long long K = 0, cge = 0;
    uint32_t stretch_cge = 0;
    struct State {
        unsigned long long p1, p2, p3;
    };
    __device__ __forceinline__ void load(State &s, uint32_t kk, uint32_t e_my, uint32_t ah) const {
        s.p1 = prev[w.mid_eid[kk & ~(uint32_t)bt::kRevHit]];
        s.p2 = prev[e_my];
        s.p3 = prev[bt::walk_anchor_edge(w, ah)];
    }
    __device__ __forceinline__ void apply(const State &s) {
        if (s.p1 == 0 || s.p2 == 0 || s.p3 == 0) return;
        unsigned long long v = s.p1 < s.p2 ? s.p1 : s.p2;
        v = v < s.p3 ? v : s.p3;
        K++;
        if (v >= H) {
            cge++;
            stretch_cge++;
        }
    }
    __device__ __forceinline__ void settle(const State &) const {}
    __device__ __forceinline__ void stretch_done() {
        const uint32_t c = __reduce_add_sync(0xffffffffu, stretch_cge);
        stretch_cge = 0;
        if ((threadIdx.x & 31) == 0 && c) atomicAdd(live, (unsigned long long)c);
    }
    __device__ __forceinline__ bool stop() const {
        unsigned long long v = 0;
        if ((threadIdx.x & 31) == 0) v = *reinterpret_cast<volatile unsigned long long *>(live);
        return __shfl_sync(0xffffffffu, v, 0) >= H;
    }
};

// a refinement pass: histogram of the values in [lo, hi), count of those >= hi
struct BinHits {
    const unsigned long long *prev;
    const bt::Walk &w;
    uint32_t *hist;
    unsigned long long lo, hi, width, above = 0;
    struct State {
        unsigned long long p1, p2, p3;
    };
    __device__ __forceinline__ void load(State &s, uint32_t kk, uint32_t e_my, uint32_t ah) const {
        s.p1 = prev[w.mid_eid[kk & ~(uint32_t)bt::kRevHit]];
        s.p2 = prev[e_my];
        s.p3 = prev[bt::walk_anchor_edge(w, ah)];
    }
    __device__ __forceinline__ void apply(const State &s) {
        if (s.p1 == 0 || s.p2 == 0 || s.p3 == 0) return;
        unsigned long long v = s.p1 < s.p2 ? s.p1 : s.p2;
        v = v < s.p3 ? v : s.p3;
        if (v >= hi) above++;
        else if (v >= lo) atomicAdd(&hist[(v - lo) / width], 1u);
    }
    __device__ __forceinline__ void settle(const State &) const {}
    __device__ __forceinline__ void stretch_done() const {}
    __device__ __forceinline__ bool stop() const { return false; }  // a histogram needs every value
};

struct HSmem {
    bt::Walk walk;
    uint32_t hist[kBuckets];
    unsigned long long red[2][kThreads / 32];
    unsigned long long e0;
    unsigned long long live;  // pass 1: values >= H counted so far (early stop)
    unsigned long long win_lo, win_hi, above, result;
    int done;
};

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block-wide sums of two per-thread counters (all threads get the result)
__device__ __forceinline__ void block_sum2(HSmem &sm, unsigned long long &a, unsigned long long &b) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        sm.red[0][warp] = a;
        sm.red[1][warp] = b;
    }
    __syncthreads();
    unsigned long long ta = 0, tb = 0;
    for (uint32_t k = 0; k < kThreads / 32; k++) {
        ta += sm.red[0][k];
        tb += sm.red[1][k];
    }
    __syncthreads();
    a = ta;
    b = tb;
}

__global__ void __launch_bounds__(kThreads) k_hidx_round(HidxArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HSmem &sm = *reinterpret_cast<HSmem *>(smem_raw);
    bt::walk_init(sm.walk);
    const unsigned long long *prev = a.prev;
    auto keep_all = [](uint32_t, uint32_t) { return true; };
    auto no_slice = [](uint32_t, bool) {};
    bool any_change = false;
    for (;;) {
        if (threadIdx.x == 0) sm.e0 = atomicAdd(a.next_edge, (unsigned long long)kEdgeChunk);
        __syncthreads();
        const unsigned long long e0 = sm.e0;
        if (e0 >= a.m) break;
        const unsigned long long e1 = e0 + kEdgeChunk < a.m ? e0 + kEdgeChunk : a.m;
        for (unsigned long long ei = e0; ei < e1; ei++) {
            const uint32_t e = a.active[ei];
            const unsigned long long H = prev[e];
            if (H == 0) {  // cpu_bitruss.cpp:155
                if (threadIdx.x == 0) a.curr[ei] = 0;
                continue;
            }
            const uint2 uv = a.ends[e];
            const uint32_t cu = a.two_hop[uv.x], cv = a.two_hop[uv.y];
            const uint32_t piv = cv <= cu ? uv.y : uv.x, anc = cv <= cu ? uv.x : uv.y;
            const uint32_t total = a.two_hop[piv];
            // pass 1: K = list length, cge = values >= H (stops at H of them);
            // the reset is seen by every thread after walk_range's first sync
            bt::Walk &w = sm.walk;
            if (threadIdx.x == 0) sm.live = 0;
            CountHits ch{prev, w, H, &sm.live};
            bt::walk_range(a.rows, a.rowpre, w, piv, anc, 0, total, 0, total, keep_all, ch, no_slice);
            unsigned long long K = ch.K, cge = ch.cge;
            block_sum2(sm, K, cge);
            unsigned long long h;
            if (cge >= H) {
                h = H;
            } else {
                // h in [0, min(H-1, K)]: refine the window [lo, hi)
                if (threadIdx.x == 0) {
                    sm.win_lo = 0;
                    sm.win_hi = (H - 1 < K ? H - 1 : K) + 1;
                    sm.done = 0;
                }
                __syncthreads();
                while (!sm.done) {
                    const unsigned long long lo = sm.win_lo, hi = sm.win_hi;
                    const unsigned long long width = (hi - lo + kBuckets - 1) / kBuckets;
                    for (uint32_t t = threadIdx.x; t < kBuckets; t += blockDim.x) sm.hist[t] = 0;
                    __syncthreads();
                    BinHits bh{prev, w, sm.hist, lo, hi, width};
                    bt::walk_range(a.rows, a.rowpre, w, piv, anc, 0, total, 0, total, keep_all, bh, no_slice);
                    unsigned long long above = bh.above, unused = 0;
                    block_sum2(sm, above, unused);
                    if (threadIdx.x == 0) {
                        // largest bucket b with count(values >= start_b) >= start_b
                        const uint32_t nb = (uint32_t)((hi - lo + width - 1) / width);
                        unsigned long long cum = above;
                        int b = (int)nb - 1;
                        for (; b >= 0; b--) {
                            cum += sm.hist[b];
                            const unsigned long long x = lo + (unsigned long long)b * width;
                            if (cum >= x) {
                                const unsigned long long xe = x + width < hi ? x + width : hi;
                                if (xe - x == 1) {
                                    sm.result = x;
                                    sm.done = 1;
                                } else {
                                    sm.win_lo = x;
                                    sm.win_hi = xe;
                                }
                                break;
                            }
                        }
                        if (b < 0) {  // cannot happen when lo == 0; be safe
                            sm.result = lo;
                            sm.done = 1;
                        }
                    }
                    __syncthreads();
                }
                h = sm.result;
            }
            if (threadIdx.x == 0) {
                a.curr[ei] = h;
                if (h != H) any_change = true;
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0 && any_change) atomicExch(a.changed, 1u);
}

__global__ void k_row_prefix(bt::Rows r, uint32_t n, uint32_t *rowpre, uint32_t *total) {
    bt::row_prefix(r, n, rowpre, total);
}

// Apply a round: every active edge whose value changed takes the new value;
// its endpoints record the lowest new and the highest old value of their
// changed edges and are listed once (stamp r).
__global__ void k_hidx_apply(uint64_t len, const uint32_t *active, const unsigned long long *nval,
                             unsigned long long *val, const uint2 *ends, uint32_t r, uint32_t *mark,
                             uint32_t *marked, uint32_t *marked_len, unsigned long long *vlo,
                             unsigned long long *vhi) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < len;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = active[k];
        const unsigned long long b = nval[k], a = val[e];
        if (b == a) continue;
        val[e] = b;
        const uint2 uv = ends[e];
        atomicMin(&vlo[uv.x], b);
        atomicMax(&vhi[uv.x], a);
        atomicMin(&vlo[uv.y], b);
        atomicMax(&vhi[uv.y], a);
        if (atomicExch(&mark[uv.x], r) != r) marked[atomicAdd(marked_len, 1u)] = uv.x;
        if (atomicExch(&mark[uv.y], r) != r) marked[atomicAdd(marked_len, 1u)] = uv.y;
    }
}

// Spread each listed vertex's (lo, hi) to itself and its neighbours (one
// warp per listed vertex).
__global__ void k_hidx_near(const uint32_t *marked, const uint32_t *marked_len, bt::Rows rows,
                            const unsigned long long *vlo, const unsigned long long *vhi,
                            unsigned long long *nlo, unsigned long long *nhi) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t len = *marked_len;
    for (uint32_t i = warp; i < len; i += nw) {
        const uint32_t z = marked[i];
        const unsigned long long lo = vlo[z], hi = vhi[z];
        const uint32_t b = rows.off[z], d = rows.deg[z];
        if (lane == 0) {
            atomicMin(&nlo[z], lo);
            atomicMax(&nhi[z], hi);
        }
        for (uint32_t j = lane; j < d; j += 32) {
            const uint32_t y = rows.nbr[b + j];
            atomicMin(&nlo[y], lo);
            atomicMax(&nhi[y], hi);
        }
    }
}

// flag of the edges the next round recomputes: value h > 0 with lo < h <= hi
// at one of its ends
__global__ void k_hidx_flags(uint64_t m, const unsigned long long *val, const uint2 *ends,
                             const unsigned long long *nlo, const unsigned long long *nhi, uint8_t *flag) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long h = val[e];
        bool f = false;
        if (h > 0) {
            const uint2 uv = ends[e];
            f = (nlo[uv.x] < h && h <= nhi[uv.x]) || (nlo[uv.y] < h && h <= nhi[uv.y]);
        }
        flag[e] = f ? 1 : 0;
    }
}

// starting values from a uint32 result (the exact peel)
__global__ void k_hidx_widen(uint64_t m, const uint32_t *in, unsigned long long *v) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x)
        v[e] = in[e];
}

__global__ void k_hidx_result(uint64_t m, const unsigned long long *v, uint32_t *out, unsigned *overflow) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        if (v[e] > 0xffffffffull) atomicExch(overflow, 1u);
        out[e] = (uint32_t)v[e];
    }
}

}  // namespace

// Start of the iteration: true = the exact peel's values, false = supports.
static bool hidx_from_peel(uint64_t m) {
    const char *v = getenv("BT_HIDX_START");
    if (v && !strcmp(v, "peel")) return true;
    if (v && !strcmp(v, "support")) return false;
    return m > (1ull << 20);
}

bt_status dev_hidx(bt_ctx *ctx, uint32_t *rounds) {
    const bool from_peel = hidx_from_peel(ctx->g.m);
    if (from_peel) {
        uint32_t lv = 0;
        BT_TRY(dev_msp(ctx, true, &lv));  // ctx->result = the exact peel's values
    } else {
        uint64_t dummy = 0;
        BT_TRY(dev_ebfc(ctx, true, &dummy));
    }
    DevGraph &g = ctx->g;
    cudaStream_t st = ctx->stream;
    const uint64_t m = g.m, n = g.n;
    const uint64_t mm = m ? m : 1, nn = n ? n : 1;
    cudaEvent_t e0 = ctx->ev[2], e1 = ctx->ev[3];
    cudaEventRecord(e0, st);
    unsigned long long *val = nullptr, *nval = nullptr, *ctr = nullptr;
    uint32_t *two_hop = nullptr, *rowpre = nullptr, *active = nullptr, *mark = nullptr;
    uint32_t *marked = nullptr;
    unsigned long long *vlo = nullptr, *vhi = nullptr, *nlo = nullptr, *nhi = nullptr;
    uint8_t *flag = nullptr;
    void *temp = nullptr;
    auto release = [&]() {
        ctx_free(ctx, val);
        ctx_free(ctx, nval);
        ctx_free(ctx, ctr);
        ctx_free(ctx, two_hop);
        ctx_free(ctx, rowpre);
        ctx_free(ctx, active);
        ctx_free(ctx, mark);
        ctx_free(ctx, vlo);
        ctx_free(ctx, vhi);
        ctx_free(ctx, nlo);
        ctx_free(ctx, nhi);
        ctx_free(ctx, marked);
        ctx_free(ctx, flag);
        ctx_free(ctx, temp);
    };
    bt_status rc;
    if ((rc = ctx_alloc_t(ctx, &val, mm)) != BT_OK || (rc = ctx_alloc_t(ctx, &nval, mm)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &ctr, 8)) != BT_OK || (rc = ctx_alloc_t(ctx, &two_hop, nn)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &rowpre, 2 * mm)) != BT_OK || (rc = ctx_alloc_t(ctx, &active, mm)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &mark, nn)) != BT_OK || (rc = ctx_alloc_t(ctx, &vlo, nn)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &vhi, nn)) != BT_OK || (rc = ctx_alloc_t(ctx, &nlo, nn)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &nhi, nn)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &marked, nn)) != BT_OK || (rc = ctx_alloc_t(ctx, &flag, mm)) != BT_OK) {
        release();
        return rc;
    }
#define C(x)                                                                  \
    do {                                                                      \
        cudaError_t _e = (x);                                                 \
        if (_e != cudaSuccess) { release(); return bt_cuda_fail(_e, #x, __FILE__, __LINE__); } \
    } while (0)
    // ctr (uint64 words): [0] work counter, [1] changed, [2] overflow, [3] marked
    // count, [4] active count
    uint32_t *marked_len = (uint32_t *)(ctr + 3);
    unsigned long long *active_len = ctr + 4;
    C(cudaMemsetAsync(mark, 0, 4 * nn, st));
    bt::Rows rows{g.off, g.deg0, g.nbr0, g.eid0, g.hub_base, g.hub_mask, g.hub_pool};
    const unsigned blk = 256, cap = (unsigned)ctx->sm_count * 8;
    const unsigned egrid = (unsigned)std::min<uint64_t>((mm + blk - 1) / blk, cap);
    if (!from_peel) {
        C(cudaMemcpyAsync(val, ctx->sup, 8 * m, cudaMemcpyDeviceToDevice, st));
    } else if (m) {
        k_hidx_widen<<<egrid, blk, 0, st>>>(m, ctx->result, val); bt_note_launches(1);
        C(cudaGetLastError());
    }
    if (n) {
        k_row_prefix<<<(unsigned)std::min<uint64_t>((n * 32 + blk - 1) / blk, cap), blk, 0, st>>>(
            rows, g.n, rowpre, two_hop); bt_note_launches(1);
        C(cudaGetLastError());
    }
    // compaction of flagged edge ids (ascending), temp sized once
    thrust::counting_iterator<uint32_t> ids(0);
    size_t tb = 0;
    C(cub::DeviceSelect::Flagged(nullptr, tb, ids, flag, active, active_len, (int64_t)mm, st));
    if ((rc = ctx_alloc(ctx, &temp, tb)) != BT_OK) {
        release();
        return rc;
    }
    const size_t smem = sizeof(HSmem);
    C(cudaFuncSetAttribute(k_hidx_round, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    C(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hidx_round, kThreads, smem));
    if (per_sm < 1) per_sm = 1;
    const unsigned nblocks = (unsigned)(ctx->sm_count * per_sm);
    // round 1 recomputes every edge
    uint64_t len = m;
    if (m) {
        C(cudaMemsetAsync(flag, 1, m, st));
        C(cub::DeviceSelect::Flagged(temp, tb, ids, flag, active, active_len, (int64_t)m, st));
    }
    uint32_t r = 0;
    uint64_t recomputed = 0;
    for (;;) {
        r++;
        recomputed += len;
        C(cudaMemsetAsync(ctr, 0, 32, st));
        if (len) {
            HidxArgs a{rows, g.ends, two_hop, rowpre, val, nval, active, len, ctr, (unsigned *)(ctr + 1)};
            k_hidx_round<<<nblocks, kThreads, smem, st>>>(a); bt_note_launches(1);
            C(cudaGetLastError());
        }
        unsigned changed = 0;
        C(cudaMemcpyAsync(&changed, ctr + 1, 4, cudaMemcpyDeviceToHost, st));
        C(cudaStreamSynchronize(st));
        if (!changed) break;
        // apply, then the next round's active edges
        C(cudaMemsetAsync(vlo, 0xff, 8 * nn, st));
        C(cudaMemsetAsync(vhi, 0, 8 * nn, st));
        C(cudaMemsetAsync(nlo, 0xff, 8 * nn, st));
        C(cudaMemsetAsync(nhi, 0, 8 * nn, st));
        k_hidx_apply<<<(unsigned)std::min<uint64_t>((len + blk - 1) / blk, cap), blk, 0, st>>>(
            len, active, nval, val, g.ends, r, mark, marked, marked_len, vlo, vhi); bt_note_launches(1);
        C(cudaGetLastError());
        k_hidx_near<<<cap, blk, 0, st>>>(marked, marked_len, rows, vlo, vhi, nlo, nhi); bt_note_launches(1);
        C(cudaGetLastError());
        k_hidx_flags<<<egrid, blk, 0, st>>>(m, val, g.ends, nlo, nhi, flag); bt_note_launches(1);
        C(cudaGetLastError());
        C(cub::DeviceSelect::Flagged(temp, tb, ids, flag, active, active_len, (int64_t)m, st));
        unsigned long long nl = 0;
        C(cudaMemcpyAsync(&nl, active_len, 8, cudaMemcpyDeviceToHost, st));
        C(cudaStreamSynchronize(st));
        len = nl;
    }
    unsigned overflow = 0;
    if (m) {
        k_hidx_result<<<egrid, blk, 0, st>>>(m, val, ctx->result, (unsigned *)(ctr + 2)); bt_note_launches(1);
        C(cudaGetLastError());
    }
    C(cudaMemcpyAsync(&overflow, ctr + 2, 4, cudaMemcpyDeviceToHost, st));
    cudaEventRecord(e1, st);
    C(cudaStreamSynchronize(st));
#undef C
    float ms = -1;
    cudaEventElapsedTime(&ms, e0, e1);
    ctx->phase_ms[PH_HIDX] = ms;
    release();
    if (overflow) return bt_fail(BT_ERR_OVERFLOW, "hidx: a bitruss number exceeds uint32");
    ctx->stats[4] = r;
    ctx->work[10] = recomputed;  // edge recomputations over all rounds
    ctx->work[11] = from_peel ? 1 : 0;
    ctx->last_result = 2;
    if (rounds) *rounds = r;
    return BT_OK;
}
