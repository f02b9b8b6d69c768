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
#include <cstdlib>

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
    const unsigned long long *prev;
    unsigned long long *curr;
    uint64_t m;
    unsigned long long *next_edge;  // work counter
    unsigned *changed;
};

// pass 1 of an edge: K = list length, cge = values >= H
struct CountHits {
    const unsigned long long *prev;
    const bt::Walk &w;
    unsigned long long H, K = 0, cge = 0;
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
        if (v >= H) cge++;
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
};

struct HSmem {
    bt::Walk walk;
    uint32_t hist[kBuckets];
    unsigned long long red[2][kThreads / 32];
    unsigned long long e0;
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
        for (unsigned long long e = e0; e < e1; e++) {
            const unsigned long long H = prev[e];
            if (H == 0) {  // cpu_bitruss.cpp:155
                if (threadIdx.x == 0) a.curr[e] = 0;
                continue;
            }
            const uint2 uv = a.ends[e];
            const uint32_t cu = a.two_hop[uv.x], cv = a.two_hop[uv.y];
            const uint32_t piv = cv <= cu ? uv.y : uv.x, anc = cv <= cu ? uv.x : uv.y;
            const uint32_t total = a.two_hop[piv];
            // pass 1: K = list length, cge = values >= H
            bt::Walk &w = sm.walk;
            CountHits ch{prev, w, H};
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
                a.curr[e] = h;
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

__global__ void k_hidx_result(uint64_t m, const unsigned long long *v, uint32_t *out, unsigned *overflow) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        if (v[e] > 0xffffffffull) atomicExch(overflow, 1u);
        out[e] = (uint32_t)v[e];
    }
}

}  // namespace

bt_status dev_hidx(bt_ctx *ctx, uint32_t *rounds) {
    uint64_t dummy = 0;
    BT_TRY(dev_ebfc(ctx, true, &dummy));
    DevGraph &g = ctx->g;
    cudaStream_t st = ctx->stream;
    const uint64_t m = g.m, n = g.n;
    cudaEvent_t e0 = ctx->ev[2], e1 = ctx->ev[3];
    cudaEventRecord(e0, st);
    unsigned long long *buf_a = nullptr, *buf_b = nullptr, *ctr = nullptr;
    uint32_t *two_hop = nullptr, *rowpre = nullptr;
    auto release = [&]() {
        ctx_free(ctx, buf_a);
        ctx_free(ctx, buf_b);
        ctx_free(ctx, ctr);
        ctx_free(ctx, two_hop);
        ctx_free(ctx, rowpre);
    };
    bt_status rc;
    if ((rc = ctx_alloc_t(ctx, &buf_a, m ? m : 1)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &buf_b, m ? m : 1)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &ctr, 4)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &two_hop, n ? n : 1)) != BT_OK ||
        (rc = ctx_alloc_t(ctx, &rowpre, m ? 2 * m : 1)) != BT_OK) {
        release();
        return rc;
    }
#define C(x)                                                                  \
    do {                                                                      \
        cudaError_t _e = (x);                                                 \
        if (_e != cudaSuccess) { release(); return bt_cuda_fail(_e, #x, __FILE__, __LINE__); } \
    } while (0)
    C(cudaMemcpyAsync(buf_a, ctx->sup, 8 * m, cudaMemcpyDeviceToDevice, st));
    bt::Rows rows{g.off, g.deg0, g.nbr0, g.eid0, g.hub_base, g.hub_mask, g.hub_pool};
    const unsigned blk = 256, cap = (unsigned)ctx->sm_count * 8;
    if (n) {
        k_row_prefix<<<(unsigned)std::min<uint64_t>((n * 32 + blk - 1) / blk, cap), blk, 0, st>>>(
            rows, g.n, rowpre, two_hop);
        C(cudaGetLastError());
    }
    const size_t smem = sizeof(HSmem);
    C(cudaFuncSetAttribute(k_hidx_round, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    C(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hidx_round, kThreads, smem));
    if (per_sm < 1) per_sm = 1;
    const unsigned nblocks = (unsigned)(ctx->sm_count * per_sm);
    uint32_t r = 0;
    unsigned long long *prev = buf_a, *curr = buf_b;
    for (;;) {
        r++;
        C(cudaMemsetAsync(ctr, 0, 32, st));
        HidxArgs a{rows, g.ends, two_hop, rowpre, prev, curr, m, ctr, (unsigned *)(ctr + 1)};
        if (m) {
            k_hidx_round<<<nblocks, kThreads, smem, st>>>(a);
            C(cudaGetLastError());
        }
        unsigned changed = 0;
        C(cudaMemcpyAsync(&changed, ctr + 1, 4, cudaMemcpyDeviceToHost, st));
        C(cudaStreamSynchronize(st));
        unsigned long long *t = prev;
        prev = curr;
        curr = t;
        if (!changed) break;
    }
    unsigned overflow = 0;
    C(cudaMemsetAsync(ctr + 2, 0, 4, st));
    if (m) {
        k_hidx_result<<<(unsigned)std::min<uint64_t>((m + blk - 1) / blk, cap), blk, 0, st>>>(
            m, prev, ctx->result, (unsigned *)(ctr + 2));
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
    ctx->last_result = 2;
    if (rounds) *rounds = r;
    return BT_OK;
}
