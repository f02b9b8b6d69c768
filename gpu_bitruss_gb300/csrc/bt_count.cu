// bt_count.cu -- vertex-priority butterfly counting (bfc) and per-edge
// butterfly support (ebfc).
//
// Same arithmetic as the reference's bfc_kernel / ebfc_kernel
// (src/bfc/bfc_vpp.cu:33-107, 126-221) and CPU ebfc (src/bfc/cpu_bfc.cpp:24-122):
// a butterfly is counted once, at its vertex u of highest priority
// p(x) = (degree, id), as a pair of wedges u-v-w, u-x-w with p(v), p(w),
// p(x) < p(u).  With c(u,w) wedges from u to w the count gains C(c,2) and
// each wedge edge (u,v), (v,w) gains c-1 support.
//
// GB300 layout: vertices are relabelled by priority rank and rows sorted by
// rank, so the lower-priority neighbours of u are a row suffix found by one
// binary search (no per-element priority test, no reads of the skipped
// prefix).  Persistent CTAs take start vertices in rank order from a work
// counter; each CTA owns a dense wedge-counter array in HBM, touched entries
// are listed and cleared after each vertex (the reference sizes one n-length
// array per block from 96% of free memory: bfc_vpp.cu:252-257; here there is
// one per resident CTA).  In a batched arena the ranks of each graph are
// contiguous, a start vertex only reaches its own graph, and the counter
// array spans the largest graph (counters are indexed from the graph's first
// rank), not the whole arena.
#include <cub/device/device_reduce.cuh>

#include "bt_internal.h"

namespace {

constexpr int kCountThreads = 512;

// first index i in row[0..len) with row[i] > key (rows ascending)
__device__ __forceinline__ uint32_t upper_bound_u32(const uint32_t *row, uint32_t len, uint32_t key) {
    uint32_t lo = 0, hi = len;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(row + mid) <= key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

struct CountArgs {
    uint32_t n, span;    // vertices; counters per CTA (largest graph of an arena, else n)
    const uint32_t *off, *deg, *nbr, *eid;
    const uint32_t *seg_base;  // per rank: first rank of its graph (NULL: one graph)
    uint32_t *cnt;       // gridDim.x * span counters (zero on entry, zero on exit)
    uint32_t *touched;   // gridDim.x * span
    unsigned long long *sup;    // m supports (PER_EDGE)
    unsigned long long *count;  // butterfly total
    uint32_t *next_vertex;      // work counter
    uint32_t *layout_error;     // set if a wedge leaves its graph's counter span
};

template <bool PER_EDGE>
__global__ void __launch_bounds__(kCountThreads) k_count(CountArgs a) {
    __shared__ uint32_t s_r, s_nt;
    __shared__ unsigned long long s_red[kCountThreads / 32];
    uint32_t *cnt0 = a.cnt + (size_t)blockIdx.x * a.span;
    uint32_t *touched = a.touched + (size_t)blockIdx.x * a.span;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned long long local = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            s_r = atomicAdd(a.next_vertex, 1u);
            s_nt = 0;
        }
        __syncthreads();
        const uint32_t r = s_r;
        if (r >= a.n) break;
        // counters of r's graph: every w reached from r lies in [base, base + span)
        const uint32_t base = a.seg_base ? a.seg_base[r] : 0u;
        uint32_t *cnt = cnt0;
        const uint32_t rb = a.off[r], rl = a.deg[r];
        const uint32_t start = upper_bound_u32(a.nbr + rb, rl, r);
        // pass 1: wedge counts c(r, w) (bfc_vpp.cu:163-187)
        for (uint32_t i = start + warp; i < rl; i += nw) {
            const uint32_t s = __ldg(a.nbr + rb + i);
            const uint32_t sb = a.off[s], sl = a.deg[s];
            const uint32_t j0 = upper_bound_u32(a.nbr + sb, sl, r);
            for (uint32_t j = j0 + lane; j < sl; j += 32) {
                const uint32_t w = __ldg(a.nbr + sb + j);
                if (w - base >= a.span) {  // not in r's graph: the arena layout is broken
                    *a.layout_error = 1;
                    continue;
                }
                const uint32_t old = atomicAdd(cnt + (w - base), 1u);
                local += old;
                if (old == 0) touched[atomicAdd(&s_nt, 1u)] = w;
            }
        }
        __syncthreads();
        if (PER_EDGE) {
            // pass 2: supports (bfc_vpp.cu:191-219)
            for (uint32_t i = start + warp; i < rl; i += nw) {
                const uint32_t s = __ldg(a.nbr + rb + i);
                const uint32_t sb = a.off[s], sl = a.deg[s];
                const uint32_t j0 = upper_bound_u32(a.nbr + sb, sl, r);
                unsigned long long acc = 0;
                for (uint32_t j = j0 + lane; j < sl; j += 32) {
                    const uint32_t w = __ldg(a.nbr + sb + j);
                    if (w - base >= a.span) continue;  // reported by pass 1
                    const uint32_t c = __ldcg(cnt + (w - base));  // written by L2 atomics: bypass L1
                    if (c > 1) {
                        atomicAdd(a.sup + __ldg(a.eid + sb + j), (unsigned long long)(c - 1));
                        acc += c - 1;
                    }
                }
                for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0 && acc) atomicAdd(a.sup + __ldg(a.eid + rb + i), acc);
            }
            __syncthreads();
        }
        const uint32_t nt = s_nt;
        for (uint32_t k = threadIdx.x; k < nt; k += blockDim.x) cnt[touched[k] - base] = 0;  // touched holds ranks
        __syncthreads();
    }
    for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if (lane == 0) s_red[warp] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (uint32_t k = 0; k < nw; k++) t += s_red[k];
        if (t) atomicAdd(a.count, t);
    }
}

}  // namespace

// resident CTAs of the counting kernel (its persistent grid)
int dev_count_ctas(bt_ctx *ctx) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_count<true>, kCountThreads, 0) != cudaSuccess)
        per_sm = 1;
    int per_sm2 = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_count<false>, kCountThreads, 0) == cudaSuccess)
        per_sm = per_sm2 > per_sm ? per_sm2 : per_sm;
    return ctx->sm_count * (per_sm < 1 ? 1 : per_sm);
}

bt_status dev_ebfc(bt_ctx *ctx, bool per_edge, uint64_t *count) {
    DevGraph &g = ctx->g;
    cudaStream_t st = ctx->stream;
    // persistent grid: resident CTAs
    int per_sm = 0;
    BT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, per_edge ? k_count<true> : k_count<false>, kCountThreads, 0));
    if (per_sm < 1) per_sm = 1;
    uint64_t nctas = (uint64_t)ctx->sm_count * per_sm;
    if (g.n && nctas > g.n) nctas = g.n;
    if (nctas < 1) nctas = 1;
    // scratch: counters + touched lists, then (bytes) [0,8) count, [8,12) work
    // counter (later the support max at [8,16)), [16,20) layout error flag
    const uint64_t nn = g.cnt_span ? g.cnt_span : 1;
    uint64_t bytes = 2 * 4 * nn * nctas + 256;
    void *scr = nullptr;
    BT_TRY(ctx_scratch(ctx, bytes, &scr));
    uint32_t *cnt = (uint32_t *)scr;
    uint32_t *touched = cnt + nn * nctas;
    unsigned long long *d_count = (unsigned long long *)(touched + nn * nctas);
    uint32_t *d_next = (uint32_t *)(d_count + 1);
    uint32_t *d_err = d_next + 2;
    BT_CUDA(cudaMemsetAsync(cnt, 0, 4 * nn * nctas, st));
    BT_CUDA(cudaMemsetAsync(d_count, 0, 32, st));
    if (per_edge) BT_CUDA(cudaMemsetAsync(ctx->sup, 0, 8 * g.m, st));
    CountArgs a;
    a.n = g.n;
    a.span = (uint32_t)nn;
    a.seg_base = g.seg_base;
    a.off = g.off;
    a.deg = g.deg0;
    a.nbr = g.nbr0;
    a.eid = g.eid0;
    a.cnt = cnt;
    a.touched = touched;
    a.sup = (unsigned long long *)ctx->sup;
    a.count = d_count;
    a.next_vertex = d_next;
    a.layout_error = d_err;
    cudaEventRecord(ctx->ev[6], st);
    if (g.n) {
        if (per_edge) k_count<true><<<(unsigned)nctas, kCountThreads, 0, st>>>(a);
        else k_count<false><<<(unsigned)nctas, kCountThreads, 0, st>>>(a);
        bt_note_launches(1);
        BT_CUDA(cudaGetLastError());
    }
    cudaEventRecord(ctx->ev[7], st);
    uint64_t h_count = 0, h_max = 0;
    uint32_t h_err = 0;
    BT_CUDA(cudaMemcpyAsync(&h_count, d_count, 8, cudaMemcpyDeviceToHost, st));
    BT_CUDA(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, st));
    if (per_edge && g.m) {
        size_t tb = 0;
        BT_CUDA(cub::DeviceReduce::Max(nullptr, tb, (unsigned long long *)ctx->sup, d_count + 1, (int64_t)g.m, st));
        void *tmp = nullptr;
        BT_TRY(ctx_alloc(ctx, &tmp, tb));
        cudaError_t e = cub::DeviceReduce::Max(tmp, tb, (unsigned long long *)ctx->sup, d_count + 1,
                                               (int64_t)g.m, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h_max, d_count + 1, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        ctx_free(ctx, tmp);
        if (e != cudaSuccess) return bt_cuda_fail(e, "support max", __FILE__, __LINE__);
    }
    BT_CUDA(cudaStreamSynchronize(st));
    if (h_err) return bt_fail(BT_ERR_INVALID, "butterfly count: a wedge left its graph in the arena layout");
    float ms = -1;
    if (cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]) == cudaSuccess) ctx->phase_ms[PH_EBFC] = ms;
    *count = h_count;
    if (per_edge) {
        ctx->last_sup_max = h_max;
        ctx->last_result = 1;
    }
    ctx->last_count = h_count;
    return BT_OK;
}
