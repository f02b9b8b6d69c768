// bt_batch.cpp -- batched arenas and the msp schedule autotuner.
//
// The reference decomposes one Graph per process (main.cu:91-128 calls
// bitruss_msp(&g) once).  A batched call packs many graphs into one arena --
// the disjoint union of the graphs, laid out exactly as the reference's
// process_graph (src/graph/graph.cpp:74-242) would number the concatenation of
// their edge lists: U vertices of graph 0, 1, ... first, then V vertices of
// graph 0, 1, ..., and graph i's edge ids offset by the edges of the graphs
// before it.  The arena is uploaded once and peeled by one persistent launch.
// The arena also records each vertex's graph, so the device layout can keep
// each graph's priority ranks contiguous (the counting kernel then sizes its
// per-CTA counters by the largest graph instead of the whole arena).
//
// Why the results are per-graph exact: a butterfly never spans two graphs, so
// a frontier edge of graph i only decrements edges of graph i, and the msp
// rule compares edge ids of one butterfly only (their order survives the
// offset).  Each level's frontier of the union is the union of the graphs'
// frontiers; a graph whose own frontier is empty at a sub-round takes no part
// in it.  So every edge receives the value it receives when its graph is
// peeled alone, and a graph's level count (the last level with a frontier
// edge) is the largest bitruss number among its edges.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "bt_internal.h"

namespace {

constexpr uint64_t kMaxArenaEdges = 0x7fffffffull;  // 32-bit CSR offsets hold 2m slots

bt_status check_graphs(const bt_graph *const *graphs, uint32_t count) {
    if (count && !graphs) return bt_fail(BT_ERR_INVALID, "null graph list");
    for (uint32_t i = 0; i < count; i++)
        if (!graphs[i]) return bt_fail(BT_ERR_INVALID, "null graph at index " + std::to_string(i));
    return BT_OK;
}

// Pack graphs[first, last) into `out` (see the file comment for the layout).
bt_status pack_range(const bt_graph *const *graphs, uint32_t first, uint32_t last, bt_graph *out) {
    const uint32_t k = last - first;
    std::vector<uint64_t> ubase(k + 1, 0), lbase(k + 1, 0), ebase(k + 1, 0);
    for (uint32_t i = 0; i < k; i++) {
        const bt_graph *g = graphs[first + i];
        ubase[i + 1] = ubase[i] + g->u_num;
        lbase[i + 1] = lbase[i] + g->l_num;
        ebase[i + 1] = ebase[i] + g->m;
    }
    const uint64_t U = ubase[k], L = lbase[k], M = ebase[k];
    if (M > kMaxArenaEdges) return bt_fail(BT_ERR_INVALID, "arena exceeds 2^31-1 edges");
    if (U + L > 0xffffffffull) return bt_fail(BT_ERR_INVALID, "arena exceeds 2^32-1 vertices");
    out->u_num = (uint32_t)U;
    out->l_num = (uint32_t)L;
    out->n = (uint32_t)(U + L);
    out->m = M;
    out->u_max = U ? (uint32_t)(U - 1) : 0;
    out->support_max = 0;
    uint32_t max_n = 0;
    for (uint32_t i = 0; i < k; i++) max_n = std::max(max_n, graphs[first + i]->n);
    out->seg_max_n = max_n;
    try {
        out->segment.assign(out->n, 0);
        out->offsets.assign((size_t)out->n + 1, 0);
        out->degrees.assign(out->n, 0);
        out->neighbors.resize(2 * M);
        out->edge_ids.resize(2 * M);
        out->edges.resize(2 * M);
    } catch (const std::bad_alloc &) {
        return bt_fail(BT_ERR_HOST_MEMORY, "host allocation of the arena failed");
    }
    out->edge_support_raw.clear();
    out->bitruss_raw.clear();
    uint32_t *off = out->offsets.data(), *deg = out->degrees.data(), *seg = out->segment.data();
    uint32_t *nbr = out->neighbors.data(), *eid = out->edge_ids.data(), *edg = out->edges.data();
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ii = 0; ii < (int64_t)k; ii++) {
        const uint32_t i = (uint32_t)ii;
        const bt_graph *g = graphs[first + i];
        const uint32_t un = g->u_num, gn = g->n;
        const uint64_t gm = g->m;
        const uint32_t ub = (uint32_t)ubase[i];             // first U vertex of graph i
        const uint32_t vb = (uint32_t)(U + lbase[i]);       // first V vertex of graph i
        const uint64_t eb = ebase[i];                       // first edge id of graph i
        // U rows occupy slots [0, M) in vertex order, V rows [M, 2M)
        for (uint32_t x = 0; x < gn; x++) {
            const bool is_u = x < un;
            const uint32_t nx = is_u ? ub + x : vb + (x - un);
            const uint64_t s0 = g->offsets[x], d = g->degrees[x];
            const uint64_t o = is_u ? eb + s0 : M + eb + (s0 - gm);
            off[nx] = (uint32_t)o;
            deg[nx] = (uint32_t)d;
            seg[nx] = i;
            for (uint64_t j = 0; j < d; j++) {
                const uint32_t y = g->neighbors[s0 + j];
                nbr[o + j] = is_u ? vb + (y - un) : ub + y;
                eid[o + j] = (uint32_t)(eb + g->edge_ids[s0 + j]);
            }
        }
        for (uint64_t e = 0; e < gm; e++) {
            edg[2 * (eb + e)] = ub + g->edges[2 * e];
            edg[2 * (eb + e) + 1] = vb + (g->edges[2 * e + 1] - un);
        }
    }
    off[out->n] = (uint32_t)(2 * M);
    return BT_OK;
}

// Arenas: consecutive runs of graphs with at most `cap` edges each (a graph
// larger than the cap gets an arena of its own).
std::vector<std::pair<uint32_t, uint32_t>> split_arenas(const bt_graph *const *graphs, uint32_t count,
                                                        uint64_t cap) {
    std::vector<std::pair<uint32_t, uint32_t>> out;
    uint32_t first = 0;
    uint64_t edges = 0;
    for (uint32_t i = 0; i < count; i++) {
        const uint64_t m = graphs[i]->m;
        if (i > first && edges + m > cap) {
            out.emplace_back(first, i);
            first = i;
            edges = 0;
        }
        edges += m;
    }
    if (count > first) out.emplace_back(first, count);
    return out;
}

bt_status enter_ctx(bt_ctx *ctx) {
    if (!ctx) return bt_fail(BT_ERR_INVALID, "null context");
    BT_CUDA(cudaSetDevice(ctx->device));
    return BT_OK;
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" bt_status bt_graph_pack(const bt_graph *const *graphs, uint32_t count, bt_graph **out,
                                   uint64_t *edge_base) {
    if (!out) return bt_fail(BT_ERR_INVALID, "null argument");
    *out = nullptr;
    BT_TRY(check_graphs(graphs, count));
    std::unique_ptr<bt_graph> g(new (std::nothrow) bt_graph());
    if (!g) return bt_fail(BT_ERR_HOST_MEMORY, "host allocation failed");
    BT_TRY(pack_range(graphs, 0, count, g.get()));
    if (edge_base) {
        edge_base[0] = 0;
        for (uint32_t i = 0; i < count; i++) edge_base[i + 1] = edge_base[i] + graphs[i]->m;
    }
    *out = g.release();
    return BT_OK;
}

extern "C" bt_status bt_ctx_set_peel_ctas(bt_ctx *ctx, uint32_t ctas) {
    if (!ctx) return bt_fail(BT_ERR_INVALID, "null context");
    ctx->peel_ctas = ctas;
    return BT_OK;
}

extern "C" bt_status bt_ctx_set_arena_edges(bt_ctx *ctx, uint64_t edges) {
    if (!ctx) return bt_fail(BT_ERR_INVALID, "null context");
    if (edges == 0 || edges > kMaxArenaEdges) return bt_fail(BT_ERR_INVALID, "arena edges must be in [1, 2^31-1]");
    ctx->arena_edges = edges;
    return BT_OK;
}

extern "C" bt_status bt_msp_batch(bt_ctx *ctx, const bt_graph *const *graphs, uint32_t count, int exact,
                                  uint32_t *bitruss, uint32_t *levels) {
    NvtxRange range("bt_msp_batch");
    BT_TRY(enter_ctx(ctx));
    BT_TRY(check_graphs(graphs, count));
    const double t0 = now_ms();
    double upload_ms = 0, msp_ms = 0, peel_ms = 0;
    uint64_t base = 0, subrounds = 0, arenas = 0;
    for (const auto &ar : split_arenas(graphs, count, ctx->arena_edges)) {
        bt_graph arena;
        BT_TRY(pack_range(graphs, ar.first, ar.second, &arena));
        const double u0 = now_ms();
        BT_TRY(dev_build_graph(ctx, &arena));  // ends with a stream synchronisation
        upload_ms += now_ms() - u0;
        uint32_t lv = 0;
        BT_TRY(dev_msp(ctx, exact != 0, &lv));
        msp_ms += ctx->phase_ms[PH_MSP] > 0 ? ctx->phase_ms[PH_MSP] : 0;
        peel_ms += ctx->phase_ms[PH_PEEL] > 0 ? ctx->phase_ms[PH_PEEL] : 0;
        subrounds += ctx->stats[1];
        arenas++;
        const uint64_t am = arena.m;
        if (bitruss || levels) {
            std::vector<uint32_t> tmp;
            uint32_t *dst = bitruss ? bitruss + base : nullptr;
            if (!dst) {
                tmp.resize(am ? am : 1);
                dst = tmp.data();
            }
            if (am) {
                BT_CUDA(cudaMemcpyAsync(dst, ctx->result, 4 * am, cudaMemcpyDeviceToHost, ctx->stream));
                BT_CUDA(cudaStreamSynchronize(ctx->stream));
            }
            if (levels) {
                uint64_t e0 = 0;
                for (uint32_t i = ar.first; i < ar.second; i++) {
                    const uint64_t gm = graphs[i]->m;
                    uint32_t mx = 0;
                    for (uint64_t e = e0; e < e0 + gm; e++) mx = dst[e] > mx ? dst[e] : mx;
                    levels[i] = mx;
                    e0 += gm;
                }
            }
        }
        base += am;
    }
    ctx->phase_ms[PH_TOTAL] = now_ms() - t0;
    ctx->phase_ms[PH_UPLOAD] = upload_ms;
    ctx->phase_ms[PH_MSP] = msp_ms;
    ctx->phase_ms[PH_PEEL] = peel_ms;
    ctx->stats[1] = subrounds;
    ctx->stats[7] = arenas;
    return BT_OK;
}

extern "C" bt_status bt_ebfc_batch(bt_ctx *ctx, const bt_graph *const *graphs, uint32_t count, uint64_t *sup,
                                   uint64_t *counts) {
    NvtxRange range("bt_ebfc_batch");
    BT_TRY(enter_ctx(ctx));
    BT_TRY(check_graphs(graphs, count));
    const double t0 = now_ms();
    uint64_t base = 0, arenas = 0;
    for (const auto &ar : split_arenas(graphs, count, ctx->arena_edges)) {
        bt_graph arena;
        BT_TRY(pack_range(graphs, ar.first, ar.second, &arena));
        BT_TRY(dev_build_graph(ctx, &arena));
        uint64_t total = 0;
        BT_TRY(dev_ebfc(ctx, true, &total));
        arenas++;
        const uint64_t am = arena.m;
        if (sup || counts) {
            std::vector<uint64_t> tmp;
            uint64_t *dst = sup ? sup + base : nullptr;
            if (!dst) {
                tmp.resize(am ? am : 1);
                dst = tmp.data();
            }
            if (am) {
                BT_CUDA(cudaMemcpyAsync(dst, ctx->sup, 8 * am, cudaMemcpyDeviceToHost, ctx->stream));
                BT_CUDA(cudaStreamSynchronize(ctx->stream));
            }
            if (counts) {
                // every butterfly holds 4 edges: count = sum of supports / 4
                uint64_t e0 = 0;
                for (uint32_t i = ar.first; i < ar.second; i++) {
                    const uint64_t gm = graphs[i]->m;
                    unsigned __int128 sum = 0;
                    for (uint64_t e = e0; e < e0 + gm; e++) sum += dst[e];
                    counts[i] = (uint64_t)(sum / 4);
                    e0 += gm;
                }
            }
        }
        base += am;
    }
    ctx->phase_ms[PH_TOTAL] = now_ms() - t0;
    ctx->stats[7] = arenas;
    return BT_OK;
}

// ---------------------------------------------------------------------------
// msp task schedule and its autotuner
// ---------------------------------------------------------------------------

extern "C" bt_status bt_ctx_set_msp_schedule(bt_ctx *ctx, uint32_t min_grain, uint32_t tasks_per_cta,
                                             uint32_t local_plan) {
    if (!ctx) return bt_fail(BT_ERR_INVALID, "null context");
    if (min_grain > (1u << 30)) return bt_fail(BT_ERR_INVALID, "min_grain above 2^30");
    if (tasks_per_cta > 64) return bt_fail(BT_ERR_INVALID, "tasks_per_cta above 64");
    if (local_plan > 512) return bt_fail(BT_ERR_INVALID, "local_plan above 512");
    ctx->msp_schedule[0] = min_grain;
    ctx->msp_schedule[1] = tasks_per_cta;
    ctx->msp_schedule[2] = local_plan;
    return BT_OK;
}

extern "C" bt_status bt_ctx_get_msp_schedule(const bt_ctx *ctx, uint32_t *out) {
    if (!ctx || !out) return bt_fail(BT_ERR_INVALID, "null argument");
    out[0] = ctx->msp_schedule[0] ? ctx->msp_schedule[0] : kMspMinGrain;
    out[1] = ctx->msp_schedule[1] ? ctx->msp_schedule[1] : kMspTasksPerCta;
    out[2] = ctx->msp_schedule[2] ? ctx->msp_schedule[2] : kMspLocalPlan;
    return BT_OK;
}

// Coordinate descent over the three schedule parameters, each from a short
// candidate list, timing the peeling kernel of bt_msp on the resident graph.
// Schedules change which CTA walks which probes and when, never the result.
extern "C" bt_status bt_msp_autotune(bt_ctx *ctx, uint32_t *out, double *best_ms) {
    BT_TRY(enter_ctx(ctx));
    if (!ctx->has_graph) return bt_fail(BT_ERR_STATE, "no graph uploaded to this context");
    static const uint32_t grains[] = {512, 1024, 2048, 4096, 8192};
    static const uint32_t tasks[] = {1, 2, 4, 8};
    static const uint32_t plans[] = {64, 256, 512};
    uint32_t cur[3];
    BT_TRY(bt_ctx_get_msp_schedule(ctx, cur));
    const uint32_t saved[3] = {ctx->msp_schedule[0], ctx->msp_schedule[1], ctx->msp_schedule[2]};
    auto time_one = [&](const uint32_t s[3], double *ms) -> bt_status {
        ctx->msp_schedule[0] = s[0];
        ctx->msp_schedule[1] = s[1];
        ctx->msp_schedule[2] = s[2];
        uint32_t lv = 0;
        bt_status rc = dev_msp(ctx, false, &lv);
        *ms = ctx->phase_ms[PH_PEEL];
        return rc;
    };
    double best = 0;
    bt_status rc = time_one(cur, &best);
    if (rc != BT_OK) {
        for (int q = 0; q < 3; q++) ctx->msp_schedule[q] = saved[q];
        return rc;
    }
    const uint32_t *lists[3] = {grains, tasks, plans};
    const int sizes[3] = {5, 4, 3};
    for (int p = 0; p < 3 && rc == BT_OK; p++) {
        for (int c = 0; c < sizes[p]; c++) {
            if (lists[p][c] == cur[p]) continue;
            uint32_t s[3] = {cur[0], cur[1], cur[2]};
            s[p] = lists[p][c];
            double ms = 0;
            rc = time_one(s, &ms);
            if (rc != BT_OK) break;
            if (ms > 0 && ms < best) {
                best = ms;
                cur[p] = s[p];
            }
        }
    }
    if (rc != BT_OK) {
        for (int q = 0; q < 3; q++) ctx->msp_schedule[q] = saved[q];
        return rc;
    }
    for (int q = 0; q < 3; q++) ctx->msp_schedule[q] = cur[q];
    if (out) {
        out[0] = cur[0];
        out[1] = cur[1];
        out[2] = cur[2];
    }
    if (best_ms) *best_ms = best;
    return BT_OK;
}
