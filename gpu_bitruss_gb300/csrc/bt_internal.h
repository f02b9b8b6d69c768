// bt_internal.h -- shared definitions of the GB300 bitruss engine.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bitruss.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

// Record a message for bt_last_error() on this host thread and return `s`.
bt_status bt_fail(bt_status s, const std::string &msg);
bt_status bt_cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define BT_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t _e = (call);                                             \
        if (_e != cudaSuccess) return bt_cuda_fail(_e, #call, __FILE__, __LINE__); \
    } while (0)

#define BT_TRY(call)                                                         \
    do {                                                                     \
        bt_status _s = (call);                                               \
        if (_s != BT_OK) return _s;                                          \
    } while (0)

// Count of this library's own kernel launches (every launch site adds its
// launches; read by bt_kernel_launches).
void bt_note_launches(uint64_t k);

// NVTX range over a scope: each public call shows up as a named range on a
// profiler's timeline (no cost without a tool attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// ---------------------------------------------------------------------------
// host graph: the reference's Graph fields (src/graph/graph.h:43-51)
// ---------------------------------------------------------------------------

struct bt_graph {
    uint32_t u_num = 0, l_num = 0, u_max = 0, n = 0;
    uint64_t m = 0;
    uint64_t support_max = 0;
    std::vector<uint32_t> offsets;    // n+1
    std::vector<uint32_t> neighbors;  // 2m
    std::vector<uint32_t> degrees;    // n
    std::vector<uint32_t> edges;      // 2m
    std::vector<uint32_t> edge_ids;   // 2m
    std::vector<uint32_t> edge_support_raw;  // m, as stored in a .bin (int32 bits)
    std::vector<uint32_t> bitruss_raw;       // m, as stored in a .bin
    // batched arena only: graph index of every vertex (empty for one graph)
    // and the vertex count of the largest graph
    std::vector<uint32_t> segment;
    uint32_t seg_max_n = 0;
};

// ---------------------------------------------------------------------------
// device graph: vertices relabelled by priority rank, rows sorted by rank
// ---------------------------------------------------------------------------
//
// Rank 0 is the vertex of highest priority p(x) = (degree, id) -- the order of
// the reference's vertex-priority counting (src/bfc/cpu_bfc.cpp:59-60).  A
// vertex's row lists its neighbours' ranks in ascending order, so "neighbours
// of lower priority than r" is the suffix of the row after r.  Edge ids stay
// the reference's ids (the msp tie rule compares them).
struct DevGraph {
    uint32_t n = 0, u_num = 0;
    uint64_t m = 0;
    uint32_t max_deg = 0;
    uint32_t *off = nullptr;    // n+1 row starts
    uint32_t *deg0 = nullptr;   // n   degree
    uint32_t *nbr0 = nullptr;   // 2m  neighbour rank, ascending per row
    uint32_t *eid0 = nullptr;   // 2m  reference edge id of each slot
    uint2 *ends = nullptr;      // m   (rank of U end, rank of V end) per edge id
    uint32_t *is_u = nullptr;   // n   1 if the rank's vertex is on the U side
    // hub index: an open-addressing hash (neighbour rank -> edge id) of every
    // row longer than the kernels' shared-memory hash; hub_mask[x] = table
    // size - 1 (0: no table), hub_base[x] = first entry in hub_pool
    uint32_t *hub_base = nullptr;
    uint32_t *hub_mask = nullptr;
    uint2 *hub_pool = nullptr;
    uint64_t hub_slots = 0;
    // batched arena: ranks are grouped by graph; seg_base[r] = first rank of
    // r's graph (NULL for one graph); cnt_span = vertices of the largest graph
    uint32_t *seg_base = nullptr;
    uint32_t cnt_span = 0;
};

// ---------------------------------------------------------------------------
// device context
// ---------------------------------------------------------------------------

struct bt_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    uint64_t budget = 0;       // 0 = unlimited
    uint64_t used = 0;
    uint64_t peak = 0;         // high-water mark of `used`
    std::vector<std::pair<void *, uint64_t>> allocs;

    DevGraph g;
    bool has_graph = false;
    uint32_t u_max = 0, l_num = 0;

    // results of the last call (by reference edge id)
    uint64_t *sup = nullptr;     // m uint64 supports (ebfc)
    uint32_t *result = nullptr;  // m uint32 bitruss (hidx / msp)
    int last_result = 0;         // 0 none, 1 supports, 2 bitruss
    uint64_t last_count = 0, last_sup_max = 0;

    // scratch reused across calls
    void *scratch = nullptr;
    uint64_t scratch_bytes = 0;

    double phase_ms[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    uint64_t stats[8] = {0};
    uint64_t work[12] = {0};  // msp work counters and phase times of the last call
    uint64_t prof[8] = {0};   // msp: SM cycles per CTA by step (task, stage, slice, probe, hits, flush, barrier, other)
    cudaEvent_t ev[8] = {};

    // msp task schedule (0 = built-in value): min grain, tasks per CTA, local-plan limit
    uint32_t msp_schedule[3] = {0, 0, 0};
    uint64_t arena_edges = 1ull << 28;  // batched calls: edges per arena, at most
    uint32_t peel_ctas = 0;             // CTAs of the peeling kernel (0 = one per SM)
};

// Default msp task schedule (bt_ctx_set_msp_schedule with 0 picks these):
// probe positions per task at least, tasks per CTA, local-plan limit.
constexpr uint32_t kMspMinGrain = 2048;
constexpr uint32_t kMspTasksPerCta = 2;
constexpr uint32_t kMspLocalPlan = 512;

enum { PH_UPLOAD = 0, PH_EBFC = 1, PH_PEEL = 2, PH_HIDX = 3, PH_TOTAL = 4, PH_MSP = 5 };

// device arena (tracked against the context's budget)
bt_status ctx_alloc(bt_ctx *ctx, void **p, uint64_t bytes);
void ctx_free(bt_ctx *ctx, void *p);
template <class T>
bt_status ctx_alloc_t(bt_ctx *ctx, T **p, uint64_t count) {
    return ctx_alloc(ctx, reinterpret_cast<void **>(p), count * sizeof(T));
}
bt_status ctx_scratch(bt_ctx *ctx, uint64_t bytes, void **p);
void ctx_release_graph(bt_ctx *ctx);

// algorithm entry points implemented in the .cu files
bt_status dev_build_graph(bt_ctx *ctx, const bt_graph *g);
bt_status dev_ebfc(bt_ctx *ctx, bool per_edge, uint64_t *count);
bt_status dev_msp(bt_ctx *ctx, bool exact, uint32_t *levels);
bt_status dev_hidx(bt_ctx *ctx, uint32_t *rounds);
