// bt_ctx.cu -- device context, device arena, graph upload and the C ABI.
//
// Upload replaces the per-call cudaMalloc + cudaMemcpy of the reference's
// host drivers (bfc_vpp.cu:245-267, bitruss_msp.cu:453-465,
// bitruss_hidx.cu:196-211): the graph is copied once and stays resident.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_segmented_sort.cuh>

#include <cstring>
#include <atomic>
#include <mutex>
#include <string>

#include "bt_device.cuh"
#include "bt_internal.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

static thread_local std::string t_last_error;

bt_status bt_fail(bt_status s, const std::string &msg) {
    t_last_error = msg;
    return s;
}

bt_status bt_cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    cudaGetLastError();  // clear a non-sticky error
    std::string msg = std::string(cudaGetErrorName(e)) + " (" + cudaGetErrorString(e) + ") in " +
                      what + " at " + file + ":" + std::to_string(line);
    if (e == cudaErrorMemoryAllocation) return bt_fail(BT_ERR_DEVICE_MEMORY, msg);
    if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice || e == cudaErrorNoKernelImageForDevice ||
        e == cudaErrorInsufficientDriver)
        return bt_fail(BT_ERR_NO_DEVICE, msg);
    return bt_fail(BT_ERR_CUDA, msg);
}

extern "C" const char *bt_last_error(void) { return t_last_error.c_str(); }

static std::atomic<uint64_t> g_kernel_launches{0};
void bt_note_launches(uint64_t k) { g_kernel_launches.fetch_add(k, std::memory_order_relaxed); }
extern "C" uint64_t bt_kernel_launches(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

extern "C" const char *bt_status_string(bt_status s) {
    switch (s) {
        case BT_OK: return "ok";
        case BT_ERR_INVALID: return "invalid argument";
        case BT_ERR_IO: return "i/o error";
        case BT_ERR_FORMAT: return "malformed input";
        case BT_ERR_HOST_MEMORY: return "host out of memory";
        case BT_ERR_DEVICE_MEMORY: return "device out of memory or over budget";
        case BT_ERR_CUDA: return "CUDA error";
        case BT_ERR_TIMEOUT: return "device wait timed out";
        case BT_ERR_STATE: return "call out of order";
        case BT_ERR_NO_DEVICE: return "no usable CUDA device";
        case BT_ERR_OVERFLOW: return "result overflows its output type";
    }
    return "unknown status";
}

// ---------------------------------------------------------------------------
// device arena
// ---------------------------------------------------------------------------

// Device memory comes from the device's stream-ordered pool
// (cudaMallocAsync / cudaFreeAsync on the context's stream): no device-wide
// synchronisation per allocation or free, so contexts on different streams
// (the serving slots) overlap, and freed blocks are reused from the pool.
namespace {
std::once_flag g_pool_once[64];

void pool_setup(int device) {
    if (device < 0 || device >= 64) return;
    std::call_once(g_pool_once[device], [device]() {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = 8ull << 30;  // keep up to 8 GiB of freed blocks for reuse
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    });
}
}  // namespace

bt_status ctx_alloc(bt_ctx *ctx, void **p, uint64_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    bytes = (bytes + 255) & ~255ull;
    if (ctx->budget && ctx->used + bytes > ctx->budget)
        return bt_fail(BT_ERR_DEVICE_MEMORY, "device budget of " + std::to_string(ctx->budget) +
                                                 " bytes exceeded (need " +
                                                 std::to_string(ctx->used + bytes) + ")");
    cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return bt_cuda_fail(e, "cudaMallocAsync", __FILE__, __LINE__);
    }
    ctx->used += bytes;
    if (ctx->used > ctx->peak) ctx->peak = ctx->used;
    ctx->allocs.emplace_back(*p, bytes);
    return BT_OK;
}

void ctx_free(bt_ctx *ctx, void *p) {
    if (!p) return;
    for (size_t i = 0; i < ctx->allocs.size(); i++) {
        if (ctx->allocs[i].first == p) {
            ctx->used -= ctx->allocs[i].second;
            ctx->allocs.erase(ctx->allocs.begin() + (long)i);
            break;
        }
    }
    cudaFreeAsync(p, ctx->stream);
}

bt_status ctx_scratch(bt_ctx *ctx, uint64_t bytes, void **p) {
    if (ctx->scratch_bytes < bytes) {
        ctx_free(ctx, ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
        BT_TRY(ctx_alloc(ctx, &ctx->scratch, bytes));
        ctx->scratch_bytes = bytes;
    }
    *p = ctx->scratch;
    return BT_OK;
}

void ctx_release_graph(bt_ctx *ctx) {
    DevGraph &g = ctx->g;
    ctx_free(ctx, g.off);
    ctx_free(ctx, g.deg0);
    ctx_free(ctx, g.nbr0);
    ctx_free(ctx, g.eid0);
    ctx_free(ctx, g.ends);
    ctx_free(ctx, g.is_u);
    ctx_free(ctx, g.hub_base);
    ctx_free(ctx, g.hub_mask);
    ctx_free(ctx, g.hub_pool);
    ctx_free(ctx, g.seg_base);
    ctx_free(ctx, ctx->sup);
    ctx_free(ctx, ctx->result);
    ctx->sup = nullptr;
    ctx->result = nullptr;
    g = DevGraph();
    ctx->has_graph = false;
    ctx->last_result = 0;
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------

extern "C" bt_status bt_ctx_create(int device, bt_ctx **out) {
    if (!out) return bt_fail(BT_ERR_INVALID, "null argument");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return bt_fail(BT_ERR_NO_DEVICE, "no CUDA device available");
    if (device < 0 || device >= count)
        return bt_fail(BT_ERR_NO_DEVICE, "gpu device id " + std::to_string(device) + " is not available");
    BT_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    BT_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3)
        return bt_fail(BT_ERR_NO_DEVICE, std::string("device ") + prop.name + " is sm_" +
                                             std::to_string(prop.major) + std::to_string(prop.minor) +
                                             "; this build targets sm_103a (GB300)");
    bt_ctx *ctx = new (std::nothrow) bt_ctx();
    if (!ctx) return bt_fail(BT_ERR_HOST_MEMORY, "host allocation failed");
    ctx->device = device;
    ctx->sm_count = prop.multiProcessorCount;
    e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return bt_cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    ctx->stream = ctx->own_stream;
    for (auto &ev : ctx->ev) cudaEventCreate(&ev);
    pool_setup(device);
    *out = ctx;
    return BT_OK;
}

extern "C" bt_status bt_ctx_set_stream(bt_ctx *ctx, void *stream) {
    if (!ctx) return bt_fail(BT_ERR_INVALID, "null context");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return BT_OK;
}

extern "C" bt_status bt_ctx_set_memory_budget(bt_ctx *ctx, uint64_t bytes) {
    if (!ctx) return bt_fail(BT_ERR_INVALID, "null context");
    ctx->budget = bytes;
    return BT_OK;
}

extern "C" bt_status bt_ctx_memory_used(const bt_ctx *ctx, uint64_t *bytes) {
    if (!ctx || !bytes) return bt_fail(BT_ERR_INVALID, "null argument");
    *bytes = ctx->used;
    return BT_OK;
}

extern "C" bt_status bt_ctx_memory_peak(bt_ctx *ctx, uint64_t *bytes, int reset) {
    if (!ctx || !bytes) return bt_fail(BT_ERR_INVALID, "null argument");
    *bytes = ctx->peak;
    if (reset) ctx->peak = ctx->used;
    return BT_OK;
}

extern "C" void bt_ctx_free(bt_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    // free in the context's own stream order (a caller's stream may be gone by now)
    ctx->stream = ctx->own_stream;
    while (!ctx->allocs.empty()) ctx_free(ctx, ctx->allocs.back().first);
    cudaStreamSynchronize(ctx->own_stream);
    for (auto &ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

extern "C" double bt_ctx_phase_ms(const bt_ctx *ctx, const char *phase) {
    if (!ctx || !phase) return -1;
    static const char *names[] = {"upload", "ebfc", "peel", "hidx", "total", "msp"};
    for (int i = 0; i < 6; i++)
        if (!strcmp(phase, names[i])) return ctx->phase_ms[i];
    return -1;
}

extern "C" bt_status bt_ctx_stats(const bt_ctx *ctx, uint64_t *out, int n) {
    if (!ctx || !out) return bt_fail(BT_ERR_INVALID, "null argument");
    for (int i = 0; i < n && i < 8; i++) out[i] = ctx->stats[i];
    for (int i = 8; i < n && i < 20; i++) out[i] = ctx->work[i - 8];
    for (int i = 20; i < n && i < 28; i++) out[i] = ctx->prof[i - 20];
    return BT_OK;
}

// ---------------------------------------------------------------------------
// graph upload: reference CSR -> rank-relabelled device CSR
// ---------------------------------------------------------------------------

namespace {

// priority sort key: ascending key = descending (degree, id)
__global__ void k_rank_keys(uint32_t n, const uint32_t *deg, unsigned long long *key, uint32_t *val) {
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
        key[x] = ((unsigned long long)(0xffffffffu - deg[x]) << 32) | (0xffffffffu - x);
        val[x] = x;
    }
}

__global__ void k_rank_scatter(uint32_t n, uint32_t u_num, const uint32_t *order, const uint32_t *deg,
                               uint32_t *rank, uint32_t *deg_r, uint32_t *is_u) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t x = order[i];
        rank[x] = i;
        deg_r[i] = deg[x];
        is_u[i] = x < u_num ? 1u : 0u;
    }
}

// copy each row into its rank position, mapping neighbour ids to ranks;
// one warp per vertex
__global__ void k_rows_relabel(uint32_t n, uint32_t u_num, const uint32_t *off, const uint32_t *nbr,
                               const uint32_t *eid, const uint32_t *rank, const uint32_t *off_r,
                               uint32_t *nbr_r, uint32_t *eid_r, uint2 *ends) {
    uint32_t lane = threadIdx.x & 31;
    uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t x = warp; x < n; x += nwarps) {
        uint32_t b = off[x], len = off[x + 1] - b, rx = rank[x], dst = off_r[rx];
        for (uint32_t j = lane; j < len; j += 32) {
            uint32_t y = nbr[b + j], e = eid[b + j], ry = rank[y];
            nbr_r[dst + j] = ry;
            eid_r[dst + j] = e;
            if (x < u_num) ends[e] = make_uint2(rx, ry);
        }
    }
}

// hub table size of each row longer than the kernels' shared hash
__global__ void k_hub_sizes(uint32_t n, const uint32_t *deg, uint32_t *size, uint32_t *mask) {
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
        uint32_t sz = 0;
        if (deg[x] > bt::kHubMinDeg) {
            sz = 64;
            while (sz < 2 * deg[x]) sz <<= 1;
        }
        size[x] = sz;
        mask[x] = sz ? sz - 1 : 0;
    }
}

__global__ void k_hub_build(bt::Rows r, uint32_t n, uint2 *pool) { bt::hub_build(r, n, pool); }

// batched arena: graph index of each vertex in priority order
__global__ void k_gather_seg(uint32_t n, const uint32_t *order, const uint32_t *seg, uint32_t *seg_r) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        seg_r[i] = seg[order[i]];
}

// first rank of each rank's graph (ranks grouped by graph, graph index ascending)
__global__ void k_seg_base(uint32_t n, const uint32_t *seg_sorted, uint32_t *base) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = seg_sorted[i];
        uint32_t lo = 0, hi = i;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (seg_sorted[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        base[i] = lo;
    }
}

inline unsigned grid_for(uint64_t n, unsigned block, unsigned cap) {
    uint64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

}  // namespace

bt_status dev_build_graph(bt_ctx *ctx, const bt_graph *hg) {
    ctx_release_graph(ctx);
    DevGraph &g = ctx->g;
    cudaStream_t st = ctx->stream;
    uint32_t n = hg->n;
    uint64_t m = hg->m;
    g.n = n;
    g.m = m;
    g.u_num = hg->u_num;
    uint32_t maxd = 0;
    for (uint32_t x = 0; x < n; x++) maxd = hg->degrees[x] > maxd ? hg->degrees[x] : maxd;
    g.max_deg = maxd;

    // persistent arrays
    BT_TRY(ctx_alloc_t(ctx, &g.off, (uint64_t)n + 1));
    BT_TRY(ctx_alloc_t(ctx, &g.deg0, n));
    BT_TRY(ctx_alloc_t(ctx, &g.nbr0, 2 * m));
    BT_TRY(ctx_alloc_t(ctx, &g.eid0, 2 * m));
    BT_TRY(ctx_alloc_t(ctx, &g.ends, m));
    BT_TRY(ctx_alloc_t(ctx, &g.is_u, n));
    BT_TRY(ctx_alloc_t(ctx, &ctx->sup, m));
    BT_TRY(ctx_alloc_t(ctx, &ctx->result, m));

    // staging: reference CSR on device (freed at the end)
    uint32_t *s_off = nullptr, *s_nbr = nullptr, *s_eid = nullptr, *s_deg = nullptr;
    uint32_t *rank = nullptr, *order = nullptr, *vals = nullptr, *t_nbr = nullptr, *t_eid = nullptr;
    uint32_t *s_seg = nullptr, *seg_r = nullptr, *seg_r2 = nullptr, *order2 = nullptr;
    unsigned long long *keys = nullptr, *keys2 = nullptr;
    void *temp = nullptr;
    bt_status rc = BT_OK;
    const bool segmented = !hg->segment.empty();
    auto cleanup = [&]() {
        ctx_free(ctx, s_off); ctx_free(ctx, s_nbr); ctx_free(ctx, s_eid); ctx_free(ctx, s_deg);
        ctx_free(ctx, rank); ctx_free(ctx, order); ctx_free(ctx, vals);
        ctx_free(ctx, t_nbr); ctx_free(ctx, t_eid);
        ctx_free(ctx, keys); ctx_free(ctx, keys2); ctx_free(ctx, temp);
        ctx_free(ctx, s_seg); ctx_free(ctx, seg_r); ctx_free(ctx, seg_r2); ctx_free(ctx, order2);
    };
#define STEP(x)                 \
    do {                        \
        rc = (x);               \
        if (rc != BT_OK) {      \
            cleanup();          \
            return rc;          \
        }                       \
    } while (0)
#define STEPC(x)                                                          \
    do {                                                                  \
        cudaError_t _e = (x);                                             \
        if (_e != cudaSuccess) {                                          \
            cleanup();                                                    \
            return bt_cuda_fail(_e, #x, __FILE__, __LINE__);              \
        }                                                                 \
    } while (0)

    STEP(ctx_alloc_t(ctx, &s_off, (uint64_t)n + 1));
    STEP(ctx_alloc_t(ctx, &s_deg, n));
    STEP(ctx_alloc_t(ctx, &s_nbr, 2 * m));
    STEP(ctx_alloc_t(ctx, &s_eid, 2 * m));
    STEP(ctx_alloc_t(ctx, &rank, n));
    STEP(ctx_alloc_t(ctx, &order, n));
    STEP(ctx_alloc_t(ctx, &vals, n));
    STEP(ctx_alloc_t(ctx, &keys, n));
    STEP(ctx_alloc_t(ctx, &keys2, n));
    STEP(ctx_alloc_t(ctx, &t_nbr, 2 * m));
    STEP(ctx_alloc_t(ctx, &t_eid, 2 * m));

    STEPC(cudaMemcpyAsync(s_off, hg->offsets.data(), 4 * ((uint64_t)n + 1), cudaMemcpyHostToDevice, st));
    STEPC(cudaMemcpyAsync(s_deg, hg->degrees.data(), 4ull * n, cudaMemcpyHostToDevice, st));
    if (m) {
        STEPC(cudaMemcpyAsync(s_nbr, hg->neighbors.data(), 8 * m, cudaMemcpyHostToDevice, st));
        STEPC(cudaMemcpyAsync(s_eid, hg->edge_ids.data(), 8 * m, cudaMemcpyHostToDevice, st));
    }

    // temp storage for the cub calls (max over the three)
    size_t t1 = 0, t2 = 0, t3 = 0;
    STEPC(cub::DeviceRadixSort::SortPairs(nullptr, t1, keys, keys2, vals, order, (int)n, 0, 64, st));
    STEPC(cub::DeviceScan::ExclusiveSum(nullptr, t2, g.deg0, g.off, (int)n + 1, st));
    STEPC(cub::DeviceSegmentedSort::SortPairs(nullptr, t3, t_nbr, g.nbr0, t_eid, g.eid0, (int64_t)(2 * m),
                                              (int64_t)n, g.off, g.off + 1, st));
    size_t tb = t1 > t2 ? t1 : t2;
    tb = tb > t3 ? tb : t3;
    int seg_bits = 1;
    if (segmented) {
        if (hg->segment.size() != n) {
            cleanup();
            return bt_fail(BT_ERR_INVALID, "arena segment array does not match the vertex count");
        }
        uint32_t maxseg = 0;
        for (uint32_t x : hg->segment) maxseg = x > maxseg ? x : maxseg;
        while (seg_bits < 32 && (maxseg >> seg_bits)) seg_bits++;
        STEP(ctx_alloc_t(ctx, &s_seg, n));
        STEP(ctx_alloc_t(ctx, &seg_r, n));
        STEP(ctx_alloc_t(ctx, &seg_r2, n));
        STEP(ctx_alloc_t(ctx, &order2, n));
        STEP(ctx_alloc_t(ctx, &g.seg_base, n));
        STEPC(cudaMemcpyAsync(s_seg, hg->segment.data(), 4ull * n, cudaMemcpyHostToDevice, st));
        size_t t5 = 0;
        STEPC(cub::DeviceRadixSort::SortPairs(nullptr, t5, seg_r, seg_r2, order, order2, (int)n, 0, seg_bits, st));
        tb = tb > t5 ? tb : t5;
    }
    g.cnt_span = segmented ? hg->seg_max_n : n;
    STEP(ctx_alloc(ctx, &temp, tb));

    unsigned blk = 256, cap = (unsigned)ctx->sm_count * 8;
    if (n) {
        k_rank_keys<<<grid_for(n, blk, cap), blk, 0, st>>>(n, s_deg, keys, vals); bt_note_launches(1);
        STEPC(cub::DeviceRadixSort::SortPairs(temp, t1, keys, keys2, vals, order, (int)n, 0, 64, st));
        if (segmented) {
            // group the ranks by graph, priority order kept within a graph (stable sort)
            k_gather_seg<<<grid_for(n, blk, cap), blk, 0, st>>>(n, order, s_seg, seg_r); bt_note_launches(1);
            size_t t5 = tb;
            STEPC(cub::DeviceRadixSort::SortPairs(temp, t5, seg_r, seg_r2, order, order2, (int)n, 0, seg_bits,
                                                  st));
            std::swap(order, order2);
            k_seg_base<<<grid_for(n, blk, cap), blk, 0, st>>>(n, seg_r2, g.seg_base); bt_note_launches(1);
            STEPC(cudaGetLastError());
        }
        k_rank_scatter<<<grid_for(n, blk, cap), blk, 0, st>>>(n, g.u_num, order, s_deg, rank, g.deg0, g.is_u); bt_note_launches(1);
    }
    // off = exclusive scan of deg0 over n+1 entries (deg0[n] read as garbage is
    // avoided by scanning n entries and setting off[n] = 2m)
    STEPC(cub::DeviceScan::ExclusiveSum(temp, t2, g.deg0, g.off, (int)n, st));
    {
        uint32_t total = (uint32_t)(2 * m);
        STEPC(cudaMemcpyAsync(g.off + n, &total, 4, cudaMemcpyHostToDevice, st));
        STEPC(cudaStreamSynchronize(st));  // `total` lives on the host stack
    }
    if (n) {
        k_rows_relabel<<<grid_for((uint64_t)n * 32, blk, cap), blk, 0, st>>>(n, g.u_num, s_off, s_nbr, s_eid,
                                                                              rank, g.off, t_nbr, t_eid, g.ends); bt_note_launches(1);
        STEPC(cudaGetLastError());
    }
    if (m) {
        STEPC(cub::DeviceSegmentedSort::SortPairs(temp, t3, t_nbr, g.nbr0, t_eid, g.eid0, (int64_t)(2 * m),
                                                  (int64_t)n, g.off, g.off + 1, st));
    }
    // hub tables
    STEP(ctx_alloc_t(ctx, &g.hub_base, n ? n : 1));
    STEP(ctx_alloc_t(ctx, &g.hub_mask, n ? n : 1));
    if (n) {
        k_hub_sizes<<<grid_for(n, blk, cap), blk, 0, st>>>(n, g.deg0, order, g.hub_mask); bt_note_launches(1);
        STEPC(cudaGetLastError());
        size_t t4 = 0;
        STEPC(cub::DeviceScan::ExclusiveSum(nullptr, t4, order, g.hub_base, (int)n, st));
        if (t4 > tb) {
            ctx_free(ctx, temp);
            temp = nullptr;
            STEP(ctx_alloc(ctx, &temp, t4));
            tb = t4;
        }
        STEPC(cub::DeviceScan::ExclusiveSum(temp, t4, order, g.hub_base, (int)n, st));
        uint32_t last_base = 0, last_size = 0;
        STEPC(cudaMemcpyAsync(&last_base, g.hub_base + n - 1, 4, cudaMemcpyDeviceToHost, st));
        STEPC(cudaMemcpyAsync(&last_size, order + n - 1, 4, cudaMemcpyDeviceToHost, st));
        STEPC(cudaStreamSynchronize(st));
        g.hub_slots = (uint64_t)last_base + last_size;
    }
    STEP(ctx_alloc_t(ctx, &g.hub_pool, g.hub_slots ? g.hub_slots : 1));
    if (g.hub_slots) {
        STEPC(cudaMemsetAsync(g.hub_pool, 0xff, 8 * g.hub_slots, st));
        bt::Rows rows{g.off, g.deg0, g.nbr0, g.eid0, g.hub_base, g.hub_mask, g.hub_pool};
        k_hub_build<<<(unsigned)ctx->sm_count * 4, 256, 0, st>>>(rows, n, g.hub_pool); bt_note_launches(1);
        STEPC(cudaGetLastError());
    }
    STEPC(cudaStreamSynchronize(st));
    cleanup();
#undef STEP
#undef STEPC
    ctx->has_graph = true;
    ctx->u_max = hg->u_max;
    ctx->l_num = hg->l_num;
    ctx->last_result = 0;
    return BT_OK;
}

// ---------------------------------------------------------------------------
// C ABI: upload and algorithms
// ---------------------------------------------------------------------------

static bt_status enter(bt_ctx *ctx) {
    if (!ctx) return bt_fail(BT_ERR_INVALID, "null context");
    BT_CUDA(cudaSetDevice(ctx->device));
    return BT_OK;
}

static bt_status need_graph(bt_ctx *ctx) {
    BT_TRY(enter(ctx));
    if (!ctx->has_graph) return bt_fail(BT_ERR_STATE, "no graph uploaded to this context");
    return BT_OK;
}

static void time_begin(bt_ctx *ctx) { cudaEventRecord(ctx->ev[0], ctx->stream); }
static void time_end(bt_ctx *ctx, int phase) {
    cudaEventRecord(ctx->ev[1], ctx->stream);
    cudaEventSynchronize(ctx->ev[1]);
    float ms = -1;
    if (cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]) == cudaSuccess) ctx->phase_ms[phase] = ms;
}

extern "C" bt_status bt_graph_upload(bt_ctx *ctx, const bt_graph *g) {
    NvtxRange range("bt_graph_upload");
    BT_TRY(enter(ctx));
    if (!g) return bt_fail(BT_ERR_INVALID, "null graph");
    time_begin(ctx);
    BT_TRY(dev_build_graph(ctx, g));
    time_end(ctx, PH_UPLOAD);
    return BT_OK;
}

static bt_status copy_out(bt_ctx *ctx, void *host, const void *dev, uint64_t bytes) {
    if (!host || bytes == 0) return BT_OK;
    BT_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    return BT_OK;
}

extern "C" bt_status bt_bfc(bt_ctx *ctx, uint64_t *count) {
    NvtxRange range("bt_bfc");
    BT_TRY(need_graph(ctx));
    time_begin(ctx);
    uint64_t c = 0;
    BT_TRY(dev_ebfc(ctx, false, &c));
    time_end(ctx, PH_TOTAL);
    if (count) *count = c;
    return BT_OK;
}

extern "C" bt_status bt_ebfc(bt_ctx *ctx, uint64_t *sup, uint64_t *count, uint64_t *support_max) {
    NvtxRange range("bt_ebfc");
    BT_TRY(need_graph(ctx));
    time_begin(ctx);
    uint64_t c = 0;
    BT_TRY(dev_ebfc(ctx, true, &c));
    time_end(ctx, PH_TOTAL);
    if (count) *count = c;
    if (support_max) *support_max = ctx->last_sup_max;
    return copy_out(ctx, sup, ctx->sup, 8 * ctx->g.m);
}

extern "C" bt_status bt_msp(bt_ctx *ctx, uint32_t *bitruss, uint32_t *levels) {
    NvtxRange range("bt_msp");
    BT_TRY(need_graph(ctx));
    time_begin(ctx);
    uint32_t lv = 0;
    BT_TRY(dev_msp(ctx, false, &lv));
    time_end(ctx, PH_TOTAL);
    if (levels) *levels = lv;
    return copy_out(ctx, bitruss, ctx->result, 4 * ctx->g.m);
}

extern "C" bt_status bt_msp_exact(bt_ctx *ctx, uint32_t *bitruss, uint32_t *levels) {
    NvtxRange range("bt_msp_exact");
    BT_TRY(need_graph(ctx));
    time_begin(ctx);
    uint32_t lv = 0;
    BT_TRY(dev_msp(ctx, true, &lv));
    time_end(ctx, PH_TOTAL);
    if (levels) *levels = lv;
    return copy_out(ctx, bitruss, ctx->result, 4 * ctx->g.m);
}

extern "C" bt_status bt_hidx(bt_ctx *ctx, uint32_t *bitruss, uint32_t *rounds) {
    NvtxRange range("bt_hidx");
    BT_TRY(need_graph(ctx));
    time_begin(ctx);
    uint32_t r = 0;
    BT_TRY(dev_hidx(ctx, &r));
    time_end(ctx, PH_TOTAL);
    if (rounds) *rounds = r;
    return copy_out(ctx, bitruss, ctx->result, 4 * ctx->g.m);
}

extern "C" bt_status bt_result_download(bt_ctx *ctx, void *host, size_t bytes) {
    BT_TRY(need_graph(ctx));
    if (!host) return bt_fail(BT_ERR_INVALID, "null host buffer");
    if (ctx->last_result == 1) {
        if (bytes < 8 * ctx->g.m) return bt_fail(BT_ERR_INVALID, "buffer smaller than m uint64");
        return copy_out(ctx, host, ctx->sup, 8 * ctx->g.m);
    }
    if (ctx->last_result == 2) {
        if (bytes < 4 * ctx->g.m) return bt_fail(BT_ERR_INVALID, "buffer smaller than m uint32");
        return copy_out(ctx, host, ctx->result, 4 * ctx->g.m);
    }
    return bt_fail(BT_ERR_STATE, "no result on this context");
}
