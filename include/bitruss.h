/*
 * bitruss.h -- C ABI of the GB300 bitruss engine (libbitruss.so).
 *
 * Drop-in for the GPU path of ShunyangLi/GPU_Bitruss
 * (`coh --gpu --algo bfc|ebfc|hidx|msp`).  Each entry point names the
 * reference interface it replaces.  All sizes are in elements unless stated;
 * every call returns a bt_status and never exits the process (the reference
 * calls exit(EXIT_FAILURE) on any CUDA error: src/util/utility.h:52-62).
 *
 * Data contract (reference layout, src/graph/graph.h:43-51):
 *   vertex ids   uint32; U vertices 0..u_num-1, V vertices u_num..n-1
 *   edge id e    rank of the edge in U-major order with sorted rows
 *                (src/graph/graph.cpp:178-194); edges[2e]=U end, edges[2e+1]=V end
 *   supports     uint64 per edge (the reference's int32 overflows on hub-hub
 *                edges of power-law graphs)
 *   bitruss      uint32 per edge
 *   butterflies  uint64 total
 *
 * Threading: one bt_ctx per host thread.  A context owns one CUDA stream and
 * the device-resident copy of one graph; calls on a context are synchronous
 * with respect to the host (they return when the result is ready).
 */
#ifndef BITRUSS_GB300_H
#define BITRUSS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    BT_OK = 0,
    BT_ERR_INVALID = 1,     /* bad argument or malformed input            */
    BT_ERR_IO = 2,          /* file could not be opened / read / written  */
    BT_ERR_FORMAT = 3,      /* .bin header or size inconsistent           */
    BT_ERR_HOST_MEMORY = 4, /* host allocation failed                     */
    BT_ERR_DEVICE_MEMORY = 5, /* device allocation failed / over budget   */
    BT_ERR_CUDA = 6,        /* CUDA runtime error                         */
    BT_ERR_TIMEOUT = 7,     /* a bounded device-side wait gave up         */
    BT_ERR_STATE = 8,       /* call out of order (e.g. no graph uploaded) */
    BT_ERR_NO_DEVICE = 9,   /* no CUDA device / wrong architecture        */
    BT_ERR_OVERFLOW = 10    /* a result does not fit its output type      */
} bt_status;

typedef struct bt_graph bt_graph; /* host CSR, reference layout */
typedef struct bt_ctx bt_ctx;     /* device context              */

/* Read-only view of a host graph's arrays (owned by the bt_graph). */
typedef struct {
    uint32_t u_num, l_num, u_max, n;
    uint64_t m;
    uint64_t support_max;       /* set by bt_ebfc / the .bin header */
    const uint32_t *offsets;    /* n+1 */
    const uint32_t *neighbors;  /* 2m  */
    const uint32_t *degrees;    /* n   */
    const uint32_t *edges;      /* 2m  */
    const uint32_t *edge_ids;   /* 2m  */
} bt_graph_view;

/* ---- host graph (replaces class Graph, src/graph/graph.h:30-52) ---------- */

/* Graph(filename, false) + load_graph_bin: src/graph/graph.cpp:261-277,335-375.
 * Unlike the reference it validates the header against the file size. */
bt_status bt_graph_load_bin(const char *path, bt_graph **out);

/* Graph(filename, true) / process_graph: src/graph/graph.cpp:74-242.
 * Parses "u v" lines (first two integers of each line; lines starting with
 * '%' and blank lines are skipped); ids must be < 99,999,999 (MAX_IDS,
 * src/util/config.h:6). */
bt_status bt_graph_load_text(const char *path, bt_graph **out);

/* process_graph on an in-memory edge list in file order (same numbering). */
bt_status bt_graph_from_edges(const uint32_t *u, const uint32_t *v, uint64_t m,
                              bt_graph **out);

/* graph_to_bin: src/graph/graph.cpp:293-318 (byte-identical output). */
bt_status bt_graph_save_bin(const bt_graph *g, const char *path);

bt_status bt_graph_get_view(const bt_graph *g, bt_graph_view *out);
void bt_graph_free(bt_graph *g);

/* ---- device context --------------------------------------------------- */

/* Select `device`, create a stream and an empty context.  Fails with
 * BT_ERR_NO_DEVICE when the device is absent or not sm_103. */
bt_status bt_ctx_create(int device, bt_ctx **out);

/* Run subsequent work on a caller-owned stream (cudaStream_t as void*);
 * NULL restores the context's own stream. */
bt_status bt_ctx_set_stream(bt_ctx *ctx, void *cuda_stream);

/* Upper bound on device bytes this context may hold (0 = no limit).
 * Allocations beyond it fail with BT_ERR_DEVICE_MEMORY. */
bt_status bt_ctx_set_memory_budget(bt_ctx *ctx, uint64_t bytes);
bt_status bt_ctx_memory_used(const bt_ctx *ctx, uint64_t *bytes);
/* High-water mark of the bytes this context held since it was created or the
 * mark was last reset (reset != 0 sets it to the current use after reading). */
bt_status bt_ctx_memory_peak(bt_ctx *ctx, uint64_t *bytes, int reset);

void bt_ctx_free(bt_ctx *ctx);

/* Copy a host graph into the context's device arena (H2D of the reference
 * CSR) and build the device layout: vertices relabelled by priority rank
 * (degree, id) and rows sorted by rank.  Replaces the per-call cudaMalloc +
 * cudaMemcpy of bfc_vpp.cu:245-267 and bitruss_msp.cu:453-465; the graph
 * stays resident until the next upload or bt_ctx_free. */
bt_status bt_graph_upload(bt_ctx *ctx, const bt_graph *g);

/* ---- algorithms (on the resident graph) ------------------------------- */

/* Global butterfly count.  Replaces bfc_vpp(Graph*): bfc_vpp.cu:321-385. */
bt_status bt_bfc(bt_ctx *ctx, uint64_t *count);

/* Per-edge butterfly support.  Replaces bfc_evpp(Graph*): bfc_vpp.cu:233-309.
 * sup: m entries, by reference edge id (NULL: keep on device only).
 * count / support_max may be NULL. */
bt_status bt_ebfc(bt_ctx *ctx, uint64_t *sup, uint64_t *count, uint64_t *support_max);

/* h-index bitruss numbers (true bitruss).  Replaces g_bitruss_hindex(Graph*):
 * bitruss_hidx.cu:179-256.  bitruss: m entries (NULL: device only);
 * rounds may be NULL.  The iteration's fixpoint does not depend on where it
 * starts between the bitruss numbers and the supports: graphs of up to 2^20
 * edges start from the supports, as the reference does (same rounds); larger
 * graphs start from the exact peel's values (bt_msp_exact), and `rounds`
 * counts the rounds that verify them (1 when they are the fixpoint).  The
 * environment variable BT_HIDX_START=support|peel picks the start. */
bt_status bt_hidx(bt_ctx *ctx, uint32_t *bitruss, uint32_t *rounds);

/* Multi-stage peeling (GBiD).  Replaces bitruss_msp(Graph*):
 * bitruss_msp.cu:440-583, bit-exact with the reference's peel rule
 * (bitruss_msp.cu:126-184).  levels: the reference's "bitruss msp with N
 * levels" figure.  bitruss / levels may be NULL. */
bt_status bt_msp(bt_ctx *ctx, uint32_t *bitruss, uint32_t *levels);

/* Peeling with the corrected one-survivor rule; equals bt_hidx.  No
 * reference counterpart (the reference's msp over-estimates some edges). */
bt_status bt_msp_exact(bt_ctx *ctx, uint32_t *bitruss, uint32_t *levels);

/* Copy the last per-edge result of this context (uint64 supports after
 * bt_ebfc, uint32 bitruss after bt_hidx / bt_msp) to host memory. */
bt_status bt_result_download(bt_ctx *ctx, void *host, size_t bytes);

/* Device time in milliseconds of the named phase of the last call
 * ("upload", "ebfc" (counting kernel), "peel" (peeling kernel), "msp" (peeling
 * set-up + kernel + result), "hidx", "total"); negative if unknown. */
double bt_ctx_phase_ms(const bt_ctx *ctx, const char *phase);

/* Counters of the last msp/hidx call: [0] levels, [1] sub-rounds,
 * [2] compressions, [3] peel tasks, [4] hidx rounds, [5] non-empty levels,
 * [6] bucket splits; msp work: [8] peel tasks run, [9] neighbour slots
 * probed, [10] anchor slots, [11] butterflies found, [12] decrements, [13] m;
 * [14..16] nanoseconds the peeling kernel spent in level transitions, peel
 * phases and finalize phases; [17] bytes per working support of the last msp
 * (4 when every support fits 32 bits, else 8); [18] edge recomputations of
 * the last hidx over all its rounds, [19] 1 if it started from the exact
 * peel's values, 0 if from the supports; [20..27] SM cycles per CTA of the peeling
 * kernel by step: task lookup, anchor staging, slice load, probe pass, hit
 * pass, flushes, grid-barrier waits, other work.  After a batched call, [1] is
 * the sub-rounds summed over its arenas and [7] the number of arenas. */
bt_status bt_ctx_stats(const bt_ctx *ctx, uint64_t *out, int n);

/* ---- peeling schedule and its autotuner ------------------------------- */

/* The msp task schedule.  min_grain: probe positions per peel task, at least;
 * tasks_per_cta: a sub-round's work is cut into about this many tasks per
 * CTA; local_plan: frontiers of at most this many edges (<= 512) are planned
 * by every CTA without a grid barrier.  0 keeps the built-in value (2048, 2,
 * 512).  Results never depend on the schedule.  No reference counterpart (the
 * reference launches one block per frontier edge: bitruss_msp.cu:286-291). */
bt_status bt_ctx_set_msp_schedule(bt_ctx *ctx, uint32_t min_grain, uint32_t tasks_per_cta,
                                  uint32_t local_plan);
/* out: 3 entries, the schedule in effect (built-in values filled in). */
bt_status bt_ctx_get_msp_schedule(const bt_ctx *ctx, uint32_t *out);

/* Autotuner: times the peeling kernel of bt_msp on the resident graph under
 * candidate schedules (coordinate descent from the current one over short
 * candidate lists), keeps the fastest on the context and returns it in out
 * (3 entries, may be NULL) with its kernel time in *best_ms (may be NULL).
 * Costs about ten msp runs of the resident graph: tune on a sample. */
bt_status bt_msp_autotune(bt_ctx *ctx, uint32_t *out, double *best_ms);

/* ---- batched arenas ---------------------------------------------------- */
/*
 * No reference counterpart: the reference decomposes one Graph per process
 * (main.cu:91-128).  A batched call packs several graphs into one device
 * arena -- their disjoint union, numbered as process_graph
 * (src/graph/graph.cpp:74-242) numbers the concatenation of their edge lists:
 * the U vertices of graph 0, 1, ... first, then their V vertices, and graph
 * i's edge ids offset by the edge counts of graphs 0..i-1 -- and decomposes it
 * with one persistent launch.  A butterfly never spans two graphs, so every
 * graph's result equals the single-graph call on that graph (bit-exact).
 * Graphs are cut, in the order given, into arenas of at most
 * bt_ctx_set_arena_edges edges (default 2^28; a larger graph gets an arena of
 * its own).  The last arena stays resident on the context afterwards.
 */

/* Pack `count` graphs into one host graph (the arena layout above).
 * edge_base: count+1 entries (may be NULL), graph i's first edge id. */
bt_status bt_graph_pack(const bt_graph *const *graphs, uint32_t count, bt_graph **out,
                        uint64_t *edge_base);

/* Largest arena, in edges, of this context's batched calls (1 .. 2^31-1). */
bt_status bt_ctx_set_arena_edges(bt_ctx *ctx, uint64_t edges);

/* CTAs of this context's peeling kernel (0, the default: one per SM, the
 * whole GPU).  No reference counterpart.  The peel is bound by the latency of
 * its chain of sub-rounds rather than by the SMs' throughput, so several
 * contexts, each with a share of the SMs, peel side by side on one GPU (the
 * server gives each slot an equal share).  Concurrent peels of one process
 * never hold more CTAs than the device keeps resident: a peel waits until
 * its share is free.  Results do not depend on it. */
bt_status bt_ctx_set_peel_ctas(bt_ctx *ctx, uint32_t ctas);

/* msp (exact = 0, the reference rule) or the corrected rule (exact = 1) of
 * every graph.  bitruss: sum of m entries, graph i's edges from edge_base[i]
 * on in its own edge-id order; levels: count entries, each graph's "msp with
 * N levels" figure.  Either may be NULL. */
bt_status bt_msp_batch(bt_ctx *ctx, const bt_graph *const *graphs, uint32_t count, int exact,
                       uint32_t *bitruss, uint32_t *levels);

/* Supports (sum of m entries, laid out as in bt_msp_batch) and butterfly
 * counts (count entries) of every graph.  Either may be NULL. */
bt_status bt_ebfc_batch(bt_ctx *ctx, const bt_graph *const *graphs, uint32_t count, uint64_t *sup,
                        uint64_t *counts);

/* ---- serving --------------------------------------------------------- */
/*
 * No reference counterpart (the reference runs one algorithm on one graph per
 * process).  A server runs count / support / decompose requests on graphs of
 * different sizes as they arrive.  It has `slots` worker threads, each with
 * its own context and stream, so their uploads, counting kernels and copies
 * overlap on the GPU (one peeling kernel runs at a time).  A request is
 * admitted when a slot is free and its device footprint (bt_job_bytes) fits
 * in what the HBM budget has left; requests are taken in arrival order, and
 * one that does not fit yet may be passed by up to 64 later admissions.
 * Continuous batching: a slot that takes a request also takes every queued
 * request of the same kind (bfc/ebfc, msp, exact msp) that fits, up to 2^26
 * edges, and runs them as one arena (bt_msp_batch layout); a request of more
 * than 2^22 edges runs alone.  Each request's
 * result is the same alone and in a batch.
 */
typedef struct bt_server bt_server;

typedef enum { BT_OP_BFC = 0, BT_OP_EBFC = 1, BT_OP_MSP = 2, BT_OP_MSP_EXACT = 3 } bt_op;

typedef struct {
    bt_status status;
    uint64_t count;        /* butterflies (bfc, ebfc) */
    uint64_t support_max;  /* largest support (ebfc; bfc when batched) */
    uint32_t levels;       /* msp level count */
    uint32_t batch_size;   /* requests that shared this request's arena */
    double queue_ms;       /* submit -> admitted */
    double run_ms;         /* admitted -> done */
    double total_ms;       /* submit -> done */
} bt_request_info;

/* hbm_budget: device bytes the server may hold at once (0 = 90% of the free
 * memory at creation).  slots: 1..64. */
bt_status bt_server_create(int device, uint32_t slots, uint64_t hbm_budget, bt_server **out);

/* Queue a request.  op: a bt_op.  out: host buffer for the per-edge result --
 * m uint32 bitruss numbers (BT_OP_MSP, BT_OP_MSP_EXACT), m uint64 supports
 * (BT_OP_EBFC) -- or NULL; the graph and `out` must stay valid until the
 * request is waited for.  *ticket identifies the request. */
bt_status bt_server_submit(bt_server *s, const bt_graph *g, int op, void *out, uint64_t *ticket);

/* Wait for a request (timeout_ms < 0: no limit).  Returns the request's own
 * status, or BT_ERR_TIMEOUT if it is not done within the limit (the ticket
 * stays valid).  A finished ticket is consumed. */
bt_status bt_server_wait(bt_server *s, uint64_t ticket, double timeout_ms, bt_request_info *info);

/* Latency percentiles (submit -> done, ms) over requests completed since the
 * server started or the last reset; completed may be NULL. */
bt_status bt_server_latency(bt_server *s, double *p50_ms, double *p99_ms, uint64_t *completed, int reset);

/* [0] budget, [1] bytes reserved by running jobs, [2] running jobs,
 * [3] queued requests, [4] batches of more than one request, [5] requests in them. */
bt_status bt_server_stats(bt_server *s, uint64_t *out, int n);

/* Finish the queued requests, stop the workers, free the contexts. */
void bt_server_free(bt_server *s);

/* Device bytes a job of `count` graphs (one arena) and this op allocates at
 * its peak on this context's device: the admission estimate of the server. */
bt_status bt_job_bytes(bt_ctx *ctx, const bt_graph *const *graphs, uint32_t count, int op, uint64_t *bytes);

/* ---- allocation-free variant ------------------------------------------ */

/* Global butterfly count that allocates no device memory.  No counterpart in
 * the reference.  For callers that may not allocate on the device -- plugin
 * hosts that own the device heap and only hand buffers in, or
 * latency-sensitive paths that cannot afford a cudaMalloc / cudaFree -- the
 * caller passes the graph and the output in its own device buffers:
 * d_offsets (n+1) and d_neighbors (2m) in the reference layout (Graph::offsets
 * and Graph::neighbors copied to the device), d_count one uint64 that receives
 * the count.  Work is enqueued on `stream` (cudaStream_t as void*, NULL =
 * default stream); the count is ready when the stream reaches that point.
 * Scratch is one 32 MiB device array inside the library, held by every GPU
 * that loads it until the process exits; graphs with more than 4,194,304
 * vertices are rejected with BT_ERR_INVALID.  The first call on a device looks
 * up that array's device address (once per device and CUDA context: a call
 * after cudaDeviceReset looks it up again) and should come before any stream
 * capture.  The call restores the caller's current device before it returns.
 * All calls share the array: calls that overlap on the GPU race and give
 * wrong counts. */
bt_status bt_bfc_noalloc(int device, const uint32_t *d_offsets, const uint32_t *d_neighbors,
                         uint32_t n, uint64_t m, unsigned long long *d_count, void *stream);

/* Number of the library's own kernel launches in this process so far (CUB
 * launches inside the library are not counted).  No reference counterpart. */
uint64_t bt_kernel_launches(void);

/* ---- errors ---------------------------------------------------------- */

const char *bt_status_string(bt_status s);
/* Message of the last failed call on this host thread ("" if none). */
const char *bt_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* BITRUSS_GB300_H */
