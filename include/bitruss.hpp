// bitruss.hpp -- C++ mirror of the reference's host interface, over the C ABI.
//
// The reference exposes class Graph (src/graph/graph.h:30-52) and four GPU
// entry points taking Graph* (src/bfc/bfc.cuh:18-19,
// src/bitruss/bitruss.cuh:17-18).  This header keeps those names and their
// meaning:
//   Graph(path, true)            text -> CSR (process_graph)
//   Graph(path, false)           load a .bin (the name must contain ".bin")
//   g.graph_to_bin(path)         write a .bin
//   bfc_vpp(&g)                  global butterfly count -> g.butterflies
//   bfc_evpp(&g)                 per-edge support -> g.edge_support, g.support_max
//   g_bitruss_hindex(&g)         bitruss numbers -> g.bitruss
//   bitruss_msp(&g)              bitruss numbers -> g.bitruss, levels -> g.levels
// Differences: supports are uint64 (the reference's int32 overflows), the
// butterfly count and level count are returned in fields instead of only
// logged, and failures throw bt::Error instead of calling exit().
#pragma once

#include <atomic>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "bitruss.h"

namespace bt {

struct Error : std::runtime_error {
    bt_status status;
    Error(bt_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

inline void check(bt_status s, const char *what) {
    if (s != BT_OK)
        throw Error(s, std::string(what) + ": " + bt_status_string(s) + ": " + bt_last_error());
}

// Per host thread: one device context (created on first use, replaced when
// another device is asked for) and the serial number of the Graph resident
// on it (0: none).
struct ThreadState {
    bt_ctx *ctx = nullptr;
    int dev = -1;
    uint64_t resident = 0;
    ThreadState() = default;
    ThreadState(const ThreadState &) = delete;
    ThreadState &operator=(const ThreadState &) = delete;
    ~ThreadState() {
        if (ctx) bt_ctx_free(ctx);
    }
};

inline ThreadState &thread_state() {
    static thread_local ThreadState s;
    return s;
}

inline bt_ctx *thread_context(int device = -1) {
    ThreadState &s = thread_state();
    if (device >= 0 && s.ctx && s.dev != device) {
        bt_ctx_free(s.ctx);
        s.ctx = nullptr;
        s.resident = 0;
    }
    if (!s.ctx) {
        int d = device >= 0 ? device : 0;
        s.resident = 0;
        check(bt_ctx_create(d, &s.ctx), "bt_ctx_create");
        s.dev = d;
    }
    return s.ctx;
}

// Every Graph gets a serial number no other Graph of the process shares, so a
// Graph built where a destroyed one lived is never mistaken for it.
inline uint64_t next_graph_serial() {
    static std::atomic<uint64_t> counter{0};
    return ++counter;
}

class Graph {
public:
    Graph(const std::string &filename, bool is_to_bin) {
        if (is_to_bin) {
            check(bt_graph_load_text(filename.c_str(), &g_), "process_graph");
        } else {
            if (filename.find(".bin") == std::string::npos)
                throw Error(BT_ERR_INVALID, "graph file should be binary file");
            check(bt_graph_load_bin(filename.c_str(), &g_), "load_graph_bin");
        }
        refresh();
    }
    Graph(const uint32_t *u, const uint32_t *v, uint64_t edges) {
        check(bt_graph_from_edges(u, v, edges, &g_), "process_graph");
        refresh();
    }
    Graph(const Graph &) = delete;
    Graph &operator=(const Graph &) = delete;
    ~Graph() {
        ThreadState &s = thread_state();
        if (s.resident == serial_) s.resident = 0;
        bt_graph_free(g_);
    }

    void graph_to_bin(const std::string &filename) const {
        check(bt_graph_save_bin(g_, filename.c_str()), "graph_to_bin");
    }

    // the reference's public fields (graph.h:43-51)
    uint32_t u_num = 0, l_num = 0, u_max = 0, n = 0;
    uint64_t m = 0;
    uint64_t support_max = 0;
    const uint32_t *neighbors = nullptr, *offsets = nullptr, *degrees = nullptr;
    const uint32_t *edges = nullptr, *edge_ids = nullptr;
    std::vector<uint64_t> edge_support;  // m
    std::vector<uint32_t> bitruss;       // m
    // facts the reference only logs
    uint64_t butterflies = 0;
    uint32_t levels = 0, rounds = 0;

    const bt_graph *handle() const { return g_; }

    // upload to the calling thread's context unless it already holds this
    // graph (keyed on the graph's serial number, not its address)
    bt_ctx *on_device(int device = -1) const {
        bt_ctx *ctx = thread_context(device);
        ThreadState &s = thread_state();
        if (s.resident != serial_) {
            s.resident = 0;  // a failed upload leaves no graph resident
            check(bt_graph_upload(ctx, g_), "graph upload");
            s.resident = serial_;
        }
        return ctx;
    }

private:
    void refresh() {
        bt_graph_view v;
        check(bt_graph_get_view(g_, &v), "graph view");
        u_num = v.u_num;
        l_num = v.l_num;
        u_max = v.u_max;
        n = v.n;
        m = v.m;
        support_max = v.support_max;
        neighbors = v.neighbors;
        offsets = v.offsets;
        degrees = v.degrees;
        edges = v.edges;
        edge_ids = v.edge_ids;
    }
    bt_graph *g_ = nullptr;
    const uint64_t serial_ = next_graph_serial();
};

// bfc_vpp(Graph*): src/bfc/bfc_vpp.cu:321-385
inline void bfc_vpp(Graph *g) {
    check(bt_bfc(g->on_device(), &g->butterflies), "bfc_vpp");
}

// bfc_evpp(Graph*): src/bfc/bfc_vpp.cu:233-309
inline void bfc_evpp(Graph *g) {
    g->edge_support.resize(g->m);
    check(bt_ebfc(g->on_device(), g->edge_support.data(), &g->butterflies, &g->support_max), "bfc_evpp");
}

// g_bitruss_hindex(Graph*): src/bitruss/bitruss_hidx.cu:179-256
inline void g_bitruss_hindex(Graph *g) {
    g->bitruss.resize(g->m);
    check(bt_hidx(g->on_device(), g->bitruss.data(), &g->rounds), "g_bitruss_hindex");
}

// bitruss_msp(Graph*): src/bitruss/bitruss_msp.cu:440-583
inline void bitruss_msp(Graph *g) {
    g->bitruss.resize(g->m);
    check(bt_msp(g->on_device(), g->bitruss.data(), &g->levels), "bitruss_msp");
}

// msp with the corrected one-survivor rule (equals g_bitruss_hindex)
inline void bitruss_msp_exact(Graph *g) {
    g->bitruss.resize(g->m);
    check(bt_msp_exact(g->on_device(), g->bitruss.data(), &g->levels), "bitruss_msp_exact");
}

}  // namespace bt
