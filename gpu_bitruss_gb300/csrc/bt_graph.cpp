// bt_graph.cpp -- host graph: text / edge list -> reference CSR, .bin I/O.
//
// The CSR and its numbering are those of the reference's
// Graph::process_graph (src/graph/graph.cpp:74-242); the .bin layout is that
// of graph_to_bin / load_graph_bin (src/graph/graph.cpp:293-375).
#include <omp.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>

#include "bt_internal.h"

namespace {

constexpr uint32_t kMaxIds = 99999999u;  // MAX_IDS, src/util/config.h:6

// Build the CSR from an edge list in file order.  U and V ids are numbered by
// first appearance (graph.cpp:99-105), V ids offset by u_num (:118-131), rows
// sorted (:134-143), edge ids assigned to U slots in order (:178-194) and the
// V-side ids found by the reference's binary search (:196-228).  Duplicate
// lines are kept, as in the reference.
bt_status build_csr(const uint32_t *us, const uint32_t *vs, uint64_t m, bt_graph *g) {
    if (m > 0x7fffffffull) return bt_fail(BT_ERR_INVALID, "edge count exceeds the 32-bit CSR offsets");
    uint32_t max_u = 0, max_v = 0;
    for (uint64_t i = 0; i < m; i++) {
        if (us[i] >= kMaxIds || vs[i] >= kMaxIds)
            return bt_fail(BT_ERR_INVALID, "vertex id " + std::to_string(std::max(us[i], vs[i])) +
                                               " >= MAX_IDS (99999999)");
        max_u = std::max(max_u, us[i]);
        max_v = std::max(max_v, vs[i]);
    }
    std::vector<uint32_t> uid, lid, eu, ev;
    try {
        uid.assign(m ? (uint64_t)max_u + 1 : 0, UINT32_MAX);
        lid.assign(m ? (uint64_t)max_v + 1 : 0, UINT32_MAX);
        eu.resize(m);
        ev.resize(m);
    } catch (const std::bad_alloc &) {
        return bt_fail(BT_ERR_HOST_MEMORY, "host allocation failed in process_graph");
    }
    uint32_t u_num = 0, l_num = 0;
    for (uint64_t i = 0; i < m; i++) {
        uint32_t &a = uid[us[i]];
        if (a == UINT32_MAX) a = u_num++;
        uint32_t &b = lid[vs[i]];
        if (b == UINT32_MAX) b = l_num++;
        eu[i] = a;
        ev[i] = b;
    }
    uint32_t n = u_num + l_num;
    try {
        g->degrees.assign(n, 0);
        g->offsets.assign((uint64_t)n + 1, 0);
        g->neighbors.resize(2 * m);
        g->edges.resize(2 * m);
        g->edge_ids.resize(2 * m);
        g->edge_support_raw.assign(m, 0);
        g->bitruss_raw.assign(m, 0);
    } catch (const std::bad_alloc &) {
        return bt_fail(BT_ERR_HOST_MEMORY, "host allocation failed in process_graph");
    }
    for (uint64_t i = 0; i < m; i++) {
        g->degrees[eu[i]]++;
        g->degrees[u_num + ev[i]]++;
    }
    for (uint32_t i = 0; i < n; i++) g->offsets[i + 1] = g->offsets[i] + g->degrees[i];
    {
        std::vector<uint32_t> fill(g->offsets.begin(), g->offsets.end() - 1);
        for (uint64_t i = 0; i < m; i++) {
            g->neighbors[fill[eu[i]]++] = u_num + ev[i];
            g->neighbors[fill[u_num + ev[i]]++] = eu[i];
        }
    }
    uint32_t *nb = g->neighbors.data();
    const uint32_t *off = g->offsets.data();
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t x = 0; x < (int64_t)n; x++) std::sort(nb + off[x], nb + off[x + 1]);
    // U rows occupy slots [0, m): slot s of a U row is edge s.
    for (uint32_t u = 0; u < u_num; u++) {
        for (uint32_t s = off[u]; s < off[u + 1]; s++) {
            g->edge_ids[s] = s;
            g->edges[2 * (uint64_t)s] = u;
            g->edges[2 * (uint64_t)s + 1] = nb[s];
        }
    }
    uint32_t *ei = g->edge_ids.data();
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t vv = u_num; vv < (int64_t)n; vv++) {
        uint32_t v = (uint32_t)vv;
        for (uint32_t i = off[v]; i < off[v + 1]; i++) {
            uint32_t u = nb[i];
            const uint32_t *row = nb + off[u];
            int left = 0, right = (int)(off[u + 1] - off[u]) - 1;
            while (left <= right) {  // graph.cpp:211-224, including its mid==0 stop
                int mid = left + ((right - left) >> 1);
                if (row[mid] == v) {
                    ei[i] = ei[off[u] + mid];
                    break;
                } else if (row[mid] < v) {
                    left = mid + 1;
                } else {
                    if (mid == 0) break;
                    right = mid - 1;
                }
            }
        }
    }
    g->u_num = u_num;
    g->l_num = l_num;
    g->u_max = u_num;
    g->n = n;
    g->m = m;
    g->support_max = 0;
    return BT_OK;
}

// Parse the first two unsigned integers of a line.  Returns 1 on success,
// 0 for a line to skip ('%' comment or blank), -1 for a malformed line.
int parse_line(const char *p, const char *end, uint64_t *a, uint64_t *b) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
    if (p == end) return 0;
    if (*p == '%') return 0;
    uint64_t vals[2];
    for (int k = 0; k < 2; k++) {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
        if (p == end || *p < '0' || *p > '9') return -1;
        uint64_t x = 0;
        while (p < end && *p >= '0' && *p <= '9') {
            x = x * 10 + (uint64_t)(*p - '0');
            if (x > 0xffffffffull) return -1;
            p++;
        }
        vals[k] = x;
    }
    *a = vals[0];
    *b = vals[1];
    return 1;
}

}  // namespace

extern "C" bt_status bt_graph_from_edges(const uint32_t *u, const uint32_t *v, uint64_t m,
                                         bt_graph **out) {
    if (!out || (m && (!u || !v))) return bt_fail(BT_ERR_INVALID, "null argument");
    *out = nullptr;
    std::unique_ptr<bt_graph> g(new (std::nothrow) bt_graph());
    if (!g) return bt_fail(BT_ERR_HOST_MEMORY, "host allocation failed");
    BT_TRY(build_csr(u, v, m, g.get()));
    *out = g.release();
    return BT_OK;
}

extern "C" bt_status bt_graph_load_text(const char *path, bt_graph **out) {
    if (!path || !out) return bt_fail(BT_ERR_INVALID, "null argument");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return bt_fail(BT_ERR_IO, std::string("cannot open ") + path + ": " + strerror(errno));
    std::string buf;
    if (fseek(f, 0, SEEK_END) == 0) {
        long sz = ftell(f);
        if (sz > 0) {
            buf.resize((size_t)sz);
            fseek(f, 0, SEEK_SET);
            if (fread(&buf[0], 1, (size_t)sz, f) != (size_t)sz) {
                fclose(f);
                return bt_fail(BT_ERR_IO, std::string("short read on ") + path);
            }
        }
    }
    fclose(f);
    // split into lines, then parse the lines in parallel chunks
    std::vector<std::pair<uint64_t, uint64_t>> lines;
    {
        uint64_t s = 0, n = buf.size();
        while (s < n) {
            const void *nl = memchr(buf.data() + s, '\n', n - s);
            uint64_t e = nl ? (uint64_t)((const char *)nl - buf.data()) : n;
            lines.emplace_back(s, e);
            s = e + 1;
        }
    }
    std::vector<uint32_t> us(lines.size()), vs(lines.size());
    std::vector<uint8_t> keep(lines.size(), 0);
    int64_t bad = -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)lines.size(); i++) {
        uint64_t a = 0, b = 0;
        int r = parse_line(buf.data() + lines[i].first, buf.data() + lines[i].second, &a, &b);
        if (r < 0 || (r > 0 && (a >= kMaxIds || b >= kMaxIds))) {
#pragma omp critical
            if (bad < 0 || i < bad) bad = i;
        } else if (r > 0) {
            us[i] = (uint32_t)a;
            vs[i] = (uint32_t)b;
            keep[i] = 1;
        }
    }
    if (bad >= 0)
        return bt_fail(BT_ERR_FORMAT, std::string(path) + ": line " + std::to_string(bad + 1) +
                                          " is not \"u v\" with ids < 99999999");
    uint64_t k = 0;
    for (uint64_t i = 0; i < lines.size(); i++)
        if (keep[i]) { us[k] = us[i]; vs[k] = vs[i]; k++; }
    return bt_graph_from_edges(us.data(), vs.data(), k, out);
}

extern "C" bt_status bt_graph_save_bin(const bt_graph *g, const char *path) {
    if (!g || !path) return bt_fail(BT_ERR_INVALID, "null argument");
    if (g->m > 0xffffffffull) return bt_fail(BT_ERR_INVALID, "edge count does not fit the .bin header");
    FILE *f = fopen(path, "wb");
    if (!f) return bt_fail(BT_ERR_IO, std::string("cannot open ") + path + ": " + strerror(errno));
    uint32_t hdr[5] = {g->u_num, g->l_num, g->u_max, (uint32_t)g->m,
                       (uint32_t)std::min<uint64_t>(g->support_max, 0xffffffffull)};
    bool ok = fwrite(hdr, 4, 5, f) == 5;
    auto put = [&](const std::vector<uint32_t> &a, uint64_t count) {
        if (!ok) return;
        if (count == 0) return;
        if (a.size() >= count) ok = fwrite(a.data(), 4, count, f) == count;
        else {
            std::vector<uint32_t> z(count, 0);
            ok = fwrite(z.data(), 4, count, f) == count;
        }
    };
    put(g->neighbors, 2 * g->m);
    put(g->offsets, (uint64_t)g->n + 1);
    put(g->degrees, g->n);
    put(g->edge_support_raw, g->m);
    put(g->edges, 2 * g->m);
    put(g->edge_ids, 2 * g->m);
    put(g->bitruss_raw, g->m);
    if (fclose(f) != 0) ok = false;
    if (!ok) return bt_fail(BT_ERR_IO, std::string("write failed on ") + path);
    return BT_OK;
}

extern "C" bt_status bt_graph_load_bin(const char *path, bt_graph **out) {
    if (!path || !out) return bt_fail(BT_ERR_INVALID, "null argument");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return bt_fail(BT_ERR_IO, std::string("cannot open ") + path + ": " + strerror(errno));
    uint32_t hdr[5];
    if (fread(hdr, 4, 5, f) != 5) {
        fclose(f);
        return bt_fail(BT_ERR_FORMAT, std::string(path) + ": truncated header");
    }
    uint64_t u_num = hdr[0], l_num = hdr[1], m = hdr[3];
    uint64_t n = u_num + l_num;
    uint64_t expect = 20 + 4 * (2 * m + (n + 1) + n + m + 2 * m + 2 * m + m);
    fseek(f, 0, SEEK_END);
    long long fsz = ftell(f);
    fseek(f, 20, SEEK_SET);
    if (n > 0xffffffffull || fsz < 0 || (uint64_t)fsz != expect) {
        fclose(f);
        return bt_fail(BT_ERR_FORMAT, std::string(path) + ": size " + std::to_string(fsz) +
                                          " does not match header (expected " +
                                          std::to_string(expect) + ")");
    }
    std::unique_ptr<bt_graph> g(new (std::nothrow) bt_graph());
    if (!g) { fclose(f); return bt_fail(BT_ERR_HOST_MEMORY, "host allocation failed"); }
    try {
        g->neighbors.resize(2 * m);
        g->offsets.resize(n + 1);
        g->degrees.resize(n);
        g->edge_support_raw.resize(m);
        g->edges.resize(2 * m);
        g->edge_ids.resize(2 * m);
        g->bitruss_raw.resize(m);
    } catch (const std::bad_alloc &) {
        fclose(f);
        return bt_fail(BT_ERR_HOST_MEMORY, "host allocation failed");
    }
    bool ok = true;
    auto get = [&](std::vector<uint32_t> &a) {
        if (ok && !a.empty()) ok = fread(a.data(), 4, a.size(), f) == a.size();
    };
    get(g->neighbors);
    get(g->offsets);
    get(g->degrees);
    get(g->edge_support_raw);
    get(g->edges);
    get(g->edge_ids);
    get(g->bitruss_raw);
    fclose(f);
    if (!ok) return bt_fail(BT_ERR_IO, std::string("read failed on ") + path);
    g->u_num = (uint32_t)u_num;
    g->l_num = (uint32_t)l_num;
    g->u_max = hdr[2];
    g->n = (uint32_t)n;
    g->m = m;
    g->support_max = hdr[4];
    // structural checks the reference only does under CHECK_GRAPH (graph.cpp:13-52)
    if (g->offsets[0] != 0 || g->offsets[n] != 2 * m)
        return bt_fail(BT_ERR_FORMAT, std::string(path) + ": offsets do not span 2m slots");
    for (uint64_t x = 0; x < n; x++) {
        if (g->offsets[x + 1] < g->offsets[x] || g->offsets[x + 1] - g->offsets[x] != g->degrees[x])
            return bt_fail(BT_ERR_FORMAT, std::string(path) + ": offsets/degrees inconsistent at vertex " +
                                              std::to_string(x));
    }
    for (uint64_t s = 0; s < 2 * m; s++) {
        if (g->neighbors[s] >= n || g->edge_ids[s] >= m)
            return bt_fail(BT_ERR_FORMAT, std::string(path) + ": neighbour or edge id out of range");
    }
    for (uint64_t e = 0; e < m; e++) {
        if (g->edges[2 * e] >= u_num || g->edges[2 * e + 1] < u_num || g->edges[2 * e + 1] >= n)
            return bt_fail(BT_ERR_FORMAT, std::string(path) + ": edge endpoints out of range");
    }
    *out = g.release();
    return BT_OK;
}

extern "C" bt_status bt_graph_get_view(const bt_graph *g, bt_graph_view *out) {
    if (!g || !out) return bt_fail(BT_ERR_INVALID, "null argument");
    out->u_num = g->u_num;
    out->l_num = g->l_num;
    out->u_max = g->u_max;
    out->n = g->n;
    out->m = g->m;
    out->support_max = g->support_max;
    out->offsets = g->offsets.data();
    out->neighbors = g->neighbors.data();
    out->degrees = g->degrees.data();
    out->edges = g->edges.data();
    out->edge_ids = g->edge_ids.data();
    return BT_OK;
}

extern "C" void bt_graph_free(bt_graph *g) { delete g; }
