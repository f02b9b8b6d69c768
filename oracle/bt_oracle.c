/*
 * bt_oracle.c -- CPU restatement of the reference bitruss algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only the test suite, the package's smoke check and the CPU
 * baseline leg of the benchmark load it, and only to check or time the CUDA
 * engine; the engine never calls it and has no CPU fallback.
 *
 * It restates, in plain C with OpenMP, the reference's CPU code paths
 * (ShunyangLi/GPU_Bitruss):
 *   og_build_csr    src/graph/graph.cpp:74-242   (Graph::process_graph)
 *   og_ebfc         src/bfc/cpu_bfc.cpp:24-122   (ebfc)
 *   og_bfc          src/bfc/cpu_bfc.cpp:137-203  (bfc)
 *   og_hidx         src/bitruss/cpu_bitruss.cpp:152-266 (compute_bitruss_hindex,
 *                                                      c_bitruss_hindex)
 *   og_msp          src/bitruss/cpu_bitruss.cpp:268-624 (c_bitruss_msp and its
 *                                                      helpers)
 * with one deliberate change: supports are uint64 instead of int32 (the
 * reference's int32 overflows on power-law graphs with hub-hub supports above
 * 2^31).  On every graph whose supports fit in int32 the results are
 * bit-identical to the reference; this is checked against the reference's own
 * sources compiled by oracle/Makefile (target "ref").
 *
 * og_msp takes a mode: the corrected peel rule (mode bit 0) must equal og_hidx;
 * the position-table intersection (mode bit 1) has the semantics of the
 * reference's merge but finishes on the large configurations, and is
 * cross-checked against the merge.
 */
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define OG_MAX_IDS 99999999u /* src/util/config.h:6 */

typedef struct {
    uint32_t n, u_num;
    uint64_t m;
    const uint32_t *offsets;   /* n+1 */
    const uint32_t *neighbors; /* 2m  */
    const uint32_t *degrees;   /* n   */
    const uint32_t *edges;     /* 2m: (u, v) of edge e at 2e, 2e+1 */
    const uint32_t *edge_ids;  /* 2m: edge id of each CSR slot */
} og_graph;

static void og_set_threads(int threads) {
    if (threads > 0) omp_set_num_threads(threads);
}

/* ------------------------------------------------------------------------ */
/* CSR construction: graph.cpp:74-242                                        */
/* ------------------------------------------------------------------------ */

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

/*
 * Build the reference CSR from an edge list in file order.
 * U and V ids are numbered by first appearance (graph.cpp:99-105); V ids are
 * offset by u_num (:118-131); rows are sorted (:134-143); edge e is the e-th
 * slot in U-major order (:178-194); the V-side edge_ids are found by the same
 * binary search as the reference (:196-228).
 * Output arrays must be sized: offsets n_max+1, degrees n_max, neighbors/
 * edges/edge_ids 2m, with n_max = distinct U + distinct V <= 2m.
 * Returns 0, or -1 if an id is >= MAX_IDS (the reference indexes a MAX_IDS
 * table with it).
 */
int og_build_csr(const uint32_t *us, const uint32_t *vs, uint64_t m,
                 uint32_t *u_num_out, uint32_t *l_num_out,
                 uint32_t *offsets, uint32_t *degrees, uint32_t *neighbors,
                 uint32_t *edges, uint32_t *edge_ids) {
    uint32_t max_u = 0, max_v = 0;
    for (uint64_t i = 0; i < m; i++) {
        if (us[i] >= OG_MAX_IDS || vs[i] >= OG_MAX_IDS) return -1;
        if (us[i] > max_u) max_u = us[i];
        if (vs[i] > max_v) max_v = vs[i];
    }
    uint32_t *uid = malloc(sizeof(uint32_t) * ((uint64_t)max_u + 1));
    uint32_t *lid = malloc(sizeof(uint32_t) * ((uint64_t)max_v + 1));
    memset(uid, 0xff, sizeof(uint32_t) * ((uint64_t)max_u + 1));
    memset(lid, 0xff, sizeof(uint32_t) * ((uint64_t)max_v + 1));
    uint32_t u_num = 0, l_num = 0;
    uint32_t *eu = malloc(sizeof(uint32_t) * (m ? m : 1));
    uint32_t *ev = malloc(sizeof(uint32_t) * (m ? m : 1));
    for (uint64_t i = 0; i < m; i++) {
        if (uid[us[i]] == UINT32_MAX) uid[us[i]] = u_num++;
        if (lid[vs[i]] == UINT32_MAX) lid[vs[i]] = l_num++;
        eu[i] = uid[us[i]];
        ev[i] = lid[vs[i]];
    }
    uint32_t n = u_num + l_num;
    memset(degrees, 0, sizeof(uint32_t) * n);
    for (uint64_t i = 0; i < m; i++) {
        degrees[eu[i]]++;
        degrees[u_num + ev[i]]++;
    }
    offsets[0] = 0;
    for (uint32_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + degrees[i];
    uint32_t *fill = malloc(sizeof(uint32_t) * (n ? n : 1));
    memcpy(fill, offsets, sizeof(uint32_t) * n);
    for (uint64_t i = 0; i < m; i++) {
        neighbors[fill[eu[i]]++] = u_num + ev[i];
        neighbors[fill[u_num + ev[i]]++] = eu[i];
    }
    for (uint32_t x = 0; x < n; x++)
        qsort(neighbors + offsets[x], degrees[x], sizeof(uint32_t), cmp_u32);
    uint64_t e = 0;
    for (uint32_t u = 0; u < u_num; u++) {
        for (uint32_t i = 0; i < degrees[u]; i++, e++) {
            edge_ids[offsets[u] + i] = (uint32_t)e;
            edges[2 * e] = u;
            edges[2 * e + 1] = neighbors[offsets[u] + i];
        }
    }
    for (uint32_t v = u_num; v < n; v++) {
        for (uint32_t i = 0; i < degrees[v]; i++) {
            uint32_t u = neighbors[offsets[v] + i];
            const uint32_t *row = neighbors + offsets[u];
            int left = 0, right = (int)degrees[u] - 1;
            while (left <= right) {
                int mid = left + ((right - left) >> 1);
                if (row[mid] == v) {
                    edge_ids[offsets[v] + i] = edge_ids[offsets[u] + mid];
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
    free(uid); free(lid); free(eu); free(ev); free(fill);
    *u_num_out = u_num;
    *l_num_out = l_num;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Butterfly counting: cpu_bfc.cpp                                            */
/* ------------------------------------------------------------------------ */

/* p(a) > p(b) with priority (degree, id): cpu_bfc.cpp:59-60 */
static inline int og_higher(const uint32_t *deg, uint32_t a, uint32_t b) {
    return deg[a] > deg[b] || (deg[a] == deg[b] && a > b);
}

/*
 * Per-edge butterfly support and global count: cpu_bfc.cpp:24-122.
 * Each vertex u counts, in last_cnt[w], the wedges u-v-w with u the highest
 * priority vertex; a butterfly adds C(c,2) to the count and c-1 to both
 * wedge edges.  sup must hold m entries (zeroed here).
 */
void og_ebfc(const og_graph *g, int threads, uint64_t *sup, uint64_t *count_out) {
    og_set_threads(threads);
    memset(sup, 0, sizeof(uint64_t) * g->m);
    uint64_t total = 0;
    const uint32_t *deg = g->degrees, *nbr = g->neighbors, *off = g->offsets;
#pragma omp parallel reduction(+ : total)
    {
        uint32_t *last_cnt = calloc(g->n ? g->n : 1, sizeof(uint32_t));
        uint32_t *last_use = malloc(sizeof(uint32_t) * (g->n ? g->n : 1));
        uint32_t used = 0;
#pragma omp for schedule(dynamic, 64)
        for (uint32_t u = 0; u < g->n; u++) {
            for (uint32_t j = 0; j < used; j++) last_cnt[last_use[j]] = 0;
            used = 0;
            for (uint32_t i = off[u]; i < off[u + 1]; i++) {
                uint32_t v = nbr[i];
                if (!og_higher(deg, u, v)) continue;
                for (uint32_t j = off[v]; j < off[v + 1]; j++) {
                    uint32_t w = nbr[j];
                    if (!og_higher(deg, u, w)) continue;
                    total += last_cnt[w];
                    if (++last_cnt[w] == 1) last_use[used++] = w;
                }
            }
            for (uint32_t i = off[u]; i < off[u + 1]; i++) {
                uint32_t v = nbr[i];
                if (!og_higher(deg, u, v)) continue;
                for (uint32_t j = off[v]; j < off[v + 1]; j++) {
                    uint32_t w = nbr[j];
                    if (!og_higher(deg, u, w)) continue;
                    uint64_t dlt = (uint64_t)last_cnt[w] - 1;
                    if (last_cnt[w] == 0 || dlt == 0) continue;
                    uint32_t uv = g->edge_ids[i], vw = g->edge_ids[j];
#pragma omp atomic
                    sup[uv] += dlt;
#pragma omp atomic
                    sup[vw] += dlt;
                }
            }
        }
        free(last_cnt);
        free(last_use);
    }
    *count_out = total;
}

/* Global butterfly count only: cpu_bfc.cpp:137-203. */
uint64_t og_bfc(const og_graph *g, int threads) {
    og_set_threads(threads);
    uint64_t total = 0;
    const uint32_t *deg = g->degrees, *nbr = g->neighbors, *off = g->offsets;
#pragma omp parallel reduction(+ : total)
    {
        uint32_t *last_cnt = calloc(g->n ? g->n : 1, sizeof(uint32_t));
        uint32_t *last_use = malloc(sizeof(uint32_t) * (g->n ? g->n : 1));
        uint32_t used = 0;
#pragma omp for schedule(dynamic, 64)
        for (uint32_t u = 0; u < g->n; u++) {
            for (uint32_t j = 0; j < used; j++) last_cnt[last_use[j]] = 0;
            used = 0;
            for (uint32_t i = off[u]; i < off[u + 1]; i++) {
                uint32_t v = nbr[i];
                if (!og_higher(deg, u, v)) continue;
                for (uint32_t j = off[v]; j < off[v + 1]; j++) {
                    uint32_t w = nbr[j];
                    if (!og_higher(deg, u, w)) continue;
                    total += last_cnt[w];
                    if (++last_cnt[w] == 1) last_use[used++] = w;
                }
            }
        }
        free(last_cnt);
        free(last_use);
    }
    return total;
}

/* ------------------------------------------------------------------------ */
/* h-index bitruss: cpu_bitruss.cpp:152-266                                   */
/* ------------------------------------------------------------------------ */

static int cmp_u64_desc(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x < y) - (x > y);
}

/*
 * One edge of one h-index round: cpu_bitruss.cpp:152-221.  Collects, over the
 * butterflies (u,v,w,x) of edge uv found by merging N(w) with N(u), the value
 * min(prev[ux], prev[wx], prev[wv]) when all three are non-zero, and returns
 * the h-index of that list (sorted descending, first i with list[i] < i+1).
 */
static uint64_t og_hidx_edge(const og_graph *g, const uint64_t *prev, uint64_t e,
                             uint64_t **buf, uint64_t *cap) {
    if (prev[e] == 0) return 0;
    uint32_t u = g->edges[2 * e], v = g->edges[2 * e + 1];
    const uint32_t *un = g->neighbors + g->offsets[u];
    uint32_t ul = g->offsets[u + 1] - g->offsets[u];
    uint64_t cnt = 0;
    for (uint32_t i = g->offsets[v]; i < g->offsets[v + 1]; i++) {
        uint32_t w = g->neighbors[i];
        if (w == u) continue;
        uint32_t wv = g->edge_ids[i];
        const uint32_t *wn = g->neighbors + g->offsets[w];
        uint32_t wl = g->offsets[w + 1] - g->offsets[w];
        uint32_t j = 0, k = 0;
        while (j < wl && k < ul) {
            if (wn[j] < un[k]) { j++; continue; }
            if (wn[j] > un[k]) { k++; continue; }
            if (wn[j] == v) { j++; k++; continue; }
            uint32_t wx = g->edge_ids[g->offsets[w] + j];
            uint32_t ux = g->edge_ids[g->offsets[u] + k];
            j++; k++;
            if (prev[ux] == 0 || prev[wx] == 0 || prev[wv] == 0) continue;
            uint64_t mv = prev[ux];
            if (prev[wx] < mv) mv = prev[wx];
            if (prev[wv] < mv) mv = prev[wv];
            if (cnt == *cap) {
                *cap = *cap ? *cap * 2 : 1024;
                *buf = realloc(*buf, sizeof(uint64_t) * *cap);
            }
            (*buf)[cnt++] = mv;
        }
    }
    qsort(*buf, cnt, sizeof(uint64_t), cmp_u64_desc);
    uint64_t h = 0;
    for (uint64_t i = 0; i < cnt; i++) {
        if ((*buf)[i] >= i + 1) h = i + 1;
        else break;
    }
    return h;
}

/*
 * h-index bitruss: cpu_bitruss.cpp:227-266.  Starts from the butterfly
 * supports and iterates synchronous h-index rounds to the fixpoint; the
 * fixpoint is the true bitruss number of every edge.  out: m entries.
 * Returns the number of rounds (the last round is the one with no change).
 */
uint32_t og_hidx(const og_graph *g, int threads, const uint64_t *sup, uint64_t *out) {
    og_set_threads(threads);
    uint64_t *prev = malloc(sizeof(uint64_t) * (g->m ? g->m : 1));
    uint64_t *curr = malloc(sizeof(uint64_t) * (g->m ? g->m : 1));
    memcpy(prev, sup, sizeof(uint64_t) * g->m);
    uint32_t rounds = 0;
    int converge = 0;
    while (!converge) {
        converge = 1;
        rounds++;
#pragma omp parallel
        {
            uint64_t *buf = NULL, cap = 0;
            int local = 1;
#pragma omp for schedule(dynamic, 16)
            for (uint64_t e = 0; e < g->m; e++) {
                curr[e] = og_hidx_edge(g, prev, e, &buf, &cap);
                if (curr[e] != prev[e]) local = 0;
            }
            if (!local) {
#pragma omp atomic write
                converge = 0;
            }
            free(buf);
        }
        uint64_t *t = prev; prev = curr; curr = t;
    }
    memcpy(out, prev, sizeof(uint64_t) * g->m);
    free(prev);
    free(curr);
    return rounds;
}

/* ------------------------------------------------------------------------ */
/* Multi-stage peeling (GBiD): cpu_bitruss.cpp:268-624                        */
/* ------------------------------------------------------------------------ */

typedef struct {
    uint64_t *sup;
    uint8_t *processed, *in_curr, *in_next;
    uint32_t *next;
    uint64_t next_len;
    uint64_t level;
    /* table mode only: the "low" list of live edges with support < low_bound
     * (see og_msp); NULL in merge mode */
    uint32_t *low;
    uint64_t low_len, low_bound;
} og_peel;

/* update_edge_support, cpu_bitruss.cpp:302-324: decrement, push the edge to
 * the next frontier when the old value was level+1, clamp at level.  In table
 * mode a decrement that takes the edge below low_bound also appends it to the
 * low list (low_bound > level, so that decrement is never clamped). */
static inline void og_dec(og_peel *p, uint32_t e) {
    uint64_t old;
#pragma omp atomic capture
    { old = p->sup[e]; p->sup[e]--; }
    if (old == p->level + 1) {
        uint64_t slot;
#pragma omp atomic capture
        slot = p->next_len++;
        p->next[slot] = e;
        p->in_next[e] = 1;
    }
    if (old <= p->level) {
#pragma omp atomic
        p->sup[e]++;
    }
    if (p->low && old == p->low_bound) {
        uint64_t slot;
#pragma omp atomic capture
        slot = p->low_len++;
        p->low[slot] = e;
    }
}

/*
 * The butterfly rule of one peeled edge uv, cpu_bitruss.cpp:328-378 (and
 * bitruss_msp.cu:126-184).  P is the set of the three other edges that are
 * not in the current frontier.
 *   |P|=3: decrement wv, wx, ux.
 *   |P|=2: decrement both iff uv is below the other frontier edge.
 *   |P|=1: the reference's chain rule: wx iff uv<ux<wv, wv iff uv<ux<wx,
 *          ux iff uv<wv<wx.  (exact == 0)
 *          The corrected rule decrements the survivor iff uv is the smallest
 *          of the three frontier edges.  (exact == 1)
 */
static inline int og_rule(og_peel *p, uint32_t uv, uint32_t wv, uint32_t wx, uint32_t ux,
                          int exact) {
    int pwv = !p->in_curr[wv], pwx = !p->in_curr[wx], pux = !p->in_curr[ux];
    int cnt = pwv + pwx + pux;
    int d = 0;  /* unit decrements applied (returned for the byte count) */
    if (cnt == 3) {
        og_dec(p, wv); og_dec(p, wx); og_dec(p, ux);
        d = 3;
    } else if (cnt == 2) {
        if (pwv && pwx && uv < ux) { og_dec(p, wv); og_dec(p, wx); d += 2; }
        if (pwv && pux && uv < wx) { og_dec(p, wv); og_dec(p, ux); d += 2; }
        if (pwx && pux && uv < wv) { og_dec(p, wx); og_dec(p, ux); d += 2; }
    } else if (cnt == 1) {
        if (!exact) {
            if (pwx && uv < ux && ux < wv) { og_dec(p, wx); d++; }
            if (pwv && uv < ux && ux < wx) { og_dec(p, wv); d++; }
            if (pux && uv < wv && wv < wx) { og_dec(p, ux); d++; }
        } else {
            if (pwx && uv < ux && uv < wv) { og_dec(p, wx); d++; }
            if (pwv && uv < ux && uv < wx) { og_dec(p, wv); d++; }
            if (pux && uv < wv && uv < wx) { og_dec(p, ux); d++; }
        }
    }
    return d;
}

/* Peel one frontier edge by merging N(w) with N(u) for every w in N(v):
 * cpu_bitruss.cpp:380-451 (peel_edges body). deg/nbr/eid are the current
 * (possibly compressed) rows. */
static void og_peel_edge_merge(const og_graph *g, og_peel *p, const uint32_t *deg,
                               const uint32_t *nbr, const uint32_t *eid, uint32_t uv,
                               int exact, uint64_t *acc) {
    uint32_t u = g->edges[2 * (uint64_t)uv], v = g->edges[2 * (uint64_t)uv + 1];
    const uint32_t *un = nbr + g->offsets[u];
    uint32_t ul = deg[u];
    for (uint32_t x = 0; x < deg[v]; x++) {
        uint32_t w = nbr[g->offsets[v] + x];
        if (w == u) continue;
        uint32_t wv = eid[g->offsets[v] + x];
        if (p->processed[wv]) continue;
        const uint32_t *wn = nbr + g->offsets[w];
        uint32_t wl = deg[w], j = 0, k = 0;
        while (j < wl && k < ul) {
            if (wn[j] < un[k]) { j++; continue; }
            if (wn[j] > un[k]) { k++; continue; }
            if (wn[j] == v) { j++; k++; continue; }
            uint32_t wx = eid[g->offsets[w] + j], ux = eid[g->offsets[u] + k];
            j++; k++;
            if (p->processed[ux] || p->processed[wx]) continue;
            acc[0]++;
            acc[1] += (uint64_t)og_rule(p, uv, wv, wx, ux, exact);
        }
    }
}

/* Two-hop sums of the current rows: two_hop[x] = sum of deg[y], y in N(x).
 * Rows change only at a compression, so this is recomputed after each. */
static void og_two_hop(const og_graph *g, const uint32_t *deg, const uint32_t *nbr,
                       uint64_t *two_hop) {
#pragma omp parallel for schedule(dynamic, 256)
    for (uint32_t x = 0; x < g->n; x++) {
        uint64_t s = 0;
        for (uint32_t i = 0; i < deg[x]; i++) s += deg[nbr[g->offsets[x] + i]];
        two_hop[x] = s;
    }
}

/* Slot of y in a sorted row of length d, or -1. */
static inline int64_t og_find(const uint32_t *row, uint32_t d, uint32_t y) {
    uint32_t lo = 0, hi = d;
    while (lo < hi) {
        uint32_t md = lo + ((hi - lo) >> 1);
        if (row[md] < y) lo = md + 1;
        else hi = md;
    }
    return lo < d && row[lo] == y ? (int64_t)lo : -1;
}

/*
 * Same butterflies as og_peel_edge_merge, found from the endpoint whose
 * two-hop sum is smaller (the pivot): each y in N(mid), mid in N(pivot), is
 * looked up in the row of the other endpoint (the anchor).  The lookup uses
 * a per-thread position table, pos[x] = 1 + slot of x in the anchor's row,
 * unless the anchor's row is long next to the probes (then filling the table
 * would cost more than the walk), in which case it is a binary search of the
 * sorted row.  A mid whose row is much longer than the anchor's is
 * intersected the other way round (the anchor's row walked, each y searched
 * in mid's sorted row).  Every butterfly of uv is visited exactly once either
 * way, so the decrements are the same.
 */
static void og_peel_edge_table(const og_graph *g, og_peel *p, const uint32_t *deg,
                               const uint32_t *nbr, const uint32_t *eid, const uint64_t *two_hop,
                               uint32_t uv, int exact, uint32_t *pos, uint64_t *acc) {
    uint32_t u = g->edges[2 * (uint64_t)uv], v = g->edges[2 * (uint64_t)uv + 1];
    uint64_t cost_v = two_hop[v], cost_u = two_hop[u];
    /* walk: iterate mid in N(piv)\anchor, probe N(mid) against N(anchor) */
    uint32_t piv = cost_v <= cost_u ? v : u;
    uint32_t anc = piv == v ? u : v;
    uint64_t probes = piv == v ? cost_v : cost_u;
    const uint32_t *arow = nbr + g->offsets[anc];
    const uint32_t ad = deg[anc];
    const int table = (uint64_t)ad <= 32 * probes;
    if (table)
        for (uint32_t i = 0; i < ad; i++) pos[arow[i]] = i + 1;
    for (uint32_t x = 0; x < deg[piv]; x++) {
        uint32_t mid = nbr[g->offsets[piv] + x];
        if (mid == anc) continue;
        uint32_t e_pm = eid[g->offsets[piv] + x];
        if (p->processed[e_pm]) continue;
        const uint32_t *mrow = nbr + g->offsets[mid];
        const uint32_t md = deg[mid];
        /* a mid row much longer than the anchor's is intersected the other
         * way: each y of the anchor's row is looked up in mid's sorted row */
        const int reverse = (uint64_t)md > 16 * (uint64_t)ad;
        const uint32_t len = reverse ? ad : md;
        for (uint32_t j = 0; j < len; j++) {
            uint32_t y = reverse ? arow[j] : mrow[j];
            if (y == piv) continue;
            int64_t jm, ka;
            if (reverse) {
                ka = j;
                jm = og_find(mrow, md, y);
            } else {
                jm = j;
                ka = table ? (int64_t)pos[y] - 1 : og_find(arow, ad, y);
            }
            if (jm < 0 || ka < 0) continue;
            uint32_t e_my = eid[g->offsets[mid] + (uint64_t)jm];
            uint32_t e_ay = eid[g->offsets[anc] + (uint64_t)ka];
            if (p->processed[e_ay] || p->processed[e_my]) continue;
            acc[0]++;
            /* name the edges as the reference does: w on u's side, x on v's */
            if (piv == v) acc[1] += (uint64_t)og_rule(p, uv, e_pm, e_my, e_ay, exact); /* mid=w, y=x */
            else acc[1] += (uint64_t)og_rule(p, uv, e_ay, e_my, e_pm, exact);          /* mid=x, y=w */
        }
    }
    if (table)
        for (uint32_t i = 0; i < ad; i++) pos[arow[i]] = 0;
}

/* ccompress_graph, cpu_bitruss.cpp:527-557: keep only edges with sup > level. */
static uint64_t og_compress(const og_graph *g, const uint64_t *sup, uint64_t level,
                            uint32_t *deg, uint32_t *nbr, uint32_t *eid) {
    uint64_t live = 0;
#pragma omp parallel for schedule(static) reduction(+ : live)
    for (uint32_t x = 0; x < g->n; x++) {
        uint32_t k = 0, base = g->offsets[x];
        for (uint32_t i = 0; i < deg[x]; i++) {
            uint32_t e = eid[base + i];
            if (sup[e] > level) {
                nbr[base + k] = nbr[base + i];
                eid[base + k] = e;
                k++;
            }
        }
        deg[x] = k;
        live += k;
    }
    return live / 2;
}

/*
 * Multi-stage peeling: c_bitruss_msp, cpu_bitruss.cpp:563-624.
 * sup: initial butterfly supports (m), overwritten with the result (the
 * reference leaves its result in edge_support).  mode 0: reference rule with
 * merge intersection; 1: corrected rule (merge); 2: reference rule with the
 * position-table intersection; 3: corrected rule with the table.
 * Compression follows the reference trigger (edge_num <= live/2 and
 * live >= m/10) and re-filters the current rows each time.
 * Returns the reference's "levels" figure (last level that peeled edges).
 * stats (optional, 8 entries): levels, sub-rounds, compressions, peeled edges,
 * then the algorithmic bytes of the peeling in the reference's own walk
 * (bitruss_msp.cu:187-274: for a frontier edge uv, u = its U end and v = its
 * V end, u's row is staged once, v's row is read with edge ids, and every
 * live w in N(v) minus u has its row merged with u's), with d_s(x) = the
 * number of x's edges unprocessed when sub-round s starts:
 *   [4] row bytes  = sum over sub-rounds s and uv in the frontier of s of
 *                    4 d_s(u) + 8 d_s(v) + sum_{live w in N(v), w != u} 4 d_s(w)
 *   [5] butterflies visited (all four edges unprocessed at the start of s)
 *   [6] unit decrements the rule applied
 *   [7] total = [4] + 8 [5] (two edge ids per butterfly) + 8 [6] (a support
 *       read-modify-write per decrement).
 * max_seconds > 0 bounds the run for timing samples: it stops after the first
 * sub-round that ends past the deadline (the result is then partial).
 */
uint64_t og_msp(const og_graph *g, int threads, uint64_t *sup, int mode, uint64_t *stats,
                double max_seconds) {
    og_set_threads(threads);
    int exact = mode & 1, table = (mode & 2) != 0;
    uint64_t m = g->m;
    og_peel p;
    p.sup = sup;
    p.processed = calloc(m ? m : 1, 1);
    p.in_curr = calloc(m ? m : 1, 1);
    p.in_next = calloc(m ? m : 1, 1);
    p.next = malloc(sizeof(uint32_t) * (m ? m : 1));
    uint32_t *curr = malloc(sizeof(uint32_t) * (m ? m : 1));
    uint32_t *deg = malloc(sizeof(uint32_t) * (g->n ? g->n : 1));
    uint32_t *nbr = malloc(sizeof(uint32_t) * (m ? 2 * m : 1));
    uint32_t *eid = malloc(sizeof(uint32_t) * (m ? 2 * m : 1));
    memcpy(deg, g->degrees, sizeof(uint32_t) * g->n);
    memcpy(nbr, g->neighbors, sizeof(uint32_t) * 2 * m);
    memcpy(eid, g->edge_ids, sizeof(uint32_t) * 2 * m);
    uint64_t subrounds = 0, compressions = 0, peeled = 0;

    /* process_support_zero, cpu_bitruss.cpp:268-283.  The unprocessed edges
     * are also kept in a compact list so a level scan costs O(live edges). */
    uint32_t *alive = malloc(sizeof(uint32_t) * (m ? m : 1));
    uint64_t alive_len = 0;
    int64_t edge_num = (int64_t)m;
    /* live degrees for the byte count: ldeg[x] = x's unprocessed edges */
    uint32_t *ldeg = malloc(sizeof(uint32_t) * (g->n ? g->n : 1));
    memcpy(ldeg, g->degrees, sizeof(uint32_t) * g->n);
    for (uint64_t e = 0; e < m; e++) {
        if (sup[e] == 0) {
            p.processed[e] = 1;
            edge_num--;
            ldeg[g->edges[2 * e]]--;
            ldeg[g->edges[2 * e + 1]]--;
        } else {
            alive[alive_len++] = (uint32_t)e;
        }
    }
    uint64_t row_bytes = 0, visited = 0, decs = 0;

    /* Table mode finds each level's frontier without scanning every live
     * edge (the reference scans all m edges per level, which is what makes a
     * 20M-edge graph with ~10^5 levels take hours).  The live edges are split
     * into a "low" list (support < low_bound) and a "high" list (the rest,
     * `alive`).  Supports only fall, and og_dec appends an edge to low when a
     * decrement takes it below low_bound, so every live edge with support
     * below low_bound is in low.  Hence when low holds a live edge the
     * smallest live support is in low; otherwise the high list is split again
     * at its minimum + width (width adapted to keep low near 2^16 entries).
     * Low may hold processed entries; they are dropped as they are met.
     * Levels with an empty frontier change nothing and are skipped.  The
     * n-sized position tables of the threads are allocated once. */
    uint32_t *low = NULL, **pos_of = NULL;
    uint64_t *two_hop = NULL;
    uint64_t width = 1;
    int nth = 1;
    p.low = NULL;
    p.low_len = 0;
    p.low_bound = 0;
    if (table) {
        low = malloc(sizeof(uint32_t) * (m ? m : 1));
        p.low = low;
        nth = omp_get_max_threads();
        pos_of = malloc(sizeof(uint32_t *) * (size_t)nth);
        for (int t = 0; t < nth; t++) pos_of[t] = calloc(g->n ? g->n : 1, sizeof(uint32_t));
        two_hop = malloc(sizeof(uint64_t) * (g->n ? g->n : 1));
        og_two_hop(g, deg, nbr, two_hop);
    }
    const uint64_t low_target = 1u << 16;

    uint64_t level = 1, live = m, last = 0;
    const double t_start = omp_get_wtime();
    int expired = 0;
    /* OG_MSP_PROGRESS=1: a progress line on stderr every 20,000 sub-rounds */
    const int progress = getenv("OG_MSP_PROGRESS") != NULL;
    while (edge_num > 0 && !expired) {
        uint64_t curr_len = 0;
        if (table) {
            uint64_t lo = UINT64_MAX;
            for (uint64_t i = 0; i < p.low_len; i++) {
                uint32_t e = low[i];
                if (!p.processed[e] && sup[e] < lo) lo = sup[e];
            }
            if (lo == UINT64_MAX) {
                /* low is dry: split the high list at its minimum + width */
                for (uint64_t i = 0; i < alive_len; i++) {
                    uint32_t e = alive[i];
                    if (!p.processed[e] && sup[e] < lo) lo = sup[e];
                }
                if (lo == UINT64_MAX) break; /* defensive: edge_num > 0 implies a live edge */
                p.low_bound = lo + width;
                p.low_len = 0;
                uint64_t k = 0;
                for (uint64_t i = 0; i < alive_len; i++) {
                    uint32_t e = alive[i];
                    if (p.processed[e]) continue;
                    if (sup[e] < p.low_bound) low[p.low_len++] = e;
                    else alive[k++] = e;
                }
                alive_len = k;
                if (p.low_len > 4 * low_target && width > 1) width >>= 1;
                else if (p.low_len < low_target / 4) width <<= 1;
            }
            level = lo; /* live supports never fall below the last level */
            p.level = level;
            /* the frontier: live low edges with support == level; the other
             * live low edges stay */
            uint64_t k = 0;
            for (uint64_t i = 0; i < p.low_len; i++) {
                uint32_t e = low[i];
                if (p.processed[e]) continue;
                if (sup[e] == level && !p.in_curr[e]) { p.in_curr[e] = 1; curr[curr_len++] = e; }
                else if (sup[e] != level) low[k++] = e;
            }
            p.low_len = k;
        } else {
            p.level = level;
            /* scan_edge, cpu_bitruss.cpp:285-299 */
            for (uint64_t i = 0; i < alive_len; i++) {
                uint32_t e = alive[i];
                if (sup[e] == level) { p.in_curr[e] = 1; curr[curr_len++] = e; }
            }
        }
        if (curr_len) last = level;
        while (curr_len) {
            edge_num -= (int64_t)curr_len;
            peeled += curr_len;
            subrounds++;
            if (progress && subrounds % 20000 == 0)
                fprintf(stderr, "og_msp: %llu sub-rounds, level %llu, %lld edges left, %.0f s\n",
                        (unsigned long long)subrounds, (unsigned long long)level,
                        (long long)edge_num, omp_get_wtime() - t_start);
            p.next_len = 0;
            uint64_t sr_bytes = 0, sr_visited = 0, sr_decs = 0;
#pragma omp parallel reduction(+ : sr_bytes, sr_visited, sr_decs)
            {
                uint32_t *pos = table ? pos_of[omp_get_thread_num()] : NULL;
#pragma omp for schedule(dynamic, 1)
                for (uint64_t i = 0; i < curr_len; i++) {
                    const uint32_t uv = curr[i];
                    /* the reference walk's row bytes for uv (see above) */
                    const uint32_t u = g->edges[2 * (uint64_t)uv], v = g->edges[2 * (uint64_t)uv + 1];
                    uint64_t b = 4ull * ldeg[u] + 8ull * ldeg[v];
                    for (uint32_t x = 0; x < deg[v]; x++) {
                        const uint32_t w = nbr[g->offsets[v] + x];
                        if (w != u && !p.processed[eid[g->offsets[v] + x]]) b += 4ull * ldeg[w];
                    }
                    sr_bytes += b;
                    uint64_t acc[2] = {0, 0};
                    if (table) og_peel_edge_table(g, &p, deg, nbr, eid, two_hop, uv, exact, pos, acc);
                    else og_peel_edge_merge(g, &p, deg, nbr, eid, uv, exact, acc);
                    sr_visited += acc[0];
                    sr_decs += acc[1];
                }
            }
            row_bytes += sr_bytes;
            visited += sr_visited;
            decs += sr_decs;
            for (uint64_t i = 0; i < curr_len; i++) {
                p.processed[curr[i]] = 1;
                p.in_curr[curr[i]] = 0;
                ldeg[g->edges[2 * (uint64_t)curr[i]]]--;
                ldeg[g->edges[2 * (uint64_t)curr[i] + 1]]--;
            }
            /* swap(curr, next), swap(is_in_curr, is_in_next) */
            memcpy(curr, p.next, sizeof(uint32_t) * p.next_len);
            curr_len = p.next_len;
            uint8_t *t = p.in_curr; p.in_curr = p.in_next; p.in_next = t;
            for (uint64_t i = 0; i < curr_len; i++) p.in_next[curr[i]] = 0;
            if (max_seconds > 0 && omp_get_wtime() - t_start > max_seconds) {
                expired = 1;
                break;
            }
        }
        if (!table) {
            uint64_t k = 0;
            for (uint64_t i = 0; i < alive_len; i++)
                if (!p.processed[alive[i]]) alive[k++] = alive[i];
            alive_len = k;
        }
        if ((double)edge_num <= (double)live * 0.5 && (double)live >= (double)m * 0.1) {
            live = og_compress(g, sup, level, deg, nbr, eid);
            compressions++;
            if (table) og_two_hop(g, deg, nbr, two_hop);
        }
        level++;
    }
    free(alive);
    free(low);
    free(two_hop);
    if (pos_of) {
        for (int t = 0; t < nth; t++) free(pos_of[t]);
        free(pos_of);
    }
    if (stats) {
        stats[0] = last;
        stats[1] = subrounds;
        stats[2] = compressions;
        stats[3] = peeled;
        stats[4] = row_bytes;
        stats[5] = visited;
        stats[6] = decs;
        stats[7] = row_bytes + 8 * visited + 8 * decs;
    }
    free(ldeg);
    free(p.processed); free(p.in_curr); free(p.in_next); free(p.next);
    free(curr); free(deg); free(nbr); free(eid);
    return last;
}
