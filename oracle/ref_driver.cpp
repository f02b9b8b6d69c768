/*
 * C entry points over the reference's own CPU code, for validating the oracle
 * restatement (oracle/bt_oracle.c).  TEST INFRASTRUCTURE ONLY: built into
 * oracle/_ref/ from the reference sources where they lie, never shipped.
 *
 *   ref_convert  Graph(text, true) + graph_to_bin      graph.cpp:261-318
 *   ref_run      Graph(bin, false) + one CPU algorithm  main.cu:91-108
 */
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "bitruss/bitruss.cuh"

/* defined in the reference's util/log.cpp, not declared in its log.h */
void log_set_fp(FILE *fp);
void log_set_quiet(int enable);

extern "C" int ref_convert(const char *text_path, const char *bin_path) {
    log_set_quiet(1);
    Graph g(text_path, true);
    g.graph_to_bin(bin_path);
    return 0;
}

/*
 * algo: 0 ebfc, 1 bfc, 2 hidx, 3 msp.  result (m entries): ebfc/msp ->
 * edge_support, hidx -> bitruss.  log_path receives the reference's log lines
 * (butterfly count, levels).  Returns m, or -1.
 */
extern "C" long long ref_run(const char *bin_path, int algo, int threads,
                             long long *result, long long cap, const char *log_path) {
    log_set_quiet(1);
    FILE *lf = fopen(log_path, "w");
    if (!lf) return -1;
    log_set_fp(lf);
    long long m;
    {
        Graph g(bin_path, false);
        m = g.m;
        if ((long long)g.m > cap) { log_set_fp(nullptr); fclose(lf); return -1; }
        if (algo == 0) ebfc(&g, threads);
        else if (algo == 1) bfc(&g, threads);
        else if (algo == 2) c_bitruss_hindex(g, threads);
        else c_bitruss_msp(&g, threads);
        for (uint e = 0; e < g.m; e++)
            result[e] = algo == 2 ? (long long)g.bitruss[e] : (long long)g.edge_support[e];
    }
    log_set_fp(nullptr);
    fclose(lf);
    return m;
}
