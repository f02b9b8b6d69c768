// coh.cpp -- command-line front end with the reference's flags (main.cu:27-133,
// src/util/utility.h:92-131):
//
//   coh --graph G.txt --bin G.bin              convert text to .bin
//   coh --graph G.bin --gpu --algo msp         run bfc | ebfc | hidx | msp
//       [--device D] [--device_info] [--threads N]
//
// Extra flags: --exact (msp with the corrected one-survivor rule) and
// --out FILE (write "u v value" per edge id; the reference keeps per-edge
// results in memory only).  --cpu is accepted for compatibility but this
// engine has no CPU algorithms; it prints a warning.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <map>
#include <string>

#include "../../include/bitruss.hpp"

namespace {

void log_line(const char *level, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
void log_line(const char *level, const char *fmt, ...) {
    char ts[32];
    time_t t = time(nullptr);
    strftime(ts, sizeof ts, "%Y-%m-%d %H:%M:%S", localtime(&t));
    printf("%s %-5s ", ts, level);
    va_list ap;
    va_start(ap, fmt);
    vprintf(fmt, ap);
    va_end(ap);
    printf("\n");
    fflush(stdout);
}

void usage() {
    printf("Usage: coh [--graph PATH] [--bin PATH] [--cpu] [--gpu] [--algo bfc|ebfc|hidx|msp]\n"
           "           [--threads N] [--device D] [--device_info] [--exact] [--out PATH]\n");
}

void device_info(int device) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) {
        log_line("WARN", "cannot query device %d", device);
        return;
    }
    printf("%-34s %s\n", "Device Number", std::to_string(device).c_str());
    printf("%-34s %s\n", "Device name", p.name);
    printf("%-34s %d\n", "Memory Bus Width (bits)", p.memoryBusWidth);
    printf("%-34s %zu\n", "Total global memory (bytes)", p.totalGlobalMem);
    printf("%-34s %.3f\n", "Total global memory (GB)", p.totalGlobalMem / (1024.0 * 1024.0 * 1024.0));
    printf("%-34s %d\n", "Number of SMs", p.multiProcessorCount);
    printf("%-34s %d%d\n", "Compute Capability", p.major, p.minor);
    printf("%-34s %zu\n", "Shared memory per block (bytes)", p.sharedMemPerBlock);
    printf("%-34s %d\n", "Max threads per SM", p.maxThreadsPerMultiProcessor);
    printf("%-34s %d\n", "Total max threads", p.maxThreadsPerMultiProcessor * p.multiProcessorCount);
}

bool write_out(const bt::Graph &g, const std::string &path, const uint64_t *v64, const uint32_t *v32) {
    FILE *f = fopen(path.c_str(), "w");
    if (!f) return false;
    for (uint64_t e = 0; e < g.m; e++)
        fprintf(f, "%u %u %llu\n", g.edges[2 * e], g.edges[2 * e + 1],
                (unsigned long long)(v64 ? v64[e] : v32[e]));
    return fclose(f) == 0;
}

}  // namespace

int main(int argc, char **argv) {
    std::map<std::string, std::string> opt;
    const char *flags[] = {"--device_info", "--cpu", "--gpu", "--exact"};
    const char *valued[] = {"--device", "--graph", "--bin", "--algo", "--threads", "--out"};
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "-h" || a == "--help") {
            usage();
            return 0;
        }
        bool ok = false;
        for (const char *f : flags)
            if (a == f) { opt[a] = "1"; ok = true; }
        for (const char *f : valued)
            if (a == f) {
                if (i + 1 >= argc) {
                    log_line("ERROR", "error: %s: expected 1 argument", f);
                    usage();
                    return EXIT_FAILURE;
                }
                opt[a] = argv[++i];
                ok = true;
            }
        if (!ok) {
            log_line("ERROR", "error: Unknown argument: %s", a.c_str());
            usage();
            return EXIT_FAILURE;
        }
    }
    int device_count = 0, device = 0;
    if (cudaGetDeviceCount(&device_count) != cudaSuccess) device_count = 0;
    if (device_count == 0) log_line("WARN", "no gpu devices supporting CUDA.");
    if (opt.count("--device")) {
        device = atoi(opt["--device"].c_str());
        if (device >= device_count) {
            log_line("ERROR", "error: gpu device id %d is not available", device);
            return EXIT_FAILURE;
        }
    }
    if (opt.count("--device_info") && device_count) device_info(device);
    if (!opt.count("--graph")) return 0;
    const std::string algo = opt.count("--algo") ? opt["--algo"] : "msp";
    try {
        if (opt.count("--bin")) {
            log_line("INFO", "processing graph file: %s", opt["--graph"].c_str());
            bt::Graph g(opt["--graph"], true);
            log_line("INFO", "graph with upper: %u, lower: %u, vertices: %u, edges: %llu", g.u_num, g.l_num,
                     g.n, (unsigned long long)g.m);
            log_line("INFO", "convert graph to binary file: %s", opt["--bin"].c_str());
            g.graph_to_bin(opt["--bin"]);
            return 0;
        }
        log_line("INFO", "loading graph from binary file: %s", opt["--graph"].c_str());
        bt::Graph g(opt["--graph"], false);
        log_line("INFO", "graph with upper: %u, lower: %u, vertices: %u, edges: %llu", g.u_num, g.l_num, g.n,
                 (unsigned long long)g.m);
        if (opt.count("--cpu"))
            log_line("WARN", "--cpu: this engine runs the algorithms on the GPU only (use --gpu)");
        if (!opt.count("--gpu")) return 0;
        if (device_count == 0) {
            log_line("ERROR", "error: no gpu devices supporting CUDA to run algorithms.");
            return EXIT_FAILURE;
        }
        g.on_device(device);
        auto t0 = std::chrono::steady_clock::now();
        const std::string out = opt.count("--out") ? opt["--out"] : "";
        bool ok = true;
        if (algo == "ebfc") {
            bt::bfc_evpp(&g);
            log_line("INFO", "butterfly counting with vertex priority on gpu, max edge support: %llu, "
                             "butterfly count: %llu",
                     (unsigned long long)g.support_max, (unsigned long long)g.butterflies);
            if (!out.empty()) ok = write_out(g, out, g.edge_support.data(), nullptr);
        } else if (algo == "bfc") {
            bt::bfc_vpp(&g);
            log_line("INFO", "butterfly counting with vertex priority on gpu, btf number: %llu",
                     (unsigned long long)g.butterflies);
        } else if (algo == "hidx") {
            bt::g_bitruss_hindex(&g);
            uint32_t kmax = g.m ? *std::max_element(g.bitruss.begin(), g.bitruss.end()) : 0;
            log_line("INFO", "k-bitruss max value %u, with %u rounds", kmax, g.rounds);
            if (!out.empty()) ok = write_out(g, out, nullptr, g.bitruss.data());
        } else {
            if (opt.count("--exact")) bt::bitruss_msp_exact(&g);
            else bt::bitruss_msp(&g);
            log_line("INFO", "bitruss msp with %u levels", g.levels);
            if (!out.empty()) ok = write_out(g, out, nullptr, g.bitruss.data());
        }
        double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        log_line("INFO", "%s finished in %.3f ms", algo.c_str(), ms);
        if (!ok) {
            log_line("ERROR", "error: cannot write %s", out.c_str());
            return EXIT_FAILURE;
        }
    } catch (const bt::Error &e) {
        log_line("ERROR", "error: %s", e.what());
        return EXIT_FAILURE;
    }
    return 0;
}
