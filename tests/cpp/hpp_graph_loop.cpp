// Drives the C++ drop-in header (include/bitruss.hpp) the way a maintainer's
// loop over graph files does: one stack Graph per iteration, so every
// iteration's Graph lives at the same address as the last one.  For each text
// file named on the command line (in order) it prints one line:
//   <butterflies> <levels> <bitruss numbers of the edges in edge-id order>
// Every Graph must be uploaded and decomposed itself; a stale resident graph
// would repeat the previous file's results.
#include <cstdio>

#include "bitruss.hpp"

int main(int argc, char **argv) {
    try {
        for (int i = 1; i < argc; i++) {
            bt::Graph g(argv[i], true);
            bt::bfc_vpp(&g);
            bt::bitruss_msp(&g);
            std::printf("%llu %u", (unsigned long long)g.butterflies, g.levels);
            for (uint64_t e = 0; e < g.m; e++) std::printf(" %u", g.bitruss[e]);
            std::printf("\n");
        }
    } catch (const bt::Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
