// Test infrastructure only: command-line front end of the CPU oracle.
//
//   fsm_port <graph.bin> <min_support> <k> [--stats] [--stream-last [--shard i/S]]
//   fsm_port --canonical      (codes on stdin, one per line: len then 5 ints
//                              per edge; prints 1 or 0 per line)
//
// Prints one line per frequent canonical pattern in the reference's format and
// order (gspan.cu:67-77), then the reference's timing line (fsm.cu:37-40).
// With --stats, a JSON line with embedding counts goes to stderr.  With
// --stream-last, the last level is counted without materialising it (same
// output; see mine_all); --shard i/S extends only the i-th of S slices of that
// level's parent rows (for timing a job in slices).
#include "gspan_port.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <omp.h>

static int canonical_mode()
{
    int len;
    while (std::scanf("%d", &len) == 1) {
        port::Code code(len);
        for (auto& e : code)
            if (std::scanf("%d%d%d%d%d", &e.from, &e.to, &e.fl, &e.el, &e.tl) != 5) return 1;
        std::printf("%d\n", port::is_canonical(code) ? 1 : 0);
    }
    return 0;
}

int main(int argc, char** argv)
{
    if (argc == 2 && std::strcmp(argv[1], "--canonical") == 0) return canonical_mode();
    if (argc < 4) {
        std::printf("usage: %s input_graph min_support k [--stats] [--stream-last]\n", argv[0]);
        return 2;
    }
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    port::Graph g;
    if (!port::load_bin(argv[1], g)) {
        std::fprintf(stderr, "failed to load %s\n", argv[1]);
        return 1;
    }
    const int min_sup = std::atoi(argv[2]);
    const int k = std::atoi(argv[3]);
    bool want_stats = false, stream_last = false;
    port::Shard shard;
    for (int a = 4; a < argc; ++a) {
        if (std::strcmp(argv[a], "--stats") == 0) want_stats = true;
        else if (std::strcmp(argv[a], "--stream-last") == 0) stream_last = true;
        else if (std::strcmp(argv[a], "--shard") == 0 && a + 1 < argc &&
                 std::sscanf(argv[a + 1], "%d/%d", &shard.index, &shard.count) == 2 && shard.count >= 1 &&
                 shard.index >= 0 && shard.index < shard.count)
            ++a;
        else {
            std::fprintf(stderr, "unknown option %s\n", argv[a]);
            return 2;
        }
    }
    const auto t1 = clk::now();
    port::Stats st;
    port::mine_all(g, k, min_sup, [](const port::Code& code, int sup) {
        for (const auto& e : code) std::printf("(%d %d %d %d %d)", e.from, e.to, e.fl, e.el, e.tl);
        std::printf(": %d\n", sup);
    }, &st, stream_last, shard);
    const auto t2 = clk::now();
    const double load_s = std::chrono::duration<double>(t1 - t0).count();
    const double fsm_s = std::chrono::duration<double>(t2 - t1).count();
    std::printf("load: %lfs prepare: %lfs fsm: %lfs\n", load_s, 0.0, fsm_s);
    if (want_stats)
        std::fprintf(stderr,
                     "{\"seeds\": %llu, \"extended\": %llu, \"patterns\": %llu, \"support_calls\": %llu, "
                     "\"fsm_s\": %.6f, \"last_s\": %.6f, \"last_extended\": %llu, \"threads\": %d}\n",
                     (unsigned long long)st.seeds, (unsigned long long)st.extended,
                     (unsigned long long)st.patterns, (unsigned long long)st.support_calls, fsm_s, st.last_s,
                     (unsigned long long)st.last_extended, omp_get_max_threads());
    return 0;
}
