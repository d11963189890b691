// `fsm <graph.bin> <min_support> <k>`: the reference's mining command
// (fsm.cu:11-43) on the GPU miner.  Prints the pattern lines, then the same
// "load: ... prepare: ... fsm: ..." timing line.  The reference tests
// `argc < 3` but reads argv[3]; this one asks for all three arguments.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>

#include "graph.h"
#include "gspan.h"

int main(int argc, char* argv[])
{
    if (argc < 4) {
        std::printf("usage: %s input_graph min_support k\n", argv[0]);
        return 0;
    }
    using namespace std::chrono;
    try {
        const auto t1 = steady_clock::now();
        CSRGraph g;
        g.load(argv[1]);
        const int min_sup = std::atoi(argv[2]);
        const int k = std::atoi(argv[3]);
        const auto t2 = steady_clock::now();
        const auto t3 = steady_clock::now();
        fsm(g, k, min_sup);
        const auto t4 = steady_clock::now();
        const auto load_us = duration_cast<microseconds>(t2 - t1).count();
        const auto prep_us = duration_cast<microseconds>(t3 - t2).count();
        const auto fsm_us = duration_cast<microseconds>(t4 - t3).count();
        std::printf("load: %lfs prepare: %lfs fsm: %lfs\n", load_us * 1e-6, prep_us * 1e-6, fsm_us * 1e-6);
    } catch (const std::exception& e) {
        std::fflush(stdout);
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
