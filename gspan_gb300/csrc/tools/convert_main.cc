// `convert <in.txt> <out.bin>`: gSpan text to binary CSR, as the reference's
// convert.cc:6-16.
#include <cstdio>
#include <stdexcept>

#include "graph.h"

int main(int argc, char* argv[])
{
    if (argc < 3) {
        std::printf("usage: %s input_name output_name\n", argv[0]);
        return 0;
    }
    try {
        Graph g = Graph::from_txt(argv[1]);
        CSRGraph csr(g);
        csr.save(argv[2]);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s", e.what());
        return 1;
    }
    return 0;
}
