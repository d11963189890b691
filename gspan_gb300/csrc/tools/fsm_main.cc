// `fsm <graph> <min_support> <k> [options]`: the reference's mining command
// (fsm.cu:11-43) on the GPU miner.  Prints the pattern lines, then the same
// "load: ... prepare: ... fsm: ..." timing line.  The reference tests
// `argc < 3` but reads argv[3]; this one asks for all three arguments.
//
// Options (none: exactly the reference's command through gspan.h fsm()):
//   --text                 <graph> is gSpan text, read on the GPU
//                          (gspan_graph_upload_text) instead of a .bin file
//   --path auto|candidate|mask
//   --domains auto|bitmap|hash
//   --hash-threshold X     auto domains: hashset when 64 * size < |V| * X
//   --device N
//   --fused-last auto|off|always
//                          next-to-last level generated inside the last
//                          level's row pass instead of stored
//   --prune                drop vertices of labels with fewer than min_support
//                          vertices before mining (the reference's prune_graph,
//                          left commented out at fsm.cu:28-29); same output
//   --stats                run statistics as one JSON object on stderr
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "graph.h"
#include "gspan.h"
#include "gspan_gb300.h"

namespace {

int print_pattern(void*, const gspan_pattern_edge* code, int32_t len, int32_t support)
{
    for (int32_t i = 0; i < len; ++i)
        std::printf("(%d %d %d %d %d)", code[i].from, code[i].to, code[i].from_label, code[i].edge_label,
                    code[i].to_label);
    std::printf(": %d\n", support);
    return 0;
}

struct Options {
    bool any = false, text = false, stats = false;
    gspan_opts o;
};

Options parse(int argc, char* argv[])
{
    Options opt;
    gspan_opts_default(&opt.o);
    for (int i = 4; i < argc; ++i) {
        const std::string a = argv[i];
        auto value = [&]() -> std::string {
            if (i + 1 >= argc) throw std::runtime_error("option " + a + " needs a value");
            return argv[++i];
        };
        opt.any = true;
        if (a == "--text") {
            opt.text = true;
        } else if (a == "--stats") {
            opt.stats = true;
        } else if (a == "--path") {
            const std::string v = value();
            if (v == "auto") opt.o.path = 0;
            else if (v == "candidate") opt.o.path = 1;
            else if (v == "mask") opt.o.path = 2;
            else throw std::runtime_error("--path: auto, candidate or mask");
        } else if (a == "--domains") {
            const std::string v = value();
            if (v == "auto") opt.o.domain_mode = 0;
            else if (v == "bitmap") opt.o.domain_mode = 1;
            else if (v == "hash") opt.o.domain_mode = 2;
            else throw std::runtime_error("--domains: auto, bitmap or hash");
        } else if (a == "--hash-threshold") {
            opt.o.hash_threshold = std::atof(value().c_str());
        } else if (a == "--device") {
            opt.o.device = std::atoi(value().c_str());
        } else if (a == "--fused-last") {
            const std::string v = value();
            if (v == "auto") opt.o.fused_last = 0;
            else if (v == "off") opt.o.fused_last = 1;
            else if (v == "always") opt.o.fused_last = 2;
            else throw std::runtime_error("--fused-last: auto, off or always");
        } else if (a == "--prune") {
            opt.o.prune = 1;
        } else {
            throw std::runtime_error("unknown option " + a);
        }
    }
    return opt;
}

std::vector<char> read_file(const char* path)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error("failed to open file\n");
    std::vector<char> buf;
    char chunk[1 << 16];
    size_t n;
    while ((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
    std::fclose(f);
    return buf;
}

void check(gspan_status s, gspan_ctx* ctx, const char* what)
{
    if (s == GSPAN_OK) return;
    std::string msg = std::string("gspan_gb300: ") + what + ": " + gspan_status_string(s);
    if (ctx && *gspan_last_error(ctx)) msg += std::string(" (") + gspan_last_error(ctx) + ")";
    throw std::runtime_error(msg);
}

void print_stats(const gspan_stats& st)
{
    std::fprintf(stderr,
                 "{\"seeds\": %llu, \"extended\": %llu, \"patterns\": %llu, \"support_keys\": %llu, "
                 "\"kernel_launches\": %llu, \"levels\": %d, \"mine_ms\": %.3f, \"frontier_rows\": %llu, "
                 "\"materialized_rows\": %llu, \"mask_parents\": %llu, \"candidate_parents\": %llu, "
                 "\"h2d_bytes\": %llu, \"d2h_bytes\": %llu, \"pruned_vertices\": %llu, \"pruned_entries\": %llu}\n",
                 (unsigned long long)st.seeds, (unsigned long long)st.extended, (unsigned long long)st.patterns,
                 (unsigned long long)st.support_keys, (unsigned long long)st.kernel_launches, st.levels, st.mine_ms,
                 (unsigned long long)st.frontier_rows, (unsigned long long)st.materialized_rows,
                 (unsigned long long)st.mask_parents, (unsigned long long)st.candidate_parents,
                 (unsigned long long)st.h2d_bytes, (unsigned long long)st.d2h_bytes,
                 (unsigned long long)st.pruned_vertices, (unsigned long long)st.pruned_entries);
}

}  // namespace

int main(int argc, char* argv[])
{
    if (argc < 4) {
        std::printf("usage: %s input_graph min_support k [--text] [--path auto|candidate|mask] "
                    "[--domains auto|bitmap|hash] [--hash-threshold X] [--device N] [--fused-last auto|off|always] [--prune] [--stats]\n",
                    argv[0]);
        return 0;
    }
    using namespace std::chrono;
    gspan_ctx* ctx = nullptr;
    gspan_graph* dg = nullptr;
    try {
        const Options opt = parse(argc, argv);
        const int min_sup = std::atoi(argv[2]);
        const int k = std::atoi(argv[3]);
        const auto t1 = steady_clock::now();
        auto t2 = t1, t3 = t1;
        if (!opt.any) {
            CSRGraph g;
            g.load(argv[1]);
            t2 = t3 = steady_clock::now();
            fsm(g, k, min_sup);
        } else {
            check(gspan_ctx_create(&opt.o, &ctx), nullptr, "context");
            if (opt.text) {
                const std::vector<char> text = read_file(argv[1]);
                t2 = steady_clock::now();
                check(gspan_graph_upload_text(ctx, text.data(), (int64_t)text.size(), &dg, nullptr, nullptr), ctx,
                      "text upload");
            } else {
                CSRGraph g;
                g.load(argv[1]);
                t2 = steady_clock::now();
                check(gspan_graph_upload(ctx, g.nr_nodes, g.nr_edges, g.offsets, g.vlabels,
                                         reinterpret_cast<const gspan_edge*>(g.edges), &dg),
                      ctx, "graph upload");
            }
            t3 = steady_clock::now();
            gspan_stats st;
            const gspan_status s = gspan_mine(ctx, dg, k, min_sup, print_pattern, nullptr, &st);
            std::fflush(stdout);
            check(s, ctx, "mining");
            if (opt.stats) print_stats(st);
            gspan_graph_free(ctx, dg);
            dg = nullptr;
            gspan_ctx_destroy(ctx);
            ctx = nullptr;
        }
        const auto t4 = steady_clock::now();
        const auto load_us = duration_cast<microseconds>(t2 - t1).count();
        const auto prep_us = duration_cast<microseconds>(t3 - t2).count();
        const auto fsm_us = duration_cast<microseconds>(t4 - t3).count();
        std::printf("load: %lfs prepare: %lfs fsm: %lfs\n", load_us * 1e-6, prep_us * 1e-6, fsm_us * 1e-6);
    } catch (const std::exception& e) {
        std::fflush(stdout);
        std::fprintf(stderr, "%s\n", e.what());
        if (ctx) {
            if (dg) gspan_graph_free(ctx, dg);
            gspan_ctx_destroy(ctx);
        }
        return 1;
    }
    return 0;
}
