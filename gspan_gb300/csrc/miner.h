// Host-side internals: context and graph objects behind the C ABI, the
// level-synchronous mining driver and the canonical-code test.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "engine.h"

namespace gs {

// A DFS-code edge.  Inside the miner labels are ranks (-1 = not fixed); codes
// are translated back to the graph's labels only when they are emitted.
struct CodeEdge {
    int from, to, fl, el, tl;
};

// The reference's minimum-DFS-code test (gspan.cu:485-606), host side.
bool is_min_code(const CodeEdge* code, int len);

// Sort key of the reference's pre-order report sequence (gspan.cu:1118-1190):
// 1-edge codes ascending by (from label, edge label, to label); below a node,
// backward children ascending by (to, edge label), then forward children by
// descending from, then ascending (edge label, to label); a node before its
// descendants.  Labels compare by rank, which preserves the order.
bool preorder_less(const std::vector<CodeEdge>& a, const std::vector<CodeEdge>& b);

}  // namespace gs

struct gspan_ctx {
    int device = 0;
    gspan_opts opts{};
    cudaStream_t stream = nullptr;
    std::string err;
    int expand_blocks = 0;
    // Small device words reused by every pass.
    uint32_t* d_status = nullptr;
    unsigned long long* d_counters = nullptr;   // [0],[2] tile counters, [1],[3] scanned entries
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_c = nullptr, ev_d = nullptr;
    int live_graphs = 0;
};

struct gspan_graph {
    gs::DevGraph g;
    gspan_ctx* owner = nullptr;
};

namespace gs {
gspan_status mine(gspan_ctx* ctx, const DevGraph& g, int k, int min_support, gspan_emit_fn emit, void* user,
                  gspan_stats* stats);
gspan_status fail(gspan_ctx* ctx, gspan_status s, const std::string& msg);
gspan_status cuda_fail(gspan_ctx* ctx, cudaError_t e, const char* what);
}  // namespace gs
