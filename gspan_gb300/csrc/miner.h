// Host-side internals: context and graph objects behind the C ABI, the
// level-synchronous mining driver and the canonical-code test.
#pragma once

#include <cstdint>
#include <functional>
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
    // Pinned host words for readbacks that are settled at a later sync.
    unsigned long long* h_pin = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_c = nullptr, ev_d = nullptr;
    // Pinned staging for the miner's device-to-host readbacks (grown on demand).
    uint8_t* h_stage = nullptr;
    size_t h_stage_cap = 0;
    // Event pairs for kernel timing (profile mode), kept across runs.
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
    int live_graphs = 0;
};

struct gspan_graph {
    gs::DevGraph g;
    gspan_ctx* owner = nullptr;
};

namespace gs {
// Receives (instance, code, length, support) in pre-order, instance by instance.
using EmitFn = std::function<int(int, const gspan_pattern_edge*, int32_t, int32_t)>;
// Mines every instance of `g` (one for a single graph) with its own minimum
// support minsup[instance].
gspan_status mine(gspan_ctx* ctx, const DevGraph& g, int k, const std::vector<int32_t>& minsup, const EmitFn& emit,
                  gspan_stats* stats);
gspan_status fail(gspan_ctx* ctx, gspan_status s, const std::string& msg);
// Builds the device store from `ninst` CSR graphs (graph_store.cc): host
// arrays, or (on_device, one graph) arrays already in device memory.
gspan_status upload_graphs(gspan_ctx* ctx, int32_t ninst, const int32_t* ns, const int32_t* ms,
                           const int32_t* const* offs, const int32_t* const* vls, const gspan_edge* const* eds,
                           gspan_graph** out, bool on_device = false);
void free_graph(gspan_graph* gr, cudaStream_t st);
// Builds the device store from gSpan text read on the device (text_loader.cu).
gspan_status load_text(gspan_ctx* ctx, const char* text, int64_t len, gspan_graph** out, int32_t* nr_nodes,
                       int32_t* nr_edges);
gspan_status cuda_fail(gspan_ctx* ctx, cudaError_t e, const char* what);
// Label-frequency pruning (prune.cu): a new store of `g` without the vertices
// whose label occurs on fewer than min_support vertices; *out stays null when
// no vertex would be dropped (or for a batch).
gspan_status prune_store(gspan_ctx* ctx, const DevGraph& g, int32_t min_support, gspan_graph** out,
                         int64_t* kept_vertices, int64_t* kept_entries);
}  // namespace gs
