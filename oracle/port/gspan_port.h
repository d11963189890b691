// Test infrastructure only: the CPU oracle for the mining path.
//
// A restatement of haozixu/gSpan's CPU algorithm (gspan.cu, graph.cc) in this
// repository's own code.  It is the checker for the CUDA engine and the timed
// CPU baseline; nothing in the product links or calls it.
//
// Parity pin: this port is validated line-by-line against the reference's own
// sources compiled here (oracle/_ref/fsm, see ref_support_shim.h), and against
// the golden outputs under tests/golden/ that the reference produced.
#pragma once

#include <cstdint>
#include <functional>
#include <vector>

namespace port {

struct Edge { int from, to, label; };            // graph.h:7-12

struct Graph {                                   // graph.h:51-65 (CSRGraph)
    int n = 0, m = 0;
    std::vector<int> offsets, vlabels;
    std::vector<Edge> edges;
};

struct PEdge {                                   // graph.h:28-47 (PatternEdge)
    int from, to, fl, el, tl;
    bool forward() const { return from < to; }
    bool operator==(const PEdge& o) const {
        return from == o.from && to == o.to && fl == o.fl && el == o.el && tl == o.tl;
    }
};
using Code = std::vector<PEdge>;

struct Stats {
    uint64_t seeds = 0;          // level-1 embeddings
    uint64_t extended = 0;       // child embeddings produced by extension
    uint64_t patterns = 0;       // reported patterns
    uint64_t support_calls = 0;  // canonical candidates whose support was counted
    double last_s = 0;           // seconds spent counting a streamed last level
    uint64_t last_extended = 0;  // the part of `extended` in a streamed last level
};

// A slice of a streamed last level: only parent rows whose last data edge
// hashes to `index` modulo `count` are extended.  Counts and times of the `count` slices add up to the whole
// level's; supports and reports are then partial (timing use only).
struct Shard {
    int index = 0, count = 1;
};

using ReportFn = std::function<void(const Code&, int support)>;

// Runs the whole mining job; calls `report` in the reference's pre-order.
//
// stream_last = false extends every level as the reference does: the children
// of a pattern are materialised as {prev_idx, edge_id} layers
// (gspan.cu:1131-1138), then each child's support walks them.
// stream_last = true changes only how the last level (patterns of k edges) is
// counted: each parent embedding's children are produced by the same three
// rules and ORed straight into per-child domain bitsets, never stored.  Output
// and counts are identical; memory no longer grows with the last level.
void mine_all(const Graph& g, int k, int min_support, const ReportFn& report, Stats* stats,
              bool stream_last = false, Shard shard = Shard{});

// The minimum-DFS-code test of gspan.cu:586-606 on its own (for unit tests).
bool is_canonical(const Code& code);

// Loads the reference's binary CSR file (graph.cc:178-200); false on a short read.
bool load_bin(const char* path, Graph& g);

}  // namespace port
