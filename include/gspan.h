// Drop-in replacement for haozixu/gSpan's gspan.h (gspan.h:1-43).
//
// `fsm` keeps the reference's signature and output: one line per frequent
// minimum DFS code, "(from to from_label edge_label to_label)...: support",
// in the reference's pre-order (gspan.cu:67-77, 1118-1199).  Mining runs on
// the GPU through the C ABI in gspan_gb300.h; if no GPU is usable, `fsm`
// throws std::runtime_error instead of printing anything.
#ifndef GSPAN_GB300_GSPAN_H_
#define GSPAN_GB300_GSPAN_H_

#include "graph.h"

// Indices into a DFSCode of the forward edges on the path v0 -> v_n, deepest
// first (gspan.h:7, gspan.cu:53-65).
using RightMostPath = std::vector<int>;

// Pointer-chained embedding (gspan.h:10-16).
struct Embedding {
    Embedding* prev;
    int edge_id;

    Embedding() {}
    Embedding(Embedding* p, int i) : prev(p), edge_id(i) {}
};

// One layer record of a layered embedding (gspan.h:18-24).
struct EmbeddingRel {
    int prev_idx;
    int edge_id;

    EmbeddingRel() {}
    EmbeddingRel(int p, int i) : prev_idx(p), edge_id(i) {}
};

using Embeddings = std::vector<Embedding>;
using EmbeddingRels = std::vector<EmbeddingRel>;
using LayeredEmbeddings = std::vector<const EmbeddingRels*>;

// The data edges of one embedding in code order (gspan.h:30-38).
struct EmbVector : std::vector<Edge> {
    bool has_edge(const Edge& e) const;   // same label, either direction
    bool has_vertex(int v) const;
    void build(const CSRGraph& g, const Embedding* p);
    void build(const CSRGraph& g, const LayeredEmbeddings& le, int emb_idx);

    EmbVector(const CSRGraph& g, const Embedding& emb) { build(g, &emb); }
    EmbVector(const CSRGraph& g, const LayeredEmbeddings& le, int emb_idx) { build(g, le, emb_idx); }
};

// Mines all frequent subgraphs of `g` with at most `k` edges and MNI support
// >= min_support, printing them to stdout (gspan.h:41).
void fsm(const CSRGraph& g, int k, int min_support);

#endif  // GSPAN_GB300_GSPAN_H_
