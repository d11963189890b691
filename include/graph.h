// Drop-in replacement for haozixu/gSpan's graph.h (graph.h:1-65).
//
// Same type names, member names, layouts and member functions, so code written
// against the reference's graph.h compiles unchanged against this header and
// links against libgspan_gb300.so.  Layouts must match because CSR files are
// read and written as raw memory: Edge is 12 bytes (from, to, label), and the
// binary file is int32 n, int32 m, int32 offsets[n+1], int32 vlabels[n],
// Edge edges[m] in native byte order (graph.cc:178-214).
#ifndef GSPAN_GB300_GRAPH_H_
#define GSPAN_GB300_GRAPH_H_

#include <map>
#include <vector>

// One directed adjacency entry (graph.h:7-12).
struct Edge {
    int from, to, label;
};

// Vertex of the text-loaded graph (graph.h:14-17).
struct Vertex {
    int label;
    std::vector<Edge> edges;
};

// Undirected graph keyed by the vertex ids of the text file (graph.h:20-26).
struct Graph : std::map<int, Vertex> {
    void add_vertex(int u, int label);
    void add_edge(int u, int v, int label);   // stores u->v and v->u

    // gSpan text: "t # id" (ignored, so several graphs merge), "v id label",
    // "e u v label".  Throws std::runtime_error if the file cannot be opened.
    static Graph from_txt(const char* filename);
};

// One edge of a DFS code (graph.h:28-47).  Labels a code does not fix are -1.
struct PatternEdge {
    int from, to, from_label, edge_label, to_label;

    PatternEdge() {}
    PatternEdge(int u, int v, int ulabel, int elabel, int vlabel)
        : from(u), to(v), from_label(ulabel), edge_label(elabel), to_label(vlabel) {}

    bool is_forward() const { return from < to; }
    bool is_backward() const { return from > to; }

    bool operator==(const PatternEdge& o) const
    {
        return from == o.from && to == o.to && from_label == o.from_label &&
               edge_label == o.edge_label && to_label == o.to_label;
    }
    bool operator!=(const PatternEdge& o) const { return !(*this == o); }
};

using DFSCode = std::vector<PatternEdge>;

// CSR graph (graph.h:51-65).  Owns its three arrays (new[]); not copyable.
struct CSRGraph {
    int nr_nodes, nr_edges;
    int *offsets, *vlabels;
    Edge* edges;

    CSRGraph() : nr_nodes(0), nr_edges(0), offsets(nullptr), vlabels(nullptr), edges(nullptr) {}
    // Vertices renumbered densely in ascending id order; each adjacency sorted by
    // (to, label) (graph.cc:66-112).
    CSRGraph(Graph&);
    // The small pattern graph of a DFS code; adjacency in reverse code order
    // (graph.cc:121-159).
    CSRGraph(const DFSCode&);
    ~CSRGraph();
    CSRGraph(const CSRGraph&) = delete;
    CSRGraph& operator=(const CSRGraph&) = delete;

    void load(const char* filename);   // throws std::runtime_error on a short read
    void save(const char* filename);
    void dump() const;
};

// Drops vertices whose label occurs fewer than min_sup times and renumbers the
// rest (graph.cc:216-266).
void prune_graph(CSRGraph& pruned, const CSRGraph& g, int min_sup);

#endif  // GSPAN_GB300_GRAPH_H_
