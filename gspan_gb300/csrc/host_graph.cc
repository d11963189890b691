// The graph.h surface (Graph, CSRGraph, prune_graph): loaders and file
// formats with the reference's exact semantics (graph.cc:1-266), in this
// library's own code.
#include "graph.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>

void Graph::add_vertex(int u, int label)
{
    (*this)[u].label = label;
}

void Graph::add_edge(int u, int v, int label)
{
    (*this)[u].edges.push_back(Edge{u, v, label});
    (*this)[v].edges.push_back(Edge{v, u, label});
}

// Reads like graph.cc:38-64, with the same scanf calls: a token starting
// with 't' is followed by one token (ignored) and an integer, 'v' by id and
// label, 'e' by both ends and the label; any other token is skipped.  Vertices
// named only by edges get label 0.
//
// Malformed records are read the reference's way.  Its three integers u, v, w
// live across records ('t' writes u; 'v' writes v, w; 'e' writes u, v, w), and
// a conversion that fails leaves its variable and the record's later ones as
// the previous record left them: the record is still added with those values,
// and the offending token is read as the next record's head.  A record that
// would use a variable no earlier record assigned (uninitialised in the
// reference, so its result is undefined) is refused with an exception.
// Tokens of 16 or more characters, and a 't' record's skipped token of 4 or
// more, overflow the reference's buffers (also undefined); here they are read
// as whole tokens of up to 63 characters.
Graph Graph::from_txt(const char* filename)
{
    FILE* f = std::fopen(filename, "r");
    if (!f) throw std::runtime_error("failed to open file\n");
    Graph g;
    char tok[64];
    int u = 0, v = 0, w = 0;
    bool has_u = false, has_v = false, has_w = false;
    long nr_edges = 0;
    auto need = [&](bool ok, const char* what) {
        if (!ok) {
            std::fclose(f);
            throw std::runtime_error(std::string("malformed record: ") + what +
                                     " is read before any record assigned it");
        }
    };
    while (std::fscanf(f, "%63s", tok) == 1) {
        if (tok[0] == 't') {
            char skip[64];
            if (std::fscanf(f, "%63s%d", skip, &u) == 2) has_u = true;
        } else if (tok[0] == 'v') {
            const int got = std::fscanf(f, "%d%d", &v, &w);
            has_v |= got >= 1;
            has_w |= got >= 2;
            need(has_v && has_w, "a vertex id or label");
            g.add_vertex(v, w);
        } else if (tok[0] == 'e') {
            const int got = std::fscanf(f, "%d%d%d", &u, &v, &w);
            has_u |= got >= 1;
            has_v |= got >= 2;
            has_w |= got >= 3;
            need(has_u && has_v && has_w, "an edge end or label");
            g.add_edge(u, v, w);
            ++nr_edges;
        }
    }
    std::fclose(f);
    std::printf("|V| = %ld |E| = %d\n", (long)g.size(), (int)nr_edges);
    return g;
}

CSRGraph::CSRGraph(Graph& g)
{
    nr_nodes = (int)g.size();
    nr_edges = 0;
    std::unordered_map<int, int> dense;
    dense.reserve(g.size() * 2 + 1);
    int next = 0;
    for (const auto& kv : g) {   // std::map: ascending old id
        dense[kv.first] = next++;
        nr_edges += (int)kv.second.edges.size();
    }
    offsets = new int[nr_nodes + 1];
    vlabels = new int[nr_nodes];
    edges = new Edge[nr_edges];
    offsets[0] = 0;
    int v = 0, at = 0;
    for (const auto& kv : g) {
        const int begin = at;
        for (const Edge& e : kv.second.edges) edges[at++] = Edge{v, dense[e.to], e.label};
        std::sort(edges + begin, edges + at, [](const Edge& a, const Edge& b) {
            return a.to != b.to ? a.to < b.to : a.label < b.label;
        });
        vlabels[v] = kv.second.label;
        offsets[++v] = at;
    }
}

// Pattern graph of a DFS code (graph.cc:121-159): each adjacency is filled from
// its end, so it lists the code's edges in reverse order.
CSRGraph::CSRGraph(const DFSCode& code)
{
    int vmax = 0;
    for (const PatternEdge& e : code) vmax = std::max(vmax, std::max(e.from, e.to));
    nr_nodes = vmax + 1;
    nr_edges = 2 * (int)code.size();
    offsets = new int[nr_nodes + 1];
    vlabels = new int[nr_nodes]();
    edges = new Edge[nr_edges];
    std::vector<int> fill(nr_nodes, 0);
    for (const PatternEdge& e : code) {
        ++fill[e.from];
        ++fill[e.to];
    }
    offsets[0] = 0;
    for (int u = 0; u < nr_nodes; ++u) offsets[u + 1] = offsets[u] + fill[u];
    for (const PatternEdge& e : code) {
        if (e.from_label != -1) vlabels[e.from] = e.from_label;
        if (e.to_label != -1) vlabels[e.to] = e.to_label;
        edges[offsets[e.from] + --fill[e.from]] = Edge{e.from, e.to, e.edge_label};
        edges[offsets[e.to] + --fill[e.to]] = Edge{e.to, e.from, e.edge_label};
    }
}

CSRGraph::~CSRGraph()
{
    delete[] offsets;
    delete[] vlabels;
    delete[] edges;
}

void CSRGraph::dump() const
{
    std::printf("vlabels:");
    for (int v = 0; v < nr_nodes; ++v) std::printf(" %d", vlabels[v]);
    std::printf("\noffsets:");
    for (int v = 0; v <= nr_nodes; ++v) std::printf(" %d", offsets[v]);
    std::printf("\nfrom: ");
    for (int i = 0; i < nr_edges; ++i) std::printf(" %d", edges[i].from);
    std::printf("\nto:");
    for (int i = 0; i < nr_edges; ++i) std::printf(" %d", edges[i].to);
    std::printf("\n");
}

namespace {
struct FileCloser {
    FILE* f;
    ~FileCloser() { if (f) std::fclose(f); }
};
}  // namespace

// Binary CSR (graph.cc:178-200): int32 n, int32 m, offsets[n+1], vlabels[n],
// Edge[m], native byte order.  The messages match the reference's.
void CSRGraph::load(const char* filename)
{
    FILE* f = std::fopen(filename, "rb");
    if (!f) throw std::runtime_error("failed to open file");
    FileCloser closer{f};
    int n = 0, m = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1) throw std::runtime_error("nr_nodes required");
    if (std::fread(&m, sizeof(m), 1, f) != 1) throw std::runtime_error("nr_edges required");
    if (n < 0 || m < 0) throw std::runtime_error("bad offsets");
    int* off = new int[(size_t)n + 1];
    int* vl = new int[(size_t)n];
    Edge* ed = new Edge[(size_t)m];
    auto drop = [&](const char* msg) {
        delete[] off;
        delete[] vl;
        delete[] ed;
        throw std::runtime_error(msg);
    };
    if (std::fread(off, sizeof(int), (size_t)n + 1, f) != (size_t)n + 1) drop("bad offsets");
    if (std::fread(vl, sizeof(int), (size_t)n, f) != (size_t)n) drop("bad vertex labels");
    if (std::fread(ed, sizeof(Edge), (size_t)m, f) != (size_t)m) drop("bad edges");
    delete[] offsets;
    delete[] vlabels;
    delete[] edges;
    nr_nodes = n;
    nr_edges = m;
    offsets = off;
    vlabels = vl;
    edges = ed;
}

void CSRGraph::save(const char* filename)
{
    FILE* f = std::fopen(filename, "wb");
    if (!f) throw std::runtime_error("failed to open file");
    FileCloser closer{f};
    std::fwrite(&nr_nodes, sizeof(nr_nodes), 1, f);
    std::fwrite(&nr_edges, sizeof(nr_edges), 1, f);
    std::fwrite(offsets, sizeof(int), (size_t)nr_nodes + 1, f);
    std::fwrite(vlabels, sizeof(int), (size_t)nr_nodes, f);
    std::fwrite(edges, sizeof(Edge), (size_t)nr_edges, f);
}

// Keeps the vertices whose label occurs at least min_sup times, renumbered in
// ascending order, and the entries between kept vertices in their original
// order (graph.cc:216-266).
void prune_graph(CSRGraph& pruned, const CSRGraph& g, int min_sup)
{
    std::unordered_map<int, int> label_count;
    for (int v = 0; v < g.nr_nodes; ++v) ++label_count[g.vlabels[v]];
    std::vector<int> dense(g.nr_nodes, -1);
    int kept = 0;
    for (int v = 0; v < g.nr_nodes; ++v)
        if (label_count[g.vlabels[v]] >= min_sup) dense[v] = kept++;
    std::vector<Edge> out;
    delete[] pruned.offsets;
    delete[] pruned.vlabels;
    delete[] pruned.edges;
    pruned.nr_nodes = kept;
    pruned.vlabels = new int[kept];
    pruned.offsets = new int[kept + 1];
    pruned.offsets[0] = 0;
    for (int v = 0; v < g.nr_nodes; ++v) {
        if (dense[v] < 0) continue;
        const int nv = dense[v];
        pruned.vlabels[nv] = g.vlabels[v];
        for (int i = g.offsets[v]; i < g.offsets[v + 1]; ++i) {
            const int to = dense[g.edges[i].to];
            if (to >= 0) out.push_back(Edge{nv, to, g.edges[i].label});
        }
        pruned.offsets[nv + 1] = (int)out.size();
    }
    pruned.nr_edges = (int)out.size();
    pruned.edges = new Edge[out.size()];
    std::copy(out.begin(), out.end(), pruned.edges);
    std::printf("|V|: %d -> %d |E|: %d -> %d\n", g.nr_nodes, pruned.nr_nodes, g.nr_edges, pruned.nr_edges);
}
