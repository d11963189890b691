// The gspan.h surface: fsm() over the C ABI, and the EmbVector helpers
// (gspan.cu:376-409).
#include "gspan.h"
#include "gspan_gb300.h"

#include <algorithm>
#include <cstdio>
#include <stdexcept>
#include <string>

void EmbVector::build(const CSRGraph& g, const Embedding* p)
{
    for (; p; p = p->prev) push_back(g.edges[p->edge_id]);
    std::reverse(begin(), end());
}

void EmbVector::build(const CSRGraph& g, const LayeredEmbeddings& le, int emb_idx)
{
    for (int layer = (int)le.size() - 1; layer >= 0; --layer) {
        const EmbeddingRel& r = (*le[layer])[emb_idx];
        push_back(g.edges[r.edge_id]);
        emb_idx = r.prev_idx;
    }
    std::reverse(begin(), end());
}

bool EmbVector::has_edge(const Edge& e) const
{
    for (const Edge& x : *this)
        if (x.label == e.label && ((x.from == e.from && x.to == e.to) || (x.to == e.from && x.from == e.to)))
            return true;
    return false;
}

bool EmbVector::has_vertex(int v) const
{
    for (const Edge& x : *this)
        if (x.from == v || x.to == v) return true;
    return false;
}

namespace {

int print_pattern(void*, const gspan_pattern_edge* code, int32_t len, int32_t support)
{
    for (int32_t i = 0; i < len; ++i)
        std::printf("(%d %d %d %d %d)", code[i].from, code[i].to, code[i].from_label, code[i].edge_label,
                    code[i].to_label);
    std::printf(": %d\n", support);
    return 0;
}

[[noreturn]] void raise(const char* what, gspan_status s, gspan_ctx* ctx)
{
    std::string msg = std::string("gspan_gb300: ") + what + ": " + gspan_status_string(s);
    if (ctx && *gspan_last_error(ctx)) msg += std::string(" (") + gspan_last_error(ctx) + ")";
    throw std::runtime_error(msg);
}

}  // namespace

// Same contract as gspan.h:41 / gspan.cu:1171-1199: prints every frequent
// minimum DFS code with its MNI support in pre-order.  Errors throw.
void fsm(const CSRGraph& g, int k, int min_support)
{
    gspan_ctx* ctx = nullptr;
    gspan_status s = gspan_ctx_create(nullptr, &ctx);
    if (s != GSPAN_OK) raise("context", s, nullptr);
    gspan_graph* dg = nullptr;
    s = gspan_graph_upload(ctx, g.nr_nodes, g.nr_edges, g.offsets, g.vlabels,
                           reinterpret_cast<const gspan_edge*>(g.edges), &dg);
    if (s != GSPAN_OK) {
        std::string err = gspan_last_error(ctx);
        gspan_ctx_destroy(ctx);
        throw std::runtime_error("gspan_gb300: graph upload: " + std::string(gspan_status_string(s)) + " (" + err +
                                 ")");
    }
    s = gspan_mine(ctx, dg, k, min_support, print_pattern, nullptr, nullptr);
    std::fflush(stdout);
    if (s != GSPAN_OK) {
        std::string err = gspan_last_error(ctx);
        gspan_graph_free(ctx, dg);
        gspan_ctx_destroy(ctx);
        throw std::runtime_error("gspan_gb300: mining: " + std::string(gspan_status_string(s)) + " (" + err + ")");
    }
    gspan_graph_free(ctx, dg);
    gspan_ctx_destroy(ctx);
}

static_assert(sizeof(Edge) == sizeof(gspan_edge), "Edge must match gspan_edge");
