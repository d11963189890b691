// Minimum-DFS-code test, host side.
//
// Decides exactly what haozixu/gSpan's is_canonical (gspan.cu:586-606) and
// projection_is_canonical (gspan.cu:485-584) decide: the code is rebuilt
// greedily on its own pattern graph, taking at every step the smallest
// extension the reference's rules allow (backward to the rightmost-path vertex
// nearest v0 with the smallest edge label; else first-forward from v_n; else
// other-forward from the deepest rightmost-path vertex that has one; then the
// smallest (edge label, to label)), and the code is canonical iff no step
// departs from it.
//
// Written as a loop over explicit embedding lists (each embedding is the list
// of pattern-graph entries it uses, in min-code order) instead of the
// reference's recursion over pointer-chained embeddings.  The pattern graph's
// adjacency order is part of the semantics: graph.cc:146-156 fills each
// adjacency from its end, so entries appear in reverse code order, and the
// backward rule takes the FIRST entry in that order (gspan.cu:428-445).
#include "miner.h"

#include <algorithm>
#include <map>
#include <tuple>

namespace gs {
namespace {

struct PEntry { int from, to, label; };

struct PatternGraph {
    int n = 0;
    std::vector<int> off, vl;
    std::vector<PEntry> ent;
};

PatternGraph build_pattern_graph(const CodeEdge* code, int len)
{
    PatternGraph p;
    for (int i = 0; i < len; ++i) p.n = std::max(p.n, std::max(code[i].from, code[i].to) + 1);
    std::vector<int> fill(p.n, 0);
    for (int i = 0; i < len; ++i) {
        ++fill[code[i].from];
        ++fill[code[i].to];
    }
    p.off.assign(p.n + 1, 0);
    for (int v = 0; v < p.n; ++v) p.off[v + 1] = p.off[v] + fill[v];
    p.vl.assign(p.n, 0);
    p.ent.resize(2 * (size_t)len);
    for (int i = 0; i < len; ++i) {
        const CodeEdge& c = code[i];
        if (c.fl != -1) p.vl[c.from] = c.fl;
        if (c.tl != -1) p.vl[c.to] = c.tl;
        p.ent[p.off[c.from] + --fill[c.from]] = PEntry{c.from, c.to, c.el};
        p.ent[p.off[c.to] + --fill[c.to]] = PEntry{c.to, c.from, c.el};
    }
    return p;
}

using Emb = std::vector<int>;   // pattern-graph entry index per min-code edge

struct View {
    const PatternGraph& p;
    const Emb& h;
    const PEntry& at(int j) const { return p.ent[h[j]]; }
    bool uses_edge(int a, int b, int label) const
    {
        for (int x : h) {
            const PEntry& e = p.ent[x];
            if (e.label == label && ((e.from == a && e.to == b) || (e.from == b && e.to == a))) return true;
        }
        return false;
    }
    bool uses_vertex(int v) const
    {
        for (int x : h)
            if (p.ent[x].from == v || p.ent[x].to == v) return true;
        return false;
    }
};

std::vector<int> rmpath_of(const std::vector<CodeEdge>& c)
{
    std::vector<int> rm;
    int want = -1;
    for (int i = (int)c.size() - 1; i >= 0; --i)
        if (c[i].from < c[i].to && (rm.empty() || c[i].to == want)) {
            rm.push_back(i);
            want = c[i].from;
        }
    return rm;
}

bool same(const CodeEdge& a, const CodeEdge& b)
{
    return a.from == b.from && a.to == b.to && a.fl == b.fl && a.el == b.el && a.tl == b.tl;
}

}  // namespace

bool is_min_code(const CodeEdge* code, int len)
{
    if (len <= 1) return true;
    const PatternGraph p = build_pattern_graph(code, len);

    // Smallest 1-edge code of the pattern graph and its embeddings.
    std::tuple<int, int, int> best{0, 0, 0};
    bool have = false;
    std::vector<Emb> embs;
    for (int u = 0; u < p.n; ++u)
        for (int i = p.off[u]; i < p.off[u + 1]; ++i) {
            const int tl = p.vl[p.ent[i].to];
            if (p.vl[u] > tl) continue;
            const std::tuple<int, int, int> key{p.vl[u], p.ent[i].label, tl};
            if (!have || key < best) {
                best = key;
                have = true;
                embs.clear();
            }
            if (key == best) embs.push_back(Emb{i});
        }
    std::vector<CodeEdge> mc{CodeEdge{0, 1, std::get<0>(best), std::get<1>(best), std::get<2>(best)}};

    for (;;) {
        const std::vector<int> rm = rmpath_of(mc);
        const int min_label = mc[0].fl;
        const int vn = mc[rm[0]].to;
        const size_t pos = mc.size();

        // Backward step.
        std::map<int, std::vector<Emb>> back;
        int back_to = -1;
        for (int i = (int)rm.size() - 1; i >= 1 && back.empty(); --i) {
            const int k = rm[i];
            for (const Emb& h : embs) {
                const View v{p, h};
                const PEntry e = v.at(k);
                const int un = v.at(rm[0]).to;
                for (int x = p.off[un]; x < p.off[un + 1]; ++x) {
                    const PEntry& cur = p.ent[x];
                    if (v.uses_edge(un, cur.to, cur.label)) continue;
                    if (cur.to == e.from && (e.label < cur.label || (e.label == cur.label && p.vl[e.to] <= p.vl[un]))) {
                        Emb nh = h;
                        nh.push_back(x);
                        back[cur.label].push_back(std::move(nh));
                        back_to = mc[k].from;
                        break;
                    }
                }
            }
        }
        if (!back.empty()) {
            const CodeEdge step{vn, back_to, -1, back.begin()->first, -1};
            if (pos >= (size_t)len || !same(code[pos], step)) return false;
            mc.push_back(step);
            embs = std::move(back.begin()->second);
            continue;
        }

        // Forward step.
        std::map<std::pair<int, int>, std::vector<Emb>> fwd;
        int fwd_from = -1;
        for (const Emb& h : embs) {
            const View v{p, h};
            const int un = v.at(rm[0]).to;
            for (int x = p.off[un]; x < p.off[un + 1]; ++x) {
                const int to = p.ent[x].to, tl = p.vl[to];
                if (tl < min_label || v.uses_vertex(to)) continue;
                Emb nh = h;
                nh.push_back(x);
                fwd[{p.ent[x].label, tl}].push_back(std::move(nh));
            }
        }
        if (!fwd.empty()) fwd_from = vn;
        for (size_t i = 0; fwd.empty() && i < rm.size(); ++i) {
            const int k = rm[i];
            for (const Emb& h : embs) {
                const View v{p, h};
                const PEntry e = v.at(k);
                const int bound = p.vl[e.to];
                for (int x = p.off[e.from]; x < p.off[e.from + 1]; ++x) {
                    const int to = p.ent[x].to, tl = p.vl[to], el = p.ent[x].label;
                    if (tl < min_label || v.uses_vertex(to)) continue;
                    if (e.label < el || (e.label == el && bound <= tl)) {
                        Emb nh = h;
                        nh.push_back(x);
                        fwd[{el, tl}].push_back(std::move(nh));
                    }
                }
            }
            if (!fwd.empty()) fwd_from = mc[k].from;
        }
        if (!fwd.empty()) {
            const CodeEdge step{fwd_from, vn + 1, -1, fwd.begin()->first.first, fwd.begin()->first.second};
            if (pos >= (size_t)len || !same(code[pos], step)) return false;
            mc.push_back(step);
            embs = std::move(fwd.begin()->second);
            continue;
        }
        return true;
    }
}

}  // namespace gs
