// Test infrastructure only: CPU oracle for the mining path (see gspan_port.h).
//
// Each function restates one piece of haozixu/gSpan and cites it.  The data
// structures follow the reference on purpose, because this port is also the
// timed CPU baseline: level-by-level {prev_idx, edge_id} embedding layers
// (gspan.h:18-28), per-embedding edge histories rebuilt by walking those layers
// (gspan.cu:385-394), OpenMP over parent embeddings with per-thread ordered
// maps merged afterwards (gspan.cu:674-780), and bitset MNI counting
// (gspan.cu:165-190 semantics).
#include "gspan_port.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <map>
#include <omp.h>

namespace port {
namespace {

struct Rel { int prev, eid; };                 // gspan.h:18-24 EmbeddingRel
using Rels = std::vector<Rel>;
using Layers = std::vector<const Rels*>;       // gspan.h:27 LayeredEmbeddings

// Rightmost path: indices of the forward code edges on the path v0 -> v_n,
// deepest first (gspan.cu:53-65).
std::vector<int> rightmost_path(const Code& c)
{
    std::vector<int> rm;
    int want = -1;
    for (int i = (int)c.size() - 1; i >= 0; --i) {
        if (c[i].forward() && (rm.empty() || c[i].to == want)) {
            rm.push_back(i);
            want = c[i].from;
        }
    }
    return rm;
}

// The data edges of one embedding, indexed by code position (EmbVector,
// gspan.cu:376-409).
struct History {
    std::vector<Edge> h;
    bool has_edge(int a, int b, int label) const      // gspan.cu:396-401
    {
        for (const Edge& x : h)
            if (x.label == label && ((x.from == a && x.to == b) || (x.to == a && x.from == b)))
                return true;
        return false;
    }
    bool has_vertex(int v) const                        // gspan.cu:403-408
    {
        for (const Edge& x : h)
            if (x.from == v || x.to == v) return true;
        return false;
    }
};

void build_history(const Graph& g, const Layers& layers, int idx, History& out)
{
    const int L = (int)layers.size();
    out.h.resize(L);
    for (int layer = L - 1; layer >= 0; --layer) {
        const Rel& r = (*layers[layer])[idx];
        out.h[layer] = g.edges[r.eid];
        idx = r.prev;
    }
}

// Backward rule (gspan.cu:428-445): the first adjacency entry of u_n that closes
// a cycle to e.from, is not already used, and passes the label order test.
bool backward_edge(const Graph& g, const Edge& e, int u_n, const History& hist, int* out)
{
    for (int i = g.offsets[u_n]; i < g.offsets[u_n + 1]; ++i) {
        const int to = g.edges[i].to, lab = g.edges[i].label;
        if (hist.has_edge(u_n, to, lab)) continue;
        if (to == e.from && (e.label < lab || (e.label == lab && g.vlabels[e.to] <= g.vlabels[u_n]))) {
            *out = i;
            return true;
        }
    }
    return false;
}

// First-forward rule (gspan.cu:447-462): every unused neighbour of u_n whose
// label is at least min_label.
template <class F>
bool first_forward(const Graph& g, int u_n, int min_label, const History& hist, F&& emit)
{
    bool any = false;
    for (int i = g.offsets[u_n]; i < g.offsets[u_n + 1]; ++i) {
        const int to = g.edges[i].to, tl = g.vlabels[to];
        if (tl < min_label || hist.has_vertex(to)) continue;
        emit(g.edges[i].label, tl, i);
        any = true;
    }
    return any;
}

// Other-forward rule (gspan.cu:464-483): unused neighbours of e.from with label
// >= min_label and (edge label, to label) not below (e.label, vlabel(e.to)).
template <class F>
bool other_forward(const Graph& g, const Edge& e, int min_label, const History& hist, F&& emit)
{
    bool any = false;
    const int bound = g.vlabels[e.to];
    for (int i = g.offsets[e.from]; i < g.offsets[e.from + 1]; ++i) {
        const int to = g.edges[i].to, tl = g.vlabels[to], el = g.edges[i].label;
        if (tl < min_label || hist.has_vertex(to)) continue;
        if (e.label < el || (e.label == el && bound <= tl)) {
            emit(el, tl, i);
            any = true;
        }
    }
    return any;
}

// ---------------------------------------------------------------------------
// Minimum DFS code test (gspan.cu:485-606) on the pattern graph built from the
// code itself (graph.cc:121-159).

Graph pattern_graph(const Code& code)
{
    Graph p;
    int vmax = 0;
    for (const PEdge& e : code) vmax = std::max(vmax, std::max(e.from, e.to));
    std::vector<int> deg(vmax + 1, 0);
    for (const PEdge& e : code) { ++deg[e.from]; ++deg[e.to]; }
    p.n = vmax + 1;
    p.m = 2 * (int)code.size();
    p.offsets.assign(p.n + 1, 0);
    p.vlabels.assign(p.n, 0);
    p.edges.resize(p.m);
    for (int v = 0; v < p.n; ++v) p.offsets[v + 1] = p.offsets[v] + deg[v];
    // Entries fill each adjacency from its end, so the adjacency order is the
    // reverse of code order (graph.cc:146-156).
    for (const PEdge& e : code) {
        if (e.fl != -1) p.vlabels[e.from] = e.fl;
        if (e.tl != -1) p.vlabels[e.to] = e.tl;
        p.edges[p.offsets[e.from] + (--deg[e.from])] = Edge{e.from, e.to, e.el};
        p.edges[p.offsets[e.to] + (--deg[e.to])] = Edge{e.to, e.from, e.el};
    }
    return p;
}

struct PEmb { const PEmb* prev; int eid; };     // gspan.h:11-16 Embedding

void chain_history(const Graph& g, const PEmb* p, History& out)
{
    out.h.clear();
    for (; p; p = p->prev) out.h.push_back(g.edges[p->eid]);
    std::reverse(out.h.begin(), out.h.end());
}

bool projection_is_canonical(const Graph& g, const std::vector<PEmb>& embs, const Code& code, Code& min_code)
{
    const std::vector<int> rm = rightmost_path(min_code);
    const int min_label = min_code[0].fl;
    const int v_n = min_code[rm[0]].to;
    History hist;

    // Smallest backward extension: the rmpath vertex nearest v0 first, then the
    // smallest edge label (gspan.cu:500-524).
    {
        bool found = false;
        int v_i = -1;
        std::map<int, std::vector<PEmb>> by_label;
        for (int i = (int)rm.size() - 1; !found && i >= 1; --i) {
            const int k = rm[i];
            for (const PEmb& emb : embs) {
                chain_history(g, &emb, hist);
                const int u_n = hist.h[rm[0]].to;
                int idx;
                if (backward_edge(g, hist.h[k], u_n, hist, &idx)) {
                    by_label[g.edges[idx].label].push_back(PEmb{&emb, idx});
                    v_i = min_code[k].from;
                    found = true;
                }
            }
        }
        if (found) {
            auto it = by_label.begin();
            const PEdge pe{v_n, v_i, -1, it->first, -1};
            if (min_code.size() >= code.size() || !(code[min_code.size()] == pe)) return false;
            min_code.push_back(pe);
            return projection_is_canonical(g, it->second, code, min_code);
        }
    }

    // Smallest forward extension: from v_n first, else from the rmpath
    // vertices deepest first; then smallest (edge label, to label)
    // (gspan.cu:526-581).
    bool found = false;
    int v_i = -1;
    std::map<int, std::map<int, std::vector<PEmb>>> by_labels;
    for (const PEmb& emb : embs) {
        chain_history(g, &emb, hist);
        const int u_n = hist.h[rm[0]].to;
        if (first_forward(g, u_n, min_label, hist, [&](int el, int tl, int idx) {
                by_labels[el][tl].push_back(PEmb{&emb, idx});
            }))
            found = true;
    }
    if (found) v_i = v_n;
    for (size_t i = 0; !found && i < rm.size(); ++i) {
        const int k = rm[i];
        for (const PEmb& emb : embs) {
            chain_history(g, &emb, hist);
            const Edge e = hist.h[k];
            if (other_forward(g, e, min_label, hist, [&](int el, int tl, int idx) {
                    by_labels[el][tl].push_back(PEmb{&emb, idx});
                }))
                found = true;
        }
        if (found) {
            v_i = min_code[k].from;
            break;
        }
    }
    if (found) {
        auto it1 = by_labels.begin();
        auto it2 = it1->second.begin();
        const PEdge pe{v_i, v_n + 1, -1, it1->first, it2->first};
        if (min_code.size() >= code.size() || !(code[min_code.size()] == pe)) return false;
        min_code.push_back(pe);
        return projection_is_canonical(g, it2->second, code, min_code);
    }
    return true;
}

// Seeds: every directed edge whose from-label <= to-label, grouped by
// (from label, edge label, to label) in ascending order (gspan.cu:41-50, 411-426).
struct SeedKey {
    int fl, el, tl;
    bool operator<(const SeedKey& o) const
    {
        if (fl != o.fl) return fl < o.fl;
        if (el != o.el) return el < o.el;
        return tl < o.tl;
    }
};

template <class F>
void for_each_seed(const Graph& g, F&& fn)
{
    for (int u = 0; u < g.n; ++u)
        for (int i = g.offsets[u]; i < g.offsets[u + 1]; ++i) {
            const int tl = g.vlabels[g.edges[i].to];
            if (g.vlabels[u] <= tl) fn(SeedKey{g.vlabels[u], g.edges[i].label, tl}, i);
        }
}

// ---------------------------------------------------------------------------
// MNI support with the reference's CUDA-path semantics (gspan.cu:165-190,
// 200-289): the domain of vertex 0 comes from layer 0's `from`, the domain of
// every other vertex from the `to` of its forward edge; min over non-empty
// domains.

int mni_support(const Graph& g, const Code& code, const Layers& layers, std::vector<uint64_t>& bits)
{
    int vmax = 0;
    for (const PEdge& e : code) vmax = std::max(vmax, std::max(e.from, e.to));
    const int nv = vmax + 1;
    const size_t words = ((size_t)g.n + 63) / 64;
    bits.assign((size_t)nv * words, 0);
    const long long last = (long long)layers.back()->size();
    const int L = (int)code.size();
    #pragma omp parallel for schedule(static)
    for (long long r = 0; r < last; ++r) {
        long long idx = r;
        for (int layer = L - 1; layer >= 0; --layer) {
            const Rel& rel = (*layers[layer])[idx];
            const Edge& de = g.edges[rel.eid];
            if (code[layer].forward())
                __atomic_fetch_or(&bits[(size_t)code[layer].to * words + (uint32_t)de.to / 64],
                                  (uint64_t)1 << ((uint32_t)de.to % 64), __ATOMIC_RELAXED);
            if (layer == 0)
                __atomic_fetch_or(&bits[(uint32_t)de.from / 64],
                                  (uint64_t)1 << ((uint32_t)de.from % 64), __ATOMIC_RELAXED);
            idx = rel.prev;
        }
    }
    int sup = 0x7fffffff;
    for (int p = 0; p < nv; ++p) {
        long long c = 0;
        for (size_t w = 0; w < words; ++w) c += __builtin_popcountll(bits[(size_t)p * words + w]);
        if (c > 0 && c < sup) sup = (int)c;
    }
    return sup;
}

// ---------------------------------------------------------------------------
// Extension of every embedding of one pattern (gspan.cu:674-780).

using BackMap = std::map<int, std::map<int, Rels>>;                  // [v_i][el]
using FwdMap = std::map<int, std::map<int, std::map<int, Rels>>>;    // [v_i][el][tl]

void extend_all(const Graph& g, const Code& code, const Layers& layers, const std::vector<int>& rm,
                BackMap& back, FwdMap& fwd)
{
    const int min_label = code[0].fl;
    const int v_n = code[rm[0]].to;
    const Rels& last = *layers.back();
    const int nthreads = omp_get_max_threads();
    std::vector<BackMap> tb(nthreads);
    std::vector<FwdMap> tf(nthreads);

    #pragma omp parallel
    {
        const int tid = omp_get_thread_num();
        BackMap& mb = tb[tid];
        FwdMap& mf = tf[tid];
        History hist;
        #pragma omp for schedule(guided)
        for (long long ei = 0; ei < (long long)last.size(); ++ei) {
            const int emb = (int)ei;
            build_history(g, layers, emb, hist);
            const int u_n = hist.h[rm[0]].to;
            for (int i = (int)rm.size() - 1; i >= 1; --i) {
                const int k = rm[i];
                int idx;
                if (backward_edge(g, hist.h[k], u_n, hist, &idx))
                    mb[code[k].from][g.edges[idx].label].push_back(Rel{emb, idx});
            }
            first_forward(g, u_n, min_label, hist, [&](int el, int tl, int idx) {
                mf[v_n][el][tl].push_back(Rel{emb, idx});
            });
            for (size_t i = 0; i < rm.size(); ++i) {
                const int k = rm[i];
                const Edge e = hist.h[k];
                const int v_i = code[k].from;
                other_forward(g, e, min_label, hist, [&](int el, int tl, int idx) {
                    mf[v_i][el][tl].push_back(Rel{emb, idx});
                });
            }
        }
    }
    // Concatenate the per-thread groups; order inside a group carries no meaning.
    for (int t = 0; t < nthreads; ++t) {
        for (auto& a : tb[t])
            for (auto& b : a.second) {
                Rels& dst = back[a.first][b.first];
                dst.insert(dst.end(), b.second.begin(), b.second.end());
            }
        for (auto& a : tf[t])
            for (auto& b : a.second)
                for (auto& c : b.second) {
                    Rels& dst = fwd[a.first][b.first][c.first];
                    dst.insert(dst.end(), c.second.begin(), c.second.end());
                }
    }
}

// ---------------------------------------------------------------------------
// Streaming last level.  Children of a pattern with k-1 edges are leaves of the
// search: the reference materialises them (gspan.cu:1131-1138), walks each
// child's layers for its MNI domains (gspan.cu:165-190, 255-260), reports it and
// stops at |code| >= k (gspan.cu:1128).  A child embedding's images are its
// parent embedding's images plus, for a forward child, the new neighbour.  So
// for each child (v_i, el[, tl]) the domain of an old pattern vertex p is
// {img_r(p) : parent row r has at least one such child}, and the new vertex's
// domain is the set of new neighbours.  One pass over the parent rows, with the
// same three rules as extend_all, accumulates exactly those sets and counts.

// Dense ranks of the labels present, so child tuples index flat arrays; rank
// order is label order, so every `<` of the reference is kept.
struct Ranks {
    std::vector<int> vlab, elab;          // sorted distinct labels
    std::vector<int> vr, er;              // rank per vertex / per directed entry
    explicit Ranks(const Graph& g)
    {
        vlab = g.vlabels;
        std::sort(vlab.begin(), vlab.end());
        vlab.erase(std::unique(vlab.begin(), vlab.end()), vlab.end());
        for (const Edge& e : g.edges) elab.push_back(e.label);
        std::sort(elab.begin(), elab.end());
        elab.erase(std::unique(elab.begin(), elab.end()), elab.end());
        vr.resize(g.n);
        for (int v = 0; v < g.n; ++v)
            vr[v] = (int)(std::lower_bound(vlab.begin(), vlab.end(), g.vlabels[v]) - vlab.begin());
        er.resize(g.m);
        for (int i = 0; i < g.m; ++i)
            er[i] = (int)(std::lower_bound(elab.begin(), elab.end(), g.edges[i].label) - elab.begin());
    }
};

inline void set_bit(uint64_t* w, uint32_t v)
{
    const uint64_t b = (uint64_t)1 << (v % 64);
    if (!(__atomic_load_n(&w[v / 64], __ATOMIC_RELAXED) & b)) __atomic_fetch_or(&w[v / 64], b, __ATOMIC_RELAXED);
}

// The slice of a parent row: a hash of the data edge id of its last layer, so
// that it does not depend on the row's position (the order of rows inside a
// materialised layer follows thread timing).
inline int row_shard(const Rels& last, long long idx, int count)
{
    uint64_t h = ((uint64_t)(uint32_t)last[idx].eid + 0x9E3779B97F4A7C15ull) * 0xBF58476D1CE4E5B9ull;
    h ^= h >> 31;
    return (int)(h % (uint64_t)count);
}

inline int min_domain(const uint64_t* bits, int nverts, size_t words)
{
    int sup = 0x7fffffff;
    for (int p = 0; p < nverts; ++p) {
        long long c = 0;
        for (size_t w = 0; w < words; ++w) c += __builtin_popcountll(bits[(size_t)p * words + w]);
        if (c > 0 && c < sup) sup = (int)c;
    }
    return sup;
}

struct Miner {
    const Graph& g;
    int k, min_support;
    const ReportFn& report;
    Stats& st;
    std::vector<uint64_t> bits;
    bool stream_last = false;
    const Ranks* ranks = nullptr;
    Shard shard;

    // The leaves below `code` (which has k-1 edges), reported in the order the
    // recursion of mine() visits them.
    void stream_children(Code& code, const Layers& layers, const std::vector<int>& rm)
    {
        const Ranks& R = *ranks;
        const int NE = (int)R.elab.size(), NV = (int)R.vlab.size();
        int nv = 0;
        for (const PEdge& e : code) nv = std::max(nv, std::max(e.from, e.to) + 1);
        const int v_n = code[rm[0]].to;
        const int min_label = code[0].fl;
        const size_t words = ((size_t)g.n + 63) / 64;
        const int nb = nv * NE, nf = nv * NE * NV;
        // Domains: a backward child has nv pattern vertices, a forward one nv+1.
        std::vector<uint64_t> bb((size_t)nb * nv * words, 0), bf((size_t)nf * (nv + 1) * words, 0);
        std::vector<uint64_t> cb(nb, 0), cf(nf, 0);
        const Rels& last = *layers.back();
        const auto t0 = std::chrono::steady_clock::now();

        #pragma omp parallel
        {
            History hist;
            std::vector<int> img(nv);
            std::vector<uint64_t> lb(nb, 0), lf(nf, 0);
            std::vector<long long> stamp_b(nb, -1), stamp_f(nf, -1);
            std::vector<int> touched_b, touched_f;
            #pragma omp for schedule(guided)
            for (long long ei = 0; ei < (long long)last.size(); ++ei) {
                if (shard.count > 1 && row_shard(last, ei, shard.count) != shard.index) continue;
                build_history(g, layers, (int)ei, hist);
                img[0] = hist.h[0].from;
                for (size_t i = 0; i < code.size(); ++i)
                    if (code[i].forward()) img[code[i].to] = hist.h[i].to;
                const int u_n = hist.h[rm[0]].to;
                touched_b.clear();
                touched_f.clear();
                for (int i = (int)rm.size() - 1; i >= 1; --i) {
                    const int kk = rm[i];
                    int idx;
                    if (backward_edge(g, hist.h[kk], u_n, hist, &idx)) {
                        const int key = code[kk].from * NE + R.er[idx];
                        ++lb[key];
                        if (stamp_b[key] != ei) { stamp_b[key] = ei; touched_b.push_back(key); }
                    }
                }
                auto fwd = [&](int v_i) {
                    return [&, v_i](int, int, int idx) {
                        const int to = g.edges[idx].to;
                        const int key = (v_i * NE + R.er[idx]) * NV + R.vr[to];
                        ++lf[key];
                        set_bit(&bf[((size_t)key * (nv + 1) + nv) * words], (uint32_t)to);
                        if (stamp_f[key] != ei) { stamp_f[key] = ei; touched_f.push_back(key); }
                    };
                };
                first_forward(g, u_n, min_label, hist, fwd(v_n));
                for (size_t i = 0; i < rm.size(); ++i)
                    other_forward(g, hist.h[rm[i]], min_label, hist, fwd(code[rm[i]].from));
                for (int key : touched_b)
                    for (int p = 0; p < nv; ++p) set_bit(&bb[((size_t)key * nv + p) * words], (uint32_t)img[p]);
                for (int key : touched_f)
                    for (int p = 0; p < nv; ++p)
                        set_bit(&bf[((size_t)key * (nv + 1) + p) * words], (uint32_t)img[p]);
            }
            #pragma omp critical
            {
                for (int q = 0; q < nb; ++q) cb[q] += lb[q];
                for (int q = 0; q < nf; ++q) cf[q] += lf[q];
            }
        }
        st.last_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

        auto leaf = [&](const PEdge& pe, uint64_t count, const uint64_t* dom, int nverts) {
            st.extended += count;
            st.last_extended += count;
            code.push_back(pe);
            if (is_canonical(code)) {
                ++st.support_calls;
                const int sup = min_domain(dom, nverts, words);
                if (sup >= min_support) {
                    ++st.patterns;
                    report(code, sup);
                }
            }
            code.pop_back();
        };
        // Backward children: ascending (v_i, edge label).
        for (int v_i = 0; v_i < nv; ++v_i)
            for (int e = 0; e < NE; ++e) {
                const int key = v_i * NE + e;
                if (cb[key])
                    leaf(PEdge{v_n, v_i, -1, R.elab[e], -1}, cb[key], &bb[(size_t)key * nv * words], nv);
            }
        // Forward children: descending v_i, then ascending (edge label, to label).
        for (int v_i = nv - 1; v_i >= 0; --v_i)
            for (int e = 0; e < NE; ++e)
                for (int t = 0; t < NV; ++t) {
                    const int key = (v_i * NE + e) * NV + t;
                    if (cf[key])
                        leaf(PEdge{v_i, v_n + 1, -1, R.elab[e], R.vlab[t]}, cf[key],
                             &bf[(size_t)key * (nv + 1) * words], nv + 1);
                }
    }

    // Pre-order recursion (gspan.cu:1118-1169).
    void mine(Code& code, Layers& layers)
    {
        if (!is_canonical(code)) return;
        ++st.support_calls;
        const int sup = mni_support(g, code, layers, bits);
        if (sup < min_support) return;
        ++st.patterns;
        report(code, sup);
        if ((int)code.size() >= k) return;

        const std::vector<int> rm = rightmost_path(code);
        const int v_n = code[rm[0]].to;
        if (stream_last && (int)code.size() + 1 == k) {
            stream_children(code, layers, rm);
            return;
        }
        BackMap back;
        FwdMap fwd;
        extend_all(g, code, layers, rm, back, fwd);
        for (auto& a : back) for (auto& b : a.second) st.extended += b.second.size();
        for (auto& a : fwd) for (auto& b : a.second) for (auto& c : b.second) st.extended += c.second.size();

        // Backward children: ascending (v_i, edge label).
        for (auto& a : back)
            for (auto& b : a.second) {
                code.push_back(PEdge{v_n, a.first, -1, b.first, -1});
                layers.push_back(&b.second);
                mine(code, layers);
                layers.pop_back();
                code.pop_back();
            }
        // Forward children: descending v_i, then ascending (edge label, to label).
        for (auto a = fwd.rbegin(); a != fwd.rend(); ++a)
            for (auto& b : a->second)
                for (auto& c : b.second) {
                    code.push_back(PEdge{a->first, v_n + 1, -1, b.first, c.first});
                    layers.push_back(&c.second);
                    mine(code, layers);
                    layers.pop_back();
                    code.pop_back();
                }
    }
};

}  // namespace

bool is_canonical(const Code& code)
{
    if (code.size() == 1) return true;
    const Graph p = pattern_graph(code);
    std::map<SeedKey, std::vector<PEmb>> seeds;
    for_each_seed(p, [&](const SeedKey& key, int i) { seeds[key].push_back(PEmb{nullptr, i}); });
    auto it = seeds.begin();
    Code min_code{PEdge{0, 1, it->first.fl, it->first.el, it->first.tl}};
    return projection_is_canonical(p, it->second, code, min_code);
}

void mine_all(const Graph& g, int k, int min_support, const ReportFn& report, Stats* stats, bool stream_last,
              Shard shard)
{
    Stats local;
    Stats& st = stats ? *stats : local;
    std::map<SeedKey, Rels> seeds;
    for_each_seed(g, [&](const SeedKey& key, int i) { seeds[key].push_back(Rel{-1, i}); });
    const Ranks ranks(g);
    Miner miner{g, k, min_support, report, st, {}, stream_last, &ranks, shard};
    for (auto& s : seeds) {
        st.seeds += s.second.size();
        Code code{PEdge{0, 1, s.first.fl, s.first.el, s.first.tl}};
        Layers layers{&s.second};
        miner.mine(code, layers);
    }
}

bool load_bin(const char* path, Graph& g)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    bool ok = std::fread(&g.n, 4, 1, f) == 1 && std::fread(&g.m, 4, 1, f) == 1 && g.n >= 0 && g.m >= 0;
    if (ok) {
        g.offsets.resize((size_t)g.n + 1);
        g.vlabels.resize(g.n);
        g.edges.resize(g.m);
        ok = std::fread(g.offsets.data(), 4, g.n + 1, f) == (size_t)g.n + 1 &&
             std::fread(g.vlabels.data(), 4, g.n, f) == (size_t)g.n &&
             std::fread(g.edges.data(), sizeof(Edge), g.m, f) == (size_t)g.m;
    }
    std::fclose(f);
    return ok;
}

}  // namespace port
