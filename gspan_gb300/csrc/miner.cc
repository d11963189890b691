// Level-synchronous mining driver (host).
//
// The reference walks the DFS-code tree depth-first, one pattern at a time
// (mine, gspan.cu:1118-1169).  Here every frequent pattern of one size is
// extended by the same kernel launch, and the reports are put back into the
// reference's pre-order at the end.  The tree is the same: a node's children
// depend only on the node's own embeddings, so visiting order changes nothing
// but the print order, which preorder_less restores.
//
// Per level:
//   1. Count pass    - histogram of child DFS-code tuples over every
//                      (embedding, adjacency entry) pair; its sum is the
//                      number of child embeddings the reference's
//                      extend_omp produces (gspan.cu:674-780).
//   2. Host          - a tuple is active when its embedding count reaches
//                      min_support (MNI support never exceeds the embedding
//                      count) and its code passes the minimum-code test, which
//                      the reference applies before support (gspan.cu:1120).
//                      Active tuples get domain sets (bitmap or hashset per
//                      tuple) and, below the last level, rows in the next
//                      level's table.
//   3. Support pass  - fills the domains and scatters child rows.
//   4. Domain sizes  - support = min over pattern vertices of the domain size
//                      (gspan.cu:282-287); frequent tuples are reported and,
//                      below k edges, become the next level's parents.
#include "miner.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <limits>

namespace gs {

gspan_status fail(gspan_ctx* ctx, gspan_status s, const std::string& msg)
{
    if (ctx) ctx->err = msg;
    return s;
}

gspan_status cuda_fail(gspan_ctx* ctx, cudaError_t e, const char* what)
{
    const gspan_status s = (e == cudaErrorMemoryAllocation) ? GSPAN_ERR_NOMEM : GSPAN_ERR_CUDA;
    return fail(ctx, s, std::string(what) + ": " + cudaGetErrorString(e));
}

#define GS_CK(call, what)                                   \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

bool preorder_less(const std::vector<CodeEdge>& a, const std::vector<CodeEdge>& b)
{
    const size_t n = std::min(a.size(), b.size());
    for (size_t j = 0; j < n; ++j) {
        const CodeEdge& x = a[j];
        const CodeEdge& y = b[j];
        if (x.from == y.from && x.to == y.to && x.fl == y.fl && x.el == y.el && x.tl == y.tl) continue;
        if (j == 0) {
            if (x.fl != y.fl) return x.fl < y.fl;
            if (x.el != y.el) return x.el < y.el;
            return x.tl < y.tl;
        }
        const bool xb = x.from > x.to, yb = y.from > y.to;
        if (xb != yb) return xb;                 // backward children first
        if (xb) {
            if (x.to != y.to) return x.to < y.to;
            return x.el < y.el;
        }
        if (x.from != y.from) return x.from > y.from;   // deeper source first
        if (x.el != y.el) return x.el < y.el;
        return x.tl < y.tl;
    }
    return a.size() < b.size();
}

namespace {

using Clock = std::chrono::steady_clock;

template <class T>
cudaError_t dalloc(T** p, size_t count, cudaStream_t st)
{
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMallocAsync(reinterpret_cast<void**>(p), count * sizeof(T), st);
}

template <class T>
void dfree(T*& p, cudaStream_t st)
{
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
}

struct Table {
    int ncols = 0;
    int64_t rows = 0;
    std::vector<int32_t*> cols;
    int32_t** d_cols = nullptr;   // device copy of `cols`

    void release(cudaStream_t st)
    {
        for (auto& c : cols) dfree(c, st);
        cols.clear();
        dfree(d_cols, st);
        ncols = 0;
        rows = 0;
    }
};

struct Parent {
    std::vector<CodeEdge> code;
    int64_t row_begin, row_end;
};

struct Found {
    std::vector<CodeEdge> code;
    int support;
};

struct Active {
    int32_t key;          // index in the level key space
    std::vector<CodeEdge> code;
    uint64_t count;       // embeddings of this child
    int nvc;              // pattern vertices of the child
};

std::vector<int> rightmost_path(const std::vector<CodeEdge>& c)
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

uint32_t next_pow2(uint64_t x)
{
    uint64_t c = 32;
    while (c < x) c <<= 1;
    return (uint32_t)std::min<uint64_t>(c, 1ull << 31);
}

// Device state of the active tuples of one level.
struct ActiveSet {
    int32_t nact = 0;
    uint32_t* pool = nullptr;
    DomDesc* d_dom = nullptr;
    long long* d_mat = nullptr;
    unsigned long long* d_cursor = nullptr;
    int32_t* d_act = nullptr;
    std::vector<DomDesc> dom;
    std::vector<long long> mat;
    uint64_t hash_domains = 0;

    void release(cudaStream_t st)
    {
        dfree(pool, st);
        dfree(d_dom, st);
        dfree(d_mat, st);
        dfree(d_cursor, st);
        dfree(d_act, st);
    }
};

struct Run {
    gspan_ctx* ctx;
    const DevGraph& g;
    int k;
    int min_support;
    uint64_t threshold;   // embedding count an active tuple needs
    gspan_stats st{};
    std::vector<Found> found;
    cudaStream_t s;
    bool profile;

    // Every host<->device copy of a mining run goes through here and is counted.
    cudaError_t copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t strm)
    {
        if (kind == cudaMemcpyHostToDevice) st.h2d_bytes += bytes;
        if (kind == cudaMemcpyDeviceToHost) st.d2h_bytes += bytes;
        return cudaMemcpyAsync(dst, src, bytes, kind, strm);
    }

    bool use_hash(uint64_t count) const
    {
        const int mode = ctx->opts.domain_mode;
        if (mode == 1) return false;
        if (mode == 2) return true;
        const double thr = ctx->opts.hash_threshold > 0 ? ctx->opts.hash_threshold : 1.0;
        return 64.0 * (double)std::min<uint64_t>(count, (uint64_t)g.n) < (double)g.n * thr;
    }

    // Domains, act[] and output rows for the active tuples; allocates `out`
    // when `materialize` is set.
    gspan_status setup_active(const std::vector<Active>& act, int64_t nkeys, bool materialize, ActiveSet& as,
                              Table& out)
    {
        as.nact = (int32_t)act.size();
        as.dom.resize(act.size());
        as.mat.assign(act.size(), -1);
        const uint32_t words = (uint32_t)std::max<int64_t>(1, ((int64_t)g.n + 31) / 32);
        uint64_t bitmap_words = 0, hash_words = 0;
        int out_cols = 0;
        int64_t out_rows = 0;
        for (size_t i = 0; i < act.size(); ++i) {
            const bool h = use_hash(act[i].count);
            DomDesc d{};
            d.nvc = (uint16_t)act[i].nvc;
            d.hash = h ? 1 : 0;
            d.cap = h ? next_pow2(2 * std::min<uint64_t>(act[i].count, (uint64_t)g.n)) : words;
            if (h) {
                d.off = hash_words;
                hash_words += (uint64_t)d.cap * d.nvc;
                as.hash_domains += d.nvc;
            } else {
                d.off = bitmap_words;
                bitmap_words += (uint64_t)d.cap * d.nvc;
            }
            as.dom[i] = d;
            if (materialize) {
                as.mat[i] = out_rows;
                out_rows += (int64_t)act[i].count;
                out_cols = std::max(out_cols, act[i].nvc);
            }
        }
        for (auto& d : as.dom)
            if (d.hash) d.off += bitmap_words;   // hashsets after all bitmaps

        std::vector<int32_t> act_h((size_t)nkeys, -1);
        for (size_t i = 0; i < act.size(); ++i) act_h[act[i].key] = (int32_t)i;

        GS_CK(dalloc(&as.d_act, (size_t)nkeys, s), "alloc act");
        GS_CK(copy(as.d_act, act_h.data(), act_h.size() * 4, cudaMemcpyHostToDevice, s), "copy act");
        if (as.nact > 0) {
            GS_CK(dalloc(&as.pool, bitmap_words + hash_words, s), "alloc domains");
            if (bitmap_words) GS_CK(cudaMemsetAsync(as.pool, 0, bitmap_words * 4, s), "clear bitmaps");
            if (hash_words)
                GS_CK(cudaMemsetAsync(as.pool + bitmap_words, 0xFF, hash_words * 4, s), "clear hashsets");
            GS_CK(dalloc(&as.d_dom, act.size(), s), "alloc dom");
            GS_CK(copy(as.d_dom, as.dom.data(), act.size() * sizeof(DomDesc), cudaMemcpyHostToDevice, s),
                  "copy dom");
            GS_CK(dalloc(&as.d_mat, act.size(), s), "alloc mat");
            GS_CK(copy(as.d_mat, as.mat.data(), act.size() * sizeof(long long), cudaMemcpyHostToDevice, s),
                  "copy mat");
            GS_CK(dalloc(&as.d_cursor, act.size(), s), "alloc cursor");
            GS_CK(cudaMemsetAsync(as.d_cursor, 0, act.size() * 8, s), "clear cursor");
        }
        if (materialize && out_rows > 0) {
            out.ncols = out_cols;
            out.rows = out_rows;
            out.cols.assign(out_cols, nullptr);
            for (int c = 0; c < out_cols; ++c) GS_CK(dalloc(&out.cols[c], (size_t)out_rows, s), "alloc level table");
            GS_CK(dalloc(&out.d_cols, (size_t)out_cols, s), "alloc column table");
            GS_CK(copy(out.d_cols, out.cols.data(), out_cols * sizeof(int32_t*), cudaMemcpyHostToDevice, s),
                  "copy column table");
            st.materialized_rows += (uint64_t)out_rows;
        }
        st.support_keys += (uint64_t)as.nact;
        st.hash_domains += as.hash_domains;
        return GSPAN_OK;
    }

    // Sizes of every domain -> support per active tuple.
    gspan_status supports(const ActiveSet& as, std::vector<int>& sup)
    {
        sup.assign(as.nact, 0);
        if (as.nact == 0) return GSPAN_OK;
        uint32_t* d_sizes = nullptr;
        GS_CK(dalloc(&d_sizes, (size_t)as.nact * kMaxV, s), "alloc sizes");
        if (profile) cudaEventRecord(ctx->ev_c, s);
        GS_CK(launch_domain_sizes(as.d_dom, as.nact, as.pool, d_sizes, s), "domain sizes launch");
        if (profile) cudaEventRecord(ctx->ev_d, s);
        ++st.kernel_launches;
        std::vector<uint32_t> h((size_t)as.nact * kMaxV);
        GS_CK(copy(h.data(), d_sizes, h.size() * 4, cudaMemcpyDeviceToHost, s), "read sizes");
        uint32_t status = 0;
        GS_CK(copy(&status, ctx->d_status, 4, cudaMemcpyDeviceToHost, s), "read status");
        GS_CK(cudaStreamSynchronize(s), "domain sizes");
        dfree(d_sizes, s);
        if (profile) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ctx->ev_c, ctx->ev_d);
            st.domain_ms += ms;
        }
        if (status) return fail(ctx, GSPAN_ERR_DEVICE, "kernel status word " + std::to_string(status));
        for (int32_t a = 0; a < as.nact; ++a) {
            uint32_t best = std::numeric_limits<uint32_t>::max();
            for (int p = 0; p < as.dom[a].nvc; ++p) {
                const uint32_t c = h[(size_t)a * kMaxV + p];
                if (c > 0 && c < best) best = c;
            }
            sup[a] = (int)std::min<uint32_t>(best, 0x7fffffffu);
        }
        return GSPAN_OK;
    }

    gspan_status seeds(std::vector<Parent>& next, Table& table)
    {
        const int64_t nkeys = (int64_t)g.nvl * g.nel * g.nvl;
        if (nkeys > (int64_t)std::numeric_limits<int32_t>::max())
            return fail(ctx, GSPAN_ERR_LIMIT, "too many distinct labels for the 1-edge key space");
        if (g.m == 0 || nkeys == 0) return GSPAN_OK;
        unsigned long long* d_counts = nullptr;
        GS_CK(dalloc(&d_counts, (size_t)nkeys, s), "alloc seed counts");
        GS_CK(cudaMemsetAsync(d_counts, 0, nkeys * 8, s), "clear seed counts");
        if (profile) cudaEventRecord(ctx->ev_a, s);
        GS_CK(launch_seed_count(g, d_counts, s), "seed count launch");
        ++st.kernel_launches;
        std::vector<unsigned long long> counts((size_t)nkeys);
        GS_CK(copy(counts.data(), d_counts, nkeys * 8, cudaMemcpyDeviceToHost, s), "read seed counts");
        GS_CK(cudaStreamSynchronize(s), "seed count");
        std::vector<Active> act;
        for (int64_t key = 0; key < nkeys; ++key) {
            const uint64_t c = counts[key];
            if (c == 0) continue;
            st.seeds += c;
            if (c < threshold) continue;
            const int fl = (int)(key / ((int64_t)g.nel * g.nvl));
            const int el = (int)((key / g.nvl) % g.nel);
            const int tl = (int)(key % g.nvl);
            act.push_back(Active{(int32_t)key, {CodeEdge{0, 1, fl, el, tl}}, c, 2});
        }
        ActiveSet as;
        const bool mat = k > 1;
        gspan_status rc = setup_active(act, nkeys, mat, as, table);
        if (rc != GSPAN_OK) return rc;
        LevelKeys keys{d_counts, as.d_act, as.d_dom, as.d_mat, as.d_cursor};
        if (as.nact > 0) {
            GS_CK(launch_seed_support(g, keys, as.pool, mat ? table.cols[0] : nullptr, mat ? table.cols[1] : nullptr,
                                      ctx->d_status, s),
                  "seed support launch");
            ++st.kernel_launches;
        }
        if (profile) cudaEventRecord(ctx->ev_b, s);
        std::vector<int> sup;
        rc = supports(as, sup);
        if (rc != GSPAN_OK) return rc;
        if (profile) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b);
            st.seed_ms += ms;
        }
        for (int32_t a = 0; a < as.nact; ++a) {
            if (sup[a] < min_support) continue;
            found.push_back(Found{act[a].code, sup[a]});
            if (k > 1) next.push_back(Parent{act[a].code, as.mat[a], as.mat[a] + (int64_t)act[a].count});
        }
        as.release(s);
        dfree(d_counts, s);
        return GSPAN_OK;
    }

    gspan_status level(int size, std::vector<Parent>& parents, Table& table, std::vector<Parent>& next, Table& out)
    {
        const int32_t LeLv = g.nel * g.nvl;
        std::vector<ParentMeta> meta(parents.size());
        std::vector<int64_t> key_span(parents.size());
        int64_t nkeys = 0, ntiles = 0;
        double read_bytes = 0;
        for (size_t i = 0; i < parents.size(); ++i) {
            const std::vector<CodeEdge>& c = parents[i].code;
            ParentMeta& P = meta[i];
            std::memset(&P, 0, sizeof(P));
            const std::vector<int> rm = rightmost_path(c);
            int nv = 0;
            for (const CodeEdge& e : c) nv = std::max(nv, std::max(e.from, e.to) + 1);
            P.nv = (int16_t)nv;
            P.vn = (int16_t)c[rm[0]].to;
            P.min_label = (int16_t)c[0].fl;
            P.vlab[0] = (int16_t)c[0].fl;
            for (const CodeEdge& e : c)
                if (e.from < e.to) P.vlab[e.to] = (int16_t)e.tl;
            P.nsrc = (int16_t)(rm.size() + 1);
            P.src_v[0] = P.vn;
            for (size_t s2 = 1; s2 <= rm.size(); ++s2) {
                const CodeEdge& e = c[rm[s2 - 1]];
                P.src_v[s2] = (int16_t)e.from;
                P.src_el[s2] = (int16_t)e.el;
                P.src_tl[s2] = P.vlab[e.to];
            }
            P.nback = (int16_t)(rm.size() - 1);
            for (int t = 0; t < P.nback; ++t) {
                const CodeEdge& e = c[rm[t + 1]];
                P.back_v[t] = (int16_t)e.from;
                P.back_el[t] = (int16_t)e.el;
                P.back_eq[t] = (int16_t)(P.vlab[e.to] <= P.vlab[P.vn]);
            }
            P.nedge = (int16_t)c.size();
            for (size_t j = 0; j < c.size(); ++j) {
                P.e_from[j] = (int8_t)c[j].from;
                P.e_to[j] = (int8_t)c[j].to;
                P.e_el[j] = (int16_t)c[j].el;
            }
            P.row_begin = parents[i].row_begin;
            P.row_end = parents[i].row_end;
            P.tile_begin = ntiles;
            ntiles += (P.row_end - P.row_begin + 31) / 32;
            P.key_base = (int32_t)nkeys;
            key_span[i] = (int64_t)P.nsrc * LeLv + (int64_t)P.nback * g.nel;
            nkeys += key_span[i];
            if (nkeys > (int64_t)std::numeric_limits<int32_t>::max())
                return fail(ctx, GSPAN_ERR_LIMIT, "child key space exceeds 2^31 tuples");
            read_bytes += (double)(P.row_end - P.row_begin) * (4.0 * nv + 8.0 * P.nsrc);
        }

        ParentMeta* d_meta = nullptr;
        unsigned long long* d_counts = nullptr;
        GS_CK(dalloc(&d_meta, meta.size(), s), "alloc parents");
        GS_CK(copy(d_meta, meta.data(), meta.size() * sizeof(ParentMeta), cudaMemcpyHostToDevice, s),
              "copy parents");
        GS_CK(dalloc(&d_counts, (size_t)nkeys, s), "alloc counts");
        GS_CK(cudaMemsetAsync(d_counts, 0, nkeys * 8, s), "clear counts");
        GS_CK(cudaMemsetAsync(ctx->d_counters, 0, 16, s), "clear counters");

        ExpandArgs x{};
        x.g = &g;
        x.parents = d_meta;
        x.nparents = (int32_t)meta.size();
        x.ntiles = ntiles;
        x.in_cols = table.ncols;
        x.in_col_ptrs = table.d_cols;
        x.out_col_ptrs = nullptr;
        x.keys.counts = d_counts;
        x.tile_counter = ctx->d_counters;
        x.scanned = ctx->d_counters + 1;
        x.status = ctx->d_status;

        if (profile) cudaEventRecord(ctx->ev_a, s);
        GS_CK(launch_expand(x, Pass::Count, s), "count pass launch");
        if (profile) cudaEventRecord(ctx->ev_b, s);
        ++st.kernel_launches;
        std::vector<unsigned long long> counts((size_t)nkeys);
        unsigned long long ctr[2] = {0, 0};
        GS_CK(copy(counts.data(), d_counts, nkeys * 8, cudaMemcpyDeviceToHost, s), "read counts");
        GS_CK(copy(ctr, ctx->d_counters, 16, cudaMemcpyDeviceToHost, s), "read counters");
        GS_CK(cudaStreamSynchronize(s), "count pass");
        if (profile) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b);
            st.expand_ms += ms;
            st.expand_launches += 1;
            st.expand_bytes += read_bytes + 8.0 * (double)ctr[1];
        }
        st.scanned_entries += ctr[1];

        const bool mat = size + 1 < k;
        std::vector<Active> act;
        for (size_t i = 0; i < parents.size(); ++i) {
            const ParentMeta& P = meta[i];
            const std::vector<CodeEdge>& c = parents[i].code;
            for (int64_t lk = 0; lk < key_span[i]; ++lk) {
                const int32_t key = P.key_base + (int32_t)lk;
                const uint64_t cnt = counts[key];
                if (cnt == 0) continue;
                st.extended += cnt;
                if (cnt < threshold) continue;
                std::vector<CodeEdge> child = c;
                int nvc;
                if (lk < (int64_t)P.nsrc * LeLv) {
                    const int s2 = (int)(lk / LeLv);
                    const int el = (int)((lk / g.nvl) % g.nel);
                    const int tl = (int)(lk % g.nvl);
                    child.push_back(CodeEdge{P.src_v[s2], P.nv, -1, el, tl});
                    nvc = P.nv + 1;
                } else {
                    const int64_t r = lk - (int64_t)P.nsrc * LeLv;
                    const int t = (int)(r / g.nel);
                    const int el = (int)(r % g.nel);
                    child.push_back(CodeEdge{P.vn, P.back_v[t], -1, el, -1});
                    nvc = P.nv;
                }
                if (!is_min_code(child.data(), (int)child.size())) continue;
                act.push_back(Active{key, std::move(child), cnt, nvc});
            }
        }

        ActiveSet as;
        gspan_status rc = setup_active(act, nkeys, mat, as, out);
        if (rc != GSPAN_OK) return rc;
        if (as.nact > 0) {
            GS_CK(cudaMemsetAsync(ctx->d_counters, 0, 8, s), "clear tile counter");
            x.keys = LevelKeys{d_counts, as.d_act, as.d_dom, as.d_mat, as.d_cursor};
            x.dom_pool = as.pool;
            x.out_col_ptrs = mat ? out.d_cols : nullptr;
            if (profile) cudaEventRecord(ctx->ev_a, s);
            GS_CK(launch_expand(x, Pass::Support, s), "support pass launch");
            if (profile) cudaEventRecord(ctx->ev_b, s);
            ++st.kernel_launches;
        }
        std::vector<int> sup;
        rc = supports(as, sup);
        if (rc != GSPAN_OK) return rc;
        if (profile && as.nact > 0) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ctx->ev_a, ctx->ev_b);
            st.expand_ms += ms;
            st.expand_launches += 1;
            double wbytes = 0;
            if (mat)
                for (const Active& a2 : act) wbytes += 4.0 * a2.nvc * (double)a2.count;
            st.expand_bytes += read_bytes + 8.0 * (double)ctr[1] + wbytes;
        }
        for (int32_t a = 0; a < as.nact; ++a) {
            if (sup[a] < min_support) continue;
            found.push_back(Found{act[a].code, sup[a]});
            if (mat) next.push_back(Parent{act[a].code, as.mat[a], as.mat[a] + (int64_t)act[a].count});
        }
        as.release(s);
        dfree(d_counts, s);
        dfree(d_meta, s);
        return GSPAN_OK;
    }
};

}  // namespace

gspan_status mine(gspan_ctx* ctx, const DevGraph& g, int k, int min_support, gspan_emit_fn emit, void* user,
                  gspan_stats* stats)
{
    const auto t0 = Clock::now();
    // The reference aborts for k < 1 (std::bad_array_new_length in its context
    // set-up); here it is an argument error.
    if (k < 1) return fail(ctx, GSPAN_ERR_INVALID, "k must be at least 1");
    if (k > kMaxE) return fail(ctx, GSPAN_ERR_LIMIT, "k exceeds the largest supported pattern size");
    Run run{ctx, g, k, min_support, (uint64_t)std::max(min_support, 1)};
    run.s = ctx->stream;
    run.profile = ctx->opts.profile != 0;
    GS_CK(cudaMemsetAsync(ctx->d_status, 0, 4, run.s), "clear status");

    std::vector<Parent> parents;
    Table table;
    gspan_status rc = run.seeds(parents, table);
    int size = 1;
    while (rc == GSPAN_OK && !parents.empty()) {
        std::vector<Parent> next;
        Table out;
        rc = run.level(size, parents, table, next, out);
        table.release(run.s);
        if (rc != GSPAN_OK) {
            out.release(run.s);
            break;
        }
        table = out;
        parents.swap(next);
        ++size;
    }
    table.release(run.s);
    run.st.levels = run.found.empty() ? 0 : size;
    if (rc != GSPAN_OK) {
        cudaStreamSynchronize(run.s);
        return rc;
    }
    GS_CK(cudaStreamSynchronize(run.s), "mine");

    std::sort(run.found.begin(), run.found.end(),
              [](const Found& a, const Found& b) { return preorder_less(a.code, b.code); });
    run.st.patterns = run.found.size();
    run.st.mine_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
    if (stats) *stats = run.st;
    if (emit) {
        std::vector<gspan_pattern_edge> buf;
        for (const Found& f : run.found) {
            buf.resize(f.code.size());
            for (size_t j = 0; j < f.code.size(); ++j) {
                const CodeEdge& e = f.code[j];
                buf[j].from = e.from;
                buf[j].to = e.to;
                buf[j].from_label = e.fl < 0 ? -1 : g.vlabel_of_rank[e.fl];
                buf[j].edge_label = e.el < 0 ? -1 : g.elabel_of_rank[e.el];
                buf[j].to_label = e.tl < 0 ? -1 : g.vlabel_of_rank[e.tl];
            }
            if (emit(user, buf.data(), (int32_t)buf.size(), f.support) != 0)
                return fail(ctx, GSPAN_ERR_ABORTED, "stopped by the emit callback");
        }
    }
    return GSPAN_OK;
}

}  // namespace gs
