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
#include <functional>
#include <limits>
#include <tuple>
#include <unordered_set>

namespace gs {

gspan_status fail(gspan_ctx* ctx, gspan_status s, const std::string& msg)
{
    if (ctx) ctx->err = msg;
    return s;
}

gspan_status cuda_fail(gspan_ctx* ctx, cudaError_t e, const char* what)
{
    const gspan_status s = (e == cudaErrorMemoryAllocation) ? GSPAN_ERR_NOMEM : GSPAN_ERR_CUDA;
    // Running out of memory leaves the context usable, but the runtime keeps
    // the error as this thread's last error, where the next launch check
    // would find it again.
    if (e == cudaErrorMemoryAllocation) cudaGetLastError();
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

// Device blocks held by the mining run on this thread.  Whatever an early
// error return leaves behind is freed when the run ends (LiveBlocks).
thread_local std::unordered_set<void*>* t_live = nullptr;

template <class T>
cudaError_t dalloc(T** p, size_t count, cudaStream_t st)
{
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(p), count * sizeof(T), st);
    if (e != cudaSuccess) *p = nullptr;
    else if (t_live) t_live->insert(*p);
    return e;
}

template <class T>
void dfree(T*& p, cudaStream_t st)
{
    if (p) {
        if (t_live) t_live->erase(p);
        cudaFreeAsync(p, st);
    }
    p = nullptr;
}

struct LiveBlocks {
    std::unordered_set<void*> blocks;
    cudaStream_t s;
    int device;
    bool out_of_memory = false;
    LiveBlocks(cudaStream_t st, int dev) : s(st), device(dev) { t_live = &blocks; }
    ~LiveBlocks()
    {
        for (void* p : blocks) cudaFreeAsync(p, s);
        t_live = nullptr;
        // A run that ran out of memory has grown the pool to the device's
        // limit: hand the unused part back, so other work (and other
        // processes) can allocate again.
        cudaMemPool_t pool;
        if (out_of_memory && cudaStreamSynchronize(s) == cudaSuccess &&
            cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess)
            cudaMemPoolTrimTo(pool, 0);
    }
};

struct Table {
    int ncols = 0;
    int ecol = -1;                // first entry column (one per pattern edge), -1 if none
    int64_t rows = 0;
    std::vector<int32_t*> cols;
    int32_t** d_cols = nullptr;   // device copy of `cols`

    void release(cudaStream_t st)
    {
        for (auto& c : cols) dfree(c, st);
        cols.clear();
        dfree(d_cols, st);
        ncols = 0;
        ecol = -1;
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
    int inst;      // mining instance (0 for a single graph)
};

struct Active {
    int32_t key;          // index in the level key space
    std::vector<CodeEdge> code;
    uint64_t count;       // embeddings of this child
    int nvc;              // pattern vertices of the child
    int32_t vbase = 0;    // the child's instance: first vertex and vertex count
    int32_t nloc = 0;
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

// Two-level last step: the parents of the last level are not materialised but
// generated from their own parents' rows by k_mask_gen.  Per parent of the
// last level: its parent's index in `up` (metas of the level above, rows in
// that level's table), the child tuple it is (kind 1 forward from source s with
// window key kc, kind 2 backward to target s with edge label kc) and its
// embedding count.
struct GenSource {
    std::vector<ParentMeta> up;
    std::vector<int32_t> up_of;
    std::vector<int16_t> kind, s;
    std::vector<int32_t> kc;
    std::vector<uint64_t> rows;
};

struct Run {
    gspan_ctx* ctx;
    const DevGraph& g;
    int k;
    const std::vector<int32_t>& minsup;   // per mining instance
    gspan_stats st{};

    // A pattern's instance follows from any of its labels (the first one's).
    int instance_of(int fl) const { return g.label_instance.empty() ? 0 : g.label_instance[fl]; }
    int min_support_of(int fl) const { return minsup[instance_of(fl)]; }
    // Embeddings a child needs before its support is worth counting: MNI
    // support never exceeds the embedding count.
    uint64_t threshold(int fl) const { return (uint64_t)std::max(min_support_of(fl), 1); }
    // Vertex and entry ranges of the instance a pattern (first label fl) lives in.
    void window(int fl, int32_t* vbase, int32_t* nloc, int32_t* ebase, int32_t* mloc) const
    {
        const int i = instance_of(fl);
        *vbase = (int32_t)g.inst_vbase[i];
        *nloc = (int32_t)(g.inst_vbase[i + 1] - g.inst_vbase[i]);
        *ebase = (int32_t)g.inst_ebase[i];
        *mloc = (int32_t)(g.inst_ebase[i + 1] - g.inst_ebase[i]);
    }
    void place(Active& a) const
    {
        int32_t eb, ml;
        window(a.code[0].fl, &a.vbase, &a.nloc, &eb, &ml);
    }
    std::vector<Found> found;
    cudaStream_t s;
    bool profile;

    // Free device memory for the size decisions (group budgets, stored or
    // generated last levels).  The query costs tens of microseconds, so it is
    // taken while kernels run - after the seed count and each level's launches -
    // and the decisions use the latest value.
    size_t free_b = 0;
    void refresh_free()
    {
        size_t f = 0, t = 0;
        if (cudaMemGetInfo(&f, &t) == cudaSuccess) free_b = f;
    }

    // A stream synchronisation, its blocked host time summed into the stats.
    cudaError_t wait(cudaStream_t strm)
    {
        const auto w0 = Clock::now();
        const cudaError_t e = cudaStreamSynchronize(strm);
        st.sync_ms += std::chrono::duration<double, std::milli>(Clock::now() - w0).count();
        return e;
    }

    // Every host<->device copy of a mining run goes through here and is counted.
    cudaError_t copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t strm)
    {
        if (kind == cudaMemcpyHostToDevice) st.h2d_bytes += bytes;
        if (kind == cudaMemcpyDeviceToHost) st.d2h_bytes += bytes;
        return cudaMemcpyAsync(dst, src, bytes, kind, strm);
    }

    // Device-to-host readbacks settled by one stream sync: the copies land in
    // the context's pinned staging buffer and are then moved to their
    // destinations (into pageable memory every copy would be a blocking round
    // trip of its own).
    struct Rb {
        void* dst;
        const void* src;
        size_t bytes;
    };
    gspan_status readback(std::initializer_list<Rb> items, const char* what)
    {
        size_t need = 0;
        for (const Rb& r : items) need += (r.bytes + 15) & ~(size_t)15;
        if (need > ctx->h_stage_cap) {
            if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
            ctx->h_stage = nullptr;
            ctx->h_stage_cap = 0;
            const size_t cap = std::max<size_t>(need + need / 2, (size_t)1 << 16);
            GS_CK(cudaMallocHost(&ctx->h_stage, cap), "alloc readback staging");
            ctx->h_stage_cap = cap;
        }
        size_t off = 0;
        for (const Rb& r : items) {
            if (r.bytes) GS_CK(copy(ctx->h_stage + off, r.src, r.bytes, cudaMemcpyDeviceToHost, s), what);
            off += (r.bytes + 15) & ~(size_t)15;
        }
        GS_CK(wait(s), what);
        off = 0;
        for (const Rb& r : items) {
            if (r.bytes) std::memcpy(r.dst, ctx->h_stage + off, r.bytes);
            off += (r.bytes + 15) & ~(size_t)15;
        }
        return GSPAN_OK;
    }

    bool use_hash(uint64_t count, int32_t nloc) const
    {
        const int mode = ctx->opts.domain_mode;
        if (mode == 1) return false;
        if (mode == 2) return true;
        const double thr = ctx->opts.hash_threshold > 0 ? ctx->opts.hash_threshold : 1.0;
        return 64.0 * (double)std::min<uint64_t>(count, (uint64_t)nloc) < (double)nloc * thr;
    }

    // Domains, act[] and output rows for the active tuples; allocates `out`
    // when `materialize` is set.
    gspan_status setup_active(const std::vector<Active>& act, int64_t nkeys, bool materialize, ActiveSet& as,
                              Table& out)
    {
        as.nact = (int32_t)act.size();
        as.dom.resize(act.size());
        as.mat.assign(act.size(), -1);

        uint64_t bitmap_words = 0, hash_words = 0;
        int out_cols = 0;
        int64_t out_rows = 0;
        for (size_t i = 0; i < act.size(); ++i) {
            const int32_t nloc = act[i].nloc;
            const bool h = use_hash(act[i].count, nloc);
            const uint32_t words = (uint32_t)std::max<int64_t>(1, ((int64_t)nloc + 31) / 32);
            DomDesc d{};
            d.nvc = (uint16_t)act[i].nvc;
            d.hash = h ? 1 : 0;
            d.vbase = act[i].vbase;
            d.cap = h ? next_pow2(2 * std::min<uint64_t>(act[i].count, (uint64_t)nloc)) : words;
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
            GS_CK(dalloc(&as.d_dom, act.size(), s), "alloc dom");
            GS_CK(copy(as.d_dom, as.dom.data(), act.size() * sizeof(DomDesc), cudaMemcpyHostToDevice, s),
                  "copy dom");
            GS_CK(dalloc(&as.d_mat, act.size(), s), "alloc mat");
            GS_CK(copy(as.d_mat, as.mat.data(), act.size() * sizeof(long long), cudaMemcpyHostToDevice, s),
                  "copy mat");
            GS_CK(dalloc(&as.d_cursor, act.size(), s), "alloc cursor");
            // Bitmaps zero, hashsets empty (~0), cursors zero: one launch.
            ClearList aclr;
            aclr.add(as.pool, (int64_t)bitmap_words);
            aclr.add(as.pool + bitmap_words, (int64_t)hash_words, 0xFFFFFFFFu);
            aclr.add(as.d_cursor, (int64_t)act.size() * 2);
            GS_CK(launch_clear(aclr, s), "clear launch");
            st.kernel_launches += aclr.n > 0;
        }
        if (materialize && out_rows > 0) {
            // One entry column (the seed's entry) follows the vertex columns.
            if (g.entry_cols) {
                out.ecol = out_cols;
                out_cols += 1;
            }
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
        uint32_t status = 0;
        gspan_status rc = readback({{h.data(), d_sizes, h.size() * 4}, {&status, ctx->d_status, 4}}, "domain sizes");
        if (rc != GSPAN_OK) return rc;
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
        const int64_t nkeys = (int64_t)g.nvl * g.nel * g.lwin;
        if (nkeys > (int64_t)std::numeric_limits<int32_t>::max())
            return fail(ctx, GSPAN_ERR_LIMIT, "too many distinct labels for the 1-edge key space");
        if (g.m == 0 || nkeys == 0) return GSPAN_OK;
        // The counts per 1-edge tuple depend on the graph alone: the store
        // keeps them (device and host copies) when its key space is small
        // enough, else they are counted here.
        const bool cached = g.seed_counts != nullptr;
        unsigned long long* d_counts = g.seed_counts;
        std::vector<unsigned long long> counted;
        if (profile) cudaEventRecord(ctx->ev_a, s);
        if (!cached) {
            GS_CK(dalloc(&d_counts, (size_t)nkeys, s), "alloc seed counts");
            GS_CK(cudaMemsetAsync(d_counts, 0, nkeys * 8, s), "clear seed counts");
            GS_CK(launch_seed_count(g, d_counts, s), "seed count launch");
            ++st.kernel_launches;
            refresh_free();
            counted.resize((size_t)nkeys);
            const gspan_status rb = readback({{counted.data(), d_counts, (size_t)nkeys * 8}}, "seed count");
            if (rb != GSPAN_OK) return rb;
        }
        const unsigned long long* const counts = cached ? g.seed_counts_h.data() : counted.data();
        std::vector<Active> act;
        for (int64_t key = 0; key < nkeys; ++key) {
            const uint64_t c = counts[key];
            if (c == 0) continue;
            st.seeds += c;
            const int fl = (int)(key / ((int64_t)g.nel * g.lwin));
            const int el = (int)((key / g.lwin) % g.nel);
            const int tl = g.win_base_h[fl] + (int)(key % g.lwin);
            if (c < threshold(fl)) continue;
            act.push_back(Active{(int32_t)key, {CodeEdge{0, 1, fl, el, tl}}, c, 2});
            place(act.back());
        }
        ActiveSet as;
        const bool mat = k > 1;
        gspan_status rc = setup_active(act, nkeys, mat, as, table);
        if (rc != GSPAN_OK) return rc;
        LevelKeys keys{d_counts, as.d_act, as.d_dom, as.d_mat, as.d_cursor};
        if (as.nact > 0) {
            GS_CK(launch_seed_support(g, keys, as.nact, as.pool, mat ? table.cols[0] : nullptr, mat ? table.cols[1] : nullptr,
                                      mat && table.ecol >= 0 ? table.cols[table.ecol] : nullptr, ctx->d_status, s),
                  "seed support launch");
            ++st.kernel_launches;
        }
        if (cached) refresh_free();
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
            if (sup[a] < min_support_of(act[a].code[0].fl)) continue;
            found.push_back(Found{act[a].code, sup[a], instance_of(act[a].code[0].fl)});
            if (k > 1) next.push_back(Parent{act[a].code, as.mat[a], as.mat[a] + (int64_t)act[a].count});
        }
        as.release(s);
        if (!cached) dfree(d_counts, s);
        return GSPAN_OK;
    }

    // Kernel timing (profile mode): event pairs resolved at the next sync.
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_free;
    std::vector<std::tuple<cudaEvent_t, cudaEvent_t, double*>> ev_pending;

    void tic(cudaEvent_t* a, cudaEvent_t* b)
    {
        if (!profile) return;
        if (ev_free.empty()) {
            cudaEvent_t x, y;
            cudaEventCreate(&x);
            cudaEventCreate(&y);
            ev_free.emplace_back(x, y);
        }
        *a = ev_free.back().first;
        *b = ev_free.back().second;
        ev_free.pop_back();
        cudaEventRecord(*a, s);
    }
    void toc(cudaEvent_t a, cudaEvent_t b, double* into)
    {
        if (!profile) return;
        cudaEventRecord(b, s);
        ev_pending.emplace_back(a, b, into);
    }
    void resolve()
    {
        for (auto& t : ev_pending) {
            float ms = 0;
            cudaEventSynchronize(std::get<1>(t));
            cudaEventElapsedTime(&ms, std::get<0>(t), std::get<1>(t));
            *std::get<2>(t) += ms;
            ev_free.emplace_back(std::get<0>(t), std::get<1>(t));
        }
        ev_pending.clear();
    }
    // The event pairs go back to the context for its next run (creating and
    // destroying them took tens of microseconds per run).
    void drop_events()
    {
        resolve();
        ctx->ev_pool.insert(ctx->ev_pool.end(), ev_free.begin(), ev_free.end());
        ev_free.clear();
    }

    struct Freq {
        int32_t key;
        std::vector<CodeEdge> code;
        uint64_t count;
        int nvc;
        int support;
    };

    // Whether the next-to-last level (children `freq` of the parents in
    // `table`) is generated inside the last level's row pass rather than
    // stored: opts.fused_last 2 always, 1 never, 0 when its table would take
    // more than half the free device memory.  Only the mask path can take
    // generated rows, so every child must fit its masks.
    bool generate_last(const std::vector<Freq>& freq, const Table& table) const
    {
        const int mode = ctx->opts.fused_last;
        if (mode == 1 || g.segw == 0 || ctx->opts.path == 1) return false;
        double bytes = 0;
        for (const Freq& f : freq) {
            const int nback = (int)rightmost_path(f.code).size() - 1;
            if ((int64_t)nback * g.nel > 32 * kMaxMaskWords) return false;
            const int ncols = f.nvc + (table.ecol >= 0 ? (int)f.code.size() : 0);
            bytes += 4.0 * ncols * (double)f.count;
        }
        if (mode == 2) return true;
        return bytes > 0.5 * (double)free_b;
    }

    // Materialisation readback waiting for a sync (see the end of level()).
    bool pending_scan = false;
    void settle()
    {
        if (!pending_scan) return;
        st.scanned_entries += ctx->h_pin[0];
        st.materialize_bytes += 8.0 * (double)ctx->h_pin[0];
        pending_scan = false;
    }

    // The code of child tuple lk (parent-local key) of a parent with code c.
    void child_of(const std::vector<CodeEdge>& c, const ParentMeta& P, int64_t lk, std::vector<CodeEdge>& child) const
    {
        const int32_t K = g.nel * g.lwin;
        child = c;
        if (lk < (int64_t)P.nsrc * K) {
            const int s2 = (int)(lk / K);
            const int el = (int)((lk % K) / g.lwin);
            const int tl = P.lbase + (int)(lk % g.lwin);
            child.push_back(CodeEdge{P.src_v[s2], P.nv, -1, el, tl});
        } else {
            const int64_t r = lk - (int64_t)P.nsrc * K;
            child.push_back(CodeEdge{P.vn, P.back_v[(int)(r / g.nel)], -1, (int)(r % g.nel), -1});
        }
    }

    gspan_status level(int size, std::vector<Parent>& parents, Table& table, std::vector<Parent>& next, Table& out,
                       const GenSource* gen = nullptr)
    {
        const int32_t K = g.nel * g.lwin;
        const int np = (int)parents.size();
        const int mode = ctx->opts.path;
        const bool mask_possible = g.segw > 0 && mode != 1;
        std::vector<ParentMeta> meta(np);
        std::vector<int64_t> key_span(np);
        std::vector<char> use_mask(np, 0);
        int64_t nkeys = 0;
        for (int i = 0; i < np; ++i) {
            const std::vector<CodeEdge>& c = parents[i].code;
            ParentMeta& P = meta[i];
            std::memset(&P, 0, sizeof(P));
            const std::vector<int> rm = rightmost_path(c);
            int nv = 0;
            for (const CodeEdge& e : c) nv = std::max(nv, std::max(e.from, e.to) + 1);
            P.nv = (int16_t)nv;
            P.vn = (int16_t)c[rm[0]].to;
            P.min_label = (int16_t)c[0].fl;
            P.lbase = g.win_base_h[c[0].fl];
            window(c[0].fl, &P.vbase, &P.nloc, &P.ebase, &P.mloc);
            P.vlab[0] = (int16_t)c[0].fl;
            for (const CodeEdge& e : c)
                if (e.from < e.to) P.vlab[e.to] = (int16_t)e.tl;
            P.nsrc = (int16_t)(rm.size() + 1);
            P.src_v[0] = P.vn;
            auto joined = [&](int v) {
                uint16_t bits = 0;
                for (const CodeEdge& e : c) {
                    if (e.from == v) bits |= (uint16_t)(1u << e.to);
                    if (e.to == v) bits |= (uint16_t)(1u << e.from);
                }
                return bits;
            };
            for (size_t s2 = 1; s2 <= rm.size(); ++s2) {
                const CodeEdge& e = c[rm[s2 - 1]];
                P.src_v[s2] = (int16_t)e.from;
                P.src_el[s2] = (int16_t)e.el;
                P.src_tl[s2] = P.vlab[e.to];
            }
            for (int s2 = 0; s2 < P.nsrc; ++s2) P.src_adj[s2] = joined(P.src_v[s2]);
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
            for (int j = 0; j < nv; ++j) P.lorder[j] = (int8_t)j;
            std::stable_sort(P.lorder, P.lorder + nv, [&](int8_t x, int8_t y) { return P.vlab[x] < P.vlab[y]; });
            std::memset(P.pair_edge, -1, sizeof(P.pair_edge));
            for (int s2 = 0; s2 < P.nsrc; ++s2)
                for (size_t q = 0; q < c.size(); ++q) {
                    if (c[q].from == P.src_v[s2]) P.pair_edge[s2][c[q].to] = (int8_t)q;
                    if (c[q].to == P.src_v[s2]) P.pair_edge[s2][c[q].from] = (int8_t)q;
                }
            for (int t = 0; t < P.nback; ++t)
                for (const CodeEdge& e : c)
                    if (e.el < 32 && ((e.from == P.vn && e.to == P.back_v[t]) || (e.to == P.vn && e.from == P.back_v[t])))
                        P.back_used[t] |= 1u << e.el;
            for (int s2 = 0; s2 < P.nsrc; ++s2) {
                const int vs = P.src_v[s2];
                const int lo_el = s2 == 0 ? 0 : P.src_el[s2];
                const int lo_tl = s2 == 0 ? P.min_label : P.src_tl[s2];
                int n = 0;
                for (int oi = 0; oi < nv; ++oi) {
                    const int j = P.lorder[oi];
                    const int t = P.vlab[j];
                    // Segment (edge label 0, t) at or above the source's lower bound.
                    if (t < P.min_label || !(0 > lo_el || (0 == lo_el && t >= lo_tl))) continue;
                    if (!g.loops && j == vs) continue;
                    const int jj = P.pair_edge[s2][j];
                    const int from_vs = jj >= 0 && P.e_from[jj] == vs ? 1 : 0;
                    P.walk[s2][n++] = (int32_t)((uint32_t)j | ((uint32_t)(jj + 1) << 4) | ((uint32_t)from_vs << 8) |
                                                ((uint32_t)t << 16));
                }
                P.walk_n[s2] = (int8_t)n;
            }
            P.row_begin = parents[i].row_begin;
            P.row_end = parents[i].row_end;
            if (gen) {
                P.row_begin = 0;
                P.row_end = (int64_t)gen->rows[i];
                P.gen_p2 = gen->up_of[i];
                P.gen_kind = gen->kind[i];
                P.gen_s = gen->s[i];
                P.gen_kc = gen->kc[i];
            }
            P.r_wide = P.row_end - P.row_begin >= ((int64_t)1 << 32) ? 1 : 0;
            P.key_base = (int32_t)nkeys;
            key_span[i] = (int64_t)P.nsrc * K + (int64_t)P.nback * g.nel;
            nkeys += key_span[i];
            if (nkeys > (int64_t)std::numeric_limits<int32_t>::max())
                return fail(ctx, GSPAN_ERR_LIMIT, "child key space exceeds 2^31 tuples");
            P.bw = (int32_t)(((int64_t)P.nback * g.nel + 31) / 32);
            if (P.bw < 1) P.bw = 1;
            // Keys of each source's valid range: to label >= min_label and
            // (edge label, to label) >= the source's lower bound.
            for (int s2 = 0; s2 < P.nsrc; ++s2) {
                const int lo_el = s2 == 0 ? 0 : P.src_el[s2];
                const int lo_tl = s2 == 0 ? P.min_label : P.src_tl[s2];
                for (int32_t kc = 0; kc < K && kc < 32 * kMaxMaskWords; ++kc) {
                    const int el = kc / g.lwin, tl = P.lbase + kc % g.lwin;
                    if (tl >= P.min_label && (el > lo_el || (el == lo_el && tl >= lo_tl)))
                        P.range[s2][kc >> 5] |= 1u << (kc & 31);
                }
            }
            if (mask_possible && P.bw <= kMaxMaskWords) {
                const int64_t rows = P.row_end - P.row_begin;
                // The mask path clears M and MB per parent (R and H are left
                // zero by its sweep); the per-candidate path examines about
                // rows x sources x (mean degree behind an embedding's vertex)
                // candidates, each far dearer than clearing a word.
                const double clear_words = (double)P.nsrc * (nv + 1) * P.nloc * g.segw + (double)nv * P.nloc * P.bw;
                const double bias = ctx->opts.mask_bias > 0 ? ctx->opts.mask_bias : 1.0;
                use_mask[i] = mode == 2 || (double)rows * P.nsrc * g.edge_biased_degree > 0.125 * bias * clear_words;
            }
            if (gen && !use_mask[i]) {
                if (!(mask_possible && P.bw <= kMaxMaskWords))
                    return fail(ctx, GSPAN_ERR_LIMIT, "generated last level needs the mask path");
                use_mask[i] = 1;
            }
        }

        // Mask-path parents run in groups whose arrays fit a memory budget;
        // per-candidate parents in one launch; all parents for materialisation.
        struct MGroup {
            std::vector<ParentMeta> metas;
            std::vector<int32_t> ps_parent;
            std::vector<MaskPlane> planes;   // mask planes counted after the sweep
            int64_t tiles = 0, r = 0, h = 0, m = 0, b = 0, t = 0, max_nloc = 0;
            double bytes = 0;
        };
        std::vector<MGroup> groups;
        std::vector<ParentMeta> cg, all = meta;
        std::vector<int64_t> sz_off(np, -1);
        int64_t ctiles = 0, atiles = 0, sz_total = 0;
        double rows_bytes = 0, cand_read_bytes = 0, all_read_bytes = 0;
        // The mask groups may hold this share of the free device memory.
        const double share = ctx->opts.mem_fraction > 0 ? std::min(0.4, ctx->opts.mem_fraction) : 0.4;
        const double budget = std::max(2.5e8, share * (double)free_b);
        for (int i = 0; i < np; ++i) {
            ParentMeta& A = all[i];
            const int64_t rows = A.row_end - A.row_begin;
            A.tile_begin = atiles;
            atiles += (rows + kMatTileRows - 1) / kMatTileRows;
            all_read_bytes += (double)rows * (4.0 * A.nv + 8.0 * A.nsrc);
            if (!use_mask[i]) {
                ParentMeta P = meta[i];
                P.tile_begin = ctiles;
                ctiles += (rows + 31) / 32;
                cand_read_bytes += (double)rows * (4.0 * P.nv + 8.0 * P.nsrc);
                cg.push_back(P);
                continue;
            }
            ParentMeta P = meta[i];
            const int64_t t_cap = std::max<int64_t>(1, std::min<int64_t>(rows, P.nloc));
            const int64_t rw = (int64_t)P.nsrc * P.nloc, hw = (int64_t)P.nsrc * P.mloc;
            const int64_t mw2 = (int64_t)P.nsrc * (P.nv + 1) * P.nloc * g.segw, bw2 = (int64_t)P.nv * P.nloc * P.bw;
            const int64_t tw = (int64_t)P.nsrc * t_cap;
            const double bytes = 4.0 * (double)(rw + hw + mw2 + bw2 + tw);
            if (groups.empty() || (!groups.back().metas.empty() && groups.back().bytes + bytes > budget))
                groups.emplace_back();
            MGroup& G = groups.back();
            P.tile_begin = G.tiles;
            if (gen) {
                const ParentMeta& Q = gen->up[(size_t)P.gen_p2];
                G.tiles += (Q.row_end - Q.row_begin + 31) / 32;
            } else {
                G.tiles += (rows + 31) / 32;
            }
            P.r_off = G.r;
            G.r += rw;
            P.h_off = G.h;
            G.h += hw;
            P.m_off = G.m;
            G.m += mw2;
            P.b_off = G.b;
            G.b += bw2;
            P.t_off = G.t;
            G.t += tw;
            P.t_cap = (int32_t)t_cap;
            P.ps_begin = (int32_t)G.ps_parent.size();
            for (int s2 = 0; s2 < P.nsrc; ++s2) G.ps_parent.push_back((int32_t)G.metas.size());
            P.sz_off = sz_total;
            sz_off[i] = sz_total;
            sz_total += (int64_t)P.nsrc * K * (P.nv + 1) + (int64_t)P.nback * g.nel * P.nv;
            G.bytes += bytes;
            // Mask ORs for the pattern vertices other than the source when
            // the sweep counts the source's own domain.
            const int mvert = K <= kSweepAccKeys ? P.nv - 1 : P.nv;
            rows_bytes += (double)rows * (4.0 * P.nv + P.nsrc * (16.0 + 4.0 * g.segw + 4.0 * mvert * g.segw) +
                                          8.0 * P.nback);
            // The parent's mask planes: per source, the old vertices' masks
            // (ORed by the row pass; the source's own when the sweep does
            // not count it) and the new vertex's (ORed by the sweep); per old
            // vertex, the backward-tuple masks.
            for (int s2 = 0; s2 < P.nsrc; ++s2)
                for (int p = 0; p <= P.nv; ++p) {
                    if (p == P.src_v[s2] && K <= kSweepAccKeys) continue;
                    G.planes.push_back(MaskPlane{P.m_off + ((int64_t)s2 * (P.nv + 1) + p) * P.nloc * g.segw,
                                                 P.sz_off + (int64_t)s2 * K * (P.nv + 1) + p, P.nloc, P.nv + 1, K,
                                                 (int16_t)g.segw, 0});
                }
            if (P.nback > 0)
                for (int p = 0; p < P.nv; ++p)
                    G.planes.push_back(MaskPlane{P.b_off + (int64_t)p * P.nloc * P.bw,
                                                 P.sz_off + (int64_t)P.nsrc * K * (P.nv + 1) + p, P.nloc, P.nv,
                                                 P.nback * g.nel, (int16_t)P.bw, 1});
            G.max_nloc = std::max<int64_t>(G.max_nloc, P.nloc);
            G.metas.push_back(P);
        }
        size_t nmask = 0;
        for (const MGroup& G : groups) nmask += G.metas.size();
        st.mask_parents += nmask;
        st.candidate_parents += cg.size();

        unsigned long long* d_counts = nullptr;
        ParentMeta *d_mg = nullptr, *d_cg = nullptr, *d_all = nullptr, *d_up = nullptr;
        uint32_t *d_R = nullptr, *d_H = nullptr, *d_M = nullptr, *d_MB = nullptr, *d_sizes = nullptr;
        uint32_t* d_tcount = nullptr;
        int32_t *d_touched = nullptr, *d_psp = nullptr;
        unsigned long long* d_tprefix = nullptr;
        MaskPlane* d_planes = nullptr;
        auto release = [&]() {
            dfree(d_up, s);
            dfree(d_counts, s);
            dfree(d_mg, s);
            dfree(d_cg, s);
            dfree(d_all, s);
            dfree(d_R, s);
            dfree(d_H, s);
            dfree(d_M, s);
            dfree(d_MB, s);
            dfree(d_sizes, s);
            dfree(d_tcount, s);
            dfree(d_touched, s);
            dfree(d_psp, s);
            dfree(d_tprefix, s);
            dfree(d_planes, s);
        };
        struct Guard {
            std::function<void()> f;
            ~Guard() { f(); }
        } guard{release};

        GS_CK(dalloc(&d_counts, (size_t)nkeys, s), "alloc counts");
        // Everything the level's first launch needs zeroed, cleared in one launch.
        ClearList clr;
        clr.add(d_counts, nkeys * 2);
        clr.add(ctx->d_counters, 8);

        cudaEvent_t e0, e1;
        int32_t gen_nv = 0;
        if (gen) {
            GS_CK(dalloc(&d_up, gen->up.size(), s), "alloc generating parents");
            GS_CK(copy(d_up, gen->up.data(), gen->up.size() * sizeof(ParentMeta), cudaMemcpyHostToDevice, s),
                  "copy generating parents");
            for (const ParentMeta& P : meta) gen_nv = std::max<int32_t>(gen_nv, std::max<int32_t>(P.nv, P.nedge));
            for (uint64_t r : gen->rows) st.fused_rows += r;
        }
        if (!groups.empty()) {
            int64_t mr = 0, mh = 0, mm = 0, mb = 0, mt = 0, mps = 0, mmeta = 0, mpl = 0;
            for (const MGroup& G : groups) {
                mpl = std::max<int64_t>(mpl, (int64_t)G.planes.size());
                mr = std::max(mr, G.r);
                mh = std::max(mh, G.h);
                mm = std::max(mm, G.m);
                mb = std::max(mb, G.b);
                mt = std::max(mt, G.t);
                mps = std::max<int64_t>(mps, (int64_t)G.ps_parent.size());
                mmeta = std::max<int64_t>(mmeta, (int64_t)G.metas.size());
            }
            GS_CK(dalloc(&d_R, (size_t)mr, s), "alloc R");
            GS_CK(dalloc(&d_H, (size_t)std::max<int64_t>(mh, 1), s), "alloc H");
            GS_CK(dalloc(&d_M, (size_t)std::max<int64_t>(mm, 1), s), "alloc M");
            GS_CK(dalloc(&d_MB, (size_t)std::max<int64_t>(mb, 1), s), "alloc MB");
            GS_CK(dalloc(&d_touched, (size_t)std::max<int64_t>(mt, 1), s), "alloc touched");
            GS_CK(dalloc(&d_tcount, (size_t)mps, s), "alloc touched counts");
            GS_CK(dalloc(&d_tprefix, (size_t)mps + 1, s), "alloc touched prefix");
            GS_CK(dalloc(&d_psp, (size_t)mps, s), "alloc slot parents");
            GS_CK(dalloc(&d_mg, (size_t)mmeta, s), "alloc mask parents");
            GS_CK(dalloc(&d_planes, (size_t)std::max<int64_t>(mpl, 1), s), "alloc mask planes");
            GS_CK(dalloc(&d_sizes, (size_t)std::max<int64_t>(sz_total, 1), s), "alloc sizes");
            clr.add(d_R, mr);
            clr.add(d_H, std::max<int64_t>(mh, 1));
            clr.add(d_sizes, std::max<int64_t>(sz_total, 1));
            for (size_t gi = 0; gi < groups.size(); ++gi) {
                const MGroup& G = groups[gi];
                GS_CK(copy(d_mg, G.metas.data(), G.metas.size() * sizeof(ParentMeta), cudaMemcpyHostToDevice, s),
                      "copy mask parents");
                GS_CK(copy(d_psp, G.ps_parent.data(), G.ps_parent.size() * 4, cudaMemcpyHostToDevice, s),
                      "copy slot parents");
                if (!G.planes.empty())
                    GS_CK(copy(d_planes, G.planes.data(), G.planes.size() * sizeof(MaskPlane), cudaMemcpyHostToDevice, s),
                          "copy mask planes");
                // Per group: its masks, touched counts and tile counter (the
                // sweep leaves R and H zero); the first group's go with the
                // level's clears.
                ClearList gclr;
                ClearList& c = gi == 0 ? clr : gclr;
                if (!(c.add(d_M, G.m) && c.add(d_MB, G.b) && c.add(d_tcount, (int64_t)G.ps_parent.size()) &&
                      c.add(ctx->d_counters + 2, 2)))
                    return fail(ctx, GSPAN_ERR_CUDA, "clear list full");
                GS_CK(launch_clear(c, s), "clear launch");
                st.kernel_launches += c.n > 0;
                c.n = 0;
                MaskArgs ma{};
                ma.g = &g;
                ma.parents = d_mg;
                ma.nparents = (int32_t)G.metas.size();
                ma.ntiles = G.tiles;
                ma.in_col_ptrs = table.d_cols;
                ma.ecol = table.ecol;
                ma.counts = d_counts;
                ma.sizes = d_sizes;
                ma.R = d_R;
                ma.H = d_H;
                ma.M = d_M;
                ma.MB = d_MB;
                ma.touched = d_touched;
                ma.tcount = d_tcount;
                ma.ps_parent = d_psp;
                ma.nps = (int32_t)G.ps_parent.size();
                ma.tprefix = d_tprefix;
                ma.tile_counter = ctx->d_counters + 2;
                ma.scanned = ctx->d_counters + 3;
                ma.status = ctx->d_status;
                ma.max_plane_nloc = G.max_nloc;
                tic(&e0, &e1);
                if (gen) {
                    ma.in_col_ptrs = nullptr;
                    ma.ecol = table.ecol >= 0 ? 0 : -1;   // generated rows carry entry columns too
                    ma.gen_parents = d_up;
                    ma.gen_cols = table.d_cols;
                    ma.gen_ecol = table.ecol;
                    ma.gen_nv = gen_nv;
                    GS_CK(launch_mask_gen(ma, s), "generated row pass launch");
                } else {
                    GS_CK(launch_mask_rows(ma, s), "mask row pass launch");
                }
                toc(e0, e1, &st.rows_ms);
                tic(&e0, &e1);
                GS_CK(launch_mask_sweep(ma, s), "mask sweep launch");
                toc(e0, e1, &st.sweep_ms);
                ma.planes = d_planes;
                ma.nplanes = (int32_t)G.planes.size();
                tic(&e0, &e1);
                GS_CK(launch_mask_popcount(ma, s), "mask popcount launch");
                toc(e0, e1, &st.domain_ms);
                // Row pass, touched lists, their prefix, sweep, popcount.
                st.kernel_launches += 5;
                st.rows_launches += 1;
            }
            st.rows_bytes += rows_bytes;
        }
        ExpandArgs x{};
        x.g = &g;
        x.in_cols = table.ncols;
        x.in_col_ptrs = table.d_cols;
        x.ecol_in = table.ecol;
        x.keys.counts = d_counts;
        x.tile_counter = ctx->d_counters;
        x.scanned = ctx->d_counters + 1;
        x.status = ctx->d_status;
        GS_CK(launch_clear(clr, s), "clear launch");   // no-op when a mask group took the list
        st.kernel_launches += clr.n > 0;
        if (!cg.empty()) {
            GS_CK(dalloc(&d_cg, cg.size(), s), "alloc parents");
            GS_CK(copy(d_cg, cg.data(), cg.size() * sizeof(ParentMeta), cudaMemcpyHostToDevice, s), "copy parents");
            x.parents = d_cg;
            x.parents_h = cg.data();
            x.nparents = (int32_t)cg.size();
            x.ntiles = ctiles;
            tic(&e0, &e1);
            GS_CK(launch_expand(x, Pass::Count, s), "count pass launch");
            toc(e0, e1, &st.expand_ms);
            ++st.kernel_launches;
            ++st.expand_launches;
        }
        refresh_free();
        // A child's code does not depend on its counts: while the GPU
        // counts, test the level's child tuples for minimum codes on the
        // host, stopping as soon as the stream is done so the GPU never
        // waits for it.  The decision below tests what is left.
        std::vector<int8_t> canon((size_t)nkeys, -1);
        {
            std::vector<CodeEdge> child;
            bool busy = true;
            for (int i = 0; i < np && busy; ++i)
                for (int64_t lk = 0; lk < key_span[i]; ++lk) {
                    if ((lk & 15) == 0 && cudaStreamQuery(s) != cudaErrorNotReady) {
                        busy = false;
                        break;
                    }
                    child_of(parents[i].code, meta[i], lk, child);
                    canon[(size_t)(meta[i].key_base + lk)] = is_min_code(child.data(), (int)child.size()) ? 1 : 0;
                }
            if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();
        }
        std::vector<unsigned long long> counts((size_t)nkeys);
        std::vector<uint32_t> sizes((size_t)sz_total);
        unsigned long long ctr[4] = {0, 0, 0, 0};
        uint32_t mstat = 0;
        {
            const gspan_status rb = readback({{counts.data(), d_counts, (size_t)nkeys * 8},
                                              {sizes.data(), d_sizes, (size_t)sz_total * 4},
                                              {ctr, ctx->d_counters, sizeof(ctr)},
                                              {&mstat, ctx->d_status, 4}},
                                             "extension count");
            if (rb != GSPAN_OK) return rb;
        }
        resolve();
        settle();
        st.scanned_entries += ctr[1] + ctr[3];
        if (!cg.empty()) st.expand_bytes += cand_read_bytes + 8.0 * (double)ctr[1];
        if (!groups.empty()) st.sweep_bytes += 12.0 * (double)ctr[3];
        if (mstat) return fail(ctx, GSPAN_ERR_DEVICE, "kernel status word " + std::to_string(mstat));
        // The mask kernels are done with their arrays.
        dfree(d_R, s);
        dfree(d_H, s);
        dfree(d_M, s);
        dfree(d_MB, s);
        dfree(d_touched, s);

        // Minimum-code tests the speculation did not reach, for children
        // with enough embeddings: independent, so spread over the host cores.
        {
            std::vector<std::pair<int, int64_t>> need;
            for (int i = 0; i < np; ++i) {
                const int fl = parents[i].code[0].fl;
                for (int64_t lk = 0; lk < key_span[i]; ++lk) {
                    const size_t key = (size_t)(meta[i].key_base + lk);
                    if (counts[key] != 0 && counts[key] >= threshold(fl) && canon[key] < 0) need.emplace_back(i, lk);
                }
            }
            if (!need.empty()) {
                const auto c0 = Clock::now();
                const int64_t nn = (int64_t)need.size();
#pragma omp parallel for schedule(dynamic, 16) if (nn > 64)
                for (int64_t q = 0; q < nn; ++q) {
                    std::vector<CodeEdge> child;
                    const int i = need[(size_t)q].first;
                    child_of(parents[i].code, meta[i], need[(size_t)q].second, child);
                    canon[(size_t)(meta[i].key_base + need[(size_t)q].second)] =
                        is_min_code(child.data(), (int)child.size()) ? 1 : 0;
                }
                st.canonical_ms += std::chrono::duration<double, std::milli>(Clock::now() - c0).count();
            }
        }
        // Which children count: enough embeddings, minimum code, and (mask
        // path) support from the domain sizes.
        std::vector<Freq> freq;
        std::vector<Active> cand_act;
        for (int i = 0; i < np; ++i) {
            const ParentMeta& P = meta[i];
            const std::vector<CodeEdge>& c = parents[i].code;
            for (int64_t lk = 0; lk < key_span[i]; ++lk) {
                const int32_t key = P.key_base + (int32_t)lk;
                const uint64_t cnt = counts[key];
                if (cnt == 0) continue;
                st.extended += cnt;
                if (cnt < threshold(c[0].fl)) continue;
                std::vector<CodeEdge> child;
                child_of(c, P, lk, child);
                const bool fwd = lk < (int64_t)P.nsrc * K;
                const int nvc = fwd ? P.nv + 1 : P.nv;
                const int64_t size_at = fwd ? sz_off[i] + lk * (P.nv + 1)
                                            : sz_off[i] + (int64_t)P.nsrc * K * (P.nv + 1) +
                                                  (lk - (int64_t)P.nsrc * K) * P.nv;
                const int stride = 1;
                ++st.canonical_checks;
                if (!canon[(size_t)key]) continue;
                if (use_mask[i]) {
                    uint32_t best = std::numeric_limits<uint32_t>::max();
                    for (int p = 0; p < nvc; ++p) {
                        const uint32_t v = sizes[(size_t)(size_at + (int64_t)p * stride)];
                        if (v > 0 && v < best) best = v;
                    }
                    const int sup = (int)std::min<uint32_t>(best, 0x7fffffffu);
                    ++st.support_keys;
                    if (sup >= min_support_of(c[0].fl)) freq.push_back(Freq{key, std::move(child), cnt, nvc, sup});
                } else {
                    cand_act.push_back(Active{key, std::move(child), cnt, nvc, P.vbase, P.nloc});
                }
            }
        }

        if (!cand_act.empty()) {
            ActiveSet as;
            Table none;
            gspan_status rc = setup_active(cand_act, nkeys, false, as, none);
            if (rc != GSPAN_OK) {
                as.release(s);
                return rc;
            }
            GS_CK(cudaMemsetAsync(ctx->d_counters, 0, 8, s), "clear tile counter");
            x.parents = d_cg;
            x.parents_h = cg.data();
            x.nparents = (int32_t)cg.size();
            x.ntiles = ctiles;
            x.keys = LevelKeys{d_counts, as.d_act, as.d_dom, as.d_mat, as.d_cursor};
            x.dom_pool = as.pool;
            tic(&e0, &e1);
            GS_CK(launch_expand(x, Pass::Support, s), "support pass launch");
            toc(e0, e1, &st.expand_ms);
            ++st.kernel_launches;
            ++st.expand_launches;
            st.expand_bytes += cand_read_bytes + 8.0 * (double)ctr[1];
            std::vector<int> sup;
            rc = supports(as, sup);
            resolve();
            as.release(s);
            if (rc != GSPAN_OK) return rc;
            for (size_t a2 = 0; a2 < cand_act.size(); ++a2)
                if (sup[a2] >= min_support_of(cand_act[a2].code[0].fl))
                    freq.push_back(Freq{cand_act[a2].key, std::move(cand_act[a2].code), cand_act[a2].count,
                                        cand_act[a2].nvc, sup[a2]});
        }

        st.frontier_rows = 0;
        for (const Freq& f : freq) {
            found.push_back(Found{f.code, f.support, instance_of(f.code[0].fl)});
            st.frontier_rows += f.count;
        }
        if (size + 1 >= k || freq.empty()) return GSPAN_OK;

        // Next-to-last level: its rows may be generated from this level's
        // rows inside the last level's row pass instead of being stored.
        if (size + 2 == k && generate_last(freq, table)) {
            GenSource gsrc;
            gsrc.up = meta;
            std::vector<Parent> last;
            for (const Freq& f : freq) {
                const int i = (int)(std::upper_bound(meta.begin(), meta.end(), f.key,
                                                     [](int32_t k2, const ParentMeta& m2) { return k2 < m2.key_base; }) -
                                    meta.begin()) - 1;
                const int64_t lk = f.key - meta[i].key_base;
                const int64_t nfwd = (int64_t)meta[i].nsrc * K;
                gsrc.up_of.push_back(i);
                if (lk < nfwd) {
                    gsrc.kind.push_back(1);
                    gsrc.s.push_back((int16_t)(lk / K));
                    gsrc.kc.push_back((int32_t)(lk % K));
                } else {
                    gsrc.kind.push_back(2);
                    gsrc.s.push_back((int16_t)((lk - nfwd) / g.nel));
                    gsrc.kc.push_back((int32_t)((lk - nfwd) % g.nel));
                }
                gsrc.rows.push_back(f.count);
                last.push_back(Parent{f.code, 0, (int64_t)f.count});
            }
            std::vector<Parent> none;
            Table unused;
            return level(size + 1, last, table, none, unused, &gsrc);
        }

        // Materialise the frequent children, grouped by tuple (offsets from the
        // counts: a one-digit counting sort of the candidates by DFS tuple).
        std::vector<int32_t> act_h((size_t)nkeys, -1);
        std::vector<long long> mat_h(freq.size());
        int64_t rows = 0;
        int ncols = 0;
        for (size_t a2 = 0; a2 < freq.size(); ++a2) {
            act_h[freq[a2].key] = (int32_t)a2;
            mat_h[a2] = rows;
            rows += (int64_t)freq[a2].count;
            ncols = std::max(ncols, freq[a2].nvc);
        }
        int32_t* d_act = nullptr;
        long long* d_mat = nullptr;
        unsigned long long* d_cur = nullptr;
        GS_CK(dalloc(&d_act, (size_t)nkeys, s), "alloc act");
        GS_CK(copy(d_act, act_h.data(), act_h.size() * 4, cudaMemcpyHostToDevice, s), "copy act");
        GS_CK(dalloc(&d_mat, freq.size(), s), "alloc mat");
        GS_CK(copy(d_mat, mat_h.data(), mat_h.size() * sizeof(long long), cudaMemcpyHostToDevice, s), "copy mat");
        GS_CK(dalloc(&d_cur, freq.size(), s), "alloc cursor");
        // Entry columns (one per pattern edge of the children) follow.
        if (table.ecol >= 0) {
            out.ecol = ncols;
            ncols += size + 1;
        }
        out.ncols = ncols;
        out.rows = rows;
        out.cols.assign(ncols, nullptr);
        for (int c2 = 0; c2 < ncols; ++c2) GS_CK(dalloc(&out.cols[c2], (size_t)rows, s), "alloc level table");
        GS_CK(dalloc(&out.d_cols, (size_t)ncols, s), "alloc column table");
        GS_CK(copy(out.d_cols, out.cols.data(), ncols * sizeof(int32_t*), cudaMemcpyHostToDevice, s),
              "copy column table");
        // Per parent, the frequent forward tuples to scan segment by segment.
        {
            std::vector<std::vector<std::pair<int16_t, uint32_t>>> segs_of(np);
            std::vector<int> key_parent;
            for (const Freq& f : freq) {
                int i = (int)(std::upper_bound(meta.begin(), meta.end(), f.key,
                                               [](int32_t k2, const ParentMeta& m2) { return k2 < m2.key_base; }) -
                              meta.begin()) - 1;
                const int64_t lk = f.key - meta[i].key_base;
                if (lk < (int64_t)meta[i].nsrc * K)
                    segs_of[i].emplace_back((int16_t)(lk / K), (uint32_t)(lk % K));
            }
            for (int i = 0; i < np; ++i) {
                ParentMeta& A = all[i];
                if ((int)segs_of[i].size() > kMaxV) {
                    A.nmseg = -1;
                    continue;
                }
                A.nmseg = (int16_t)segs_of[i].size();
                for (size_t q = 0; q < segs_of[i].size(); ++q) {
                    A.mseg_s[q] = segs_of[i][q].first;
                    A.mseg_kc[q] = segs_of[i][q].second;
                }
            }
        }
        GS_CK(dalloc(&d_all, all.size(), s), "alloc parents");
        GS_CK(copy(d_all, all.data(), all.size() * sizeof(ParentMeta), cudaMemcpyHostToDevice, s), "copy parents");
        {
            ClearList mclr;
            mclr.add(d_cur, (int64_t)freq.size() * 2);
            mclr.add(ctx->d_counters, 4);
            GS_CK(launch_clear(mclr, s), "clear launch");
            st.kernel_launches += mclr.n > 0;
        }
        x.parents = d_all;
        x.parents_h = all.data();
        x.nparents = (int32_t)all.size();
        x.ntiles = atiles;
        x.keys = LevelKeys{d_counts, d_act, nullptr, d_mat, d_cur};
        x.out_col_ptrs = out.d_cols;
        x.ecol_out = out.ecol;
        tic(&e0, &e1);
        GS_CK(launch_expand(x, Pass::Materialize, s), "materialise launch");
        toc(e0, e1, &st.materialize_ms);
        ++st.kernel_launches;
        ++st.materialize_launches;
        // No sync here: the next level's host work overlaps this pass.  Its
        // status bits are read with the next level's counts (the status
        // word accumulates over the run) and its scanned-entry counter lands
        // in pinned memory, settled after that sync.
        GS_CK(copy(ctx->h_pin, ctx->d_counters + 1, 8, cudaMemcpyDeviceToHost, s), "read counters");
        pending_scan = true;
        st.materialized_rows += (uint64_t)rows;
        double wbytes = 0;
        for (const Freq& f : freq) wbytes += 4.0 * f.nvc * (double)f.count;
        st.materialize_bytes += all_read_bytes + wbytes;
        for (size_t a2 = 0; a2 < freq.size(); ++a2)
            next.push_back(Parent{freq[a2].code, mat_h[a2], mat_h[a2] + (int64_t)freq[a2].count});
        dfree(d_act, s);
        dfree(d_mat, s);
        dfree(d_cur, s);
        return GSPAN_OK;
    }
};

}  // namespace

gspan_status mine(gspan_ctx* ctx, const DevGraph& g, int k, const std::vector<int32_t>& minsup, const EmitFn& emit,
                  gspan_stats* stats)
{
    const auto t0 = Clock::now();
    // The reference aborts for k < 1 (std::bad_array_new_length in its context
    // set-up); here it is an argument error.
    if (k < 1) return fail(ctx, GSPAN_ERR_INVALID, "k must be at least 1");
    if (k > kMaxE) return fail(ctx, GSPAN_ERR_LIMIT, "k exceeds the largest supported pattern size");
    if (ctx->opts.prune && g.ninst == 1 && minsup[0] > 1) {
        // Mine a copy of the store without the vertices of infrequent labels
        // (prune.cu); patterns and supports are the same, the work is less.
        gspan_graph* pruned = nullptr;
        int64_t kv = 0, ke = 0;
        gspan_status rc = prune_store(ctx, g, minsup[0], &pruned, &kv, &ke);
        if (rc != GSPAN_OK) return rc;
        if (pruned) {
            ctx->opts.prune = 0;
            rc = mine(ctx, pruned->g, k, minsup, emit, stats);
            ctx->opts.prune = 1;
            free_graph(pruned, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
            delete pruned;
            --ctx->live_graphs;
            if (stats) {
                stats->pruned_vertices = (uint64_t)(g.n - kv);
                stats->pruned_entries = (uint64_t)(g.m - ke);
                stats->mine_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
            }
            return rc;
        }
    }
    LiveBlocks live(ctx->stream, ctx->device);
    Run run{ctx, g, k, minsup};
    run.s = ctx->stream;
    run.profile = ctx->opts.profile != 0;
    run.ev_free.swap(ctx->ev_pool);
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
    run.drop_events();
    run.st.levels = run.found.empty() ? 0 : size;
    if (rc != GSPAN_OK) {
        live.out_of_memory = rc == GSPAN_ERR_NOMEM;
        cudaStreamSynchronize(run.s);
        return rc;
    }
    GS_CK(run.wait(run.s), "mine");
    run.settle();

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
            if (emit(f.inst, buf.data(), (int32_t)buf.size(), f.support) != 0)
                return fail(ctx, GSPAN_ERR_ABORTED, "stopped by the emit callback");
        }
    }
    return GSPAN_OK;
}

}  // namespace gs
