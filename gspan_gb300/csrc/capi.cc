// The C ABI (gspan_gb300.h): contexts, the device graph store and the mining
// entry point.  No exception crosses this boundary; every failure becomes a
// status code with a message in gspan_last_error.
#include "miner.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>

namespace {

using gs::cuda_fail;
using gs::fail;

#define GS_CK(call, what)                                   \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

// Ranks of the distinct values of `vals` (ascending).  Small value ranges use
// a presence table, anything else a sort.
void rank_labels(const int32_t* vals, size_t n, size_t stride_ints, std::vector<int32_t>& distinct,
                 std::vector<int32_t>* rank_of_each)
{
    distinct.clear();
    if (n == 0) {
        if (rank_of_each) rank_of_each->clear();
        return;
    }
    int64_t lo = vals[0], hi = vals[0];
    for (size_t i = 0; i < n; ++i) {
        const int64_t v = vals[i * stride_ints];
        lo = std::min(lo, v);
        hi = std::max(hi, v);
    }
    const int64_t range = hi - lo + 1;
    if (range <= (int64_t)1 << 22) {
        std::vector<int32_t> slot((size_t)range, -1);
        for (size_t i = 0; i < n; ++i) slot[(size_t)(vals[i * stride_ints] - lo)] = 0;
        int32_t r = 0;
        for (int64_t v = 0; v < range; ++v)
            if (slot[(size_t)v] == 0) {
                slot[(size_t)v] = r++;
                distinct.push_back((int32_t)(v + lo));
            }
        if (rank_of_each) {
            rank_of_each->resize(n);
            for (size_t i = 0; i < n; ++i) (*rank_of_each)[i] = slot[(size_t)(vals[i * stride_ints] - lo)];
        }
        return;
    }
    distinct.reserve(n);
    for (size_t i = 0; i < n; ++i) distinct.push_back(vals[i * stride_ints]);
    std::sort(distinct.begin(), distinct.end());
    distinct.erase(std::unique(distinct.begin(), distinct.end()), distinct.end());
    if (rank_of_each) {
        rank_of_each->resize(n);
        for (size_t i = 0; i < n; ++i)
            (*rank_of_each)[i] =
                (int32_t)(std::lower_bound(distinct.begin(), distinct.end(), vals[i * stride_ints]) - distinct.begin());
    }
}

void free_graph(gspan_graph* gr, cudaStream_t st)
{
    gs::DevGraph& g = gr->g;
    if (g.offsets) cudaFreeAsync(g.offsets, st);
    if (g.adj) cudaFreeAsync(g.adj, st);
    if (g.src) cudaFreeAsync(g.src, st);
    if (g.vrank) cudaFreeAsync(g.vrank, st);
    if (g.segmask) cudaFreeAsync(g.segmask, st);
    if (g.selfloop) cudaFreeAsync(g.selfloop, st);
    g.segmask = nullptr;
    g.selfloop = nullptr;
    g.offsets = nullptr;
    g.adj = nullptr;
    g.src = nullptr;
    g.vrank = nullptr;
}

}  // namespace

extern "C" {

void gspan_opts_default(gspan_opts* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->device = 0;
    o->domain_mode = 0;
    o->hash_threshold = 1.0;
    o->mem_fraction = 0.85;
    o->profile = 0;
    o->path = 0;
}

const char* gspan_status_string(gspan_status s)
{
    switch (s) {
    case GSPAN_OK: return "ok";
    case GSPAN_ERR_INVALID: return "invalid argument";
    case GSPAN_ERR_CUDA: return "CUDA error";
    case GSPAN_ERR_NOMEM: return "out of memory";
    case GSPAN_ERR_LIMIT: return "size limit exceeded";
    case GSPAN_ERR_DEVICE: return "device-side error";
    case GSPAN_ERR_ABORTED: return "aborted by callback";
    case GSPAN_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

const char* gspan_last_error(const gspan_ctx* ctx)
{
    return ctx ? ctx->err.c_str() : "";
}

int32_t gspan_max_pattern_edges(void)
{
    return gs::kMaxE;
}

gspan_status gspan_ctx_create(const gspan_opts* opts, gspan_ctx** out)
{
    if (!out) return GSPAN_ERR_INVALID;
    *out = nullptr;
    gspan_opts o;
    gspan_opts_default(&o);
    if (opts) o = *opts;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return GSPAN_ERR_NO_DEVICE;
    }
    if (o.device < 0 || o.device >= ndev) return GSPAN_ERR_INVALID;
    gspan_ctx* ctx = new (std::nothrow) gspan_ctx();
    if (!ctx) return GSPAN_ERR_NOMEM;
    ctx->device = o.device;
    ctx->opts = o;
    auto bail = [&](cudaError_t e) {
        ctx->err = cudaGetErrorString(e);
        gspan_ctx_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? GSPAN_ERR_NOMEM : GSPAN_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return bail(e);
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
    for (cudaEvent_t* ev : {&ctx->ev_a, &ctx->ev_b, &ctx->ev_c, &ctx->ev_d})
        if ((e = cudaEventCreate(ev)) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc(&ctx->d_status, 4)) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc(&ctx->d_counters, 32)) != cudaSuccess) return bail(e);
    // Keep freed stream-ordered blocks cached in this process, so the many
    // per-level buffers of repeated mining runs do not go back to the driver.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    ctx->expand_blocks = gs::expand_grid_blocks(ctx->device);
    *out = ctx;
    return GSPAN_OK;
}

void gspan_ctx_destroy(gspan_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    for (cudaEvent_t ev : {ctx->ev_a, ctx->ev_b, ctx->ev_c, ctx->ev_d})
        if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

gspan_status gspan_graph_upload(gspan_ctx* ctx, int32_t n, int32_t m, const int32_t* offsets,
                                const int32_t* vlabels, const gspan_edge* edges, gspan_graph** out)
{
    if (!ctx || !out) return GSPAN_ERR_INVALID;
    *out = nullptr;
    if (n < 0 || m < 0) return fail(ctx, GSPAN_ERR_INVALID, "negative graph size");
    if (!offsets || (n > 0 && !vlabels) || (m > 0 && !edges))
        return fail(ctx, GSPAN_ERR_INVALID, "null graph array");
    if (offsets[0] != 0 || offsets[n] != m)
        return fail(ctx, GSPAN_ERR_INVALID, "offsets must start at 0 and end at nr_edges");
    GS_CK(cudaSetDevice(ctx->device), "set device");
    cudaStream_t s = ctx->stream;

    gspan_graph* gr = new (std::nothrow) gspan_graph();
    if (!gr) return fail(ctx, GSPAN_ERR_NOMEM, "host allocation");
    gr->owner = ctx;
    gs::DevGraph& g = gr->g;
    g.n = n;
    g.m = m;

    // Temporaries of the build, freed on every path.
    gspan_edge* d_edges = nullptr;
    int32_t *d_vl = nullptr, *d_minmax = nullptr, *d_vtab = nullptr, *d_etab = nullptr, *d_elabels = nullptr;
    uint8_t *d_vflag = nullptr, *d_eflag = nullptr;
    uint64_t* d_tmp = nullptr;
    auto cleanup = [&]() {
        for (void* p : {(void*)d_edges, (void*)d_vl, (void*)d_minmax, (void*)d_vtab, (void*)d_etab, (void*)d_elabels,
                        (void*)d_vflag, (void*)d_eflag, (void*)d_tmp})
            if (p) cudaFreeAsync(p, s);
        d_edges = nullptr;
        d_vl = d_minmax = d_vtab = d_etab = d_elabels = nullptr;
        d_vflag = d_eflag = nullptr;
        d_tmp = nullptr;
    };
    auto drop = [&]() {
        cleanup();
        free_graph(gr, s);
        cudaStreamSynchronize(s);
        delete gr;
    };
    auto bail = [&](cudaError_t e, const char* what) {
        drop();
        return cuda_fail(ctx, e, what);
    };
    cudaError_t e;
#define UP_CK(call, what) \
    if ((e = (call)) != cudaSuccess) return bail(e, what)
    UP_CK(cudaMallocAsync(&g.offsets, ((size_t)n + 1) * 4, s), "alloc offsets");
    UP_CK(cudaMemcpyAsync(g.offsets, offsets, ((size_t)n + 1) * 4, cudaMemcpyHostToDevice, s), "copy offsets");
    if (n > 0) {
        UP_CK(cudaMallocAsync(&d_vl, (size_t)n * 4, s), "alloc labels");
        UP_CK(cudaMemcpyAsync(d_vl, vlabels, (size_t)n * 4, cudaMemcpyHostToDevice, s), "copy labels");
        UP_CK(cudaMallocAsync(&g.vrank, (size_t)n * 4, s), "alloc vrank");
    }
    if (m > 0) {
        UP_CK(cudaMallocAsync(&d_edges, (size_t)m * sizeof(gspan_edge), s), "alloc edges");
        UP_CK(cudaMemcpyAsync(d_edges, edges, (size_t)m * sizeof(gspan_edge), cudaMemcpyHostToDevice, s),
              "copy edges");
    }

    // Label ranks: min/max and presence on the device, rank tables on the host
    // (O(label range)); sparse ranges beyond 2^24 values rank on the host.
    constexpr int64_t kDenseRange = (int64_t)1 << 24;
    int32_t mm[4] = {INT32_MAX, INT32_MIN, INT32_MAX, INT32_MIN};
    UP_CK(cudaMallocAsync(&d_minmax, sizeof(mm), s), "alloc minmax");
    UP_CK(cudaMemcpyAsync(d_minmax, mm, sizeof(mm), cudaMemcpyHostToDevice, s), "init minmax");
    if (n > 0 || m > 0) UP_CK(gs::launch_label_minmax(n, d_vl, m, d_edges, d_minmax, s), "label minmax launch");
    UP_CK(cudaMemcpyAsync(mm, d_minmax, sizeof(mm), cudaMemcpyDeviceToHost, s), "read minmax");
    UP_CK(cudaStreamSynchronize(s), "label minmax");
    const int64_t vrange = n > 0 ? (int64_t)mm[1] - mm[0] + 1 : 0;
    const int64_t erange = m > 0 ? (int64_t)mm[3] - mm[2] + 1 : 0;
    int32_t elo = mm[2];
    if (vrange <= kDenseRange && erange <= kDenseRange) {
        std::vector<uint8_t> vflag((size_t)vrange), eflag((size_t)erange);
        if (vrange) UP_CK(cudaMallocAsync(&d_vflag, (size_t)vrange, s), "alloc flags");
        if (erange) UP_CK(cudaMallocAsync(&d_eflag, (size_t)erange, s), "alloc flags");
        if (vrange) UP_CK(cudaMemsetAsync(d_vflag, 0, (size_t)vrange, s), "clear flags");
        if (erange) UP_CK(cudaMemsetAsync(d_eflag, 0, (size_t)erange, s), "clear flags");
        UP_CK(gs::launch_label_presence(n, d_vl, mm[0], d_vflag, m, d_edges, elo, d_eflag, s), "presence launch");
        if (vrange) UP_CK(cudaMemcpyAsync(vflag.data(), d_vflag, (size_t)vrange, cudaMemcpyDeviceToHost, s), "flags");
        if (erange) UP_CK(cudaMemcpyAsync(eflag.data(), d_eflag, (size_t)erange, cudaMemcpyDeviceToHost, s), "flags");
        UP_CK(cudaStreamSynchronize(s), "label presence");
        std::vector<int32_t> vtab((size_t)vrange, -1), etab((size_t)erange, -1);
        for (int64_t v = 0; v < vrange; ++v)
            if (vflag[(size_t)v]) {
                vtab[(size_t)v] = (int32_t)g.vlabel_of_rank.size();
                g.vlabel_of_rank.push_back((int32_t)(v + mm[0]));
            }
        for (int64_t v = 0; v < erange; ++v)
            if (eflag[(size_t)v]) {
                etab[(size_t)v] = (int32_t)g.elabel_of_rank.size();
                g.elabel_of_rank.push_back((int32_t)(v + elo));
            }
        if (vrange) {
            UP_CK(cudaMallocAsync(&d_vtab, (size_t)vrange * 4, s), "alloc rank table");
            UP_CK(cudaMemcpyAsync(d_vtab, vtab.data(), (size_t)vrange * 4, cudaMemcpyHostToDevice, s), "rank table");
            UP_CK(gs::launch_vertex_ranks(n, d_vl, mm[0], d_vtab, g.vrank, s), "vertex ranks launch");
        }
        if (erange) {
            UP_CK(cudaMallocAsync(&d_etab, (size_t)erange * 4, s), "alloc rank table");
            UP_CK(cudaMemcpyAsync(d_etab, etab.data(), (size_t)erange * 4, cudaMemcpyHostToDevice, s), "rank table");
        }
        UP_CK(cudaStreamSynchronize(s), "rank tables");   // host tables leave scope
    } else {
        std::vector<int32_t> vrank;
        rank_labels(vlabels, (size_t)n, 1, g.vlabel_of_rank, &vrank);
        rank_labels(m > 0 ? &edges[0].label : nullptr, (size_t)m, 3, g.elabel_of_rank, nullptr);
        if (n > 0)
            UP_CK(cudaMemcpyAsync(g.vrank, vrank.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s), "copy vrank");
        if (!g.elabel_of_rank.empty()) {
            UP_CK(cudaMallocAsync(&d_elabels, g.elabel_of_rank.size() * 4, s), "alloc edge labels");
            UP_CK(cudaMemcpyAsync(d_elabels, g.elabel_of_rank.data(), g.elabel_of_rank.size() * 4,
                                  cudaMemcpyHostToDevice, s),
                  "copy edge labels");
        }
        UP_CK(cudaStreamSynchronize(s), "host ranks");
    }
    g.nvl = (int32_t)g.vlabel_of_rank.size();
    g.nel = (int32_t)g.elabel_of_rank.size();
    if (g.nvl > 0xFFFF || g.nel > 0xFFFF) {
        drop();
        return fail(ctx, GSPAN_ERR_LIMIT, "more than 65535 distinct vertex or edge labels");
    }
    // Mean degree behind an edge, for the kernel-path choice.
    {
        double d1 = 0, d2 = 0;
        for (int32_t v = 0; v < n; ++v) {
            const double d = (double)offsets[v + 1] - offsets[v];
            d1 += d;
            d2 += d * d;
        }
        g.edge_biased_degree = d1 > 0 ? d2 / d1 : 0.0;
    }

    if (m > 0) {
        UP_CK(cudaMallocAsync(&d_tmp, (size_t)m * 8, s), "alloc keys");
        UP_CK(cudaMallocAsync(&g.adj, (size_t)m * 8, s), "alloc adjacency");
        UP_CK(cudaMallocAsync(&g.src, (size_t)m * 4, s), "alloc sources");
    }
    UP_CK(cudaMemsetAsync(ctx->d_status, 0, 4, s), "clear status");
    UP_CK(gs::launch_build_adjacency(g.offsets, d_edges, d_etab, elo, d_elabels, g, d_tmp, ctx->d_status, s),
          "build adjacency launch");
    // Per-vertex masks of the (edge label, to label) segments present, for the
    // mask extension path; only when the tuple space fits the mask width.
    {
        const int64_t K = (int64_t)g.nel * g.nvl;
        if (n > 0 && K > 0 && K <= 32 * gs::kMaxMaskWords) {
            g.segw = (int32_t)((K + 31) / 32);
            UP_CK(cudaMallocAsync(&g.segmask, (size_t)n * g.segw * 4, s), "alloc segment masks");
            UP_CK(gs::launch_segmask(g, s), "segment mask launch");
        }
    }
    uint32_t status = 0;
    UP_CK(cudaMemcpyAsync(&status, ctx->d_status, 4, cudaMemcpyDeviceToHost, s), "read status");
    cleanup();
    UP_CK(cudaStreamSynchronize(s), "graph upload");
    if (status & gs::kErrBadGraph) {
        drop();
        return fail(ctx, GSPAN_ERR_INVALID, "malformed graph: offsets not monotone, an entry's `from` differs from "
                                            "its vertex, or a `to` is out of range");
    }
    // Self-loop bits and the symmetry check, on the validated adjacency.
    {
        const size_t words = ((size_t)n + 31) / 32 + 1;
        uint32_t flags = 0;
        UP_CK(cudaMallocAsync(&g.selfloop, words * 4, s), "alloc self-loop bits");
        UP_CK(cudaMemsetAsync(g.selfloop, 0, words * 4, s), "clear self-loop bits");
        UP_CK(cudaMemsetAsync(ctx->d_status, 0, 4, s), "clear status");
        UP_CK(gs::launch_graph_flags(g, ctx->d_status, s), "graph flags launch");
        UP_CK(cudaMemcpyAsync(&flags, ctx->d_status, 4, cudaMemcpyDeviceToHost, s), "read flags");
        UP_CK(cudaStreamSynchronize(s), "graph flags");
        g.symmetric = !(flags & gs::kErrAsymmetric);
    }
#undef UP_CK
    ++ctx->live_graphs;
    *out = gr;
    return GSPAN_OK;
}

gspan_status gspan_graph_free(gspan_ctx* ctx, gspan_graph* graph)
{
    if (!ctx || !graph) return GSPAN_ERR_INVALID;
    if (graph->owner != ctx) return fail(ctx, GSPAN_ERR_INVALID, "graph belongs to another context");
    cudaSetDevice(ctx->device);
    free_graph(graph, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    delete graph;
    --ctx->live_graphs;
    return GSPAN_OK;
}

gspan_status gspan_mine(gspan_ctx* ctx, const gspan_graph* graph, int32_t k, int32_t min_support,
                        gspan_emit_fn emit, void* user, gspan_stats* stats)
{
    if (!ctx || !graph) return GSPAN_ERR_INVALID;
    if (graph->owner != ctx) return fail(ctx, GSPAN_ERR_INVALID, "graph belongs to another context");
    ctx->err.clear();
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set device");
    try {
        return gs::mine(ctx, graph->g, k, min_support, emit, user, stats);
    } catch (const std::bad_alloc&) {
        return fail(ctx, GSPAN_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& ex) {
        return fail(ctx, GSPAN_ERR_INVALID, ex.what());
    }
}

gspan_status gspan_is_canonical(const gspan_pattern_edge* code, int32_t len, int32_t* out)
{
    if (!code || !out || len < 1 || len > 4096) return GSPAN_ERR_INVALID;
    std::vector<gs::CodeEdge> c((size_t)len);
    for (int32_t i = 0; i < len; ++i) {
        const gspan_pattern_edge& e = code[i];
        if (e.from < 0 || e.to < 0 || e.from == e.to || e.from > len || e.to > len)
            return GSPAN_ERR_INVALID;
        c[i] = gs::CodeEdge{e.from, e.to, e.from_label, e.edge_label, e.to_label};
    }
    try {
        *out = gs::is_min_code(c.data(), len) ? 1 : 0;
    } catch (...) {
        return GSPAN_ERR_NOMEM;
    }
    return GSPAN_OK;
}

}  // extern "C"
