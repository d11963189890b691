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
    o->mask_bias = 1.0;
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
    if ((e = cudaMallocHost(&ctx->h_pin, 64)) != cudaSuccess) return bail(e);
    // Keep freed stream-ordered blocks cached in this process, so the
    // per-level buffers of repeated mining runs are not mapped again each
    // run.  A run that fails for want of memory gives the cache back (see
    // gs::mine).
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
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
    if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    for (cudaEvent_t ev : {ctx->ev_a, ctx->ev_b, ctx->ev_c, ctx->ev_d})
        if (ev) cudaEventDestroy(ev);
    for (auto& p : ctx->ev_pool) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

gspan_status gspan_graph_upload(gspan_ctx* ctx, int32_t n, int32_t m, const int32_t* offsets,
                                const int32_t* vlabels, const gspan_edge* edges, gspan_graph** out)
{
    if (!ctx || !out) return GSPAN_ERR_INVALID;
    *out = nullptr;
    const int32_t ns[1] = {n}, ms[1] = {m};
    const int32_t* offs[1] = {offsets};
    const int32_t* vls[1] = {vlabels};
    const gspan_edge* eds[1] = {edges};
    return gs::upload_graphs(ctx, 1, ns, ms, offs, vls, eds, out);
}

gspan_status gspan_graph_upload_text(gspan_ctx* ctx, const char* text, int64_t len, gspan_graph** out,
                                     int32_t* nr_nodes, int32_t* nr_edges)
{
    if (!ctx || !out) return GSPAN_ERR_INVALID;
    *out = nullptr;
    ctx->err.clear();
    try {
        return gs::load_text(ctx, text, len, out, nr_nodes, nr_edges);
    } catch (const std::bad_alloc&) {
        return fail(ctx, GSPAN_ERR_NOMEM, "host allocation failed");
    }
}

gspan_status gspan_batch_upload(gspan_ctx* ctx, int32_t ninst, const int32_t* nr_nodes, const int32_t* nr_edges,
                                const int32_t* const* offsets, const int32_t* const* vlabels,
                                const gspan_edge* const* edges, gspan_graph** out)
{
    if (!ctx || !out || ninst < 1 || !nr_nodes || !nr_edges || !offsets || !vlabels || !edges)
        return GSPAN_ERR_INVALID;
    *out = nullptr;
    return gs::upload_graphs(ctx, ninst, nr_nodes, nr_edges, offsets, vlabels, edges, out);
}

gspan_status gspan_graph_free(gspan_ctx* ctx, gspan_graph* graph)
{
    if (!ctx || !graph) return GSPAN_ERR_INVALID;
    if (graph->owner != ctx) return fail(ctx, GSPAN_ERR_INVALID, "graph belongs to another context");
    cudaSetDevice(ctx->device);
    gs::free_graph(graph, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    delete graph;
    --ctx->live_graphs;
    return GSPAN_OK;
}

gspan_status gspan_mine(gspan_ctx* ctx, const gspan_graph* graph, int32_t k, int32_t min_support,
                        gspan_emit_fn emit, void* user, gspan_stats* stats)
{
    if (!ctx || !graph) return GSPAN_ERR_INVALID;
    if (graph->owner->device != ctx->device)
        return fail(ctx, GSPAN_ERR_INVALID, "graph was uploaded to another device");
    ctx->err.clear();
    if (graph->g.ninst != 1) return fail(ctx, GSPAN_ERR_INVALID, "a batch is mined with gspan_mine_batch");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set device");
    try {
        const std::vector<int32_t> minsup{min_support};
        gs::EmitFn fn;
        if (emit)
            fn = [emit, user](int, const gspan_pattern_edge* c, int32_t len, int32_t sup) {
                return emit(user, c, len, sup);
            };
        return gs::mine(ctx, graph->g, k, minsup, fn, stats);
    } catch (const std::bad_alloc&) {
        return fail(ctx, GSPAN_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& ex) {
        return fail(ctx, GSPAN_ERR_INVALID, ex.what());
    }
}

gspan_status gspan_mine_batch(gspan_ctx* ctx, const gspan_graph* batch, int32_t k, const int32_t* min_support,
                              gspan_batch_emit_fn emit, void* user, gspan_stats* stats)
{
    if (!ctx || !batch || !min_support) return GSPAN_ERR_INVALID;
    if (batch->owner->device != ctx->device)
        return fail(ctx, GSPAN_ERR_INVALID, "graph was uploaded to another device");
    ctx->err.clear();
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set device");
    try {
        const std::vector<int32_t> minsup(min_support, min_support + batch->g.ninst);
        gs::EmitFn fn;
        if (emit)
            fn = [emit, user](int inst, const gspan_pattern_edge* c, int32_t len, int32_t sup) {
                return emit(user, inst, c, len, sup);
            };
        return gs::mine(ctx, batch->g, k, minsup, fn, stats);
    } catch (const std::bad_alloc&) {
        return fail(ctx, GSPAN_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& ex) {
        return fail(ctx, GSPAN_ERR_INVALID, ex.what());
    }
}

int32_t gspan_graph_instances(const gspan_graph* graph)
{
    return graph ? graph->g.ninst : 0;
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
