// Label-frequency pruning of a device store before mining: the reference's
// prune_graph (graph.cc:216-266), which its CLI leaves commented out
// (fsm.cu:28-29), applied on the GPU.
//
// A vertex whose label occurs on fewer than min_support vertices can be the
// image of no pattern vertex of a frequent pattern: that pattern vertex's MNI
// domain would hold fewer than min_support vertices.  So dropping such vertices
// and their entries keeps every frequent pattern's embeddings (their images
// all carry frequent labels) and every support, and removes only children that
// could never be frequent.  Patterns are reported in label space, so the
// renumbering is invisible in the output.  What changes is the work, and the
// extended-embedding count, which then counts children in the pruned graph.
//
// Kept vertices are renumbered densely in ascending order, and each kept
// vertex keeps its entries to kept vertices, as in the reference.  The pruned
// CSR is built in device memory and handed to the device-input store build.
#include "device_scan.cuh"
#include "miner.h"

#include <vector>

namespace gs {
namespace {

// Vertices per label rank (warp-aggregated atomics).
__global__ void k_rank_hist(int32_t n, const int32_t* __restrict__ vrank, unsigned long long* __restrict__ hist)
{
    const int lane = threadIdx.x & 31;
    // Warp per 32 consecutive vertices (the stride is a multiple of 32).
    for (int64_t base = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & ~31ll; base < n;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = base + lane;
        const bool live = v < n;
        const int32_t r = live ? vrank[v] : -1;
        const unsigned lm = __ballot_sync(kAll, live);
        if (live) {
            const unsigned peers = __match_any_sync(lm, r);
            if (lane == __ffs(peers) - 1) atomicAdd(hist + r, (unsigned long long)__popc(peers));
        }
    }
}

__global__ void k_keep_flags(int32_t n, const int32_t* __restrict__ vrank, const uint8_t* __restrict__ keep_rank,
                             uint8_t* __restrict__ flag)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        flag[v] = keep_rank[vrank[v]];
}

// Kept entries per kept vertex (its new degree), at its new id.
__global__ void k_kept_degrees(int32_t n, const int32_t* __restrict__ offsets, const uint64_t* __restrict__ adj,
                               const int32_t* __restrict__ rank, int64_t* __restrict__ deg)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t nv = rank[v];
        if (nv < 0) continue;
        int64_t d = 0;
        for (int32_t i = offsets[v]; i < offsets[v + 1]; ++i) d += rank[entry_to(adj[i])] >= 0;
        deg[nv] = d;
    }
}

// The pruned CSR: labels and edges in the graph's own label values; each kept
// vertex's entries in store order, written from its new offset.
__global__ void k_kept_entries(int32_t n, const int32_t* __restrict__ offsets, const uint64_t* __restrict__ adj,
                               const int32_t* __restrict__ vrank, const int32_t* __restrict__ rank,
                               const int64_t* __restrict__ off64, const int32_t* __restrict__ vlabel_of_rank,
                               const int32_t* __restrict__ elabel_of_rank, int32_t* __restrict__ out_off,
                               int32_t* __restrict__ out_vl, gspan_edge* __restrict__ out_edges)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t nv = rank[v];
        if (nv < 0) continue;
        out_vl[nv] = vlabel_of_rank[vrank[v]];
        int64_t at = off64[nv];
        out_off[nv] = (int32_t)at;
        for (int32_t i = offsets[v]; i < offsets[v + 1]; ++i) {
            const uint64_t e = adj[i];
            const int32_t to = rank[entry_to(e)];
            if (to >= 0) out_edges[at++] = gspan_edge{nv, to, elabel_of_rank[entry_el(e)]};
        }
    }
}

int grid_for_n(int64_t work)
{
    const int64_t b = (work + kThreads - 1) / kThreads;
    return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace

gspan_status prune_store(gspan_ctx* ctx, const DevGraph& g, int32_t min_support, gspan_graph** out,
                         int64_t* kept_vertices, int64_t* kept_entries)
{
    *out = nullptr;
    *kept_vertices = g.n;
    *kept_entries = g.m;
    if (g.ninst != 1 || g.n == 0 || g.nvl == 0) return GSPAN_OK;
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    std::vector<void*> tmp;
    auto freeall = [&]() {
        for (void* p : tmp) cudaFreeAsync(p, s);
        cudaStreamSynchronize(s);
        tmp.clear();
    };
    auto alloc = [&](void** p, size_t bytes) {
        *p = nullptr;
        const cudaError_t r = cudaMallocAsync(p, bytes < 16 ? 16 : bytes, s);
        if (r == cudaSuccess) tmp.push_back(*p);
        return r;
    };
#define PR_CK(call, what)                      \
    do {                                       \
        if ((e = (call)) != cudaSuccess) {     \
            freeall();                         \
            return cuda_fail(ctx, e, what);    \
        }                                      \
    } while (0)
    auto read = [&](void* dst, const void* src, size_t bytes) {
        cudaError_t r = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
        if (r == cudaSuccess) r = cudaStreamSynchronize(s);
        return r;
    };

    // Which labels are frequent enough to keep.
    unsigned long long* d_hist = nullptr;
    PR_CK(alloc((void**)&d_hist, (size_t)g.nvl * 8), "alloc label counts");
    PR_CK(cudaMemsetAsync(d_hist, 0, (size_t)g.nvl * 8, s), "clear label counts");
    k_rank_hist<<<grid_for_n(g.n), kThreads, 0, s>>>(g.n, g.vrank, d_hist);
    PR_CK(cudaGetLastError(), "label count launch");
    std::vector<unsigned long long> hist((size_t)g.nvl);
    PR_CK(read(hist.data(), d_hist, hist.size() * 8), "label counts");
    std::vector<uint8_t> keep_rank((size_t)g.nvl);
    bool any_dropped = false;
    for (int32_t r = 0; r < g.nvl; ++r) {
        keep_rank[r] = hist[r] >= (unsigned long long)std::max(min_support, 0) ? 1 : 0;
        any_dropped |= hist[r] > 0 && !keep_rank[r];
    }
    if (!any_dropped) {
        freeall();
        return GSPAN_OK;
    }

    // Dense new ids of the kept vertices, ascending.
    uint8_t *d_keep_rank = nullptr, *d_flag = nullptr;
    int32_t* d_rank = nullptr;
    PR_CK(alloc((void**)&d_keep_rank, keep_rank.size()), "alloc keep flags");
    PR_CK(cudaMemcpyAsync(d_keep_rank, keep_rank.data(), keep_rank.size(), cudaMemcpyHostToDevice, s), "copy keep flags");
    PR_CK(alloc((void**)&d_flag, (size_t)g.n), "alloc keep flags");
    PR_CK(alloc((void**)&d_rank, (size_t)g.n * 4), "alloc new ids");
    k_keep_flags<<<grid_for_n(g.n), kThreads, 0, s>>>(g.n, g.vrank, d_keep_rank, d_flag);
    const int64_t fb = ((int64_t)g.n + kChunk - 1) / kChunk;
    int64_t *d_fc = nullptr, *d_fo = nullptr;
    PR_CK(alloc((void**)&d_fc, (size_t)(fb + 1) * 8), "alloc id scan");
    PR_CK(alloc((void**)&d_fo, (size_t)(fb + 1) * 8), "alloc id scan");
    k_flag_count<<<(int)fb, kThreads, 0, s>>>(d_flag, g.n, d_fc);
    k_scan_small<<<1, 1024, 0, s>>>(d_fc, d_fo, fb);
    k_flag_rank<<<(int)fb, kThreads, 0, s>>>(d_flag, g.n, d_fo, d_rank);
    PR_CK(cudaGetLastError(), "new id launches");
    int64_t n2 = 0;
    PR_CK(read(&n2, d_fo + fb, 8), "kept vertex count");

    // Degrees, offsets and entries of the pruned graph.
    int64_t *d_deg = nullptr, *d_off64 = nullptr;
    int32_t *d_off = nullptr, *d_vl = nullptr, *d_lv = nullptr, *d_le = nullptr;
    PR_CK(alloc((void**)&d_deg, (size_t)(n2 + 1) * 8), "alloc degrees");
    PR_CK(alloc((void**)&d_off64, (size_t)(n2 + 2) * 8), "alloc offsets");
    PR_CK(alloc((void**)&d_off, (size_t)(n2 + 1) * 4), "alloc offsets");
    PR_CK(alloc((void**)&d_vl, (size_t)n2 * 4), "alloc labels");
    PR_CK(alloc((void**)&d_lv, g.vlabel_of_rank.size() * 4), "alloc label values");
    PR_CK(alloc((void**)&d_le, g.elabel_of_rank.size() * 4), "alloc label values");
    PR_CK(cudaMemcpyAsync(d_lv, g.vlabel_of_rank.data(), g.vlabel_of_rank.size() * 4, cudaMemcpyHostToDevice, s),
          "copy label values");
    PR_CK(cudaMemcpyAsync(d_le, g.elabel_of_rank.data(), g.elabel_of_rank.size() * 4, cudaMemcpyHostToDevice, s),
          "copy label values");
    PR_CK(cudaMemsetAsync(d_deg, 0, (size_t)(n2 + 1) * 8, s), "clear degrees");
    k_kept_degrees<<<grid_for_n(g.n), kThreads, 0, s>>>(g.n, g.offsets, g.adj, d_rank, d_deg);
    k_scan_small<<<1, 1024, 0, s>>>(d_deg, d_off64, n2);
    PR_CK(cudaGetLastError(), "degree launches");
    int64_t m2 = 0;
    PR_CK(read(&m2, d_off64 + n2, 8), "kept entry count");
    gspan_edge* d_edges = nullptr;
    PR_CK(alloc((void**)&d_edges, (size_t)m2 * sizeof(gspan_edge)), "alloc edges");
    k_kept_entries<<<grid_for_n(g.n), kThreads, 0, s>>>(g.n, g.offsets, g.adj, g.vrank, d_rank, d_off64, d_lv, d_le,
                                                         d_off, d_vl, d_edges);
    PR_CK(cudaGetLastError(), "entry launch");
    const int32_t m2i = (int32_t)m2;
    PR_CK(cudaMemcpyAsync(d_off + n2, &m2i, 4, cudaMemcpyHostToDevice, s), "close offsets");
    PR_CK(cudaStreamSynchronize(s), "pruned graph");
    const int32_t N = (int32_t)n2, M = m2i;
    const int32_t* offs[1] = {d_off};
    const int32_t* vls[1] = {d_vl};
    const gspan_edge* eds[1] = {d_edges};
    const gspan_status rc = upload_graphs(ctx, 1, &N, &M, offs, vls, eds, out, /*on_device=*/true);
    freeall();
#undef PR_CK
    if (rc == GSPAN_OK) {
        *kept_vertices = n2;
        *kept_entries = m2;
    }
    return rc;
}

}  // namespace gs
