// Graph store: host arrays in the reference's CSR layout (graph.h:51-65) ->
// the device store (DevGraph).  Either one graph, or a batch of independent
// graphs ("instances") placed one after another, whose vertex labels are
// ranked per instance so that every instance owns a contiguous range of label
// ranks (its label window).
#include "miner.h"

#include <algorithm>
#include <cstring>
#include <climits>
#include <new>

namespace gs {

namespace {

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

}  // namespace

void free_graph(gspan_graph* gr, cudaStream_t st)
{
    gs::DevGraph& g = gr->g;
    if (g.offsets) cudaFreeAsync(g.offsets, st);
    if (g.adj) cudaFreeAsync(g.adj, st);
    if (g.src) cudaFreeAsync(g.src, st);
    if (g.vrank) cudaFreeAsync(g.vrank, st);
    if (g.segmask) cudaFreeAsync(g.segmask, st);
    if (g.segone) cudaFreeAsync(g.segone, st);
    g.segone = nullptr;
    if (g.segstart) cudaFreeAsync(g.segstart, st);
    g.segstart = nullptr;
    if (g.selfloop) cudaFreeAsync(g.selfloop, st);
    if (g.rev) cudaFreeAsync(g.rev, st);
    g.rev = nullptr;
    if (g.eidx) cudaFreeAsync(g.eidx, st);
    g.eidx = nullptr;
    g.eidx_cap = 0;
    if (g.win_base) cudaFreeAsync(g.win_base, st);
    g.win_base = nullptr;
    if (g.seed_counts) cudaFreeAsync(g.seed_counts, st);
    g.seed_counts = nullptr;
    g.seed_counts_h.clear();
    g.segmask = nullptr;
    g.selfloop = nullptr;
    g.offsets = nullptr;
    g.adj = nullptr;
    g.src = nullptr;
    g.vrank = nullptr;
}


gspan_status upload_graphs(gspan_ctx* ctx, int32_t ninst, const int32_t* ns, const int32_t* ms,
                           const int32_t* const* offs_in, const int32_t* const* vls_in, const gspan_edge* const* eds_in,
                           gspan_graph** out, bool on_device)
{
    // Device-resident input (one graph): the host reads only a copy of the
    // offsets here, and of labels and edges for sparse label values below.
    const int32_t* const* offs = offs_in;
    const int32_t* const* vls = vls_in;
    const gspan_edge* const* eds = eds_in;
    std::vector<int32_t> h_off, h_vl;
    std::vector<gspan_edge> h_ed;
    const int32_t* h_offp[1] = {nullptr};
    const int32_t* h_vlp[1] = {nullptr};
    const gspan_edge* h_edp[1] = {nullptr};
    const cudaMemcpyKind kin = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (on_device) {
        if (ninst != 1 || ns[0] < 0 || ms[0] < 0 || !offs_in[0]) return fail(ctx, GSPAN_ERR_INVALID, "bad device graph");
        cudaError_t e0 = cudaSetDevice(ctx->device);
        if (e0 == cudaSuccess) {
            h_off.resize((size_t)ns[0] + 1);
            e0 = cudaMemcpyAsync(h_off.data(), offs_in[0], h_off.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
        }
        if (e0 == cudaSuccess) e0 = cudaStreamSynchronize(ctx->stream);
        if (e0 != cudaSuccess) return cuda_fail(ctx, e0, "read offsets");
        h_offp[0] = h_off.data();
        offs = h_offp;
    }
    std::vector<int64_t> vbase((size_t)ninst + 1, 0), ebase((size_t)ninst + 1, 0);
    for (int32_t i = 0; i < ninst; ++i) {
        const int32_t n = ns[i], m = ms[i];
        if (n < 0 || m < 0) return fail(ctx, GSPAN_ERR_INVALID, "negative graph size");
        if (!offs[i] || (n > 0 && !vls_in[i]) || (m > 0 && !eds_in[i]))
            return fail(ctx, GSPAN_ERR_INVALID, "null graph array");
        if (offs[i][0] != 0 || offs[i][n] != m)
            return fail(ctx, GSPAN_ERR_INVALID, "offsets must start at 0 and end at nr_edges");
        vbase[(size_t)i + 1] = vbase[i] + n;
        ebase[(size_t)i + 1] = ebase[i] + m;
    }
    if (vbase[ninst] >= INT32_MAX || ebase[ninst] > INT32_MAX)
        return fail(ctx, GSPAN_ERR_LIMIT, "more than 2^31 vertices or entries in one upload");
    const int32_t N = (int32_t)vbase[ninst], M = (int32_t)ebase[ninst];
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set device");
    cudaStream_t s = ctx->stream;

    gspan_graph* gr = new (std::nothrow) gspan_graph();
    if (!gr) return fail(ctx, GSPAN_ERR_NOMEM, "host allocation");
    gr->owner = ctx;
    DevGraph& g = gr->g;
    g.n = N;
    g.m = M;
    g.ninst = ninst;

    // Temporaries of the build, freed on every path.
    gspan_edge* d_edges = nullptr;
    int32_t *d_vl = nullptr, *d_minmax = nullptr, *d_vtab = nullptr, *d_etab = nullptr, *d_elabels = nullptr;
    int64_t *d_vbase = nullptr, *d_ebase = nullptr;
    uint8_t *d_vflag = nullptr, *d_eflag = nullptr;
    uint64_t* d_tmp = nullptr;
    auto cleanup = [&]() {
        for (void* p : {(void*)d_edges, (void*)d_vl, (void*)d_minmax, (void*)d_vtab, (void*)d_etab, (void*)d_elabels,
                        (void*)d_vbase, (void*)d_ebase, (void*)d_vflag, (void*)d_eflag, (void*)d_tmp})
            if (p) cudaFreeAsync(p, s);
        d_edges = nullptr;
        d_vl = d_minmax = d_vtab = d_etab = d_elabels = nullptr;
        d_vbase = d_ebase = nullptr;
        d_vflag = d_eflag = nullptr;
        d_tmp = nullptr;
    };
    auto drop = [&]() {
        cleanup();
        free_graph(gr, s);
        cudaStreamSynchronize(s);
        delete gr;
    };
    auto bail = [&](cudaError_t err, const char* what) {
        drop();
        return cuda_fail(ctx, err, what);
    };
#define UP_CK(call, what) \
    if ((e = (call)) != cudaSuccess) return bail(e, what)
    UP_CK(cudaMallocAsync(&g.offsets, ((size_t)N + 1) * 4, s), "alloc offsets");
    if (M > 0) UP_CK(cudaMallocAsync(&d_edges, (size_t)M * sizeof(gspan_edge), s), "alloc edges");
    if (N > 0) UP_CK(cudaMallocAsync(&g.vrank, (size_t)N * 4, s), "alloc vrank");
    for (int32_t i = 0; i < ninst; ++i) {
        if (ns[i] > 0)
            UP_CK(cudaMemcpyAsync(g.offsets + vbase[i], offs[i], (size_t)ns[i] * 4, cudaMemcpyHostToDevice, s),
                  "copy offsets");
        if (ms[i] > 0)
            UP_CK(cudaMemcpyAsync(d_edges + ebase[i], eds[i], (size_t)ms[i] * sizeof(gspan_edge), kin, s),
                  "copy edges");
    }
    UP_CK(cudaMemcpyAsync(g.offsets + N, &M, 4, cudaMemcpyHostToDevice, s), "copy offsets");
    UP_CK(cudaMemsetAsync(ctx->d_status, 0, 4, s), "clear status");
    if (ninst > 1) {
        // Instance-local ids -> batch ids; an id outside its own instance is rejected.
        UP_CK(cudaMallocAsync(&d_vbase, vbase.size() * 8, s), "alloc bases");
        UP_CK(cudaMallocAsync(&d_ebase, ebase.size() * 8, s), "alloc bases");
        UP_CK(cudaMemcpyAsync(d_vbase, vbase.data(), vbase.size() * 8, cudaMemcpyHostToDevice, s), "copy bases");
        UP_CK(cudaMemcpyAsync(d_ebase, ebase.data(), ebase.size() * 8, cudaMemcpyHostToDevice, s), "copy bases");
        UP_CK(launch_batch_fixup(ninst, d_vbase, d_ebase, N, M, g.offsets, d_edges, ctx->d_status, s),
              "batch fix-up launch");
    }

    // Vertex label ranks.  One graph: min/max and presence on the device, rank
    // tables on the host (O(label range)).  A batch: per instance on the host,
    // instance-major, so each instance's labels form one window.
    constexpr int64_t kDenseRange = (int64_t)1 << 24;
    int32_t mm[4] = {INT32_MAX, INT32_MIN, INT32_MAX, INT32_MIN};
    const int32_t nv_dev = ninst == 1 ? N : 0;   // vertices ranked on the device
    if (nv_dev > 0) {
        UP_CK(cudaMallocAsync(&d_vl, (size_t)N * 4, s), "alloc labels");
        UP_CK(cudaMemcpyAsync(d_vl, vls[0], (size_t)N * 4, kin, s), "copy labels");
    }
    UP_CK(cudaMallocAsync(&d_minmax, sizeof(mm), s), "alloc minmax");
    UP_CK(cudaMemcpyAsync(d_minmax, mm, sizeof(mm), cudaMemcpyHostToDevice, s), "init minmax");
    if (nv_dev > 0 || M > 0) UP_CK(launch_label_minmax(nv_dev, d_vl, M, d_edges, d_minmax, s), "label minmax launch");
    UP_CK(cudaMemcpyAsync(mm, d_minmax, sizeof(mm), cudaMemcpyDeviceToHost, s), "read minmax");
    UP_CK(cudaStreamSynchronize(s), "label minmax");
    const int64_t vrange = nv_dev > 0 ? (int64_t)mm[1] - mm[0] + 1 : 0;
    const int64_t erange = M > 0 ? (int64_t)mm[3] - mm[2] + 1 : 0;
    const int32_t elo = mm[2];
    bool dense = vrange <= kDenseRange && erange <= kDenseRange;
    // Host sources of copies still in flight: they live until the upload's
    // status sync below (every early return syncs the stream first).
    std::vector<int32_t> vtab, etab, vrank;
    if (dense) {
        std::vector<uint8_t> vflag((size_t)vrange), eflag((size_t)erange);
        if (vrange) UP_CK(cudaMallocAsync(&d_vflag, (size_t)vrange, s), "alloc flags");
        if (erange) UP_CK(cudaMallocAsync(&d_eflag, (size_t)erange, s), "alloc flags");
        if (vrange) UP_CK(cudaMemsetAsync(d_vflag, 0, (size_t)vrange, s), "clear flags");
        if (erange) UP_CK(cudaMemsetAsync(d_eflag, 0, (size_t)erange, s), "clear flags");
        UP_CK(launch_label_presence(nv_dev, d_vl, mm[0], d_vflag, M, d_edges, elo, d_eflag, s), "presence launch");
        if (vrange) UP_CK(cudaMemcpyAsync(vflag.data(), d_vflag, (size_t)vrange, cudaMemcpyDeviceToHost, s), "flags");
        if (erange) UP_CK(cudaMemcpyAsync(eflag.data(), d_eflag, (size_t)erange, cudaMemcpyDeviceToHost, s), "flags");
        UP_CK(cudaStreamSynchronize(s), "label presence");
        vtab.assign((size_t)vrange, -1);
        etab.assign((size_t)erange, -1);
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
            UP_CK(launch_vertex_ranks(N, d_vl, mm[0], d_vtab, g.vrank, s), "vertex ranks launch");
        }
        if (erange) {
            UP_CK(cudaMallocAsync(&d_etab, (size_t)erange * 4, s), "alloc rank table");
            UP_CK(cudaMemcpyAsync(d_etab, etab.data(), (size_t)erange * 4, cudaMemcpyHostToDevice, s), "rank table");
        }
    } else {
        // Sparse label values: rank on the host.
        if (on_device) {
            h_vl.resize((size_t)N);
            h_ed.resize((size_t)M);
            if (N > 0) UP_CK(cudaMemcpyAsync(h_vl.data(), vls_in[0], (size_t)N * 4, cudaMemcpyDeviceToHost, s), "read labels");
            if (M > 0)
                UP_CK(cudaMemcpyAsync(h_ed.data(), eds_in[0], (size_t)M * sizeof(gspan_edge), cudaMemcpyDeviceToHost, s),
                      "read edges");
            UP_CK(cudaStreamSynchronize(s), "read labels");
            h_vlp[0] = h_vl.data();
            h_edp[0] = h_ed.data();
            vls = h_vlp;
            eds = h_edp;
        }
        std::vector<int32_t> dist;
        for (int32_t i = 0; i < ninst; ++i) {
            if (ms[i] == 0) continue;
            std::vector<int32_t> d2;
            rank_labels(&eds[i][0].label, (size_t)ms[i], 3, d2, nullptr);
            dist.insert(dist.end(), d2.begin(), d2.end());
        }
        std::sort(dist.begin(), dist.end());
        dist.erase(std::unique(dist.begin(), dist.end()), dist.end());
        g.elabel_of_rank = dist;
        if (nv_dev > 0) {
            rank_labels(vls[0], (size_t)N, 1, g.vlabel_of_rank, &vrank);
            UP_CK(cudaMemcpyAsync(g.vrank, vrank.data(), (size_t)N * 4, cudaMemcpyHostToDevice, s), "copy vrank");
        }
        if (!g.elabel_of_rank.empty()) {
            UP_CK(cudaMallocAsync(&d_elabels, g.elabel_of_rank.size() * 4, s), "alloc edge labels");
            UP_CK(cudaMemcpyAsync(d_elabels, g.elabel_of_rank.data(), g.elabel_of_rank.size() * 4,
                                  cudaMemcpyHostToDevice, s),
                  "copy edge labels");
        }
    }
    if (ninst == 1) {
        g.lwin = (int32_t)g.vlabel_of_rank.size();
        g.win_base_h.assign(g.vlabel_of_rank.size(), 0);
    } else {
        vrank.assign((size_t)N, 0);
        for (int32_t i = 0; i < ninst; ++i) {
            std::vector<int32_t> distinct, local;
            rank_labels(vls[i], (size_t)ns[i], 1, distinct, &local);
            const int32_t base = (int32_t)g.vlabel_of_rank.size();
            for (int32_t v = 0; v < ns[i]; ++v) vrank[(size_t)vbase[i] + v] = base + local[(size_t)v];
            for (int32_t lab : distinct) {
                g.vlabel_of_rank.push_back(lab);
                g.label_instance.push_back(i);
                g.win_base_h.push_back(base);
            }
            g.lwin = std::max(g.lwin, (int32_t)distinct.size());
        }
        if (N > 0)
            UP_CK(cudaMemcpyAsync(g.vrank, vrank.data(), (size_t)N * 4, cudaMemcpyHostToDevice, s), "copy vrank");
    }
    g.inst_vbase = vbase;
    g.inst_ebase = ebase;
    g.nvl = (int32_t)g.vlabel_of_rank.size();
    g.nel = (int32_t)g.elabel_of_rank.size();
    if (g.nvl > 0xFFFF || g.nel > 0xFFFF) {
        drop();
        return fail(ctx, GSPAN_ERR_LIMIT, "more than 65535 distinct vertex or edge labels (all instances together)");
    }
    if (g.nvl > 0) {
        UP_CK(cudaMallocAsync(&g.win_base, (size_t)g.nvl * 4, s), "alloc label windows");
        UP_CK(cudaMemcpyAsync(g.win_base, g.win_base_h.data(), (size_t)g.nvl * 4, cudaMemcpyHostToDevice, s),
              "copy label windows");
    }
    // Mean degree behind an edge, for the kernel-path choice.
    {
        double d1 = 0, d2 = 0;
        for (int32_t i = 0; i < ninst; ++i)
            for (int32_t v = 0; v < ns[i]; ++v) {
                const double d = (double)offs[i][v + 1] - offs[i][v];
                d1 += d;
                d2 += d * d;
            }
        g.edge_biased_degree = d1 > 0 ? d2 / d1 : 0.0;
    }

    if (M > 0) {
        UP_CK(cudaMallocAsync(&d_tmp, (size_t)M * 8, s), "alloc keys");
        UP_CK(cudaMallocAsync(&g.adj, (size_t)M * 8, s), "alloc adjacency");
        UP_CK(cudaMallocAsync(&g.src, (size_t)M * 4, s), "alloc sources");
    }
    UP_CK(launch_build_adjacency(g.offsets, d_edges, d_etab, elo, d_elabels, g, d_tmp, ctx->d_status, s),
          "build adjacency launch");
    uint32_t status = 0;
    UP_CK(cudaMemcpyAsync(&status, ctx->d_status, 4, cudaMemcpyDeviceToHost, s), "read status");
    cleanup();
    UP_CK(cudaStreamSynchronize(s), "graph upload");
    if (status & kErrBadGraph) {
        drop();
        return fail(ctx, GSPAN_ERR_INVALID, "malformed graph: offsets not monotone, an entry's `from` differs from "
                                            "its vertex, or a `to` is out of range");
    }
    // On the validated adjacency, with one sync for all their flags:
    // per-vertex segment masks and starts (for the mask extension path, when
    // the window's tuple space fits the mask width), self-loop bits and the
    // symmetry check, and the edge index (load factor in (3/8, 3/4]).
    // Everything these passes need zeroed (or, for the edge index, ~0) is
    // allocated first and cleared by one launch.
    ClearList clr;
    clr.add(ctx->d_status, 1);
    {
        const int64_t K = (int64_t)g.nel * g.lwin;
        if (N > 0 && K > 0 && K <= 32 * kMaxMaskWords) {
            g.segw = (int32_t)((K + 31) / 32);
            UP_CK(cudaMallocAsync(&g.segmask, (size_t)N * g.segw * 4, s), "alloc segment masks");
            UP_CK(cudaMallocAsync(&g.segone, (size_t)N * g.segw * 4, s), "alloc segment masks");
            clr.add(g.segmask, (int64_t)N * g.segw);
            clr.add(g.segone, (int64_t)N * g.segw);
            const int64_t k1 = K + 1;
            if ((double)N * k1 * 4 <= 4.0 * (1u << 30))
                UP_CK(cudaMallocAsync(&g.segstart, (size_t)N * k1 * 4, s), "alloc segment starts");
        }
    }
    {
        const size_t words = ((size_t)N + 31) / 32 + 1;
        UP_CK(cudaMallocAsync(&g.selfloop, words * 4, s), "alloc self-loop bits");
        if (M > 0) UP_CK(cudaMallocAsync(&g.rev, (size_t)M * 4, s), "alloc reverse entries");
        clr.add(g.selfloop, (int64_t)words);
    }
    if (M > 0 && M <= (1 << 30)) {
        uint32_t cap = 64;
        while ((uint64_t)cap < (uint64_t)M + M / 3) cap <<= 1;
        UP_CK(cudaMallocAsync(&g.eidx, (size_t)cap * 8, s), "alloc edge index");
        g.eidx_cap = cap;
        clr.add(g.eidx, (int64_t)cap * 2, 0xFFFFFFFFu);
    }
    // Seed counts: a property of the graph alone, counted once here and read
    // with the flags, so mining runs start from them.
    const int64_t seed_keys = (int64_t)g.nvl * g.nel * g.lwin;
    const bool keep_seeds = M > 0 && seed_keys > 0 && seed_keys <= kSeedCacheKeys;
    if (keep_seeds) {
        UP_CK(cudaMallocAsync(&g.seed_counts, (size_t)seed_keys * 8, s), "alloc seed counts");
        clr.add(g.seed_counts, seed_keys * 2);
    }
    UP_CK(launch_clear(clr, s), "clear launch");
    if (g.segw > 0) UP_CK(launch_segments(g, s), "segment launch");
    UP_CK(launch_entry_flags(g, ctx->d_status, s), "entry flags launch");
    if (keep_seeds) UP_CK(launch_seed_count(g, g.seed_counts, s), "seed count launch");
    {
        // Flags and seed counts come back through the context's pinned
        // staging, settled by one sync.
        const size_t seed_bytes = keep_seeds ? (size_t)seed_keys * 8 : 0;
        const size_t need = 16 + seed_bytes;
        if (need > ctx->h_stage_cap) {
            if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
            ctx->h_stage = nullptr;
            ctx->h_stage_cap = 0;
            const size_t cap = std::max<size_t>(need + need / 2, (size_t)1 << 16);
            UP_CK(cudaMallocHost(&ctx->h_stage, cap), "alloc readback staging");
            ctx->h_stage_cap = cap;
        }
        UP_CK(cudaMemcpyAsync(ctx->h_stage, ctx->d_status, 4, cudaMemcpyDeviceToHost, s), "read flags");
        if (keep_seeds)
            UP_CK(cudaMemcpyAsync(ctx->h_stage + 16, g.seed_counts, seed_bytes, cudaMemcpyDeviceToHost, s),
                  "read seed counts");
        UP_CK(cudaStreamSynchronize(s), "graph flags");
        uint32_t flags = 0;
        std::memcpy(&flags, ctx->h_stage, 4);
        if (keep_seeds) {
            g.seed_counts_h.resize((size_t)seed_keys);
            std::memcpy(g.seed_counts_h.data(), ctx->h_stage + 16, seed_bytes);
        }
        if (flags & kErrHashFull) {
            drop();
            return fail(ctx, GSPAN_ERR_CUDA, "edge index: a probe ran through the table");
        }
        g.symmetric = !(flags & kErrAsymmetric);
        g.loops = (flags & kFlagSelfLoop) != 0;
        g.entry_cols = g.symmetric && g.nel == 1;
        g.parallel = !g.eidx || (flags & kFlagParallel) != 0;
    }
#undef UP_CK
    ++ctx->live_graphs;
    *out = gr;
    return GSPAN_OK;
}

}  // namespace gs
