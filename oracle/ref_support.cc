// Test infrastructure only (CPU oracle).  MNI support with the semantics of the
// reference's active CUDA path, support_gpu + support_kernel_v2
// (gspan.cu:200-289, 165-190):
//   * one domain per pattern vertex 0..v_max (gspan.cu:206-211);
//   * walking each last-level embedding from the last layer back to layer 0,
//     a forward code edge j adds edges[edge_id].to to the domain of
//     dfs_code[j].to (op_array, gspan.cu:255-260, kernel :179-183);
//   * layer 0 adds edges[edge_id].from to the domain of vertex 0 (:185-188);
//   * support = min over domains with a non-zero size (:282-287).
// Domains are bitsets over graph vertices, filled by OpenMP threads with
// atomic OR and counted afterwards by popcount.
#include "ref_support_shim.h"

#include <cstdint>
#include <vector>
#include <omp.h>

int support_gpu(const CSRGraph& g, DFSCode& dfs_code, LayeredEmbeddings& layered_embeddings)
{
    int v_max = 0;
    for (const auto& e : dfs_code) {
        if (e.from > v_max) v_max = e.from;
        if (e.to > v_max) v_max = e.to;
    }
    const int nr_pattern_nodes = v_max + 1;
    const int nr_layers = (int)dfs_code.size();
    const size_t words = ((size_t)g.nr_nodes + 63) / 64;
    std::vector<uint64_t> dom((size_t)nr_pattern_nodes * words, 0);

    const long long n_last = (long long)layered_embeddings.back()->size();
    #pragma omp parallel for schedule(static)
    for (long long r = 0; r < n_last; ++r) {
        long long idx = r;
        for (int layer = nr_layers - 1; layer >= 0; --layer) {
            const EmbeddingRel& rel = (*layered_embeddings[layer])[idx];
            const Edge& de = g.edges[rel.edge_id];
            if (dfs_code[layer].from < dfs_code[layer].to) {
                uint32_t u = (uint32_t)de.to;
                __atomic_fetch_or(&dom[(size_t)dfs_code[layer].to * words + u / 64],
                                  (uint64_t)1 << (u % 64), __ATOMIC_RELAXED);
            }
            if (layer == 0) {
                uint32_t u = (uint32_t)de.from;
                __atomic_fetch_or(&dom[u / 64], (uint64_t)1 << (u % 64), __ATOMIC_RELAXED);
            }
            idx = rel.prev_idx;
        }
    }

    int sup = 0x7fffffff;
    for (int p = 0; p < nr_pattern_nodes; ++p) {
        long long cnt = 0;
        for (size_t w = 0; w < words; ++w)
            cnt += __builtin_popcountll(dom[(size_t)p * words + w]);
        if (cnt > 0 && cnt < sup)
            sup = (int)cnt;
    }
    return sup;
}
