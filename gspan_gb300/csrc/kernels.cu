// CUDA kernels of the miner, written for sm_103a.
//
// Everything here is integer work on the graph store and on column-oriented
// embedding tables; none of it is a dense contraction, so tensor cores are not
// used.  The bounds are HBM / L2 bandwidth (adjacency and table streams) and
// L2 atomic throughput (domain sets).
//
//  * build_adjacency : packs every CSR entry as (edge label, to label, to) and
//                      sorts each vertex's entries by that key (warp per vertex).
//  * seed_count / seed_support : 1-edge patterns (gspan.cu:411-426, 1176-1190).
//  * expand          : one pass over the embeddings of every parent pattern of a
//                      level, evaluating the backward / first-forward /
//                      other-forward rules of gspan.cu:428-483 for each
//                      (embedding, adjacency entry) pair.  Pass::Count builds the
//                      histogram of child DFS-code tuples; Pass::Support fills
//                      the MNI domains of the active tuples and, when the level
//                      is not the last, scatters the child rows grouped by tuple
//                      (a one-digit counting sort whose offsets the host derived
//                      from the Count histogram).
//  * domain_sizes    : popcount / occupied-slot count of every domain.
#include "engine.h"

#include <algorithm>

namespace gs {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kExpandWarps = 8;
constexpr int kExpandThreads = kExpandWarps * 32;

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------------------
// Domain sets.

__device__ __forceinline__ void bitmap_insert(uint32_t* words, uint32_t v)
{
    uint32_t* w = words + (v >> 5);
    const uint32_t bit = 1u << (v & 31u);
    // Bits only go 0 -> 1, so a stale read can cost an extra atomic but never
    // loses an insert.  __ldcg reads L2, where the atomics land.
    if (!(__ldcg(w) & bit)) atomicOr(w, bit);
}

__device__ __forceinline__ uint32_t hash_slot(uint32_t v, uint32_t cap)
{
    // Fibonacci hashing scaled to [0, cap) by a 32x32->64 multiply.
    return (uint32_t)(((uint64_t)(v * 2654435769u) * cap) >> 32);
}

__device__ void hash_insert(uint32_t* table, uint32_t cap, uint32_t v, uint32_t* status)
{
    uint32_t slot = hash_slot(v, cap);
    for (uint32_t probe = 0; probe < cap; ++probe) {
        uint32_t cur = __ldcg(table + slot);
        if (cur == v) return;
        if (cur == kHashEmpty) {
            cur = atomicCAS(table + slot, kHashEmpty, v);
            if (cur == kHashEmpty || cur == v) return;
        }
        slot = (slot + 1u) & (cap - 1u);
    }
    atomicOr(status, kErrHashFull);   // capacity is >= 2x the largest possible size: unreachable
}

__device__ __forceinline__ void dom_insert(uint32_t* pool, const DomDesc& d, int p, uint32_t v, uint32_t* status)
{
    uint32_t* base = pool + d.off + (uint64_t)p * d.cap;
    v -= (uint32_t)d.vbase;   // ids local to the tuple's instance
    if (d.hash)
        hash_insert(base, d.cap, v, status);
    else
        bitmap_insert(base, v);
}

// First index in adj[b, e) whose packed key is >= key.
__device__ __forceinline__ int32_t lower_bound_entry(const uint64_t* __restrict__ adj, int32_t b, int32_t e, uint64_t key)
{
    while (b < e) {
        const int32_t mid = b + ((e - b) >> 1);
        if (__ldg(adj + mid) < key)
            b = mid + 1;
        else
            e = mid;
    }
    return b;
}

// Edge index hash of (vertex, edge label, to): the 64-bit finaliser of
// MurmurHash3 over the packed triple.  Low bits pick the slot, high 32 bits
// are the slot's fingerprint.
__device__ __forceinline__ uint64_t edge_hash(uint32_t u, uint32_t el, uint32_t to)
{
    uint64_t h = (((uint64_t)u << 32) | to) + (uint64_t)(el + 1) * 0x9E3779B97F4A7C15ull;
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 33;
    return h;
}

// First index of `key` (packed edge label, to label, to) in u's adjacency
// adj[b, e), or -1: probes the edge index from the key's slot to the first
// empty slot.  A slot is taken only when its entry lies in [b, e) and holds
// `key`, so fingerprint collisions cannot give a wrong answer.
__device__ __forceinline__ int32_t edge_find(const uint64_t* __restrict__ eidx, uint32_t cap,
                                             const uint64_t* __restrict__ adj, int32_t b, int32_t e, uint32_t u,
                                             uint64_t key)
{
    const uint64_t h = edge_hash(u, entry_el(key), entry_to(key));
    const uint32_t fp = (uint32_t)(h >> 32);
    uint32_t i = (uint32_t)h & (cap - 1);
    for (uint32_t probe = 0; probe < cap; ++probe) {
        const uint64_t slot = __ldg(eidx + i);
        const uint32_t pos = (uint32_t)slot;
        if (pos == 0xFFFFFFFFu) return -1;
        if ((uint32_t)(slot >> 32) == fp && (int32_t)pos >= b && (int32_t)pos < e && __ldg(adj + pos) == key)
            return (int32_t)pos;
        i = (i + 1) & (cap - 1);
    }
    return -1;
}

// ---------------------------------------------------------------------------
// Graph store build.

// Label ranks on the device: min/max, then presence flags over the value
// range; the host turns the flags into rank tables.
__global__ void k_label_minmax(int32_t n, const int32_t* __restrict__ vlabels, int32_t m,
                               const gspan_edge* __restrict__ edges, int32_t* __restrict__ out)
{
    int32_t vmin = INT32_MAX, vmax = INT32_MIN, emin = INT32_MAX, emax = INT32_MIN;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        vmin = min(vmin, vlabels[i]);
        vmax = max(vmax, vlabels[i]);
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride) {
        emin = min(emin, edges[i].label);
        emax = max(emax, edges[i].label);
    }
    for (int o = 16; o > 0; o >>= 1) {
        vmin = min(vmin, __shfl_xor_sync(kFull, vmin, o));
        vmax = max(vmax, __shfl_xor_sync(kFull, vmax, o));
        emin = min(emin, __shfl_xor_sync(kFull, emin, o));
        emax = max(emax, __shfl_xor_sync(kFull, emax, o));
    }
    // Block-wide first, so the four global words see one atomic per block
    // instead of one per warp.
    __shared__ int32_t part[4][32];
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        part[0][w] = vmin;
        part[1][w] = vmax;
        part[2][w] = emin;
        part[3][w] = emax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < nw; ++q) {
            vmin = min(vmin, part[0][q]);
            vmax = max(vmax, part[1][q]);
            emin = min(emin, part[2][q]);
            emax = max(emax, part[3][q]);
        }
        if (vmin != INT32_MAX) atomicMin(out + 0, vmin);
        if (vmax != INT32_MIN) atomicMax(out + 1, vmax);
        if (emin != INT32_MAX) atomicMin(out + 2, emin);
        if (emax != INT32_MIN) atomicMax(out + 3, emax);
    }
}

__global__ void k_label_presence(int32_t n, const int32_t* __restrict__ vlabels, int32_t vlo,
                                 uint8_t* __restrict__ vflag, int32_t m, const gspan_edge* __restrict__ edges,
                                 int32_t elo, uint8_t* __restrict__ eflag)
{
    // Few distinct labels over many elements: one writer per distinct label
    // per warp, and only where the flag is not yet set (a read, not a store,
    // for the common case).  The loops are warp-uniform (stride and bounds
    // rounded to whole warps).
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t first = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & ~31ll;
    for (int64_t base = first; base < n; base += stride) {
        const int64_t i = base + lane;
        const bool live = i < n;
        const int32_t x = live ? vlabels[i] : 0;
        const unsigned lm = __ballot_sync(kFull, live);
        if (live && lane == __ffs(__match_any_sync(lm, x)) - 1 && !vflag[(int64_t)x - vlo])
            vflag[(int64_t)x - vlo] = 1;
    }
    for (int64_t base = first; base < m; base += stride) {
        const int64_t i = base + lane;
        const bool live = i < m;
        const int32_t x = live ? edges[i].label : 0;
        const unsigned lm = __ballot_sync(kFull, live);
        if (live && lane == __ffs(__match_any_sync(lm, x)) - 1 && !eflag[(int64_t)x - elo])
            eflag[(int64_t)x - elo] = 1;
    }
}

__device__ __forceinline__ int32_t last_at_most(const int64_t* base, int32_t n, int64_t x)
{
    int32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (base[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_batch_fixup(int32_t ninst, const int64_t* __restrict__ vbase, const int64_t* __restrict__ ebase,
                              int32_t N, int32_t M, int32_t* __restrict__ offsets, gspan_edge* __restrict__ edges,
                              uint32_t* status)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += stride)
        offsets[v] += (int32_t)ebase[last_at_most(vbase, ninst, v)];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += stride) {
        const int32_t inst = last_at_most(ebase, ninst, i);
        const int64_t nloc = vbase[inst + 1] - vbase[inst];
        gspan_edge ed = edges[i];
        if (ed.from < 0 || ed.from >= nloc || ed.to < 0 || ed.to >= nloc) atomicOr(status, kErrBadGraph);
        ed.from += (int32_t)vbase[inst];
        ed.to += (int32_t)vbase[inst];
        edges[i] = ed;
    }
}

__global__ void k_vertex_ranks(int32_t n, const int32_t* __restrict__ vlabels, int32_t vlo,
                               const int32_t* __restrict__ vtab, int32_t* __restrict__ vrank)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        vrank[i] = vtab[(int64_t)vlabels[i] - vlo];
}

// Packed key of every entry.  Edge-label ranks come from a dense table
// (etab, indexed by label - elo) or, for sparse label ranges, from a binary
// search over the sorted distinct labels.
__global__ void k_entry_keys(int32_t m, int32_t n, const gspan_edge* __restrict__ edges,
                             const int32_t* __restrict__ vrank, const int32_t* __restrict__ etab, int32_t elo,
                             const int32_t* __restrict__ elabels, int32_t nel, uint64_t* __restrict__ keys,
                             uint32_t* status)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const gspan_edge e = edges[i];
        if (e.to < 0 || e.to >= n) {
            atomicOr(status, kErrBadGraph);
            keys[i] = 0;
            continue;
        }
        int32_t lo;
        if (etab) {
            lo = etab[(int64_t)e.label - elo];
        } else {
            lo = 0;
            int32_t hi = nel - 1;
            while (lo < hi) {
                const int32_t mid = (lo + hi) >> 1;
                if (elabels[mid] < e.label) lo = mid + 1; else hi = mid;
            }
        }
        keys[i] = pack_entry((uint32_t)lo, (uint32_t)vrank[e.to], (uint32_t)e.to);
    }
}

constexpr int kSortBuckets = 128;

// Warp per vertex.  The reference's CSR lists each adjacency by (to, label);
// then a stable counting sort by the (edge label, to label) tuple yields the
// (edge label, to label, to) order in O(degree).  Input in any other order,
// or a tuple space wider than kSortBuckets, falls back to ranking every entry
// against its segment (O(degree^2), still stable).
__global__ void __launch_bounds__(256) k_sort_segments(int32_t n, int32_t m, int32_t lwin, int32_t K,
                                                       const int32_t* __restrict__ vrank,
                                                       const int32_t* __restrict__ win_base,
                                                       const int32_t* __restrict__ offsets,
                                                       const gspan_edge* __restrict__ edges,
                                                       const uint64_t* __restrict__ keys, uint64_t* __restrict__ adj,
                                                       int32_t* __restrict__ src, uint32_t* status)
{
    __shared__ uint32_t cnt_s[8][kSortBuckets];
    uint32_t* cnt = cnt_s[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = warp; v < n; v += nwarps) {
        const int32_t b = offsets[v], e = offsets[v + 1];
        if (b < 0 || e < b || e > m) {
            if (lane == 0) atomicOr(status, kErrBadGraph);
            continue;
        }
        bool sorted = true;
        for (int32_t j = b + lane; j < e; j += 32) {
            const gspan_edge c = edges[j];
            if (c.from != (int32_t)v) atomicOr(status, kErrBadGraph);
            src[j] = (int32_t)v;
            if (j > b) {
                const gspan_edge pv = edges[j - 1];
                sorted &= pv.to < c.to || (pv.to == c.to && pv.label <= c.label);
            }
        }
        // Counting sort needs every neighbour label inside the vertex's window.
        const uint32_t wbase = (uint32_t)win_base[vrank[v]];
        for (int32_t j = b + lane; j < e; j += 32)
            sorted &= entry_tl(__ldg(keys + j)) - wbase < (uint32_t)lwin;
        sorted = __all_sync(kFull, sorted);
        if (!sorted || K > kSortBuckets) {
            for (int32_t j = b + lane; j < e; j += 32) {
                const uint64_t kj = __ldg(keys + j);
                int32_t rank = 0;
                for (int32_t i = b; i < e; ++i) {
                    const uint64_t ki = __ldg(keys + i);
                    rank += (ki < kj) || (ki == kj && i < j);
                }
                adj[b + rank] = kj;
            }
            continue;
        }
        const uint32_t wb = wbase;
        for (int i = lane; i < kSortBuckets; i += 32) cnt[i] = 0;
        __syncwarp();
        for (int32_t j = b + lane; j < e; j += 32) {
            const uint64_t kj = __ldg(keys + j);
            atomicAdd(&cnt[entry_el(kj) * (uint32_t)lwin + entry_tl(kj) - wb], 1u);
        }
        __syncwarp();
        // Exclusive scan of the bucket counts; lane i owns buckets 4i .. 4i+3.
        uint32_t c[4], local = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            c[q] = cnt[4 * lane + q];
            local += c[q];
        }
        uint32_t incl = local;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += t;
        }
        uint32_t run = incl - local;
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            cnt[4 * lane + q] = run;
            run += c[q];
        }
        __syncwarp();
        for (int32_t base = b; base < e; base += 32) {
            const int32_t j = base + lane;
            const bool valid = j < e;
            uint64_t kj = 0;
            uint32_t bucket = 0;
            if (valid) {
                kj = __ldg(keys + j);
                bucket = entry_el(kj) * (uint32_t)lwin + entry_tl(kj) - wb;
            }
            const unsigned vm = __ballot_sync(kFull, valid);
            unsigned peers = 0;
            if (valid) {
                peers = __match_any_sync(vm, bucket);
                adj[b + cnt[bucket] + __popc(peers & lanemask_lt())] = kj;
            }
            __syncwarp();
            if (valid && lane == __ffs(peers) - 1) cnt[bucket] += __popc(peers);
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// Seeds: every directed entry u->w with label(u) <= label(w) is an embedding of
// the 1-edge code (0,1,label(u),edge label,label(w)).

__device__ __forceinline__ bool seed_key(const int32_t* __restrict__ src, const uint64_t* __restrict__ adj,
                                         const int32_t* __restrict__ vrank, const int32_t* __restrict__ win_base,
                                         int32_t lwin, int32_t nel, int64_t i, int32_t* key, uint32_t* u, uint32_t* w)
{
    const uint64_t e = adj[i];
    *u = (uint32_t)src[i];
    *w = entry_to(e);
    const int32_t fl = vrank[*u];
    const int32_t tl = (int32_t)entry_tl(e);
    const int32_t local = tl - win_base[fl];
    *key = (fl * nel + (int32_t)entry_el(e)) * lwin + local;
    return fl <= tl && (uint32_t)local < (uint32_t)lwin;
}

// Seed tuples whose block-level counters fit shared memory (8 bytes each).
constexpr int kSeedSmemKeys = 4096;

// Embedding count per seed tuple.  With `smem_keys` > 0 (the key space fits
// shared memory), each block counts into its own histogram first and adds
// its non-zero bins once, so the few hot tuples (frequent label pairs) take
// one global atomic per block instead of one per warp.
__global__ void k_seed_count(int32_t m, const int32_t* __restrict__ src, const uint64_t* __restrict__ adj,
                             const int32_t* __restrict__ vrank, const int32_t* __restrict__ win_base, int32_t lwin,
                             int32_t nel, unsigned long long* __restrict__ counts, int32_t smem_keys)
{
    extern __shared__ unsigned long long seed_hist[];
    if (smem_keys > 0) {
        for (int32_t q = threadIdx.x; q < smem_keys; q += blockDim.x) seed_hist[q] = 0;
        __syncthreads();
    }
    unsigned long long* const tgt = smem_keys > 0 ? seed_hist : counts;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < m; base += nwarps * 32) {
        const int64_t i = base + lane;
        int32_t key = 0;
        uint32_t u, w;
        const bool ok = i < m && seed_key(src, adj, vrank, win_base, lwin, nel, i, &key, &u, &w);
        // Entries are sorted per vertex, so equal keys come in runs of
        // consecutive lanes: one atomic per run (`ok` is a function of the key).
        const unsigned okm = __ballot_sync(kFull, ok);
        const int32_t prev = __shfl_up_sync(kFull, key, 1);
        const unsigned heads = __ballot_sync(kFull, ok && (lane == 0 || !((okm >> (lane - 1)) & 1u) || prev != key));
        if ((heads >> lane) & 1u) {
            const unsigned stop = (heads | ~okm) & ~((2u << lane) - 1u);
            const int end = stop ? __ffs(stop) - 1 : 32;
            atomicAdd(tgt + key, (unsigned long long)(end - lane));
        }
    }
    if (smem_keys > 0) {
        __syncthreads();
        for (int32_t q = threadIdx.x; q < smem_keys; q += blockDim.x)
            if (seed_hist[q]) atomicAdd(counts + q, seed_hist[q]);
    }
}

// Seed domains and (when materialising) the level-1 table.  With `smem_act` >
// 0 (the active tuples fit shared memory), a block first counts its rows per
// active tuple, reserves one range per tuple in the global cursor, and then
// hands out slots from a shared cursor, so the hot tuples' global cursors
// take one atomic per block.  Rows of a tuple may land in any order.
__global__ void k_seed_support(int32_t m, const int32_t* __restrict__ src, const uint64_t* __restrict__ adj,
                               const int32_t* __restrict__ vrank, const int32_t* __restrict__ win_base,
                               int32_t lwin, int32_t nel, LevelKeys keys,
                               uint32_t* __restrict__ pool, int32_t* __restrict__ col0, int32_t* __restrict__ col1,
                               int32_t* __restrict__ col2, uint32_t* status, int32_t smem_act)
{
    extern __shared__ unsigned long long seed_cur[];   // [smem_act] block counts, then [smem_act] cursors
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool local = smem_act > 0 && col0 != nullptr;
    if (local) {
        for (int32_t q = threadIdx.x; q < 2 * smem_act; q += blockDim.x) seed_cur[q] = 0;
        __syncthreads();
        // This block's rows per active tuple (the same entries, in the same
        // order, as the pass below).
        for (int64_t base = warp * 32; base < m; base += nwarps * 32) {
            const int64_t i = base + lane;
            int32_t key = 0;
            uint32_t u = 0, w = 0;
            bool ok = i < m && seed_key(src, adj, vrank, win_base, lwin, nel, i, &key, &u, &w);
            const int32_t a = ok ? keys.act[key] : -1;
            const bool mat = a >= 0 && keys.mat_off[a] >= 0;
            const unsigned mm = __ballot_sync(kFull, mat);
            const int32_t prev = __shfl_up_sync(kFull, a, 1);
            const unsigned heads = __ballot_sync(kFull, mat && (lane == 0 || !((mm >> (lane - 1)) & 1u) || prev != a));
            if ((heads >> lane) & 1u) {
                const unsigned stop = (heads | ~mm) & ~((2u << lane) - 1u);
                const int end = stop ? __ffs(stop) - 1 : 32;
                atomicAdd(seed_cur + a, (unsigned long long)(end - lane));
            }
        }
        __syncthreads();
        for (int32_t q = threadIdx.x; q < smem_act; q += blockDim.x)
            if (seed_cur[q]) seed_cur[smem_act + q] = atomicAdd(keys.cursor + q, seed_cur[q]);
        __syncthreads();
    }
    unsigned long long* const cursor = local ? seed_cur + smem_act : keys.cursor;
    for (int64_t base = warp * 32; base < m; base += nwarps * 32) {
        const int64_t i = base + lane;
        int32_t key = 0;
        uint32_t u = 0, w = 0;
        bool ok = i < m && seed_key(src, adj, vrank, win_base, lwin, nel, i, &key, &u, &w);
        const int32_t a = ok ? keys.act[key] : -1;
        ok = a >= 0;
        // Runs of consecutive lanes with equal (active key, source vertex):
        // the source goes into its domain once per run.
        const unsigned okm = __ballot_sync(kFull, ok);
        const uint64_t rk = ((uint64_t)(uint32_t)a << 32) | u;
        const uint64_t prev = __shfl_up_sync(kFull, rk, 1);
        const unsigned heads = __ballot_sync(kFull, ok && (lane == 0 || !((okm >> (lane - 1)) & 1u) || prev != rk));
        if (ok) {
            const DomDesc d = keys.dom[a];
            if ((heads >> lane) & 1u) dom_insert(pool, d, 0, u, status);
            dom_insert(pool, d, 1, w, status);
        }
        const bool mat = ok && keys.mat_off[a] >= 0;
        const unsigned mm = __ballot_sync(kFull, mat);
        if (mat) {
            // One cursor reservation per run (materialisation depends on the key only).
            const int h = 31 - __clz(heads & ((2u << lane) - 1u));
            const unsigned stop = (heads | ~mm) & ~((2u << h) - 1u);
            const int end = stop ? __ffs(stop) - 1 : 32;
            unsigned long long at = 0;
            if (lane == h) at = atomicAdd(cursor + a, (unsigned long long)(end - h));
            at = __shfl_sync(mm, at, h);
            const unsigned long long slot = at + (unsigned long long)(lane - h);
            if (slot < keys.counts[key]) {
                const long long row = keys.mat_off[a] + (long long)slot;
                col0[row] = (int32_t)u;
                col1[row] = (int32_t)w;
                if (col2) col2[row] = (int32_t)i;
            } else {
                atomicOr(status, kErrCursor);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Extension.

struct ExpandDev {
    const int32_t* offsets;
    const uint64_t* adj;
    const int32_t* segstart;     // segment starts per vertex (null: binary search)
    const uint64_t* eidx;        // edge index (null: binary search)
    uint32_t eidx_cap;
    int32_t nvl, nel, lwin;
    const ParentMeta* parents;
    int32_t nparents;
    int64_t ntiles;
    int32_t* const* in_cols;
    int32_t* const* out_cols;
    int32_t ecol_in, ecol_out;   // first entry column of the parent / child table (-1: none)
    int32_t vs, ss;              // scratch strides: >= every parent's vertices / ranges, odd
    LevelKeys keys;
    uint32_t* pool;
    unsigned long long* tile_counter;
    unsigned long long* scanned;
    uint32_t* status;
};

// Per-warp scratch in dynamic shared memory, sized per launch by the level's
// largest parent: img [32][vs] (row images, one row per lane), start and cnt
// [32][ss] (per row and range: first adjacency entry, entries), pre [32]
// (exclusive prefix of the rows' entry counts).  vs, ss are odd (no bank
// conflicts between lanes).
// Materialize also keeps a per-slot 64-bit cursor [ss] (2 * ss ints) after
// them, then per slot a 64-bit row limit [ss] and an active index (2 * ss
// ints), and the records of up to kMatChunk candidates [3][kMatChunk].
constexpr int kMatChunk = 256;
__host__ __device__ inline int expand_warp_ints(int vs, int ss, bool mat)
{
    return 32 * (vs + 2 * ss + 1) + 2 * ss + (mat ? 4 * ss + 3 * kMatChunk : 0);
}

template <Pass kPass>
__global__ void __launch_bounds__(kExpandThreads) k_expand(ExpandDev a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int32_t* const Wimg = reinterpret_cast<int32_t*>(smem_raw) +
                          (threadIdx.x >> 5) * expand_warp_ints(a.vs, a.ss, kPass == Pass::Materialize);
    int32_t* const Wstart = Wimg + 32 * a.vs;
    int32_t* const Wcnt = Wstart + 32 * a.ss;
    int32_t* const Wpre = Wcnt + 32 * a.ss;
    unsigned long long* const Wcur = reinterpret_cast<unsigned long long*>(Wpre + 32);
    unsigned long long* const Wlim = Wcur + a.ss;                       // Materialize only
    int32_t* const Wai = reinterpret_cast<int32_t*>(Wlim + a.ss);      // Materialize only
    int32_t* const Wrec = Wai + 2 * a.ss;                                // Materialize only
    const int lane = threadIdx.x & 31;
    const int32_t LeLv = a.nel * a.lwin;

    for (;;) {
        long long tile = 0;
        if (lane == 0) tile = (long long)atomicAdd(a.tile_counter, 1ull);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= a.ntiles) break;

        // Parent owning this tile: last parent whose first tile is <= tile.
        int32_t lo = 0, hi = a.nparents - 1;
        while (lo < hi) {
            const int32_t mid = (lo + hi + 1) >> 1;
            if (a.parents[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
        }
        const ParentMeta& P = a.parents[lo];
        const int nv = P.nv, nsrc = P.nsrc, nback = P.nback;
        const int32_t key_base = P.key_base;
        const int min_label = P.min_label;
        constexpr int kRows = kPass == Pass::Materialize ? kMatTileRows : 32;
        const int64_t row = P.row_begin + (tile - P.tile_begin) * kRows + lane;
        const bool live = lane < kRows && row < P.row_end;

        for (int p = 0; p < nv; ++p) Wimg[(lane) * a.vs + (p)] = live ? __ldcs(a.in_cols[p] + row) : -1;

        // Ranges to scan per row: one per source (the source's valid suffix),
        // or, when materialising with few frequent tuples, one per frequent
        // tuple segment (slot q covers source mseg_s[q], tuple mseg_kc[q]).
        const bool segs = kPass == Pass::Materialize && P.nmseg >= 0;
        const int nslot = segs ? P.nmseg : nsrc;
        int32_t work = 0;
        for (int q = 0; q < nslot; ++q) {
            int32_t st = 0, c = 0;
            if (live) {
                const int sq = segs ? P.mseg_s[q] : q;
                const int32_t u = Wimg[(lane) * a.vs + (P.src_v[sq])];
                const int32_t b = __ldg(a.offsets + u), e = __ldg(a.offsets + u + 1);
                const int32_t K1 = a.nel * a.lwin + 1;
                if (segs) {
                    const uint32_t kc = P.mseg_kc[q];
                    if (a.segstart) {
                        st = __ldg(a.segstart + (int64_t)u * K1 + kc);
                        c = __ldg(a.segstart + (int64_t)u * K1 + kc + 1) - st;
                    } else {
                        const uint32_t el = kc / (uint32_t)a.lwin;
                        const uint32_t tl = (uint32_t)P.lbase + kc % (uint32_t)a.lwin;
                        st = lower_bound_entry(a.adj, b, e, pack_entry(el, tl, 0));
                        c = lower_bound_entry(a.adj, st, e, pack_entry(el, tl + 1, 0)) - st;
                    }
                } else {
                    if (a.segstart) {
                        const int32_t kc = sq == 0 ? min_label - P.lbase : P.src_el[sq] * a.lwin + P.src_tl[sq] - P.lbase;
                        st = __ldg(a.segstart + (int64_t)u * K1 + kc);
                    } else {
                        const uint64_t lo_key = sq == 0 ? pack_entry(0, (uint32_t)min_label, 0)
                                                        : pack_entry((uint32_t)P.src_el[sq], (uint32_t)P.src_tl[sq], 0);
                        st = lower_bound_entry(a.adj, b, e, lo_key);
                    }
                    c = e - st;
                }
            }
            Wstart[(lane) * a.ss + (q)] = st;
            Wcnt[(lane) * a.ss + (q)] = c;
            work += c;
        }
        int32_t incl = work;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t t = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += t;
        }
        Wpre[lane] = incl - work;
        const int32_t total = __shfl_sync(kFull, incl, 31);
        __syncwarp();
        if (kPass != Pass::Support && lane == 0 && total > 0)
            atomicAdd(a.scanned, (unsigned long long)total);

        // Backward candidates: at most one per (row, rightmost-path target).
        for (int t = 0; t < nback; ++t) {
            bool ok = false;
            int32_t bel = 0;
            int32_t bpos = 0;   // entry index of the backward edge found
            if (live) {
                const int bv = P.back_v[t];
                const int32_t x = Wimg[(lane) * a.vs + (bv)];
                const int32_t un = Wimg[(lane) * a.vs + (P.vn)];
                const uint32_t tlx = (uint32_t)P.vlab[bv];
                const int32_t b = __ldg(a.offsets + un), e = __ldg(a.offsets + un + 1);
                for (int32_t el = P.back_eq[t] ? P.back_el[t] : P.back_el[t] + 1; el < a.nel && !ok; ++el) {
                    const uint64_t want = pack_entry((uint32_t)el, tlx, (uint32_t)x);
                    int32_t pos;
                    if (a.eidx) {
                        pos = edge_find(a.eidx, a.eidx_cap, a.adj, b, e, (uint32_t)un, want);
                    } else {
                        pos = lower_bound_entry(a.adj, b, e, want);
                        if (pos >= e || __ldg(a.adj + pos) != want) pos = -1;
                    }
                    if (pos >= 0) {
                        bool used = false;
                        for (int j = 0; j < P.nedge; ++j) {
                            if (P.e_el[j] != el) continue;
                            const int32_t f = Wimg[(lane) * a.vs + (P.e_from[j])], g2 = Wimg[(lane) * a.vs + (P.e_to[j])];
                            if ((f == un && g2 == x) || (g2 == un && f == x)) used = true;
                        }
                        if (!used) {
                            ok = true;
                            bel = el;
                            bpos = pos;
                        }
                    }
                }
            }
            const int32_t key = key_base + nsrc * LeLv + t * a.nel + bel;
            const unsigned mask = __ballot_sync(kFull, ok);
            if (kPass == Pass::Count) {
                if (ok) {
                    const unsigned peers = __match_any_sync(mask, key);
                    if (lane == __ffs(peers) - 1) atomicAdd(a.keys.counts + key, (unsigned long long)__popc(peers));
                }
            } else {
                const int32_t ai = ok ? a.keys.act[key] : -1;
                const bool sup = ai >= 0;
                if (kPass == Pass::Support && sup) {
                    const DomDesc d = a.keys.dom[ai];
                    for (int p = 0; p < nv; ++p) dom_insert(a.pool, d, p, (uint32_t)Wimg[(lane) * a.vs + (p)], a.status);
                }
                const bool mat = kPass == Pass::Materialize && sup;
                const unsigned mm = __ballot_sync(kFull, mat);
                if (mat) {
                    const unsigned peers = __match_any_sync(mm, ai);
                    const int leader = __ffs(peers) - 1;
                    unsigned long long at = 0;
                    if (lane == leader) at = atomicAdd(a.keys.cursor + ai, (unsigned long long)__popc(peers));
                    at = __shfl_sync(mm, at, leader);
                    const unsigned long long slot = at + __popc(peers & lanemask_lt());
                    if (slot < a.keys.counts[key]) {
                        const long long r = a.keys.mat_off[ai] + (long long)slot;
                        for (int p = 0; p < nv; ++p) a.out_cols[p][r] = Wimg[(lane) * a.vs + (p)];
                        if (a.ecol_out >= 0) {
                            for (int j = 0; j < P.nedge; ++j)
                                a.out_cols[a.ecol_out + j][r] = __ldg(a.in_cols[a.ecol_in + j] + row);
                            a.out_cols[a.ecol_out + P.nedge][r] = bpos;
                        }
                    } else {
                        atomicOr(a.status, kErrCursor);   // more candidates than counted: never write past the range
                    }
                }
            }
        }

        if (kPass == Pass::Materialize && segs) {
            // Few frequent tuples, one per slot: count the tile's rows per
            // slot, reserve each slot's range with one global atomic, then
            // write from a per-warp cursor (the hot tuples' global cursors
            // see one atomic per tile instead of one per 32 candidates).
            // The candidate of item: its owner row, slot and entry, and
            // whether it is a child (its `to` not an image of the row).
            auto candidate = [&](int32_t item, int* owner, int* slot, int32_t* eidx, uint32_t* to) {
                int l2 = 0, h2 = 31;
                while (l2 < h2) {
                    const int mid = (l2 + h2 + 1) >> 1;
                    if (Wpre[mid] <= item) l2 = mid; else h2 = mid - 1;
                }
                *owner = l2;
                int32_t j = item - Wpre[l2];
                int q = 0;
                while (j >= Wcnt[l2 * a.ss + q]) {
                    j -= Wcnt[l2 * a.ss + q];
                    ++q;
                }
                *slot = q;
                *eidx = Wstart[l2 * a.ss + q] + j;
                *to = entry_to(__ldg(a.adj + *eidx));
                bool fresh = true;
                for (int p = 0; p < nv; ++p) fresh &= Wimg[l2 * a.vs + p] != (int32_t)*to;
                return fresh;
            };
            // Candidates go in chunks of kMatChunk: the counting pass keeps
            // each one's `to` (-1: not a child), entry and (owner, slot) in
            // shared memory, so the writing pass reads them back instead of
            // searching for them again.
            int32_t* const Rto = Wrec;
            int32_t* const Rei = Wrec + kMatChunk;
            int32_t* const Roq = Wrec + 2 * kMatChunk;
            for (int32_t cb = 0; cb < total; cb += kMatChunk) {
                const int32_t cn = min(kMatChunk, total - cb);
                if (lane < nslot) Wcur[lane] = 0;
                __syncwarp();
                for (int32_t base = 0; base < cn; base += 32) {
                    const int32_t item = base + lane;
                    int owner = 0, q = 0;
                    int32_t ei = 0;
                    uint32_t to = 0;
                    const bool ok = item < cn && candidate(cb + item, &owner, &q, &ei, &to);
                    if (item < cn) {
                        Rto[item] = ok ? (int32_t)to : -1;
                        Rei[item] = ei;
                        Roq[item] = (owner << 8) | q;
                    }
                    const unsigned m = __ballot_sync(kFull, ok);
                    if (ok) {
                        const unsigned peers = __match_any_sync(m, q);
                        if (lane == __ffs(peers) - 1) atomicAdd(Wcur + q, (unsigned long long)__popc(peers));
                    }
                }
                __syncwarp();
                if (lane < nslot) {
                    const int32_t key = key_base + P.mseg_s[lane] * LeLv + (int32_t)P.mseg_kc[lane];
                    const int32_t ai = a.keys.act[key];
                    const unsigned long long n = Wcur[lane];
                    Wcur[lane] = (n && ai >= 0) ? atomicAdd(a.keys.cursor + ai, n) : 0ull;
                    Wai[lane] = ai;
                    Wlim[lane] = a.keys.counts[key];
                }
                __syncwarp();
                for (int32_t base = 0; base < cn; base += 32) {
                    const int32_t item = base + lane;
                    int32_t to = -1, ei = 0, oq = 0;
                    if (item < cn) {
                        to = Rto[item];
                        ei = Rei[item];
                        oq = Roq[item];
                    }
                    const int q = oq & 0xFF, owner = oq >> 8;
                    const int32_t ai = to >= 0 ? Wai[q] : -1;
                    const bool mat = ai >= 0;
                    const unsigned mm = __ballot_sync(kFull, mat);
                    if (mat) {
                        const unsigned peers = __match_any_sync(mm, q);
                        const int leader = __ffs(peers) - 1;
                        unsigned long long at = 0;
                        if (lane == leader) at = atomicAdd(Wcur + q, (unsigned long long)__popc(peers));
                        at = __shfl_sync(mm, at, leader);
                        const unsigned long long slot = at + __popc(peers & lanemask_lt());
                        if (slot < Wlim[q]) {
                            const long long r = a.keys.mat_off[ai] + (long long)slot;
                            for (int p = 0; p < nv; ++p) a.out_cols[p][r] = Wimg[owner * a.vs + p];
                            a.out_cols[nv][r] = to;
                            if (a.ecol_out >= 0) {
                                const int64_t orow = P.row_begin + (tile - P.tile_begin) * kRows + owner;
                                for (int jj = 0; jj < P.nedge; ++jj)
                                    a.out_cols[a.ecol_out + jj][r] = __ldg(a.in_cols[a.ecol_in + jj] + orow);
                                a.out_cols[a.ecol_out + P.nedge][r] = ei;
                            }
                        } else {
                            atomicOr(a.status, kErrCursor);
                        }
                    }
                }
                __syncwarp();
            }
            __syncwarp();
            continue;
        }

        // Forward candidates: the tile's adjacency ranges, 32 entries at a time.
        for (int32_t base = 0; base < total; base += 32) {
            const int32_t item = base + lane;
            bool ok = item < total;
            int owner = 0;
            uint32_t to = 0;
            int32_t eidx = 0;   // index of the candidate entry
            int32_t key = 0;
            if (ok) {
                int l2 = 0, h2 = 31;
                while (l2 < h2) {
                    const int mid = (l2 + h2 + 1) >> 1;
                    if (Wpre[mid] <= item) l2 = mid; else h2 = mid - 1;
                }
                owner = l2;
                int32_t j = item - Wpre[owner];
                int s = 0;
                while (j >= Wcnt[(owner) * a.ss + (s)]) {
                    j -= Wcnt[(owner) * a.ss + (s)];
                    ++s;
                }
                eidx = Wstart[(owner) * a.ss + (s)] + j;
                const uint64_t e = __ldg(a.adj + eidx);
                to = entry_to(e);
                const int32_t tl = (int32_t)entry_tl(e);
                bool fresh = tl >= min_label && (uint32_t)(tl - P.lbase) < (uint32_t)a.lwin;
                for (int p = 0; p < nv; ++p) fresh &= Wimg[(owner) * a.vs + (p)] != (int32_t)to;
                ok = fresh;
                key = key_base + (segs ? P.mseg_s[s] : s) * LeLv + (int32_t)entry_el(e) * a.lwin + (tl - P.lbase);
            }
            const unsigned mask = __ballot_sync(kFull, ok);
            if (kPass == Pass::Count) {
                if (ok) {
                    const unsigned peers = __match_any_sync(mask, key);
                    if (lane == __ffs(peers) - 1) atomicAdd(a.keys.counts + key, (unsigned long long)__popc(peers));
                }
            } else {
                const int32_t ai = ok ? a.keys.act[key] : -1;
                const bool sup = ai >= 0;
                if (kPass == Pass::Support) {
                    const unsigned sm = __ballot_sync(kFull, sup);
                    if (sup) {
                        const DomDesc d = a.keys.dom[ai];
                        dom_insert(a.pool, d, nv, to, a.status);
                        // The parent row's images go in once per (row, child tuple) in this chunk.
                        const unsigned peers = __match_any_sync(sm, ((unsigned long long)owner << 32) | (unsigned)ai);
                        if (lane == __ffs(peers) - 1)
                            for (int p = 0; p < nv; ++p) dom_insert(a.pool, d, p, (uint32_t)Wimg[(owner) * a.vs + (p)], a.status);
                    }
                }
                const bool mat = kPass == Pass::Materialize && sup;
                const unsigned mm = __ballot_sync(kFull, mat);
                if (mat) {
                    const unsigned peers = __match_any_sync(mm, ai);
                    const int leader = __ffs(peers) - 1;
                    unsigned long long at = 0;
                    if (lane == leader) at = atomicAdd(a.keys.cursor + ai, (unsigned long long)__popc(peers));
                    at = __shfl_sync(mm, at, leader);
                    const unsigned long long slot = at + __popc(peers & lanemask_lt());
                    if (slot < a.keys.counts[key]) {
                        const long long r = a.keys.mat_off[ai] + (long long)slot;
                        for (int p = 0; p < nv; ++p) a.out_cols[p][r] = Wimg[(owner) * a.vs + (p)];
                        a.out_cols[nv][r] = (int32_t)to;
                        if (a.ecol_out >= 0) {
                            const int64_t orow = P.row_begin + (tile - P.tile_begin) * kRows + owner;
                            for (int jj = 0; jj < P.nedge; ++jj)
                                a.out_cols[a.ecol_out + jj][r] = __ldg(a.in_cols[a.ecol_in + jj] + orow);
                            a.out_cols[a.ecol_out + P.nedge][r] = eidx;
                        }
                    } else {
                        atomicOr(a.status, kErrCursor);
                    }
                }
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Mask path: counts and MNI domains of every child tuple without visiting
// candidates one by one.
//
// For parent pattern P, source s (a rightmost-path vertex) and row r, let u_r be
// the row's image of the source and seg(u, c) the adjacency entries of u with
// (edge label, to label) = c.  The reference emits one child embedding per
// entry e of seg(u_r, c) whose `to` is not an image of r (gspan.cu:447-483).
// With
//   R[u] = rows whose source image is u,
//   H[e] = rows whose source image owns entry e and that have to(e) as an image,
// the child count of tuple (s, c) is sum over entries e of seg(u, c) of
// R[u] - H[e], and the new vertex's domain is {to(e) : R[u] > H[e]}.  An old
// vertex p's domain for (s, c) is {img_r(p) : row r has an entry of
// seg(u_r, c) outside its images}; the row pass ORs the set of such c (a
// bitmask over the tuple space) into M[p][img_r(p)], the sweep the new
// vertex's bits, and k_mask_popcount counts the set bits of every mask plane
// into the domain sizes afterwards.  All of it is exact.
//
// k_mask_touched lists every vertex with a non-zero R (`touched`), so the
// sweep visits only those vertices; the sweep also resets the R and H entries
// it reads, leaving both arrays zero for the next group of parents.

constexpr int kMaskWarps = 8;
// Pattern vertices whose mask words the row pass reads together (one word each).
constexpr int kMaskBatch = 4;

struct MaskDev {
    const int32_t* offsets;
    const uint64_t* adj;
    const uint32_t* segmask;
    const uint32_t* segone;      // segments of exactly one entry
    const int32_t* segstart;     // segment starts per vertex (null: binary search)
    const uint32_t* selfloop;
    const int32_t* rev;
    const uint64_t* eidx;        // edge index (null: binary search)
    uint32_t eidx_cap;
    int32_t ecol;
    bool symmetric;
    bool parallel;               // equal entries may follow each other
    bool loops;                  // self-loops present: images of a row may repeat
    int32_t n, m, nvl, nel, mw, lwin;
    const ParentMeta* parents;
    int32_t nparents;
    int64_t ntiles;
    int32_t* const* in_cols;
    unsigned long long* counts;
    uint32_t* sizes;
    uint32_t* R;
    uint32_t* H;
    uint32_t* M;
    uint32_t* MB;
    int32_t* touched;
    uint32_t* tcount;
    const int32_t* ps_parent;
    int32_t nps;
    unsigned long long* tprefix;
    unsigned long long* tile_counter;
    unsigned long long* scanned;
    uint32_t* status;
    const ParentMeta* gen_parents;
    int32_t* const* gen_cols;
    int32_t gen_ecol;
    int32_t gen_vs, gen_es;      // shared-memory strides of generated rows (odd)
};

// OR `bits` into *p without waiting for the old value (the atomic's result
// is unused); a word already holding them costs one L2 read and no atomic.
__device__ __forceinline__ void or_bits(uint32_t* p, uint32_t bits)
{
    if (bits && (__ldcg(p) & bits) != bits) atomicOr(p, bits);
}

// Warp per vertex, over its entries (sorted by window key kc): the entry
// that opens segment kc sets bit kc of segmask, and of segone when it also
// closes it; segstart[v][k] (when not null) = the first entry whose key is
// >= k, for k in [0, K], each k written once (by the entry that opens it, or
// by the tail for keys after the last entry).  segmask and segone start zero.
__global__ void k_segments(int32_t n, int32_t m, int32_t lwin, int32_t K, int32_t segw,
                           const int32_t* __restrict__ vrank, const int32_t* __restrict__ win_base,
                           const int32_t* __restrict__ offsets, const uint64_t* __restrict__ adj,
                           uint32_t* __restrict__ segmask, uint32_t* __restrict__ segone,
                           int32_t* __restrict__ segstart)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = warp; v < n; v += nwarps) {
        const int32_t wb = win_base[vrank[v]];
        const int32_t b = offsets[v], e = offsets[v + 1];
        if (b < 0 || e < b || e > m) continue;   // malformed range (rejected by the upload)
        auto key = [&](int32_t j) { return (int32_t)(entry_el(adj[j]) * (uint32_t)lwin + entry_tl(adj[j])) - wb; };
        int32_t* out = segstart ? segstart + v * (int64_t)(K + 1) : nullptr;
        for (int32_t j = b + lane; j < e; j += 32) {
            const int32_t kc = key(j);
            const int32_t kp = j > b ? key(j - 1) : -1;
            if (kp < kc && kc >= 0 && kc < 32 * segw) {
                const int64_t w = v * segw + (kc >> 5);
                const uint32_t bit = 1u << (kc & 31);
                atomicOr(segmask + w, bit);
                if (j + 1 == e || key(j + 1) > kc) atomicOr(segone + w, bit);
            }
            if (out)
                for (int32_t k = kp + 1; k <= kc && k <= K; ++k) out[k] = j;
        }
        if (out) {
            const int32_t kl = e > b ? key(e - 1) : -1;
            for (int32_t k = kl + 1 + lane; k <= K; k += 32) out[k] = e;
        }
    }
}


// Thread per entry: self-loop bits, the entry's reverse entry (the k-th of
// a run of equal entries pairs with the k-th of the reverse run) and the
// symmetry check; and the edge index: the first entry of each run of equal
// entries is inserted (linear probing, bounded by the table size).
__global__ void k_entry_flags(int32_t m, const int32_t* __restrict__ src, const int32_t* __restrict__ offsets,
                              const uint64_t* __restrict__ adj, const int32_t* __restrict__ vrank,
                              const int32_t* __restrict__ segstart, const int32_t* __restrict__ win_base,
                              int32_t lwin, int32_t K, uint32_t* __restrict__ selfloop, int32_t* __restrict__ rev,
                              unsigned long long* __restrict__ eidx, uint32_t cap, uint32_t* status)
{
    bool asym = false, loop = false, parallel = false, full = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t ent = adj[i];
        const uint32_t u = (uint32_t)src[i], x = entry_to(ent);
        const int32_t bu = offsets[u];
        const bool repeat = i > bu && adj[i - 1] == ent;
        parallel |= repeat;
        if (eidx && !repeat) {
            const uint64_t h = edge_hash(u, entry_el(ent), x);
            const unsigned long long val = ((h >> 32) << 32) | (uint32_t)i;
            uint32_t j = (uint32_t)h & (cap - 1);
            uint32_t probe = 0;
            for (; probe < cap; ++probe) {
                if (atomicCAS(eidx + j, ~0ull, val) == ~0ull) break;
                j = (j + 1) & (cap - 1);
            }
            full |= probe == cap;
        }
        if (u == x) {
            atomicOr(selfloop + (u >> 5), 1u << (u & 31));
            rev[i] = (int32_t)i;
            loop = true;
            continue;
        }
        // Rank of i among the equal entries before it (parallel edges with one label).
        int32_t r0 = (int32_t)i;
        while (r0 > bu && adj[r0 - 1] == ent) --r0;
        const uint64_t rk = pack_entry(entry_el(ent), (uint32_t)vrank[u], u);
        int32_t b = offsets[x], e = offsets[x + 1];
        if (segstart) {
            // The reverse entry lies in x's segment of (edge label, u's label):
            // search that segment only.
            const int32_t local = vrank[u] - win_base[vrank[x]];
            if ((uint32_t)local < (uint32_t)lwin) {
                const int64_t so = (int64_t)x * (K + 1) + (int64_t)entry_el(ent) * lwin + local;
                b = segstart[so];
                e = segstart[so + 1];
            } else {
                e = b;
            }
        }
        const int32_t q = lower_bound_entry(adj, b, e, rk) + ((int32_t)i - r0);
        const bool found = q < e && adj[q] == rk;
        rev[i] = found ? q : -1;
        asym |= !found;
    }
    const unsigned am = __ballot_sync(kFull, asym), lm = __ballot_sync(kFull, loop);
    const unsigned pm = __ballot_sync(kFull, parallel), fm = __ballot_sync(kFull, full);
    if ((threadIdx.x & 31) == 0 && (am | lm | pm | fm))
        atomicOr(status, (am ? kErrAsymmetric : 0u) | (lm ? kFlagSelfLoop : 0u) | (pm ? kFlagParallel : 0u) |
                             (fm ? kErrHashFull : 0u));
}

__device__ __forceinline__ int32_t find_parent_tile(const ParentMeta* parents, int32_t np, long long tile)
{
    int32_t lo = 0, hi = np - 1;
    while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (parents[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Entry column j (the adjacency index of pattern edge j's image) of the lane's
// row: from the level table ...
struct EcolFromTable {
    int32_t* const* cols;
    int32_t base;
    int64_t row;
    __device__ __forceinline__ int32_t operator()(int j) const { return __ldg(cols[base + j] + row); }
};

// ... or from a row generated in shared memory (two-level last step).
struct EcolFromShared {
    const int32_t* e;
    __device__ __forceinline__ int32_t operator()(int j) const { return e[j]; }
};

// The row pass's work for one row per lane of parent P: updates R (listing new
// source images), H and M for every source, and counts and MB masks for
// backward tuples (at most one per row and rightmost-path target).  `img` holds
// the lane's row images; lanes with !live take part in the warp-wide steps only.
// Warp-uniform running sums of backward-tuple counts (one edge label: one
// tuple per parent and target), added to the global counts when the key
// changes and at the end of the kernel, instead of one atomic per row batch
// on a handful of hot counters.
struct BackAcc {
    static constexpr int kTargets = 2;
    // Per-warp slots in shared memory, touched by lane 0 only.
    int32_t* key;                  // [kTargets], -1 when empty
    unsigned long long* n;         // [kTargets]
    __device__ __forceinline__ void init(int lane)
    {
        if (lane == 0)
            for (int t = 0; t < kTargets; ++t) {
                key[t] = -1;
                n[t] = 0;
            }
    }
    __device__ __forceinline__ void add(unsigned long long* counts, int t, int32_t k, unsigned long long c, int lane)
    {
        if (lane != 0) return;
        if (key[t] != k) {
            if (n[t]) atomicAdd(counts + key[t], n[t]);
            key[t] = k;
            n[t] = 0;
        }
        n[t] += c;
    }
    __device__ __forceinline__ void flush(unsigned long long* counts, int lane)
    {
        if (lane != 0) return;
        for (int t = 0; t < kTargets; ++t)
            if (n[t]) atomicAdd(counts + key[t], n[t]);
    }
};

// Bit of the unordered pattern-vertex pair {i, j} in a 32-bit set; a vertex
// paired with itself (a self-loop query) and pairs with a vertex beyond the
// eighth have none.
__device__ __forceinline__ uint32_t pair_bit(int i, int j)
{
    const int lo = min(i, j), hi = max(i, j);
    return hi < 8 && lo != hi ? 1u << (hi * (hi - 1) / 2 + lo) : 0u;
}

template <int MW, class Ecol>
__device__ __forceinline__ void mask_row(const MaskDev& a, const ParentMeta& P, const int32_t* img, const Ecol& ecol,
                                         bool live, int lane, BackAcc& acc)
{
    const int32_t K = a.nel * a.lwin;
    const int mw = a.mw;
    const int nv = P.nv, nsrc = P.nsrc;
    const int min_label = P.min_label;
    // Pairs of the row's images found not adjacent through the edge index
    // (one edge label, symmetric graph: the entry-column case), so a pair
    // probed from one source is not probed again from the other end or as a
    // backward target.
    uint32_t absent = 0;
    for (int s = 0; s < nsrc; ++s) {
        const int32_t u = live ? img[P.src_v[s]] : -1;
        const unsigned lm = __ballot_sync(kFull, live);
        if (live) {
            // One add per group of lanes with the same source image; the
            // touched lists are built from R afterwards (k_mask_touched), so
            // the old value is not waited for - except for a parent with
            // 2^32 rows or more, where a 32-bit counter (R, and H <= R) could
            // wrap: that fails the job.
            const unsigned peers = __match_any_sync(lm, u);
            if (lane == __ffs(peers) - 1) {
                uint32_t* const Ru = a.R + P.r_off + (int64_t)s * P.nloc + (u - P.vbase);
                const uint32_t add = (uint32_t)__popc(peers);
                if (P.r_wide) {
                    if (atomicAdd(Ru, add) > 0xFFFFFFFFu - add) atomicOr(a.status, kErrCounter);
                } else {
                    atomicAdd(Ru, add);
                }
            }
        }
        uint32_t mk[MW] = {};
        if (live) {
        const int32_t b = __ldg(a.offsets + u), e = __ldg(a.offsets + u + 1);
        const uint64_t lo = s == 0 ? pack_entry(0, (uint32_t)min_label, 0)
                                   : pack_entry((uint32_t)P.src_el[s], (uint32_t)P.src_tl[s], 0);
        // H of this source, indexed by batch-wide entry index.
        uint32_t* Hs = a.H + P.h_off + (int64_t)s * P.mloc - P.ebase;
        uint32_t ex[MW] = {};
        if (a.ecol >= 0) {
            // One edge label.  Images joined to the source by a pattern
            // edge are found through the row's entry columns (or their
            // reverse entries); the others through the edge index (or by
            // search, after a cheap existence test from the shorter side).
            // Vertices are visited in label order, so each label's hits
            // are summed on the fly: a segment is lost to the row when
            // its images fill all of it.
            // The walk (see ParentMeta::walk) holds only the vertices that
            // can hit: one load per vertex, the static filters done on the host.
            const int vs = P.src_v[s];
            const int nwalk = P.walk_n[s];
            const int32_t* const walk = P.walk[s];
            int cur_t = -1, gstart = 0;
            int32_t hits = 0, minlb = e, maxub = b;
            for (int oi = 0; oi <= nwalk; ++oi) {
                const int32_t wk = oi < nwalk ? walk[oi] : 0;
                const int j = wk & 15;
                const int t = oi < nwalk ? (wk >> 16) & 0xFFFF : -1;
                if (t != cur_t) {
                    if (hits > 0) {
                        const uint32_t kc = (uint32_t)(cur_t - P.lbase);
                        bool lost;
                        if (hits == 1) {
                            // One hit fills its segment only when the segment has one entry.
                            lost = (__ldg(a.segone + (int64_t)u * mw + (kc >> 5)) >> (kc & 31u)) & 1u;
                        } else {
                            const uint32_t segk = (uint32_t)(pack_entry(0, (uint32_t)cur_t, 0) >> 32);
                            const bool first = minlb == b || (uint32_t)(__ldg(a.adj + minlb - 1) >> 32) != segk;
                            const bool last = maxub == e || (uint32_t)(__ldg(a.adj + maxub) >> 32) != segk;
                            lost = first && last && maxub - minlb == hits;
                        }
                        if (lost) {
#pragma unroll
                            for (int w = 0; w < MW; ++w)
                                ex[w] |= (uint32_t)(w == (int)(kc >> 5)) << (kc & 31u);
                        }
                    }
                    cur_t = t;
                    gstart = oi;
                    hits = 0;
                    minlb = e;
                    maxub = b;
                }
                if (oi == nwalk) break;
                const uint64_t seg0 = pack_entry(0, (uint32_t)t, 0);
                const int32_t x = img[j];
                if (a.loops) {
                    // Images may repeat: one hit per distinct image (equal
                    // images have equal labels, so within the group).
                    bool dup = false;
                    for (int q = gstart; q < oi; ++q) dup |= img[walk[q] & 15] == x;
                    if (dup) continue;
                }
                const uint64_t key = seg0 | (uint32_t)x;
                const int jj = ((wk >> 4) & 15) - 1;
                int32_t pos = -1;
                if (jj >= 0) {
                    const int32_t stored = ecol(jj);
                    pos = (wk >> 8) & 1 ? stored : __ldg(a.rev + stored);
                    // The entry column holds the image edge's entry (or, from its
                    // other end, the reverse entry): inside u's list it is the key.
                    if (pos < b || pos >= e) pos = -1;
                }
                if (pos < 0) {
                    if (x == u && !((__ldg(a.selfloop + (u >> 5)) >> (u & 31)) & 1u)) continue;
                    if (a.eidx) {
                        const uint32_t pb = pair_bit(vs, j);
                        if (absent & pb) continue;
                        pos = edge_find(a.eidx, a.eidx_cap, a.adj, b, e, (uint32_t)u, key);
                        if (pos < 0) {
                            absent |= pb;
                            continue;
                        }
                    } else {
                        if (x != u && jj < 0 && a.symmetric) {
                            const int32_t xb = __ldg(a.offsets + x), xe = __ldg(a.offsets + x + 1);
                            if (4 * (xe - xb) < e - b) {
                                const uint64_t rk = pack_entry(0, (uint32_t)P.vlab[vs], (uint32_t)u);
                                const int32_t rp = lower_bound_entry(a.adj, xb, xe, rk);
                                if (rp >= xe || __ldg(a.adj + rp) != rk) continue;
                            }
                        }
                        pos = lower_bound_entry(a.adj, b, e, key);
                        if (pos >= e || __ldg(a.adj + pos) != key) continue;
                    }
                }
                int32_t lb = pos, ub = pos + 1;
                if (a.parallel) {
                    while (lb > b && __ldg(a.adj + lb - 1) == key) --lb;
                    while (ub < e && __ldg(a.adj + ub) == key) ++ub;
                }
                for (int32_t q = lb; q < ub; ++q) atomicAdd(Hs + q, 1u);
                hits += ub - lb;
                minlb = min(minlb, lb);
                maxub = max(maxub, ub);
            }
        } else
        for (int el = 0; el < a.nel; ++el) {
            for (int i = 0; i < nv; ++i) {
                const int t = P.vlab[i];
                const uint64_t seg0 = pack_entry((uint32_t)el, (uint32_t)t, 0);
                if (t < min_label || seg0 < lo) continue;
                bool lead = true;   // first pattern vertex of this label handles the label group
                for (int q = 0; q < i; ++q) lead &= P.vlab[q] != t;
                if (!lead) continue;
                int32_t hits = 0, minlb = e, maxub = b;
                for (int j = i; j < nv; ++j) {
                    if (P.vlab[j] != t) continue;
                    const int32_t x = img[j];
                    if (a.loops) {
                        bool dup = false;
                        for (int q = i; q < j; ++q) dup |= img[q] == x;
                        if (dup) continue;
                    }
                    // Most image pairs are not adjacent.  A vertex reaches
                    // itself only through a self-loop; a pair that the
                    // pattern does not join is first looked up from the
                    // shorter side when the graph is symmetric.
                    if (x == u) {
                        if (!((__ldg(a.selfloop + (u >> 5)) >> (u & 31)) & 1u)) continue;
                    } else if (!a.eidx && a.symmetric && !((P.src_adj[s] >> j) & 1)) {
                        const int32_t xb = __ldg(a.offsets + x), xe = __ldg(a.offsets + x + 1);
                        if (4 * (xe - xb) < e - b) {
                            const uint64_t rk = pack_entry((uint32_t)el, (uint32_t)P.vlab[P.src_v[s]], (uint32_t)u);
                            const int32_t rp = lower_bound_entry(a.adj, xb, xe, rk);
                            if (rp >= xe || __ldg(a.adj + rp) != rk) continue;
                        }
                    }
                    const uint64_t key = seg0 | (uint32_t)x;
                    int32_t lb;
                    if (a.eidx) {
                        lb = edge_find(a.eidx, a.eidx_cap, a.adj, b, e, (uint32_t)u, key);
                        if (lb < 0) continue;
                    } else {
                        lb = lower_bound_entry(a.adj, b, e, key);
                    }
                    int32_t ub = lb;
                    while (ub < e && __ldg(a.adj + ub) == key) {
                        atomicAdd(Hs + ub, 1u);
                        ++ub;
                    }
                    if (ub > lb) {
                        hits += ub - lb;
                        minlb = min(minlb, lb);
                        maxub = max(maxub, ub);
                    }
                }
                if (hits > 0) {
                    // The row has no child in this segment when its images fill all of it.
                    const uint32_t segk = (uint32_t)(seg0 >> 32);
                    const bool first = minlb == b || (uint32_t)(__ldg(a.adj + minlb - 1) >> 32) != segk;
                    const bool last = maxub == e || (uint32_t)(__ldg(a.adj + maxub) >> 32) != segk;
                    if (first && last && maxub - minlb == hits) {
                        const uint32_t kc = (uint32_t)(el * a.lwin + t - P.lbase);
#pragma unroll
                        for (int w = 0; w < MW; ++w)
                            ex[w] |= (uint32_t)(w == (int)(kc >> 5)) << (kc & 31u);
                    }
                }
            }
        }
#pragma unroll
        for (int w = 0; w < MW; ++w)
            mk[w] = w < mw ? (__ldg(a.segmask + (int64_t)u * mw + w) & P.range[s][w] & ~ex[w]) : 0u;
        }
        // The source vertex's own domain is counted by the sweep when the
        // tuple space is small (see k_mask_sweep); the other vertices' masks
        // are ORed here and counted afterwards (k_mask_popcount).
        const int skip_p = K <= kSweepAccKeys ? P.src_v[s] : -1;
        if (mw == 1 && nv <= kMaskBatch) {
            // One mask word per vertex: read every vertex's word first, so
            // the L2 round trips overlap, then OR where bits are missing.
            uint32_t* const mrow = a.M + P.m_off + (int64_t)s * (nv + 1) * P.nloc;
            uint32_t cur[kMaskBatch];
#pragma unroll
            for (int p = 0; p < kMaskBatch; ++p)
                cur[p] = p < nv && p != skip_p && mk[0] ? __ldcg(mrow + (int64_t)p * P.nloc + (img[p] - P.vbase)) : ~0u;
#pragma unroll
            for (int p = 0; p < kMaskBatch; ++p) {
                if (p >= nv) break;
                if (p == skip_p) continue;
                if (mk[0] & ~cur[p]) atomicOr(mrow + (int64_t)p * P.nloc + (img[p] - P.vbase), mk[0]);
            }
        } else {
            for (int p = 0; p < nv; ++p) {
                if (p == skip_p) continue;
                uint32_t* rowm = a.M + P.m_off + (((int64_t)s * (nv + 1) + p) * P.nloc + (live ? img[p] - P.vbase : 0)) * mw;
                for (int w = 0; w < mw; ++w) or_bits(rowm + w, mk[w]);
            }
        }
    }

    for (int t = 0; t < P.nback; ++t) {
        bool ok = false;
        int32_t bel = 0;
        if (live) {
            const int bv = P.back_v[t];
            const int32_t x = img[bv];
            const int32_t un = img[P.vn];
            const uint32_t tlx = (uint32_t)P.vlab[bv];
            const int32_t b = __ldg(a.offsets + un), e = __ldg(a.offsets + un + 1);
            for (int32_t el = P.back_eq[t] ? P.back_el[t] : P.back_el[t] + 1; el < a.nel && !ok; ++el) {
                const uint64_t want = pack_entry((uint32_t)el, tlx, (uint32_t)x);
                int32_t pos;
                if (a.eidx) {
                    pos = a.ecol >= 0 && (absent & pair_bit(P.vn, bv))
                              ? -1
                              : edge_find(a.eidx, a.eidx_cap, a.adj, b, e, (uint32_t)un, want);
                } else {
                    pos = lower_bound_entry(a.adj, b, e, want);
                    if (pos >= e || __ldg(a.adj + pos) != want) pos = -1;
                }
                if (pos >= 0) {
                    // has_edge: the row already uses an edge (un, x, el).
                    // Without self-loops images are distinct, so that is
                    // a code edge joining v_n and the target.
                    bool used = false;
                    if (!a.loops && el < 32) {
                        used = (P.back_used[t] >> el) & 1u;
                    } else {
                        for (int j = 0; j < P.nedge; ++j) {
                            if (P.e_el[j] != el) continue;
                            const int32_t f = img[P.e_from[j]], g2 = img[P.e_to[j]];
                            if ((f == un && g2 == x) || (g2 == un && f == x)) used = true;
                        }
                    }
                    if (!used) {
                        ok = true;
                        bel = el;
                    }
                }
            }
        }
        const int32_t bk = t * a.nel + bel;
        const int32_t key = P.key_base + nsrc * K + bk;
        const unsigned mask = __ballot_sync(kFull, ok);
        if (a.nel == 1 && t < BackAcc::kTargets) {
            // One edge label: one backward tuple per target, the same in
            // every lane; summed per warp and added once per parent.
            if (mask) acc.add(a.counts, t, key, (unsigned long long)__popc(mask), lane);
        } else if (ok) {
            const unsigned peers = __match_any_sync(mask, key);
            if (lane == __ffs(peers) - 1) atomicAdd(a.counts + key, (unsigned long long)__popc(peers));
        }
        if (ok)
            for (int p = 0; p < nv; ++p)
                or_bits(a.MB + P.b_off + ((int64_t)p * P.nloc + (img[p] - P.vbase)) * P.bw + (bk >> 5), 1u << (bk & 31));
    }
}

// Row pass: lane per row of the level table.
template <int MW>
__global__ void __launch_bounds__(kMaskWarps * 32, MW <= kNarrowMaskWords ? 5 : 2) k_mask_rows(MaskDev a)
{
    __shared__ int32_t img_s[kMaskWarps][32][kMaxV + 1];
    int32_t (*img_all)[kMaxV + 1] = img_s[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    int32_t* img = img_all[lane];
    __shared__ int32_t acc_key[kMaskWarps][BackAcc::kTargets];
    __shared__ unsigned long long acc_n[kMaskWarps][BackAcc::kTargets];
    BackAcc acc{acc_key[threadIdx.x >> 5], acc_n[threadIdx.x >> 5]};
    acc.init(lane);

    for (;;) {
        long long tile = 0;
        if (lane == 0) tile = (long long)atomicAdd(a.tile_counter, 1ull);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= a.ntiles) break;
        const ParentMeta& P = a.parents[find_parent_tile(a.parents, a.nparents, tile)];
        const int nv = P.nv;
        const int64_t row = P.row_begin + (tile - P.tile_begin) * 32 + lane;
        const bool live = row < P.row_end;
        for (int p = 0; p < nv; ++p) img[p] = live ? __ldcs(a.in_cols[p] + row) : -1;
        mask_row<MW>(a, P, img, EcolFromTable{a.in_cols, a.ecol, row}, live, lane, acc);
        __syncwarp();
    }
    acc.flush(a.counts, lane);
}

// Two-level last step: warp per tile of 32 rows of a parent's own parent Q
// (one level up).  The parent F is Q's child tuple; its rows are generated here
// exactly as the Materialize pass of k_expand would write them - a forward
// tuple's rows are the entries of the tuple's segment of the source image
// that are not images of the Q row, a backward tuple's the Q rows whose first
// valid closing edge (gspan.cu:428-445) has the tuple's label - and go through
// mask_row in batches of 32, one per lane, never stored.
//
// Per-warp dynamic shared memory (ints): Q images [32][vs], Q entry columns
// [32][es], generated images [32][vs], generated entry columns [32][es],
// segment start, length and exclusive prefix [32] each.
__host__ __device__ inline int gen_warp_ints(int vs, int es) { return 32 * (2 * vs + 2 * es + 3); }

// Five blocks per SM (48 registers, a few spilled): on large jobs, the only
// ones that generate rows by default, the extra warps beat the spills
// (2.40 against 2.57 s on the 3.7M graph at k = 4, support 100,000).
template <int MW>
__global__ void __launch_bounds__(kMaskWarps * 32, MW <= kNarrowMaskWords ? 5 : 2) k_mask_gen(MaskDev a)
{
    extern __shared__ __align__(16) int32_t gen_smem[];
    const int lane = threadIdx.x & 31;
    const int vs = a.gen_vs, es = a.gen_es;
    int32_t* const qimg = gen_smem + (threadIdx.x >> 5) * gen_warp_ints(vs, es);
    int32_t* const qec = qimg + 32 * vs;
    int32_t* const gimg = qec + 32 * es;
    int32_t* const gec = gimg + 32 * vs;
    int32_t* const wst = gec + 32 * es;
    int32_t* const wcnt = wst + 32;
    int32_t* const wpre = wcnt + 32;
    const bool ecols = a.gen_ecol >= 0;
    __shared__ int32_t acc_key[kMaskWarps][BackAcc::kTargets];
    __shared__ unsigned long long acc_n[kMaskWarps][BackAcc::kTargets];
    BackAcc acc{acc_key[threadIdx.x >> 5], acc_n[threadIdx.x >> 5]};
    acc.init(lane);

    for (;;) {
        long long tile = 0;
        if (lane == 0) tile = (long long)atomicAdd(a.tile_counter, 1ull);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= a.ntiles) break;
        const ParentMeta& F = a.parents[find_parent_tile(a.parents, a.nparents, tile)];
        const ParentMeta& Q = a.gen_parents[F.gen_p2];
        const int nq = Q.nv, eq = Q.nedge;
        const int64_t qrow = Q.row_begin + (tile - F.tile_begin) * 32 + lane;
        const bool qlive = qrow < Q.row_end;
        for (int p = 0; p < nq; ++p) qimg[lane * vs + p] = qlive ? __ldcs(a.gen_cols[p] + qrow) : -1;
        if (ecols)
            for (int j = 0; j < eq; ++j) qec[lane * es + j] = qlive ? __ldcs(a.gen_cols[a.gen_ecol + j] + qrow) : -1;

        if (F.gen_kind == 2) {
            // Backward tuple (target t, label el): the Q row itself, when its
            // smallest unused closing edge label is el.
            bool ok = false;
            int32_t bpos = 0;
            if (qlive) {
                const int t = F.gen_s;
                const int bv = Q.back_v[t];
                const int32_t x = qimg[lane * vs + bv];
                const int32_t un = qimg[lane * vs + Q.vn];
                const uint32_t tlx = (uint32_t)Q.vlab[bv];
                const int32_t b = __ldg(a.offsets + un), e = __ldg(a.offsets + un + 1);
                for (int32_t el = Q.back_eq[t] ? Q.back_el[t] : Q.back_el[t] + 1; el < a.nel; ++el) {
                    const uint64_t want = pack_entry((uint32_t)el, tlx, (uint32_t)x);
                    int32_t pos;
                    if (a.eidx) {
                        pos = edge_find(a.eidx, a.eidx_cap, a.adj, b, e, (uint32_t)un, want);
                    } else {
                        pos = lower_bound_entry(a.adj, b, e, want);
                        if (pos >= e || __ldg(a.adj + pos) != want) pos = -1;
                    }
                    if (pos < 0) continue;
                    bool used = false;
                    for (int j = 0; j < eq; ++j) {
                        if (Q.e_el[j] != el) continue;
                        const int32_t f = qimg[lane * vs + Q.e_from[j]], g2 = qimg[lane * vs + Q.e_to[j]];
                        if ((f == un && g2 == x) || (g2 == un && f == x)) used = true;
                    }
                    if (used) continue;
                    ok = el == F.gen_kc;
                    bpos = pos;
                    break;
                }
            }
            for (int p = 0; p < nq; ++p) gimg[lane * vs + p] = qimg[lane * vs + p];
            if (ecols) {
                for (int j = 0; j < eq; ++j) gec[lane * es + j] = qec[lane * es + j];
                gec[lane * es + eq] = bpos;
            }
            __syncwarp();
            mask_row<MW>(a, F, gimg + lane * vs, EcolFromShared{gec + lane * es}, ok, lane, acc);
            __syncwarp();
            continue;
        }

        // Forward tuple (source s, window key kc): the entries of the
        // segment (s, kc) of each Q row's source image, minus the row's images.
        int32_t st = 0, c = 0;
        if (qlive) {
            const int32_t u = qimg[lane * vs + Q.src_v[F.gen_s]];
            const uint32_t kc = (uint32_t)F.gen_kc;
            if (a.segstart) {
                const int64_t K1 = (int64_t)a.nel * a.lwin + 1;
                st = __ldg(a.segstart + (int64_t)u * K1 + kc);
                c = __ldg(a.segstart + (int64_t)u * K1 + kc + 1) - st;
            } else {
                const int32_t b = __ldg(a.offsets + u), e = __ldg(a.offsets + u + 1);
                const uint32_t el = kc / (uint32_t)a.lwin;
                const uint32_t tl = (uint32_t)Q.lbase + kc % (uint32_t)a.lwin;
                st = lower_bound_entry(a.adj, b, e, pack_entry(el, tl, 0));
                c = lower_bound_entry(a.adj, st, e, pack_entry(el, tl + 1, 0)) - st;
            }
        }
        wst[lane] = st;
        wcnt[lane] = c;
        int32_t incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t t = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += t;
        }
        wpre[lane] = incl - c;
        const int32_t total = __shfl_sync(kFull, incl, 31);
        __syncwarp();
        for (int32_t base = 0; base < total; base += 32) {
            const int32_t item = base + lane;
            bool ok = item < total;
            if (ok) {
                int l2 = 0, h2 = 31;
                while (l2 < h2) {
                    const int mid = (l2 + h2 + 1) >> 1;
                    if (wpre[mid] <= item) l2 = mid; else h2 = mid - 1;
                }
                const int owner = l2;
                const int32_t ei = wst[owner] + (item - wpre[owner]);
                const int32_t to = (int32_t)entry_to(__ldg(a.adj + ei));
                for (int p = 0; p < nq; ++p) {
                    const int32_t x = qimg[owner * vs + p];
                    ok &= x != to;
                    gimg[lane * vs + p] = x;
                }
                gimg[lane * vs + nq] = to;
                if (ecols) {
                    for (int j = 0; j < eq; ++j) gec[lane * es + j] = qec[owner * es + j];
                    gec[lane * es + eq] = ei;
                }
            }
            __syncwarp();
            mask_row<MW>(a, F, gimg + lane * vs, EcolFromShared{gec + lane * es}, ok, lane, acc);
            __syncwarp();
        }
    }
    acc.flush(a.counts, lane);
}

// Transposes the warp's 32x32 bit matrix (lane i's word is row i): afterwards
// lane b holds column b, bit i of it being bit b of lane i's word.  Five
// exchange steps, each swapping the off-diagonal blocks of the next smaller
// block size (the recursive block transpose, done across lanes).
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, int lane)
{
    const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const int j = 16 >> k;
        const uint32_t m = masks[k];
        const uint32_t y = __shfl_xor_sync(kFull, x, j);
        x = (lane & j) ? (x & ~m) | ((y & ~m) >> j) : (x & m) | ((y & m) << j);
    }
    return x;
}

// Domain sizes from the mask planes: each set bit of a plane word adds one
// vertex to its tuple's domain.  Block per (plane, run of 256 vertices) in
// grid-stride loops; a warp transposes its 32 vertices' word w, so lane b
// counts bit b with one popcount, summed per block in shared memory and
// added once per block.
__global__ void __launch_bounds__(256) k_mask_popcount(const MaskPlane* __restrict__ planes, int32_t nplanes,
                                                     const uint32_t* __restrict__ M, const uint32_t* __restrict__ MB,
                                                     uint32_t* __restrict__ sizes)
{
    __shared__ uint32_t hist[32 * kMaxMaskWords];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int32_t pl = blockIdx.y; pl < nplanes; pl += gridDim.y) {
        const MaskPlane P = planes[pl];
        const uint32_t* const base = (P.mb ? MB : M) + P.off;
        const int W = P.words;
        for (int i = threadIdx.x; i < 32 * W; i += blockDim.x) hist[i] = 0u;
        __syncthreads();
        for (int64_t v0 = (int64_t)blockIdx.x * blockDim.x + warp * 32; v0 < P.nloc;
             v0 += (int64_t)gridDim.x * blockDim.x) {
            const int64_t v = v0 + lane;
            for (int w = 0; w < W; ++w) {
                const uint32_t word = v < P.nloc ? __ldcs(base + v * W + w) : 0u;
                if (!__any_sync(kFull, word)) continue;
                const uint32_t c = (uint32_t)__popc(warp_transpose32(word, lane));
                if (c) atomicAdd(hist + w * 32 + lane, c);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 32 * W; i += blockDim.x) {
            const uint32_t c = hist[i];
            if (c && i < P.nbits) atomicAdd(sizes + P.sz_base + (int64_t)i * P.sz_stride, c);
        }
        __syncthreads();
    }
}

// Touched lists from R: every vertex of a (parent, source) slot's window
// whose row counter is non-zero, in vertex order.  Block rows (blockIdx.y)
// walk the slots, blocks along x the window in runs of 256 vertices, with one
// reservation in the slot's count per run.
__global__ void __launch_bounds__(256) k_mask_touched(MaskDev a)
{
    __shared__ uint32_t wcnt[8];
    __shared__ uint32_t run_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int32_t q = blockIdx.y; q < a.nps; q += gridDim.y) {
        const ParentMeta& P = a.parents[a.ps_parent[q]];
        const int s = q - P.ps_begin;
        const uint32_t* const Rs = a.R + P.r_off + (int64_t)s * P.nloc;
        int32_t* const out = a.touched + P.t_off + (int64_t)s * P.t_cap;
        for (int64_t b0 = (int64_t)blockIdx.x * blockDim.x; b0 < P.nloc; b0 += (int64_t)gridDim.x * blockDim.x) {
            const int64_t v = b0 + threadIdx.x;
            const bool hit = v < P.nloc && __ldcg(Rs + v) != 0u;
            const unsigned hm = __ballot_sync(kFull, hit);
            if (lane == 0) wcnt[warp] = (uint32_t)__popc(hm);
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t run = 0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                    const uint32_t c = wcnt[w];
                    wcnt[w] = run;
                    run += c;
                }
                run_base = run ? atomicAdd(a.tcount + q, run) : 0u;
            }
            __syncthreads();
            if (hit) {
                const uint32_t slot = run_base + wcnt[warp] + (uint32_t)__popc(hm & lanemask_lt());
                if (slot < (uint32_t)P.t_cap)
                    out[slot] = (int32_t)(P.vbase + v);
                else
                    atomicOr(a.status, kErrCursor);
            }
            __syncthreads();
        }
    }
}

// Exclusive prefix of the touched-list lengths: the sweep's task numbering.
__global__ void k_mask_prefix(int32_t nps, const uint32_t* __restrict__ tcount, unsigned long long* __restrict__ tprefix)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long run = 0;
    for (int32_t i = 0; i < nps; ++i) {
        tprefix[i] = run;
        run += tcount[i];
    }
    tprefix[nps] = run;
}

// Sweep: warp per touched (parent, source, vertex u) over u's entries in the
// source's range: child counts by tuple and the new vertex's domain masks.
// R[u] and the H entries it reads are reset to zero.
__global__ void __launch_bounds__(256) k_mask_sweep(MaskDev a)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int32_t K = a.nel * a.lwin;
    const int mw = a.mw;
    const unsigned long long total = a.tprefix[a.nps];
    unsigned long long scanned = 0;
    // Forward counts of the current (parent, source) slot, summed per tuple in
    // shared memory when the tuple space is small; flushed to the global
    // counts when the warp moves to another slot and at the end.
    // With the same small tuple space, the source vertex's own domain for
    // tuple c: every touched u with some entry e of seg(u, c) where
    // R[u] > H[e], i.e. some row with source image u has a child in c
    // (exactly the rows whose mask would have included c).  R - H >= 0 for
    // every entry, so a run of equal keys has a child exactly when its sum is
    // positive: the lane that ends the run flags the key (wflag), and at the
    // end of the task lane q moves the flags of keys q and q + 32 into the
    // per-key counts (wsrc), flushed with the forward counts.
    __shared__ unsigned long long sweep_acc[8][kSweepAccKeys];
    __shared__ uint32_t sweep_src[8][kSweepAccKeys];
    __shared__ uint32_t sweep_flag[8][kSweepAccKeys];
    unsigned long long* const wacc = sweep_acc[threadIdx.x >> 5];
    uint32_t* const wsrc = sweep_src[threadIdx.x >> 5];
    uint32_t* const wflag = sweep_flag[threadIdx.x >> 5];
    const bool use_acc = K <= kSweepAccKeys && (blockDim.x >> 5) <= 8;
    unsigned long long* acc_cnt = nullptr;   // global counts the accumulator belongs to
    int64_t acc_src = 0;                     // sizes index of the source domain of key 0
    int32_t acc_stride = 0;
    if (use_acc) {
        for (int q = lane; q < kSweepAccKeys; q += 32) {
            wacc[q] = 0;
            wsrc[q] = 0;
            wflag[q] = 0;
        }
        __syncwarp();
    }
    auto flush = [&]() {
        if (!acc_cnt) return;
        __syncwarp();
        for (int q = lane; q < K; q += 32) {
            const unsigned long long v = wacc[q];
            if (v) {
                atomicAdd(acc_cnt + q, v);
                wacc[q] = 0;
            }
            const uint32_t d = wsrc[q];
            if (d) {
                atomicAdd(a.sizes + acc_src + (int64_t)q * acc_stride, d);
                wsrc[q] = 0;
            }
        }
        __syncwarp();
    };
    for (unsigned long long task = warp; task < total; task += nwarps) {
        int32_t lo = 0, hi = a.nps - 1;
        while (lo < hi) {
            const int32_t mid = (lo + hi + 1) >> 1;
            if (a.tprefix[mid] <= task) lo = mid; else hi = mid - 1;
        }
        const ParentMeta& P = a.parents[a.ps_parent[lo]];
        const int s = lo - P.ps_begin;
        const int64_t idx = (int64_t)(task - a.tprefix[lo]);
        if (idx >= P.t_cap) continue;   // the row pass flagged an overflow; never read past the list
        const int32_t u = a.touched[P.t_off + (int64_t)s * P.t_cap + idx];
        uint32_t* Ru = a.R + P.r_off + (int64_t)s * P.nloc + (u - P.vbase);
        const uint32_t r = *Ru;
        __syncwarp();
        const int min_label = P.min_label;
        const int32_t b = __ldg(a.offsets + u), e = __ldg(a.offsets + u + 1);
        const uint64_t lo_key = s == 0 ? pack_entry(0, (uint32_t)min_label, 0)
                                       : pack_entry((uint32_t)P.src_el[s], (uint32_t)P.src_tl[s], 0);
        const int32_t st = a.segstart ? __ldg(a.segstart + (int64_t)u * (a.nel * a.lwin + 1) +
                                              (s == 0 ? min_label - P.lbase
                                                      : P.src_el[s] * a.lwin + P.src_tl[s] - P.lbase))
                                      : lower_bound_entry(a.adj, b, e, lo_key);
        uint32_t* Hs = a.H + P.h_off + (int64_t)s * P.mloc - P.ebase;
        uint32_t* NM = a.M + P.m_off + ((int64_t)s * (P.nv + 1) + P.nv) * P.nloc * mw;
        unsigned long long* cnt = a.counts + P.key_base + (int64_t)s * K;
        if (use_acc && cnt != acc_cnt) {
            flush();
            acc_cnt = cnt;
            acc_src = P.sz_off + (int64_t)s * K * (P.nv + 1) + P.src_v[s];
            acc_stride = P.nv + 1;
        }
        scanned += (unsigned long long)(e - st);
        for (int32_t base = st; base < e; base += 32) {
            const int32_t i = base + lane;
            bool ok = false;
            int32_t kc = 0;
            uint32_t diff = 0, to = 0;
            if (i < e) {
                const uint64_t ent = __ldg(a.adj + i);
                const int32_t tl = (int32_t)entry_tl(ent);
                ok = tl >= min_label && (uint32_t)(tl - P.lbase) < (uint32_t)a.lwin;
                kc = (int32_t)entry_el(ent) * a.lwin + tl - P.lbase;
                to = entry_to(ent);
                const uint32_t h = Hs[i];
                if (h) Hs[i] = 0u;
                diff = r - h;
            }
            // Entries are sorted by tuple, so equal tuples sit in adjacent lanes.
            const int32_t segk = ok ? kc : (int32_t)(0x40000000 + lane);
            unsigned long long v = ok ? diff : 0ull;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long uv = __shfl_up_sync(kFull, v, d);
                const int32_t uk = __shfl_up_sync(kFull, segk, d);
                if (lane >= d && uk == segk) v += uv;
            }
            const int32_t nk = __shfl_down_sync(kFull, segk, 1);
            if (ok && (lane == 31 || nk != segk) && v) {
                if (use_acc) {
                    atomicAdd(wacc + kc, v);
                    wflag[kc] = 1u;
                } else {
                    atomicAdd(cnt + kc, v);
                }
            }
            if (ok && diff > 0) or_bits(NM + (int64_t)(to - P.vbase) * mw + (kc >> 5), 1u << (kc & 31));
        }
        __syncwarp();
        if (use_acc) {
            wsrc[lane] += wflag[lane];
            wsrc[lane + 32] += wflag[lane + 32];
            wflag[lane] = 0u;
            wflag[lane + 32] = 0u;
        }
        __syncwarp();
        if (lane == 0) *Ru = 0u;
    }
    flush();
    // `scanned` is the same in every lane of the warp.
    if (lane == 0 && scanned) atomicAdd(a.scanned, scanned);
}

// Block per (active tuple, pattern vertex): the size of that domain.
__global__ void k_domain_sizes(const DomDesc* __restrict__ dom, const uint32_t* __restrict__ pool,
                               uint32_t* __restrict__ sizes)
{
    const int32_t ai = blockIdx.x / kMaxV;
    const int p = blockIdx.x % kMaxV;
    const DomDesc d = dom[ai];
    if (p >= d.nvc) return;
    const uint32_t* base = pool + d.off + (uint64_t)p * d.cap;
    uint32_t c = 0;
    for (uint32_t i = threadIdx.x; i < d.cap; i += blockDim.x) {
        const uint32_t w = base[i];
        c += d.hash ? (w != kHashEmpty) : __popc(w);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(kFull, c, o);
    __shared__ uint32_t part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x < 32) {
        c = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(kFull, c, o);
        if (threadIdx.x == 0) sizes[blockIdx.x] = c;
    }
}

int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

int grid_for(int64_t work, int threads)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (work + threads - 1) / threads;
    const int64_t cap = (int64_t)sms * 16;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

cudaError_t launch_label_minmax(int32_t n, const int32_t* d_vlabels, int32_t m, const gspan_edge* d_edges,
                                int32_t* d_out, cudaStream_t st)
{
    k_label_minmax<<<grid_for(std::max<int64_t>(n, m), 256), 256, 0, st>>>(n, d_vlabels, m, d_edges, d_out);
    return cudaGetLastError();
}

cudaError_t launch_label_presence(int32_t n, const int32_t* d_vlabels, int32_t vlo, uint8_t* d_vflag, int32_t m,
                                  const gspan_edge* d_edges, int32_t elo, uint8_t* d_eflag, cudaStream_t st)
{
    k_label_presence<<<grid_for(std::max<int64_t>(n, m), 256), 256, 0, st>>>(n, d_vlabels, vlo, d_vflag, m, d_edges,
                                                                             elo, d_eflag);
    return cudaGetLastError();
}

cudaError_t launch_batch_fixup(int32_t ninst, const int64_t* d_vbase, const int64_t* d_ebase, int32_t N, int32_t M,
                               int32_t* d_offsets, gspan_edge* d_edges, uint32_t* d_status, cudaStream_t st)
{
    if (N == 0 && M == 0) return cudaSuccess;
    k_batch_fixup<<<grid_for(std::max<int64_t>(N, M), 256), 256, 0, st>>>(ninst, d_vbase, d_ebase, N, M, d_offsets,
                                                                          d_edges, d_status);
    return cudaGetLastError();
}

cudaError_t launch_vertex_ranks(int32_t n, const int32_t* d_vlabels, int32_t vlo, const int32_t* d_vtab,
                                int32_t* d_vrank, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_vertex_ranks<<<grid_for(n, 256), 256, 0, st>>>(n, d_vlabels, vlo, d_vtab, d_vrank);
    return cudaGetLastError();
}

cudaError_t launch_build_adjacency(const int32_t* d_offsets, const gspan_edge* d_edges, const int32_t* d_etab,
                                   int32_t elo, const int32_t* d_elabels_sorted, DevGraph& g, uint64_t* d_tmp,
                                   uint32_t* d_status, cudaStream_t st)
{
    if (g.m > 0) {
        k_entry_keys<<<grid_for(g.m, 256), 256, 0, st>>>(g.m, g.n, d_edges, g.vrank, d_etab, elo, d_elabels_sorted,
                                                         g.nel, d_tmp, d_status);
    }
    if (g.n > 0) {
        k_sort_segments<<<grid_for((int64_t)g.n * 32, 256), 256, 0, st>>>(
            g.n, g.m, g.lwin, g.nel * g.lwin, g.vrank, g.win_base, d_offsets, d_edges, d_tmp, g.adj, g.src, d_status);
    }
    return cudaGetLastError();
}

cudaError_t launch_seed_count(const DevGraph& g, unsigned long long* counts, cudaStream_t st)
{
    if (g.m == 0) return cudaSuccess;
    const int64_t nkeys = (int64_t)g.nvl * g.nel * g.lwin;
    const int32_t smem_keys = nkeys <= kSeedSmemKeys ? (int32_t)nkeys : 0;
    // Few blocks when each flushes a histogram: a couple per SM.
    const int grid = smem_keys ? std::min(grid_for(g.m, 256), sm_count() * 2) : grid_for(g.m, 256);
    k_seed_count<<<grid, 256, (size_t)smem_keys * 8, st>>>(g.m, g.src, g.adj, g.vrank, g.win_base, g.lwin, g.nel,
                                                          counts, smem_keys);
    return cudaGetLastError();
}

cudaError_t launch_seed_support(const DevGraph& g, LevelKeys keys, int32_t nact, uint32_t* pool, int32_t* col0,
                                int32_t* col1, int32_t* col2, uint32_t* status, cudaStream_t st)
{
    if (g.m == 0) return cudaSuccess;
    const int32_t smem_act = nact <= kSeedSmemKeys / 2 ? nact : 0;
    const int grid = smem_act && col0 ? std::min(grid_for(g.m, 256), sm_count() * 2) : grid_for(g.m, 256);
    k_seed_support<<<grid, 256, (size_t)smem_act * 16, st>>>(g.m, g.src, g.adj, g.vrank, g.win_base, g.lwin, g.nel,
                                                            keys, pool, col0, col1, col2, status, smem_act);
    return cudaGetLastError();
}

int expand_grid_blocks(int device)
{
    // Allow the largest scratch (kMaxV vertices and ranges) on this device.
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const size_t smem = (size_t)kExpandWarps * 4 * expand_warp_ints(kMaxV | 1, kMaxV | 1, false);
    const size_t smem_mat = (size_t)kExpandWarps * 4 * expand_warp_ints(kMaxV | 1, kMaxV | 1, true);
    cudaFuncSetAttribute(k_expand<Pass::Count>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_expand<Pass::Support>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_expand<Pass::Materialize>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_mat);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_expand<Pass::Support>, kExpandThreads, smem);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

cudaError_t launch_expand(const ExpandArgs& x, Pass pass, cudaStream_t st)
{
    if (x.ntiles == 0) return cudaSuccess;
    ExpandDev a;
    a.offsets = x.g->offsets;
    a.adj = x.g->adj;
    a.segstart = x.g->segstart;
    a.eidx = x.g->eidx;
    a.eidx_cap = x.g->eidx_cap;
    a.nvl = x.g->nvl;
    a.nel = x.g->nel;
    a.lwin = x.g->lwin;
    a.parents = x.parents;
    a.nparents = x.nparents;
    a.ntiles = x.ntiles;
    a.in_cols = x.in_col_ptrs;
    a.out_cols = x.out_col_ptrs;
    a.ecol_in = x.ecol_in;
    a.ecol_out = x.ecol_out;
    a.keys = x.keys;
    a.pool = x.dom_pool;
    a.tile_counter = x.tile_counter;
    a.scanned = x.scanned;
    a.status = x.status;
    // Scratch strides from the largest parent of this launch.
    int maxv = 1, maxs = 1;
    for (int32_t i = 0; i < x.nparents; ++i) {
        const ParentMeta& P = x.parents_h[i];
        maxv = std::max(maxv, (int)P.nv);
        maxs = std::max(maxs, pass == Pass::Materialize && P.nmseg >= 0 ? (int)P.nmseg : (int)P.nsrc);
    }
    a.vs = maxv | 1;
    a.ss = maxs | 1;
    const size_t smem = (size_t)kExpandWarps * 4 * expand_warp_ints(a.vs, a.ss, pass == Pass::Materialize);
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (pass == Pass::Count)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_expand<Pass::Count>, kExpandThreads, smem);
    else if (pass == Pass::Support)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_expand<Pass::Support>, kExpandThreads, smem);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_expand<Pass::Materialize>, kExpandThreads, smem);
    const int64_t cap = (int64_t)sms * std::max(per_sm, 1);
    const int64_t need = (x.ntiles + kExpandWarps - 1) / kExpandWarps;
    const int grid = (int)(need < cap ? need : cap);
    if (pass == Pass::Count)
        k_expand<Pass::Count><<<grid, kExpandThreads, smem, st>>>(a);
    else if (pass == Pass::Support)
        k_expand<Pass::Support><<<grid, kExpandThreads, smem, st>>>(a);
    else
        k_expand<Pass::Materialize><<<grid, kExpandThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_entry_flags(DevGraph& g, uint32_t* status, cudaStream_t st)
{
    if (g.m == 0) return cudaSuccess;
    k_entry_flags<<<grid_for(g.m, 256), 256, 0, st>>>(g.m, g.src, g.offsets, g.adj, g.vrank, g.segstart, g.win_base,
                                                      g.lwin, g.nel * g.lwin, g.selfloop, g.rev,
                                                      reinterpret_cast<unsigned long long*>(g.eidx), g.eidx_cap,
                                                      status);
    return cudaGetLastError();
}



cudaError_t launch_segments(DevGraph& g, cudaStream_t st)
{
    if (g.n == 0 || g.segw == 0) return cudaSuccess;
    k_segments<<<grid_for((int64_t)g.n * 32, 256), 256, 0, st>>>(g.n, g.m, g.lwin, g.nel * g.lwin, g.segw, g.vrank,
                                                                 g.win_base, g.offsets, g.adj, g.segmask, g.segone,
                                                                 g.segstart);
    return cudaGetLastError();
}

namespace {
MaskDev mask_dev(const MaskArgs& x)
{
    MaskDev a;
    a.offsets = x.g->offsets;
    a.adj = x.g->adj;
    a.segmask = x.g->segmask;
    a.segone = x.g->segone;
    a.segstart = x.g->segstart;
    a.selfloop = x.g->selfloop;
    a.rev = x.g->rev;
    a.eidx = x.g->eidx;
    a.eidx_cap = x.g->eidx_cap;
    a.parallel = x.g->parallel;
    a.loops = x.g->loops;
    a.ecol = x.ecol;
    a.symmetric = x.g->symmetric;
    a.n = x.g->n;
    a.m = x.g->m;
    a.nvl = x.g->nvl;
    a.nel = x.g->nel;
    a.mw = x.g->segw;
    a.lwin = x.g->lwin;
    a.parents = x.parents;
    a.nparents = x.nparents;
    a.ntiles = x.ntiles;
    a.in_cols = x.in_col_ptrs;
    a.counts = x.counts;
    a.sizes = x.sizes;
    a.R = x.R;
    a.H = x.H;
    a.M = x.M;
    a.MB = x.MB;
    a.touched = x.touched;
    a.tcount = x.tcount;
    a.ps_parent = x.ps_parent;
    a.nps = x.nps;
    a.tprefix = x.tprefix;
    a.tile_counter = x.tile_counter;
    a.scanned = x.scanned;
    a.status = x.status;
    a.gen_parents = x.gen_parents;
    a.gen_cols = x.gen_cols;
    a.gen_ecol = x.gen_ecol;
    // gen_nv >= every generated row's vertices and pattern edges, so image
    // p < nv and entry column j < nedge stay inside their strides.
    a.gen_vs = (x.gen_nv + 1) | 1;
    a.gen_es = (x.gen_nv + 1) | 1;
    return a;
}

}  // namespace

cudaError_t launch_mask_rows(const MaskArgs& x, cudaStream_t st)
{
    if (x.ntiles == 0) return cudaSuccess;
    const int64_t need = (x.ntiles + kMaskWarps - 1) / kMaskWarps;
    const int64_t cap = (int64_t)sm_count() * 8;
    const int grid = (int)(need < cap ? need : cap);
    if (x.g->segw <= kNarrowMaskWords)
        k_mask_rows<kNarrowMaskWords><<<grid, kMaskWarps * 32, 0, st>>>(mask_dev(x));
    else
        k_mask_rows<kMaxMaskWords><<<grid, kMaskWarps * 32, 0, st>>>(mask_dev(x));
    return cudaGetLastError();
}

cudaError_t launch_mask_gen(const MaskArgs& x, cudaStream_t st)
{
    if (x.ntiles == 0) return cudaSuccess;
    const MaskDev a = mask_dev(x);
    const size_t smem = (size_t)kMaskWarps * gen_warp_ints(a.gen_vs, a.gen_es) * sizeof(int32_t);
    const int64_t need = (x.ntiles + kMaskWarps - 1) / kMaskWarps;
    const int64_t cap = (int64_t)sm_count() * 8;
    const int grid = (int)(need < cap ? need : cap);
    cudaError_t e;
    if (x.g->segw <= 2) {
        // Up to 64 tuples (37 vertex labels and one edge label on the 3.7M
        // graph): the two-word build spills less at the same 48 registers
        // (k = 4 on that graph: 2.31 against 2.40 s at support 100,000,
        // 38.7 against 40.6 s at 50,000).
        if ((e = cudaFuncSetAttribute(k_mask_gen<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem)) != cudaSuccess)
            return e;
        k_mask_gen<2><<<grid, kMaskWarps * 32, smem, st>>>(a);
    } else if (x.g->segw <= kNarrowMaskWords) {
        if ((e = cudaFuncSetAttribute(k_mask_gen<kNarrowMaskWords>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem)) != cudaSuccess)
            return e;
        k_mask_gen<kNarrowMaskWords><<<grid, kMaskWarps * 32, smem, st>>>(a);
    } else {
        if ((e = cudaFuncSetAttribute(k_mask_gen<kMaxMaskWords>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem)) != cudaSuccess)
            return e;
        k_mask_gen<kMaxMaskWords><<<grid, kMaskWarps * 32, smem, st>>>(a);
    }
    return cudaGetLastError();
}

namespace {
// blockIdx.y picks the span; 16-byte stores where the span is 16-byte
// aligned (stream-ordered allocations are), 4-byte stores for the rest.
__global__ void k_clear(ClearList l)
{
    const ClearSpan sp = l.span[blockIdx.y];
    uint32_t* p = static_cast<uint32_t*>(sp.p);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t head = 0;
    if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
        const int64_t n4 = sp.words >> 2;
        const uint4 v = make_uint4(sp.value, sp.value, sp.value, sp.value);
        uint4* p4 = reinterpret_cast<uint4*>(p);
        for (int64_t i = t; i < n4; i += stride) p4[i] = v;
        head = n4 << 2;
    }
    for (int64_t i = head + t; i < sp.words; i += stride) p[i] = sp.value;
}
}  // namespace

cudaError_t launch_clear(const ClearList& l, cudaStream_t st)
{
    if (l.n == 0) return cudaSuccess;
    int64_t most = 0;
    for (int i = 0; i < l.n; ++i) most = std::max(most, l.span[i].words);
    const int64_t want = (most / 4 + 255) / 256;
    const int64_t cap = (int64_t)sm_count() * 8;
    const int gx = (int)std::max<int64_t>(1, std::min(want, cap));
    k_clear<<<dim3(gx, l.n), 256, 0, st>>>(l);
    return cudaGetLastError();
}

cudaError_t launch_mask_popcount(const MaskArgs& x, cudaStream_t st)
{
    if (x.nplanes == 0) return cudaSuccess;
    const int gy = (int)std::min<int64_t>(x.nplanes, 65535);
    const int64_t runs = (x.max_plane_nloc + 255) / 256;
    const int64_t want = ((int64_t)sm_count() * 16 + gy - 1) / gy;
    const int gx = (int)std::max<int64_t>(1, std::min(runs, want));
    k_mask_popcount<<<dim3(gx, gy), 256, 0, st>>>(x.planes, x.nplanes, x.M, x.MB, x.sizes);
    return cudaGetLastError();
}

cudaError_t launch_mask_sweep(const MaskArgs& x, cudaStream_t st)
{
    if (x.nps == 0) return cudaSuccess;
    {
        const int gy = (int)std::min<int64_t>(x.nps, 65535);
        const int64_t runs = (x.max_plane_nloc + 255) / 256;
        const int64_t want = ((int64_t)sm_count() * 16 + gy - 1) / gy;
        const int gx = (int)std::max<int64_t>(1, std::min(runs, want));
        k_mask_touched<<<dim3(gx, gy), 256, 0, st>>>(mask_dev(x));
    }
    k_mask_prefix<<<1, 32, 0, st>>>(x.nps, x.tcount, x.tprefix);
    k_mask_sweep<<<sm_count() * 8, 256, 0, st>>>(mask_dev(x));
    return cudaGetLastError();
}

cudaError_t launch_domain_sizes(const DomDesc* dom, int32_t nact, const uint32_t* pool, uint32_t* sizes,
                                cudaStream_t st)
{
    if (nact == 0) return cudaSuccess;
    k_domain_sizes<<<nact * kMaxV, 256, 0, st>>>(dom, pool, sizes);
    return cudaGetLastError();
}

}  // namespace gs
