// Internal declarations shared by the host orchestration (miner.cc, capi.cc)
// and the CUDA kernels (kernels.cu).  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gspan_gb300.h"

namespace gs {

// Largest pattern (in edges) the kernels handle; a pattern of E edges has at
// most E+1 vertices.  Row images and per-source state live in shared memory
// sized by kMaxV.
constexpr int kMaxE = 15;
constexpr int kMaxV = kMaxE + 1;

// Packed adjacency entry: (edge-label rank << 48) | (to-label rank << 32) | to.
// Each vertex's entries are sorted ascending, i.e. by (edge label, to label, to).
__host__ __device__ inline uint64_t pack_entry(uint32_t el, uint32_t tl, uint32_t to)
{
    return ((uint64_t)el << 48) | ((uint64_t)tl << 32) | (uint64_t)to;
}
__host__ __device__ inline uint32_t entry_to(uint64_t e) { return (uint32_t)e; }
__host__ __device__ inline uint32_t entry_tl(uint64_t e) { return (uint32_t)(e >> 32) & 0xFFFFu; }
__host__ __device__ inline uint32_t entry_el(uint64_t e) { return (uint32_t)(e >> 48); }

// Device-side status word bits (set by kernels, read by the host after a pass).
enum : uint32_t {
    kErrHashFull = 1u << 0,     // a hashset probe ran through its whole table
    kErrBadGraph = 1u << 1,     // upload validation: offsets or entries inconsistent
    kErrCursor = 1u << 2,       // a materialisation cursor ran past its reserved rows
    kErrAsymmetric = 1u << 3,   // upload: an entry without its reverse entry (not an error)
    kFlagParallel = 1u << 4,    // upload: two equal entries of one vertex (parallel edges; not an error)
    kFlagSelfLoop = 1u << 5,    // upload: some vertex has an entry to itself (not an error)
    kErrCounter = 1u << 6,      // a 32-bit per-vertex row counter (R) of the mask path would wrap
};

// The graph in HBM.  Labels are replaced by their rank among the distinct
// labels present, which preserves every `<` / `<=` test of the reference.
struct DevGraph {
    int32_t n = 0;              // vertices
    int32_t m = 0;              // directed entries (2 per undirected edge)
    int32_t nvl = 0, nel = 0;   // distinct vertex / edge labels
    int32_t ninst = 1;          // mining instances (independent graphs) in this store
    // Label windows: the neighbours of a vertex with label rank r have label
    // ranks in [win_base[r], win_base[r] + lwin).  One window of all labels for
    // a single graph; one window per instance for a batch (instance-tagged
    // labels never meet across instances).  Tuple keys are window-local.
    int32_t lwin = 0;
    int32_t* win_base = nullptr;        // [nvl] device
    std::vector<int32_t> win_base_h;    // [nvl] host copy
    std::vector<int32_t> label_instance;  // [nvl] instance of each label rank (batch)
    std::vector<int64_t> inst_vbase, inst_ebase;  // [ninst + 1] vertex / entry prefix of the instances
    int32_t* offsets = nullptr; // [n+1]
    uint64_t* adj = nullptr;    // [m] packed entries, sorted per vertex
    int32_t* src = nullptr;     // [m] owning vertex of each entry
    int32_t* vrank = nullptr;   // [n] vertex label rank
    // Per vertex, `segw` words with bit (el * nvl + tl) set when the vertex has
    // a neighbour entry with that (edge label, to label).  Built when the key
    // space nel * nvl fits kMaxMaskWords words, else null (segw = 0).
    uint32_t* segmask = nullptr;
    int32_t segw = 0;
    // Same layout: bit set when that segment holds exactly one entry.
    uint32_t* segone = nullptr;
    // Per vertex, nel * lwin + 1 entry indices: where each (edge label, to
    // label) key's segment starts in the adjacency (the lower bound of the
    // key; the last one is the list's end).  Replaces the binary searches for
    // range starts.  Built with segmask when it fits 4 GB, else null.
    int32_t* segstart = nullptr;
    // Bit v set when vertex v has an entry to itself.
    uint32_t* selfloop = nullptr;
    // Every entry u->x with edge label l has a reverse entry x->u with label l
    // (checked at upload; true for every graph built by the text loader).
    bool symmetric = false;
    // rev[e]: index of the reverse entry of e (the k-th of a run of equal
    // entries pairs with the k-th of the reverse run); built with the symmetry
    // check.  When the graph is symmetric and has one edge label, level tables
    // also carry each pattern edge's entry index (entry_cols), which replaces
    // most adjacency searches of the mask row pass.
    int32_t* rev = nullptr;
    bool entry_cols = false;
    // Edge index: open addressing over `eidx_cap` (a power of two) 64-bit
    // slots, one per run of equal entries, keyed by (vertex, edge label, to):
    // slot = fingerprint << 32 | index of the run's first entry, empty = ~0.
    // An edge lookup is one or two L2 probes instead of a binary search over
    // the adjacency.  Not built (null) above 2^30 entries.
    uint64_t* eidx = nullptr;
    uint32_t eidx_cap = 0;
    // Embeddings per 1-edge tuple (nvl * nel * lwin keys), counted once at
    // upload: device and host copies, null / empty when the key space is
    // larger than kSeedCacheKeys (mining counts them per run then).
    unsigned long long* seed_counts = nullptr;
    std::vector<unsigned long long> seed_counts_h;
    // Some vertex has two equal entries (parallel edges with one label).
    bool parallel = true;
    // Some vertex has an entry to itself.  Without self-loops every embedding
    // maps distinct pattern vertices to distinct graph vertices.
    bool loops = true;
    // Mean degree of a vertex reached through an edge (sum d^2 / sum d): the
    // expected adjacency length behind an embedding's vertex.
    double edge_biased_degree = 0;
    std::vector<int32_t> vlabel_of_rank, elabel_of_rank;
};

// Rows per tile of the Materialize pass (the other passes: 32, one per
// lane).  Fewer rows give the tile queue more, lighter units to balance when
// some rows' frequent segments are long (hubs).
constexpr int kMatTileRows = 8;

// Tuples per source (nel * lwin) up to which the sweep sums forward counts
// per warp in shared memory and counts the source vertex's own domains (the
// row pass then leaves those domains out of M).
constexpr int kSweepAccKeys = 64;

// Widest per-vertex key mask the mask kernels handle (x 32 keys).
constexpr int kMaxMaskWords = 16;
// Largest 1-edge key space whose seed counts the store keeps.
constexpr int64_t kSeedCacheKeys = (int64_t)1 << 22;
// Mask words of the row pass's fast build (<= 128 tuple keys per label
// window); wider label spaces use the kMaxMaskWords build.
constexpr int kNarrowMaskWords = 4;

// Where a domain (set of graph vertices that one pattern vertex maps to)
// lives: `nvc` consecutive tables of `cap` 32-bit words starting at `off` in
// the domain pool.  Bitmap: cap = ceil(n/32) words.  Hashset: cap = power of
// two slots holding vertex ids, empty = 0xFFFFFFFF.
struct DomDesc {
    uint64_t off;
    uint32_t cap;
    uint16_t nvc;
    uint16_t hash;
    int32_t vbase;              // first vertex of the tuple's instance (ids are stored relative to it)
    int32_t pad;
};

constexpr uint32_t kHashEmpty = 0xFFFFFFFFu;

// One parent pattern of an extension level, as the kernels see it.
// Sources: s = 0 is the first-forward source v_n; s >= 1 are the tails of the
// rightmost-path edges rmpath[s-1] (other-forward), each with the (edge label,
// to label) lower bound (src_el, src_tl) of gspan.cu:464-483.
// Backward targets t: rmpath[t+1] tails (gspan.cu:702-711), with the label test
// of gspan.cu:437-439 reduced to: edge label > back_el, or == back_el when
// back_eq is set.
struct ParentMeta {
    int64_t row_begin;          // first row in the level table
    int64_t row_end;
    int64_t tile_begin;         // first 32-row tile index of this parent
    int32_t key_base;           // first key of this parent in the level key space
    int16_t nv;                 // pattern vertices
    int16_t nsrc;
    int16_t nback;
    int16_t nedge;
    int16_t vn;                 // rightmost vertex v_n
    int16_t min_label;          // vertex-label rank of v0
    int32_t lbase;              // first label rank of this pattern's label window
    // Vertices [vbase, vbase + nloc) and entries [ebase, ebase + mloc) of this
    // pattern's instance: the dense per-parent arrays cover only these.
    int32_t vbase, nloc, ebase, mloc;
    int16_t vlab[kMaxV];        // vertex-label rank of each pattern vertex
    int16_t src_v[kMaxV];
    int16_t src_el[kMaxV];
    int16_t src_tl[kMaxV];
    int16_t back_v[kMaxV];
    int16_t back_el[kMaxV];
    int16_t back_eq[kMaxV];
    int8_t e_from[kMaxE];       // parent code edges, for the has_edge test
    int8_t e_to[kMaxE];
    int16_t e_el[kMaxE];
    uint16_t src_adj[kMaxV];    // per source: pattern vertices joined to it by a code edge
    // Pattern vertices in (stable) label order: equal labels are adjacent.
    int8_t lorder[kMaxV];
    // Per source and pattern vertex: the (last) code edge joining them, -1 if none.
    int8_t pair_edge[kMaxV][kMaxV];
    // Per backward target: bit el (el < 32) when a code edge with label el
    // joins v_n and the target.
    uint32_t back_used[kMaxV];
    // Materialisation: the frequent forward tuples as (source, el * nvl + tl),
    // scanned segment by segment; nmseg = -1 scans every source's full range.
    int16_t nmseg;
    int16_t mseg_s[kMaxV];
    uint32_t mseg_kc[kMaxV];
    // Mask path (see k_mask_rows): offsets of this parent's arrays in the
    // buffers of its parent group.
    int32_t bw;                 // words per backward-key mask
    int32_t ps_begin;           // first (parent, source) slot of this parent in the group
    int32_t t_cap;              // touched-list capacity per source: min(rows, n)
    int64_t t_off;              // touched lists: nsrc x t_cap vertices
    int64_t r_off;              // R: nsrc x n row counters
    int64_t h_off;              // H: nsrc x m entry counters
    int64_t m_off;              // M: nsrc x (nv+1) x n x segw words
    int64_t b_off;              // MB: nv x n x bw words
    int64_t sz_off;             // domain sizes: nsrc*K*(nv+1) forward, then nback*nel*nv backward
    uint32_t range[kMaxV][kMaxMaskWords];   // per source: keys inside its valid range
    // Two-level last step (k_mask_gen): this parent's rows are not in a table
    // but generated from the rows of its own parent gen_p2 (one level up) as
    // that parent's child tuple: forward (gen_kind 1) from source gen_s with
    // window key gen_kc, or backward (gen_kind 2) to target gen_s with edge
    // label gen_kc.  gen_kind 0: rows come from the level table.  tile_begin
    // then counts 32-row tiles of gen_p2's rows.
    int32_t gen_p2;
    int16_t gen_kind;
    int16_t gen_s;
    int32_t gen_kc;
    // 2^32 rows or more: the row pass checks its 32-bit counters for a wrap.
    int32_t r_wide;
    // One edge label (entry-column row walk): per source, the pattern vertices
    // the walk visits, in label order - labels inside the source's valid
    // range and, without self-loops, not the source itself - packed as
    // j | (code edge joining j and the source + 1) << 4 | (that edge starts at
    // the source) << 8 | label rank << 16.
    int8_t walk_n[kMaxV];
    int32_t walk[kMaxV][kMaxV];
};

// Per-level key space arrays on the device.
struct LevelKeys {
    unsigned long long* counts = nullptr;   // [nkeys]
    int32_t* act = nullptr;                 // [nkeys] active-key index or -1
    DomDesc* dom = nullptr;                 // [nact]
    long long* mat_off = nullptr;           // [nact] first output row, or -1
    unsigned long long* cursor = nullptr;   // [nact]
};

enum class Pass : int { Count = 0, Support = 1, Materialize = 2 };

struct ExpandArgs {
    const DevGraph* g;                 // host copy; device pointers inside are used
    const ParentMeta* parents;         // device
    const ParentMeta* parents_h;       // host copy of the same parents (sizes the launch's scratch)
    int32_t nparents;
    int64_t ntiles;
    int32_t in_cols;                   // columns of the parent table
    int32_t ecol_in = -1;              // first entry column of the parent table, -1 if none
    int32_t ecol_out = -1;             // first entry column of the child table, -1 if none
    int32_t* const* in_col_ptrs;       // device array [in_cols] of column pointers
    int32_t* const* out_col_ptrs;      // device array [out_cols] (support pass with materialisation)
    LevelKeys keys;
    uint32_t* dom_pool;
    unsigned long long* tile_counter;  // device scratch, zeroed before launch
    unsigned long long* scanned;       // device accumulator of adjacency entries read
    uint32_t* status;
};

// Kernel launchers (kernels.cu).  All are asynchronous on `st`.
// Graph store build: label min/max ([vmin, vmax, emin, emax], initialised
// by the caller to INT32_MAX / INT32_MIN), presence flags over the label
// ranges, vertex label ranks from a dense table, then packed + sorted entries.
cudaError_t launch_label_minmax(int32_t n, const int32_t* d_vlabels, int32_t m, const gspan_edge* d_edges,
                                int32_t* d_out, cudaStream_t st);
cudaError_t launch_label_presence(int32_t n, const int32_t* d_vlabels, int32_t vlo, uint8_t* d_vflag, int32_t m,
                                  const gspan_edge* d_edges, int32_t elo, uint8_t* d_eflag, cudaStream_t st);
// Batch: instance-local offsets and ids -> batch-wide (vbase/ebase: [ninst+1]
// prefix sums of vertex and entry counts); an id outside its instance sets
// kErrBadGraph.
cudaError_t launch_batch_fixup(int32_t ninst, const int64_t* d_vbase, const int64_t* d_ebase, int32_t N, int32_t M,
                               int32_t* d_offsets, gspan_edge* d_edges, uint32_t* d_status, cudaStream_t st);
cudaError_t launch_vertex_ranks(int32_t n, const int32_t* d_vlabels, int32_t vlo, const int32_t* d_vtab,
                                int32_t* d_vrank, cudaStream_t st);
// Edge-label ranks from d_etab[label - elo] when d_etab is set, else by binary
// search over d_elabels_sorted (g.nel entries).  g.vrank must be filled.
cudaError_t launch_build_adjacency(const int32_t* d_offsets, const gspan_edge* d_edges, const int32_t* d_etab,
                                   int32_t elo, const int32_t* d_elabels_sorted, DevGraph& g, uint64_t* d_tmp,
                                   uint32_t* d_status, cudaStream_t st);
cudaError_t launch_seed_count(const DevGraph& g, unsigned long long* counts, cudaStream_t st);
// col2 (may be null) receives each seed's entry index.
cudaError_t launch_seed_support(const DevGraph& g, LevelKeys keys, int32_t nact, uint32_t* pool, int32_t* col0,
                                int32_t* col1, int32_t* col2, uint32_t* status, cudaStream_t st);
cudaError_t launch_expand(const ExpandArgs& a, Pass pass, cudaStream_t st);
cudaError_t launch_domain_sizes(const DomDesc* dom, int32_t nact, const uint32_t* pool,
                                uint32_t* sizes /* [nact * kMaxV] */, cudaStream_t st);

int expand_grid_blocks(int device);

// Mask path.
// One plane of mask words (M: per parent, source and pattern vertex; MB:
// per parent and pattern vertex): `words` words per vertex of the parent's
// window, bit i of a vertex's words counting into sizes[sz_base + i * sz_stride]
// for i < nbits.
struct MaskPlane {
    int64_t off;       // first word in M (mb = 0) or MB (mb = 1)
    int64_t sz_base;
    int32_t nloc;
    int32_t sz_stride;
    int32_t nbits;
    int16_t words;
    int16_t mb;
};

struct MaskArgs {
    const DevGraph* g;
    const ParentMeta* parents;   // device, one group of mask-path parents
    int32_t nparents;
    int64_t ntiles;
    int32_t* const* in_col_ptrs;
    int32_t ecol = -1;           // first entry column of the parent table, -1 if none
    unsigned long long* counts;  // level key space
    uint32_t* sizes;             // domain sizes, indexed from ParentMeta::sz_off
    uint32_t* R;                 // zero on entry; the sweep leaves it zero
    uint32_t* H;                 // zero on entry; the sweep leaves it zero
    uint32_t* M;                 // zero on entry
    uint32_t* MB;                // zero on entry
    int32_t* touched;
    uint32_t* tcount;            // [nps], zero on entry
    const int32_t* ps_parent;    // [nps] parent index of each (parent, source) slot
    int32_t nps;
    unsigned long long* tprefix; // [nps + 1] scratch
    unsigned long long* tile_counter;
    unsigned long long* scanned; // adjacency entries read by the sweep
    uint32_t* status;
    // Two-level last step only: the parents' own parents (one level up), the
    // table of their rows and its first entry column (-1 if none).
    const ParentMeta* gen_parents = nullptr;
    int32_t* const* gen_cols = nullptr;
    int32_t gen_ecol = -1;
    int32_t gen_nv = 0;          // most vertices of any generated row
    // The group's mask planes, counted into `sizes` after the sweep.
    const MaskPlane* planes = nullptr;
    int32_t nplanes = 0;
    int64_t max_plane_nloc = 0;
};
// Segment masks (zeroed by the caller), singleton masks and, when
// allocated, segment starts, in one pass over each vertex's entries.
cudaError_t launch_segments(DevGraph& g, cudaStream_t st);
// One pass over the entries: self-loop bitmap (zeroed by the caller), reverse
// entries and the symmetry check (kErrAsymmetric), the edge index when
// g.eidx is allocated (all slots ~0 on entry; kFlagParallel, kErrHashFull),
// and kFlagSelfLoop.
cudaError_t launch_entry_flags(DevGraph& g, uint32_t* status, cudaStream_t st);
cudaError_t launch_mask_rows(const MaskArgs& a, cudaStream_t st);
// Two-level last step: the row pass over rows generated from gen_parents'
// rows (every parent has gen_kind != 0), none of them stored.
cudaError_t launch_mask_gen(const MaskArgs& a, cudaStream_t st);
// Touched lists from R, their prefix, then the sweep (three launches).
cudaError_t launch_mask_sweep(const MaskArgs& a, cudaStream_t st);
// Domain sizes of the group's tuples from its mask planes (after the sweep).
cudaError_t launch_mask_popcount(const MaskArgs& a, cudaStream_t st);

// Several buffers set to one 32-bit value each, in one launch instead of a
// memset per buffer (each memset is an API call and a stream operation of
// its own).  Spans with no words are skipped.
constexpr int kMaxClearSpans = 12;
struct ClearSpan {
    void* p;
    int64_t words;    // 32-bit words
    uint32_t value;
};
struct ClearList {
    ClearSpan span[kMaxClearSpans];
    int n = 0;
    // Adds a span; false when the list is full.
    bool add(void* p, int64_t words, uint32_t value = 0)
    {
        if (!p || words <= 0) return true;
        if (n == kMaxClearSpans) return false;
        span[n++] = ClearSpan{p, words, value};
        return true;
    }
};
cudaError_t launch_clear(const ClearList& l, cudaStream_t st);

}  // namespace gs
