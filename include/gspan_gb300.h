/*
 * gspan_gb300 — C ABI of the GB300 frequent-subgraph miner.
 *
 * gSpan pattern growth over ONE undirected, vertex- and edge-labelled graph with
 * MNI (minimum-image) support, computed by CUDA kernels on one GPU.  The ABI
 * takes plain pointers and sizes; every call returns a status code and never
 * throws.  Results (pattern, support) come back through a callback in the same
 * order in which haozixu/gSpan prints them.
 *
 * Reference interfaces replaced (file:line in haozixu/gSpan):
 *   gspan_graph_upload  <- CSRGraph + init_gpu_context      (graph.h:51-65, gspan.cu:97-127)
 *   gspan_mine          <- void fsm(const CSRGraph&, int k, int min_support)
 *                                                           (gspan.h:41, gspan.cu:1171-1199)
 *   gspan_emit_fn       <- report()/print_dfs_code()        (gspan.cu:67-77)
 *   gspan_is_canonical  <- is_canonical(const DFSCode&)     (gspan.cu:586-606)
 *
 * Threading: a context is used by one host thread at a time.  A context owns
 * its CUDA stream and all device memory it allocates.  A graph is freed by
 * the context that uploaded it (before that context is destroyed) and may be
 * mined by any context on the same device, from any number of threads at
 * once: mining only reads it.
 */
#ifndef GSPAN_GB300_H_
#define GSPAN_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gspan_status {
    GSPAN_OK = 0,
    GSPAN_ERR_INVALID = 1,   /* bad argument or malformed graph */
    GSPAN_ERR_CUDA = 2,      /* a CUDA runtime call failed (message in gspan_last_error) */
    GSPAN_ERR_NOMEM = 3,     /* device or host allocation failed, or over the memory budget */
    GSPAN_ERR_LIMIT = 4,     /* beyond a documented size limit (pattern size, label count) */
    GSPAN_ERR_DEVICE = 5,    /* a kernel reported an internal error through its status word */
    GSPAN_ERR_ABORTED = 6,   /* the emit callback asked to stop */
    GSPAN_ERR_NO_DEVICE = 7  /* no CUDA device is visible */
} gspan_status;

/* One directed CSR entry, layout-identical to the reference's `Edge`
 * (graph.h:7-12): 12 bytes, from / to / label. */
typedef struct gspan_edge {
    int32_t from, to, label;
} gspan_edge;

/* One DFS-code edge, layout-identical to the reference's `PatternEdge`
 * (graph.h:28-47).  Labels that the code does not fix are -1. */
typedef struct gspan_pattern_edge {
    int32_t from, to, from_label, edge_label, to_label;
} gspan_pattern_edge;

typedef struct gspan_opts {
    int32_t device;              /* CUDA device ordinal (default 0) */
    int32_t domain_mode;         /* 0 auto (bitmap or hashset per domain), 1 bitmaps only, 2 hashsets only */
    double hash_threshold;       /* auto mode: a domain uses a hashset when 64 * max_size < |V| * hash_threshold.
                                    0 selects the default (1.0) */
    double mem_fraction;         /* share of free device memory one level's mask-path arrays may hold
                                    (capped at 0.4; 0 selects 0.4) */
    int32_t profile;             /* 1: time every kernel launch with CUDA events into gspan_stats */
    int32_t path;                /* extension kernels: 0 auto, 1 per-candidate only, 2 mask path wherever the
                                    label space allows (both give identical results) */
    double mask_bias;            /* auto path: a parent takes the mask path when its estimated candidate work
                                    exceeds mask_bias / 8 x the dense words the mask path clears.
                                    0 selects the default (1.0) */
    int32_t prune;               /* 1: before mining a single graph, drop every vertex whose label occurs on
                                    fewer than min_support vertices, with its edges (the reference's unused
                                    prune_graph, graph.cc:216-266, done on the device).  Patterns and
                                    supports are unchanged; `extended` then counts the pruned graph's
                                    children.  Ignored for batches.  Default 0 */
    int32_t fused_last;          /* the next-to-last level's embeddings: 0 auto (generated on the fly inside the
                                    last level's row pass when storing them would take more than half the free
                                    device memory, else stored), 1 always stored, 2 always generated (needs the
                                    mask path; both give identical results) */
} gspan_opts;

/* Run statistics.  Counts are exact and identical to those of the reference's
 * CPU path on the same input (extension outputs of every extended pattern). */
typedef struct gspan_stats {
    uint64_t seeds;              /* level-1 embeddings (directed edges with from_label <= to_label) */
    uint64_t extended;           /* child embeddings produced by extending frequent patterns */
    uint64_t patterns;           /* reported (frequent, minimum-code) patterns */
    uint64_t support_keys;       /* candidate patterns whose MNI support was counted */
    uint64_t hash_domains;       /* of their vertex domains, how many used hashsets */
    uint64_t scanned_entries;    /* adjacency entries read by the extension kernels */
    uint64_t materialized_rows;  /* child embedding rows written to HBM */
    uint64_t kernel_launches;    /* kernels of this library launched during gspan_mine */
    int32_t levels;              /* deepest pattern size reached */
    double mine_ms;              /* host wall time of gspan_mine */
    uint64_t h2d_bytes;          /* host->device bytes copied by gspan_mine */
    uint64_t d2h_bytes;          /* device->host bytes copied by gspan_mine */
    uint64_t frontier_rows;      /* embeddings of the frequent patterns of the deepest level mined */
    uint64_t mask_parents;       /* parent patterns extended by the mask kernels */
    uint64_t candidate_parents;  /* parent patterns extended by the per-candidate kernels */
    /* Per kernel family: launches, algorithmic bytes, and (profile == 1 only)
     * CUDA-event time summed over launches. */
    double expand_ms;            /* per-candidate kernels, Count and Support passes */
    uint64_t expand_launches;
    double expand_bytes;
    double rows_ms;              /* mask path: row pass */
    uint64_t rows_launches;
    double rows_bytes;
    double sweep_ms;             /* mask path: adjacency sweep */
    double sweep_bytes;
    double materialize_ms;       /* child-row scatter of frequent children */
    uint64_t materialize_launches;
    double materialize_bytes;
    double seed_ms;
    double domain_ms;            /* domain-size reductions */
    uint64_t canonical_checks;   /* children that needed the minimum-code test (host) */
    double canonical_ms;         /* host time in tests not already done while the GPU counted */
    uint64_t pruned_vertices;    /* opts.prune: vertices dropped before mining (0 otherwise) */
    uint64_t pruned_entries;     /* opts.prune: directed entries dropped with them */
    uint64_t fused_rows;         /* next-to-last-level embeddings generated inside the last level's row pass
                                    instead of being stored */
    double sync_ms;              /* host time blocked in stream synchronisations (the rest of mine_ms is host
                                    work and launch calls) */
} gspan_stats;

typedef struct gspan_ctx gspan_ctx;
typedef struct gspan_graph gspan_graph;

/* Receives one frequent pattern: `code[0..len)` and its MNI support.  Return 0
 * to continue, non-zero to stop mining (gspan_mine then returns ABORTED). */
typedef int (*gspan_emit_fn)(void* user, const gspan_pattern_edge* code, int32_t len, int32_t support);

void gspan_opts_default(gspan_opts* opts);

/* Creates a context on opts->device (NULL: defaults).  Fails with NO_DEVICE
 * when no GPU is visible: there is no CPU fallback. */
gspan_status gspan_ctx_create(const gspan_opts* opts, gspan_ctx** out);
void gspan_ctx_destroy(gspan_ctx* ctx);

/* Copies a host CSR graph in the reference's layout (graph.h:51-65: offsets[n+1],
 * vlabels[n], edges[m], every undirected edge stored in both directions) into
 * the device store.  The host arrays are not retained. */
gspan_status gspan_graph_upload(gspan_ctx* ctx, int32_t nr_nodes, int32_t nr_edges,
                                const int32_t* offsets, const int32_t* vlabels,
                                const gspan_edge* edges, gspan_graph** out);

/* Device-side loader: builds the same device store from the bytes of a gSpan
 * text file (the format convert.cc / graph.cc:38-64 read: 't # id', 'v id
 * label', 'e from to label' records; other tokens skipped; the first integer
 * that fails to parse ends the reading), parsed and turned into a CSR on the
 * GPU.  Equivalent to reading the file with Graph::from_txt, building its
 * CSRGraph and calling gspan_graph_upload.  Refuses (GSPAN_ERR_INVALID) the
 * inputs a token-level parser cannot read like the reference's scanf-based
 * reader: an integer directly followed by other characters, an integer
 * outside int32, a token of 64 characters or more.  Vertex ids must span at
 * most 2^28 values.  nr_nodes / nr_edges (may be null) receive the CSR's
 * vertex and directed-entry counts. */
gspan_status gspan_graph_upload_text(gspan_ctx* ctx, const char* text, int64_t len, gspan_graph** out,
                                     int32_t* nr_nodes, int32_t* nr_edges);
gspan_status gspan_graph_free(gspan_ctx* ctx, gspan_graph* graph);

/* Mines every frequent pattern with at most `k` edges whose MNI support is
 * >= min_support, and emits them in the reference's pre-order.  k < 1 returns
 * INVALID (the reference aborts on it); k > gspan_max_pattern_edges() returns
 * LIMIT.  `stats` may be NULL. */
gspan_status gspan_mine(gspan_ctx* ctx, const gspan_graph* graph, int32_t k, int32_t min_support,
                        gspan_emit_fn emit, void* user, gspan_stats* stats);

/* ---- Batches: many independent mining instances in one device store ----
 * No counterpart in the reference, which mines one graph per process.  Each
 * instance is a separate CSR graph (vertex ids local to it); its results are
 * exactly those of gspan_mine on that graph alone with its own min_support,
 * while every extension level of all instances runs in the same kernel
 * launches.  Vertex labels are ranked per instance, so all instances together
 * may hold at most 65535 distinct (instance, label) pairs. */
typedef int (*gspan_batch_emit_fn)(void* user, int32_t instance, const gspan_pattern_edge* code, int32_t len,
                                   int32_t support);

/* Uploads `ninst` graphs (arrays per instance, layout as gspan_graph_upload).
 * An edge whose ends are outside its own instance returns INVALID. */
gspan_status gspan_batch_upload(gspan_ctx* ctx, int32_t ninst, const int32_t* nr_nodes, const int32_t* nr_edges,
                                const int32_t* const* offsets, const int32_t* const* vlabels,
                                const gspan_edge* const* edges, gspan_graph** out);

/* Mines every instance of a batch with min_support[instance]; emits instance
 * by instance (ascending), each in the reference's pre-order.  gspan_mine on
 * a batch of more than one instance returns INVALID. */
gspan_status gspan_mine_batch(gspan_ctx* ctx, const gspan_graph* batch, int32_t k, const int32_t* min_support,
                              gspan_batch_emit_fn emit, void* user, gspan_stats* stats);

/* Number of instances in an uploaded graph (1 for gspan_graph_upload). */
int32_t gspan_graph_instances(const gspan_graph* graph);

/* Result collector: an emit target that appends every pattern to one flat
 * int32 buffer, per pattern [instance, length, support, then length x (from,
 * to, from_label, edge_label, to_label)], for callers that take all results
 * at once instead of one callback per pattern.  Pass gspan_results_emit (or
 * gspan_results_batch_emit) as the emit function and the collector as
 * `user`.  Not thread-safe: one collector per concurrent mining call. */
typedef struct gspan_results gspan_results;
gspan_results* gspan_results_create(void);
void gspan_results_destroy(gspan_results* results);
void gspan_results_clear(gspan_results* results);
int gspan_results_emit(void* results, const gspan_pattern_edge* code, int32_t len, int32_t support);
int gspan_results_batch_emit(void* results, int32_t instance, const gspan_pattern_edge* code, int32_t len,
                             int32_t support);
int64_t gspan_results_patterns(const gspan_results* results);
/* The buffer (valid until the next emit, clear or destroy) and its length in words. */
const int32_t* gspan_results_data(const gspan_results* results, int64_t* nwords);

/* Autotuner: mines (graph, k, min_support) under each of `ncand` option sets
 * (device and profile are taken from the context), one untimed run then
 * `repeats` timed runs each, and checks that every set returns the same
 * patterns and supports (GSPAN_ERR_DEVICE if not).  The fastest set goes to
 * *best and each set's median wall time to ms[] (may be null).
 * candidates == NULL uses the first min(ncand, 6) sets of a built-in grid
 * over path, mask_bias and domain_mode.  min_support holds one threshold per instance
 * (gspan_graph_instances).  No counterpart in the reference. */
gspan_status gspan_autotune(gspan_ctx* ctx, const gspan_graph* graph, int32_t k, const int32_t* min_support,
                            const gspan_opts* candidates, int32_t ncand, int32_t repeats, gspan_opts* best,
                            double* ms);

/* ---- Serving: requests accepted as they arrive, overlapping on the GPU ----
 * No counterpart in the reference (one graph per process run).  Graphs are
 * uploaded once and stay resident.  `slots` worker threads, each with its
 * own context and stream, run admitted jobs concurrently; a job is exactly a
 * gspan_mine call, so its result is the same alone or in a mix.  Admission is
 * first come, first served: the oldest waiting job starts when a slot is free
 * and its predicted working bytes fit `budget_bytes` (0: 60 % of the free
 * device memory) beside the running jobs; a job that runs out of device
 * memory beside others is re-run alone.  add_graph, submit and wait may be
 * called from any host threads (each job id is waited once); destroy only
 * when no other call on the server is in progress. */
typedef struct gspan_server gspan_server;

typedef struct gspan_job_info {
    gspan_status status;
    double queued_ms;            /* submit -> start */
    double run_ms;               /* start -> done */
    double latency_ms;           /* submit -> done */
    double predicted_bytes;      /* admission estimate */
    int32_t retried_alone;       /* 1: ran out of memory beside others and was re-run alone */
    gspan_stats stats;
} gspan_job_info;

gspan_status gspan_server_create(int32_t device, int32_t slots, double budget_bytes, gspan_server** out);
/* Lets the running jobs finish, drops the queued ones, then frees the
 * graphs, contexts and server. */
void gspan_server_destroy(gspan_server* server);
gspan_status gspan_server_add_graph(gspan_server* server, int32_t nr_nodes, int32_t nr_edges, const int32_t* offsets,
                                    const int32_t* vlabels, const gspan_edge* edges, int32_t* graph_id);
/* Queues a job; returns at once with its id. */
gspan_status gspan_server_submit(gspan_server* server, int32_t graph_id, int32_t k, int32_t min_support,
                                 int64_t* job_id);
/* Blocks until the job is done, emits its patterns (pre-order) and fills
 * `info` (may be NULL); returns the job's status.  Each id is waited once. */
gspan_status gspan_server_wait(gspan_server* server, int64_t job_id, gspan_emit_fn emit, void* user,
                               gspan_job_info* info);

/* MNI support of an embedding table in device memory (the reference's
 * support_gpu, gspan.cu:200-289, for a column table): `cols` is a host array
 * of `ncols` (1..16) device pointers, each to `nrows` int32 vertex ids in
 * [0, nr_nodes), one column per pattern vertex.  Writes to the device array
 * `out[ncols + 1]` the distinct-id count of every column and, at out[ncols],
 * the support: the smallest non-zero count (0x7fffffff when nrows == 0).
 * Runs on the context's stream and returns when `out` is ready.  An id
 * outside [0, nr_nodes) returns INVALID. */
gspan_status gspan_table_support(gspan_ctx* ctx, int32_t nr_nodes, const int32_t* const* cols, int32_t ncols,
                                 int64_t nrows, uint32_t* out);

/* Allocation-free gspan_table_support.  No counterpart in the reference: it is
 * for callers that cannot let a library allocate device memory - a process
 * that fixed its device-memory budget at start-up, a latency-critical loop
 * that cannot take the synchronisation cudaMalloc/cudaFree may cause, or an
 * application whose own allocator owns all device memory.  It needs no
 * context and allocates nothing: the domain bitmaps live in an 8 MiB array
 * compiled into the library, which every GPU that loads the library holds
 * until the process exits.
 *   - Same inputs and outputs as gspan_table_support, on the current device,
 *     enqueued on `stream` (a cudaStream_t; NULL = the legacy default stream)
 *     and asynchronous: `out` is ready when the stream reaches this work.
 *   - ncols * ceil(nr_nodes / 32) must be at most 2,097,088 (LIMIT otherwise).
 *   - An id outside [0, nr_nodes) cannot be returned as an error by an
 *     asynchronous call; out[ncols] is then 0xFFFFFFFF.
 *   - The first call on a device looks up the array's device address; make
 *     that first call before any stream capture on that device.
 *   - All calls share the array: calls whose GPU work overlaps race.
 *   - If a CUDA error of earlier work is pending on the calling thread, the
 *     call launches nothing, leaves that error in place and returns CUDA. */
gspan_status gspan_table_support_noalloc(int32_t nr_nodes, const int32_t* const* cols, int32_t ncols,
                                         int64_t nrows, uint32_t* out, void* stream);

/* Host-only: whether `code` is a minimum DFS code by the reference's test
 * (gspan.cu:586-606).  Writes 1 or 0 to *out. */
gspan_status gspan_is_canonical(const gspan_pattern_edge* code, int32_t len, int32_t* out);

const char* gspan_status_string(gspan_status s);
/* Message of the last failure on this context (empty if none). */
const char* gspan_last_error(const gspan_ctx* ctx);

/* Largest supported pattern size in edges (k beyond it returns LIMIT). */
int32_t gspan_max_pattern_edges(void);

#ifdef __cplusplus
}
#endif

#endif /* GSPAN_GB300_H_ */
