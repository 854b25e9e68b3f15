/*
 * kcore.h -- C ABI of the pico_gb300 k-core engine (libkcore.so).
 *
 * GB300-native replacement for the k-core path of chriszhao13/pico.  The
 * reference has no library interface: each method is a CUDA executable whose
 * main() loads a MatrixMarket file, builds a graph on the host, iterates its
 * kernels from a host loop and prints a report.  This header exposes that
 * path as plain C entry points (pointers and sizes only) so any host language
 * can bind it; each declaration names the reference code it replaces.
 *
 * Conventions
 *   - Every call returns an int status: KC_OK (0) or a KC_ERR_* code.  Nothing
 *     here exits the process or traps the GPU; kc_last_error() returns a
 *     message for the calling thread's last failure.
 *   - A kc_graph owns a device-resident CSR (int64 row offsets, uint32 column
 *     ids, both directions of every edge, no self-loops) plus the work buffers
 *     of the decomposition.  One graph is used by one host thread at a time;
 *     different graphs are independent.
 *   - `stream` arguments are cudaStream_t values passed as void*; NULL selects
 *     the graph's own stream.
 *   - Core numbers are uint32, one per vertex in [0, n).
 */
#ifndef PICO_GB300_KCORE_H
#define PICO_GB300_KCORE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KC_ABI_VERSION 1

/* Status codes. */
enum {
    KC_OK = 0,
    KC_ERR_INVALID = 1,     /* bad argument, id out of range, malformed input line */
    KC_ERR_IO = 2,          /* file cannot be opened or read */
    KC_ERR_CUDA = 3,        /* CUDA runtime error (message in kc_last_error) */
    KC_ERR_NOMEM = 4,       /* device or host allocation failed / not admitted */
    KC_ERR_CAPACITY = 5,    /* a bounded device queue or table overflowed */
    KC_ERR_TIMEOUT = 6,     /* a device-side wait exceeded its limit; results invalid */
    KC_ERR_UNSUPPORTED = 7, /* feature not available (e.g. no cooperative launch) */
    KC_ERR_STATE = 8        /* call not valid in the object's current state */
};

/* Decomposition methods: the seven reference drivers plus automatic choice.
 * All produce the exact core numbers; KC_GPP additionally reports core 1 for
 * degree-0 vertices, as peel/gppeel.cu:35-39 does. */
enum {
    KC_HISTO = 0,       /* index2core/HistoCore.cu   h-index iteration        */
    KC_CNT = 1,         /* index2core/CntCore.cu     h-index iteration        */
    KC_NBR = 2,         /* index2core/NbrCore.cu     h-index iteration        */
    KC_PEELONE = 3,     /* peel/peelone.cu           bucket peel              */
    KC_GPP = 4,         /* peel/gppeel.cu            bucket peel (+ deg0 -> 1) */
    KC_PEELONE_DYN = 5, /* peel/src/peelone-dyn.cc   bucket peel              */
    KC_PEEL_DYN = 6,    /* peel/src/peel-dyn.cc      bucket peel              */
    KC_AUTO = 7         /* engine's choice: see kc_graph_autotune             */
};

/* MatrixMarket loader semantics. */
enum {
    /* Graph::ReadGraph + VirtualGraph (index2core/shared/graph.cpp:17-95,
     * virtual_graph.cpp:16-44): skip 2 lines, keep duplicate lines as parallel
     * edges, drop self-loops; n = max id (+1 if id 0 occurs); ids shifted to
     * 0-based when id 0 does not occur. */
    KC_LOAD_COO = 0,
    /* Graph::readFile (peel/src/graph.cpp:58-133): 1-based ids, self-loops
     * dropped, neighbours de-duplicated and sorted, V = max id. */
    KC_LOAD_CSR_DEDUP = 1
};

/* Flags for kc_graph_from_edges*. */
#define KC_EDGES_DEDUP 1u      /* remove parallel edges, sort each row */
#define KC_EDGES_SORT_ROWS 2u  /* sort each row by neighbour id (keeps parallel edges) */

typedef struct kc_graph kc_graph;

typedef struct kc_stats {
    uint32_t method;      /* method actually run */
    /* peel: level indices processed; h-index: Gauss-Seidel sweeps.  The CLI
     * drivers print this as "Number of iterations"; the reference prints its
     * own synchronous schedule's count there (HistoCore.cu:346, CntCore.cu:421,
     * NbrCore.cu:302, peelone.cu:191, gppeel.cu:231), which the engine's
     * schedule does not follow, so the two numbers differ. */
    uint32_t iterations;
    uint32_t levels;      /* peel: distinct non-empty levels (= distinct core values) */
    uint32_t kmax;        /* largest core number ("Max K") */
    uint32_t kmin;        /* reference's "Min K": min(10, smallest core) (util.cpp:6-22) */
    uint32_t reserved;
    uint64_t n;           /* vertices */
    uint64_t nnz;         /* directed CSR entries (2 x undirected edges) */
    double ms;            /* device time of the decomposition (CUDA events) */
    double build_ms;      /* device time of the CSR build that made this graph */
} kc_stats;

/* ---- library ---------------------------------------------------------- */
int kc_abi_version(void);
/* Message describing the calling thread's most recent failure ("" if none). */
const char *kc_last_error(void);
/* Number of CUDA devices visible (0 without a GPU; never fails). */
int kc_device_count(void);

/* ---- graph construction ----------------------------------------------- */
/* Load a MatrixMarket file (mode = KC_LOAD_*) and build it on `device`.
 * Replaces Graph::ReadGraph + VirtualGraph::MakeUGraph + the cudaMemcpy block
 * of each index2core/peel main() (e.g. HistoCore.cu:207-286), and the
 * Graph(std::string) + malloc_graph_gpu_memory of peel/main.cu:65 /
 * peel/src/gpu_memory_allocation.cu:4-12. */
int kc_graph_from_mtx(const char *path, int mode, int device, kc_graph **out);

/* Parse a MatrixMarket file on the host only (no GPU needed).  On success
 * *src / *dst hold *m 0-based endpoints (self-loops already dropped) in file
 * order, and *n the vertex count, with `mode` semantics.  Free with
 * kc_host_free_edges.  Restates the two loaders above for host callers. */
int kc_parse_mtx(const char *path, int mode, uint32_t *n, uint64_t *m, uint32_t **src, uint32_t **dst);
void kc_host_free_edges(uint32_t *src, uint32_t *dst);

/* Build from an undirected edge list in HOST memory: endpoints are 0-based
 * and < n; self-loops are dropped; both directions are stored.  flags:
 * KC_EDGES_DEDUP / KC_EDGES_SORT_ROWS; without either, each row keeps the
 * edge-list order (the order MakeUGraph produces, virtual_graph.cpp:142-163).
 * The device build: degree count, exclusive scan to int64 offsets, scatter,
 * segmented row sort and unique. */
int kc_graph_from_edges(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n,
                        uint32_t flags, int device, kc_graph **out);
/* Same with endpoints already in device memory of `device`. */
int kc_graph_from_edges_device(const uint32_t *d_src, const uint32_t *d_dst, uint64_t m, uint32_t n,
                               uint32_t flags, int device, kc_graph **out);

/* Build from a CSR in HOST memory (rowptr[n+1] int64, col[rowptr[n]]).  The
 * CSR must be symmetric without self-loops (not checked; see
 * kc_graph_validate). */
int kc_graph_from_csr(const int64_t *rowptr, const uint32_t *col, uint32_t n, int device, kc_graph **out);
/* Same from device memory; the graph copies the arrays. */
int kc_graph_from_csr_device(const int64_t *d_rowptr, const uint32_t *d_col, uint32_t n, int device,
                             kc_graph **out);

/* Binary edge list: a file of little-endian uint32 (src, dst) pairs, 0-based
 * ids, n = largest id + 1, read through mmap (no text parsing); flags as for
 * kc_graph_from_edges.  The fast input path for graphs whose MatrixMarket
 * text takes minutes to parse (the reference parses text only,
 * index2core/shared/graph.cpp:17-95, peel/src/graph.cpp:58-133). */
int kc_graph_from_edge_file(const char *path, uint32_t flags, int device, kc_graph **out);

/* Binary snapshot of a graph and, when a decomposition has completed, its core
 * numbers: a 64-byte header (magic "KCSNAP01", version, flags, n, nnz, a 64-bit
 * content hash of the payload) followed by rowptr int64[n+1], col uint32[nnz]
 * (padded to 8 bytes) and core uint32[n].  kc_graph_load rejects a file whose
 * size or content hash does not match its header, and restores the core
 * numbers (kc_graph_device_core works without a new decomposition).  Replaces
 * the reference's text CSR cache (peel/src/graph.cpp:9-54,151), which is keyed
 * by the input's basename only. */
int kc_graph_save(const kc_graph *g, const char *path);
int kc_graph_load(const char *path, int device, kc_graph **out);

/* Check symmetry / self-loops / id range on the device.  *bad = number of
 * offending entries (0 for a valid graph). */
int kc_graph_validate(kc_graph *g, uint64_t *bad);

int kc_graph_free(kc_graph *g);

/* Sizes: n, directed entries, max degree, number of 32-wide virtual nodes. */
int kc_graph_info(const kc_graph *g, uint32_t *n, uint64_t *nnz, uint32_t *max_degree,
                  uint64_t *num_vnodes);
/* Device pointers of the resident CSR (valid until kc_graph_free). */
int kc_graph_device_csr(const kc_graph *g, const int64_t **d_rowptr, const uint32_t **d_col);
/* Copy the CSR to host buffers (rowptr[n+1], col[nnz]). */
int kc_graph_copy_csr(const kc_graph *g, int64_t *rowptr, uint32_t *col);
/* Degrees (host buffer, n entries). */
int kc_graph_degrees(const kc_graph *g, uint32_t *deg);

/* Export the reference's virtual-graph layout built on the device
 * (VirtualGraph::MakeUGraph, virtual_graph.cpp:96-192): nodePointer[n]
 * (uint32 slot of deg(v)), edgeList[nnz+n] (deg(v) then the row), and
 * parts[2*numParts] = {node, part} with ceil(deg/part_size) parts per vertex.
 * Host output buffers; *num_parts receives numParts.  Pass parts == NULL to
 * query *num_parts only.  Offsets must fit uint32 as in the reference. */
int kc_graph_virtual_layout(kc_graph *g, uint32_t part_size, uint32_t *node_pointer,
                            uint32_t *edge_list, uint32_t *parts, uint64_t *num_parts);

/* ---- decomposition ----------------------------------------------------- */
/* Core number of every vertex.  Replaces the timed loops of HistoCore.cu:292-341,
 * CntCore.cu:344-417, NbrCore.cu:244-297, peelone.cu:157-186,
 * gppeel.cu:186-228, int peelone_dyn(Graph&) (peelone-dyn.cc:120-168) and
 * int peel_dyn(Graph&) (peel-dyn.cc:133-182).  core_out: n uint32 in host
 * memory (out_on_device = 0) or device memory of the graph's device
 * (out_on_device = 1); may be NULL to keep the result on the device only
 * (see kc_graph_device_core).  stats may be NULL. */
int kc_decompose(kc_graph *g, int method, uint32_t *core_out, int out_on_device, kc_stats *stats,
                 void *stream);
/* Chooses what KC_AUTO runs on this graph by timing it: the bucket peel
 * with its default tunables, the peel with the other row-chunk size (1024 /
 * 2048 entries), the peel keeping more cascade items per CTA ("peel.spill"
 * 2 x + 16), and the h-index iteration, each warmed up once and timed twice;
 * the fastest (method and peel tunables) is kept in the graph.  *method receives the chosen KC_*
 * method, *best_ms its time (either may be NULL).  The first
 * kc_decompose(KC_AUTO) of a graph calls this itself, so that call takes
 * about eight decompositions longer; later KC_AUTO calls reuse the choice.
 * No counterpart in the reference, which runs one fixed method per binary. */
int kc_graph_autotune(kc_graph *g, int *method, double *best_ms);
/* CUDA-event timings of the last decomposition on this graph: *total_ms
 * covers every kernel of the call (initialisation included), *kernel_ms the
 * main decomposition kernel alone.  Either pointer may be NULL. */
int kc_graph_last_timing(const kc_graph *g, double *total_ms, double *kernel_ms);
/* Tunables of the decomposition kernels, set per graph (the autotuner and
 * the benchmarks use these).  Names: "peel.chunk" (row entries per peel work
 * item; 0, the default, picks 1024, or 2048 for graphs of 2^29 entries or
 * more), "peel.spill" (cascade items a CTA keeps before publishing to the
 * shared queues, default 16), "peel.steal" (most items reserved per steal,
 * 1..64, default 32), "peel.queues" (number
 * of shared queues, 1..64), "peel.ctas_per_sm" (0 = occupancy maximum),
 * "peel.unroll" (row entries each lane keeps in flight, 4 or 8),
 * "peel.threads" (threads per CTA, 512 or 256), "peel.balanced" (1 = each
 * processing round spreads at most "peel.round_entries" row entries evenly
 * over the CTA's threads), "peel.scan_unroll" (alive-list entries per
 * thread per scan tile, 4 or 8), "peel.aggregate" (1 = lanes of a warp that
 * decrement the same vertex issue one atomicSub of their count; exact either
 * way, off by default because it measured slower), "hindex.warp_rows" (h-index: after the
 * first sweep, rows up to this many entries are re-examined by one warp,
 * longer ones by a whole CTA; default 8192), "hindex.order" (1 = each
 * h-index decomposition first copies the rows above "hindex.order_min"
 * entries with the neighbours in descending buckets of floor(log2(degree)),
 * so that its passes read only the prefix of a row that can hold the values
 * they need; default 1; the copy takes 5 bytes per row entry and about 1 byte
 * per entry more for the bucket table), "hindex.order_min" (default 128,
 * at least 128),
 * "trace" (1 = record a per-level trace of the next decompositions),
 * "update.incremental_max" (largest update batch, in edges, maintained
 * incrementally by kc_graph_update; default 512),
 * "update.deletion_incremental_max" (the same for batches of deletions only;
 * default 500,000), "wait.timeout_us" (limit of one
 * inter-CTA wait of the peel and h-index kernels, default 2 s; a wait that
 * runs out makes the call return KC_ERR_TIMEOUT), "test.withhold" (1 = one
 * CTA never signals the others, so their waits run out: exercises the
 * timeout path without faulting the GPU; off by default). */
int kc_graph_set_param(kc_graph *g, const char *name, int64_t value);

/* Per-level trace of the last peel decomposition (recorded when the "trace"
 * parameter is 1): one record per level index.  After an h-index
 * decomposition (KC_HISTO / KC_CNT / KC_NBR) the records are per sweep:
 * level = sweep index, claimed = estimates lowered, scan_len = vertices
 * re-evaluated by one warp each, spilled = vertices re-evaluated by a whole
 * CTA (rows above 512 entries), max_steal = the longest such row,
 * t_work_end_ns = when the last CTA finished the sweep's vertices, cta_ns =
 * CTA time on long rows, on short rows and in the sweep's barriers (the
 * fourth is 0), steals = estimates lowered among the long rows; steal_fail
 * and rounds are 0. */
typedef struct kc_level_trace {
    uint64_t t_start_ns;  /* GPU global timer when the level began (CTA 0) */
    uint32_t level;       /* level value L */
    uint32_t claimed;     /* vertices peeled at this level */
    uint32_t scan_len;    /* alive-list length scanned */
    uint32_t spilled;     /* items published on the shared queues */
    uint32_t steals;      /* successful steals */
    uint32_t steal_fail;  /* failed steal attempts */
    uint64_t t_work_end_ns; /* GPU global timer when the last CTA handed back its work credit */
    uint32_t rounds;      /* most processing rounds of one CTA */
    uint32_t max_steal;   /* largest single steal (items) */
    uint64_t cta_ns[4];   /* CTA time summed over CTAs: scanning, processing rows, stealing, idle */
} kc_level_trace;
int kc_graph_trace(const kc_graph *g, kc_level_trace *out, uint32_t cap, uint32_t *count);

/* Device pointer of the last decomposition's core array (n uint32). */
int kc_graph_device_core(const kc_graph *g, const uint32_t **d_core);

/* The induced k-core of the last decomposition as a graph of its own: the
 * vertices with core >= k, renumbered in increasing id order, and the edges
 * among them (rows keep their order).  map_out (optional; host memory, or
 * device memory when map_on_device is 1) receives the original id of each new
 * vertex and needs room for every vertex with core >= k.  The reference prints
 * only the largest and smallest core (util.cpp:6-22); this extends its result
 * writers (utility::SaveResults, util.cpp:70-89). */
int kc_graph_kcore_subgraph(const kc_graph *g, uint32_t k, kc_graph **out, uint32_t *map_out, int map_on_device);

/* ---- dynamic graphs: exact core maintenance under edge batches ---------- */
/* No counterpart in the reference (its "dyn" drivers use dynamic work
 * queues, not edge updates).  Applies a batch to a graph built with
 * KC_EDGES_DEDUP (sorted rows, no parallel edges) and keeps the core numbers
 * exact: deletions first, then insertions; deleting an absent edge or
 * inserting a present one is ignored; self-loops are ignored.  Batches of at
 * most "update.incremental_max" edges (kc_graph_set_param), and batches of
 * deletions only up to "update.deletion_incremental_max" edges, are maintained
 * incrementally (h-index iteration from the old cores for deletions;
 * matching rounds with subcore candidate sets for insertions); larger ones
 * are applied in one rewrite followed by a full decomposition.  Edge lists in
 * host memory; core_out as in kc_decompose (may be NULL). */
typedef struct kc_update_stats {
    uint64_t inserted;    /* undirected edges added */
    uint64_t deleted;     /* undirected edges removed */
    uint32_t rounds;      /* insertion matchings processed */
    uint32_t sweeps;      /* h-index sweeps, summed */
    uint64_t candidates;  /* vertices re-examined after insertions */
    uint32_t recomputed;  /* 1 = applied through a full decomposition */
    uint32_t reserved;
    double ms;            /* wall time of the call */
} kc_update_stats;
int kc_graph_update(kc_graph *g, const uint32_t *ins_src, const uint32_t *ins_dst, uint64_t n_ins,
                    const uint32_t *del_src, const uint32_t *del_dst, uint64_t n_del, uint32_t *core_out,
                    int out_on_device, kc_update_stats *stats);

/* ---- batched decomposition -------------------------------------------- */
/* Many independent graphs decomposed together.  The graphs are packed into
 * one kc_graph (a segmented CSR): graph i owns vertices [vbase[i],
 * vbase[i+1]) and its rows reference only its own vertices (checked at
 * creation).  The reference decomposes one graph per program run; the plain
 * equivalent here is one kc_decompose per graph (see kc_graph_from_segment).
 * A kc_batch holds the plan (size classes, work lists, tuning, captured CUDA
 * graph) and uses the kc_graph's core array for its results. */
typedef struct kc_batch kc_batch;
int kc_batch_create(kc_graph *g, const uint32_t *vbase, uint32_t num_graphs, kc_batch **out);
/* Parameters: "batch.small_n" (largest graph, in vertices, of the small-CTA
 * class), "batch.small_threads", "batch.large_threads", "batch.chunk" (row
 * entries per work item), "batch.large_shared" (1 = graphs above small_n
 * keep degrees in shared memory, one CTA per SM; 0 = in global memory, as many
 * CTAs per SM as fit), "batch.cuda_graph" (1 = capture once, replay),
 * "trace" (1 = record per-graph timings, see kc_batch_trace). */
int kc_batch_set_param(kc_batch *b, const char *name, int64_t value);
int kc_batch_get_param(const kc_batch *b, const char *name, int64_t *value);
/* Times a grid of configurations on this batch and keeps the fastest;
 * *best_ms receives its time. */
int kc_batch_autotune(kc_batch *b, double *best_ms);
/* Core numbers of every packed vertex (n uint32, host or device buffer; NULL
 * keeps them in the graph's core array).  stats->ms = device time. */
int kc_batch_decompose(kc_batch *b, uint32_t *core_out, int out_on_device, kc_stats *stats, void *stream);
/* With parameter "trace" = 1, each decomposition records per graph i the GPU
 * timer at its start and end and the SM that ran it: out[3i], out[3i+1],
 * out[3i+2] (cap = number of uint64 slots of out). */
int kc_batch_trace(const kc_batch *b, uint64_t *out, uint32_t cap);
int kc_batch_free(kc_batch *b);
/* A standalone graph made of vertices [lo, hi) of g, ids rebased to 0; the
 * rows of those vertices must reference only [lo, hi). */
int kc_graph_from_segment(const kc_graph *g, uint32_t lo, uint32_t hi, kc_graph **out);

/* ---- serving: continuous batching of requests on one GPU --------------- */
/* No counterpart in the reference.  A server keeps `resident` on the device
 * and runs two request kinds concurrently on separate CUDA streams:
 * updates (edge batches on the resident graph, exact core maintenance, in
 * submission order) and decompositions (a graph sent with the request).
 * Waiting decompositions are admitted as lanes free up and device memory
 * allows (cudaMemGetInfo minus hbm_reserve_bytes minus what admitted requests
 * may still allocate); a lane packs all admissible waiting requests (up to
 * max_batch_graphs / max_batch_bytes) into one batched launch.  Inputs are
 * copied at submission.  Latency = submission to result on the host. */
typedef struct kc_server kc_server;
typedef struct kc_server_config {
    uint32_t decompose_slots;   /* concurrent decomposition lanes (default 2) */
    uint32_t max_batch_graphs;  /* requests packed per launch (default 64) */
    uint64_t max_batch_bytes;   /* estimated device bytes per launch (default 256 MiB) */
    uint64_t hbm_reserve_bytes; /* device memory left free (0 = none) */
} kc_server_config;
typedef struct kc_request_result {
    int32_t status;             /* KC_OK or the request's error */
    uint32_t kind;              /* 0 update, 1 decompose */
    uint32_t n;                 /* vertices of the result */
    uint32_t kmax;              /* largest core number */
    uint64_t digest;            /* sum of core[v] * splitmix64(v + 1) mod 2^64 */
    double latency_ms;          /* submission -> result on host */
    double queue_ms;            /* submission -> start of work */
    kc_update_stats update;     /* update requests */
    uint32_t has_core;          /* a core array is available for kc_server_wait */
    uint32_t reserved;
} kc_request_result;
typedef struct kc_server_stats {
    uint64_t completed_updates, completed_decompositions, failed;
    double p50_update_ms, p99_update_ms, p50_decompose_ms, p99_decompose_ms;
    double elapsed_ms;          /* first submission -> last completion */
    uint64_t edges_decomposed;  /* undirected edges of completed decompositions */
    uint64_t edges_updated;     /* edges in completed update batches */
    uint64_t decompose_launches;
    uint32_t max_inflight;      /* most requests groups running at once */
    uint32_t reserved;
} kc_server_stats;
/* cfg may be NULL for defaults.  Decomposes `resident` first if needed. */
int kc_server_create(kc_graph *resident, const kc_server_config *cfg, kc_server **out);
/* want_core: keep a copy of the full resident core array for kc_server_wait. */
int kc_server_submit_update(kc_server *s, const uint32_t *ins_src, const uint32_t *ins_dst, uint64_t n_ins,
                            const uint32_t *del_src, const uint32_t *del_dst, uint64_t n_del, int want_core,
                            uint64_t *ticket);
/* A symmetric CSR without self-loops (host memory). */
int kc_server_submit_decompose(kc_server *s, const int64_t *rowptr, const uint32_t *col, uint32_t n,
                               uint64_t *ticket);
/* Blocks until the request is done; fills res, and core_out (capacity
 * core_cap entries) when a core array is available.  Returns the request's
 * status.  Each ticket can be waited for once. */
int kc_server_wait(kc_server *s, uint64_t ticket, kc_request_result *res, uint32_t *core_out, uint64_t core_cap);
int kc_server_get_stats(kc_server *s, kc_server_stats *st);
/* Finishes every submitted request, then stops the lanes. */
int kc_server_free(kc_server *s);

/* ---- allocation-free decomposition -------------------------------------- */
/* No counterpart in the reference.  Core numbers of one small graph for
 * callers that cannot allocate device memory on this path (a framework that
 * owns all device memory through its own pool, a latency-critical loop where
 * cudaMalloc/cudaFree would synchronize the device).  Inputs and output are
 * device pointers on the current device: rowptr[n+1] (int64), col[rowptr[n]]
 * (symmetric, no self-loops), core[n].  Limits: n <= 50,000 vertices and
 * rowptr[n] <= 4,194,304 entries; larger graphs get KC_ERR_CAPACITY.  The
 * only scratch is a fixed array of about 663 KB inside the library that every
 * GPU loading it holds until exit; it is looked up on the first call on each
 * device.  All calls share it: calls that overlap on the GPU race and must be
 * serialised by the caller.  Nothing is allocated.  Blocks until the result
 * is in core (it reads a status word back and synchronises the stream), so a
 * call can never be captured into a CUDA graph. */
int kc_decompose_noalloc(const int64_t *d_rowptr, const uint32_t *d_col, uint32_t n, uint32_t *d_core,
                         void *stream);

/* ---- memory helpers ----------------------------------------------------
 * The reference allocates and copies inside each driver
 * (peel/src/gpu_memory_allocation.cu:4-21, HistoCore.cu:259-286); callers of
 * this library use these to stage inputs and outputs. */
/* Pinned host memory (fast host<->device copies). */
int kc_host_alloc(void **p, size_t bytes);
int kc_host_free(void *p);
/* Device memory on `device` (stream-ordered pool).  Free a buffer only after
 * the work that uses it has completed. */
int kc_device_alloc(void **p, size_t bytes, int device);
int kc_device_free(void *p);
/* Blocking copy; kind: 1 = host->device, 2 = device->host, 3 = device->device. */
int kc_memcpy(void *dst, const void *src, size_t bytes, int kind);
/* Wait for all work on `device` to finish. */
int kc_device_synchronize(int device);

/* ---- seeded graph generators (device) ---------------------------------- */
/* Generators write an undirected edge list (src, dst; 0-based) to DEVICE
 * buffers of capacity `cap` edges and report the count in *m.  Counter-based
 * hashing (splitmix64 finaliser) makes the output independent of the launch
 * shape, so a host restatement reproduces it bit for bit. */
/* R-MAT: 2^scale ids, edge_factor*2^scale draws, quadrant probabilities a,b,c
 * (d = 1-a-b-c).  Self-loops and duplicates are kept (the builder drops them). */
int kc_gen_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c, uint64_t seed,
                uint32_t *d_src, uint32_t *d_dst, void *stream);
/* Erdos-Renyi G(n, m): m distinct unordered pairs {u<v}, sampled without
 * replacement through a keyed Feistel permutation of the pair index space. */
int kc_gen_er(uint32_t n, uint64_t m, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, void *stream);
/* Planted dense subgraph: `k` distinct members of [0, n) chosen by a keyed
 * permutation; each member pair is an edge with probability p.  Writes at
 * most cap edges; *m receives the count (KC_ERR_CAPACITY if cap is short). */
int kc_gen_planted(uint32_t n, uint32_t k, double p, uint64_t seed, uint32_t *d_src, uint32_t *d_dst,
                   uint64_t cap, uint64_t *m, void *stream);

/* R-MAT over [0, n) for any n >= 2: 2^ceil(log2 n) ids, draws with an
 * endpoint >= n are rejected and written as the self-loop (0, 0). */
int kc_gen_rmat_bounded(uint32_t n, uint64_t num_edges, double a, double b, double c, uint64_t seed,
                        uint32_t *d_src, uint32_t *d_dst, void *stream);
/* Barabasi-Albert preferential attachment: n vertices, d edges per vertex
 * (n*d edges; vertex v creates edges v*d .. v*d+d-1 towards endpoints of
 * earlier edges), in the copy-model formulation of Batagelj and Brandes. */
int kc_gen_ba(uint32_t n, uint32_t d, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, void *stream);
/* Add `offset` to every endpoint of a device edge list (packing graphs into
 * one id space). */
int kc_edges_offset(uint32_t *d_src, uint32_t *d_dst, uint64_t m, uint32_t offset, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PICO_GB300_KCORE_H */
