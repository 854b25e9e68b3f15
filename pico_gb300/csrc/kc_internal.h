// Internal declarations shared by the translation units of libkcore.so.
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/kcore.h"

namespace kc {

// Records a formatted message for kc_last_error() and returns `code`.
int fail(int code, const char *fmt, ...);

// Named range on profiler timelines (NVTX), open for the lifetime of the
// object; free when no profiler is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
// Free device memory of the current device, including what this process's
// allocator pool holds for reuse (api.cu).
size_t device_free_bytes(size_t *total);
// Non-blocking streams of `device` from a per-process pool (api.cu); a stream
// is handed back idle.
cudaError_t acquire_stream(int device, cudaStream_t *s);
void release_stream(int device, cudaStream_t s);
// Timing events of the current device from a per-process pool (api.cu).
cudaError_t acquire_event(cudaEvent_t *e);
void release_event(cudaEvent_t e);
void clear_error();

#define KC_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return ::kc::fail(KC_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,          \
                              cudaGetErrorString(e_));                                         \
    } while (0)

#define KC_TRY(expr)                 \
    do {                             \
        int rc_ = (expr);            \
        if (rc_ != KC_OK) return rc_; \
    } while (0)

// Device allocation helpers: report KC_ERR_NOMEM with the size on failure.
int dmalloc(void **p, size_t bytes, const char *what);
void dfree(void *p);

template <class T>
int dalloc(T **p, size_t count, const char *what) {
    return dmalloc(reinterpret_cast<void **>(p), count * sizeof(T) + 16, what);
}

// Control block of the persistent bucket peel (one per graph, device memory).
// Slots [i % 3] belong to level index i; see peel.cu.
constexpr int PEEL_MAX_QUEUES = 64;

// One shared work queue: producer and consumer index on separate lines.
struct alignas(128) PeelQueue {
    unsigned long long head;
    unsigned long long pad0[15];
    unsigned long long tail;
    unsigned long long pad1[15];
};

struct PeelCtl {
    unsigned long long pending[3];   // outstanding work credits of level i
    unsigned long long scan_cursor[3];  // next alive-list tile of level i
    unsigned long long out_len[3];   // survivors appended by level i's scan
    unsigned int next_min[3];        // smallest residual degree above level i
    unsigned int nonempty[3];        // some vertex was claimed at level i
    unsigned int err;                // KC_ERR_* raised on the device
    unsigned int err_info;           // where it was raised
    unsigned int level_indices;      // level indices processed
    unsigned int levels;             // non-empty levels
    unsigned int kmax;               // largest level with a claim
    unsigned int pad;
    PeelQueue q[3][PEEL_MAX_QUEUES]; // shared spill queues of level i (slot i % 3)
};

// Per-level trace record (layout of kc_level_trace).
struct PeelTrace {
    unsigned long long t_start_ns;
    unsigned int level, claimed, scan_len, spilled, steals, steal_fail;
    unsigned long long t_work_end_ns;
    unsigned int rounds, max_steal;
    unsigned long long cta_ns[4];  // CTA time summed over CTAs: scan, process, steal, idle
};

struct Tuning {
    int peel_chunk = 0;  // 0: by graph size (1024 entries, 2048 from 2^29 entries up)
    int peel_spill = 16;  // measured best with 32-item steals (R-MAT scale 22 and 25)
    int peel_steal = 32;
    int peel_queues = 1;
    int peel_ctas_per_sm = 0;
    int peel_unroll = 4;  // row entries in flight per lane: 4 or 8
    int peel_threads = 512;  // threads per CTA: 512 (2 per SM) or 256 (4 per SM)
    int peel_balanced = 1;   // 1: rounds spread a bounded number of row entries over the whole CTA
    int peel_round_entries = 16384;
    int peel_scan_unroll = 4;  // alive-list entries per thread per scan tile: 4 or 8
    int peel_aggregate = 0;    // 1: warp-aggregated decrements (measured 5-9% slower: repeats within a warp are rare)
    int trace = 0;
    int64_t hindex_warp_rows = 8192;  // h-index: rows up to this length re-examined by one warp
    int hindex_order = 1;  // h-index: long rows read from a copy ordered by neighbour degree (prefix reads)
    int64_t hindex_order_min = 128;  // h-index: rows above this length get the ordered copy
    int64_t update_incremental_max = 512;  // larger update batches: full recompute (measured crossover ~1000 edges)
    int64_t update_deletion_incremental_max = 500000;  // deletion-only batches (crossover ~600,000 on R-MAT 22)
    int64_t wait_timeout_us = 2000000;       // limit of one inter-CTA wait
    int withhold = 0;  // failure-detection hook: one CTA never signals, so the others' waits run out
};

// Control block of the h-index iteration.
struct HindexCtl {
    unsigned long long list_len[2];  // active list lengths (ping-pong)
    unsigned long long big_len[2];   // high-degree active list lengths
    unsigned long long mid_len[2];   // medium rows, stored from the far end of list[]
    unsigned long long mid_cursor;   // work cursor (medium rows)
    unsigned long long cursor;       // work cursor (short-row items)
    unsigned long long big_cursor;   // work cursor (high-degree items)
    unsigned int go_on;              // another sweep follows
    unsigned int bar_count;          // grid barrier arrivals
    unsigned int bar_gen;            // grid barrier generation
    unsigned int sweeps;
    unsigned int changed;
    unsigned int err;
    unsigned int err_info;
    unsigned long long ord_len;   // rows of 129..8192 entries given an ordered copy
    unsigned long long ord_huge;  // rows above 8192 entries given an ordered copy
    unsigned long long ord_cursor, ord_huge_cursor;  // work cursors of the copy
};

struct Graph {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    uint32_t n = 0;
    uint64_t nnz = 0;
    uint32_t max_deg = 0;
    uint64_t num_vnodes = 0;
    double build_ms = 0.0;

    int64_t *rowptr = nullptr;  // [n+1]
    uint32_t *col = nullptr;    // [nnz]
    uint32_t *core = nullptr;   // [n]  residual degree / estimate -> core numbers
    bool core_valid = false;

    // decomposition work buffers (allocated on first use, kept for reuse)
    uint32_t *bitmap = nullptr;       // [ceil(n/32)]  claimed / active flags
    uint32_t *alive = nullptr;        // [2n]          alive lists (ping-pong by level)
    unsigned long long *gq = nullptr; // spill queues of work items (sentinel = ~0)
    unsigned long long gq_cap = 0;    // capacity of each of the 3 x gq_nq queues
    unsigned gq_nq = 0;
    unsigned long long gq_items = 0;  // queue sizing basis (n + nnz / MIN_CHUNK)
    PeelTrace *trace = nullptr;       // per-level trace (when enabled)
    uint32_t trace_cap = 0, trace_count = 0;
    Tuning tune;
    bool gq_clean = false;            // gq holds only sentinels
    PeelCtl *peel_ctl = nullptr;
    uint32_t *list[2] = {nullptr, nullptr};  // h-index active lists
    uint32_t *big[2] = {nullptr, nullptr};   // h-index high-degree lists
    uint32_t *hx_bitmap = nullptr;           // h-index pending bitmap of odd sweeps (even: bitmap)
    HindexCtl *hctl = nullptr;
    // h-index: rows above 128 entries copied in descending log2-degree buckets of the neighbours
    uint32_t *hx_ord = nullptr;   // [nnz] (same positions as col; short rows unused)
    uint32_t *hx_lid = nullptr;   // [n] index of a long row in hx_pref
    uint32_t *hx_pref = nullptr;  // [32 per long row] entries in buckets >= b
    uint8_t *hx_bk = nullptr;     // [nnz] bucket of each long-row entry (scratch of the copy)
    uint8_t *hx_vb = nullptr;     // [n] floor(log2(degree)) of every vertex
    uint64_t hx_ord_cap = 0, hx_lid_cap = 0, hx_pref_rows = 0;
    uint32_t *red = nullptr;          // small reduction scratch (min/max)
    // dynamic-graph maintenance
    uint32_t *mfront[2] = {nullptr, nullptr};
    uint32_t *mcand = nullptr;
    uint32_t *mvisit = nullptr;
    unsigned long long *mcount = nullptr;
    bool simple_checked = false;
    std::vector<uint32_t> color_count;
    int auto_method = -1;             // method KC_AUTO runs (set by the autotuner; -1: not tuned yet)
    double auto_ms = 0.0;             // its time when it was tuned
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
    double last_ms = 0.0, last_kernel_ms = 0.0;

    ~Graph();
};

// csr_build.cu
int build_csr_from_edges(Graph *g, const uint32_t *d_src, const uint32_t *d_dst, uint64_t m, uint32_t n,
                         uint32_t flags);
int exclusive_scan_u32_i64(const uint32_t *d_in, int64_t *d_out, uint64_t n, cudaStream_t s);
int graph_finish(Graph *g);  // max degree, vnode count
int graph_validate(Graph *g, uint64_t *bad);
int virtual_layout(Graph *g, uint32_t part_size, uint32_t *h_node_pointer, uint32_t *h_edge_list,
                   uint32_t *h_parts, uint64_t *num_parts);

// peel.cu
int peel_run(Graph *g, cudaStream_t s, bool gpp_zero_to_one, kc_stats *st);
// hindex.cu
int hindex_run(Graph *g, cudaStream_t s, kc_stats *st);
int hindex_run_from(Graph *g, const uint32_t *d_list, uint64_t len, cudaStream_t s, kc_stats *st);

// maintain.cu
int graph_update(Graph *g, const uint32_t *ins_src, const uint32_t *ins_dst, uint64_t n_ins, const uint32_t *del_src,
                 const uint32_t *del_dst, uint64_t n_del, kc_update_stats *st);

// mtx_loader.cpp
int parse_mtx(const char *path, int mode, uint32_t *n, uint64_t *m, uint32_t **src, uint32_t **dst);

// gen.cu
int gen_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c, uint64_t seed,
             uint32_t *d_src, uint32_t *d_dst, cudaStream_t s);
int gen_er(uint32_t n, uint64_t m, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, cudaStream_t s);
int gen_planted(uint32_t n, uint32_t k, double p, uint64_t seed, uint32_t *d_src, uint32_t *d_dst,
                uint64_t cap, uint64_t *m, cudaStream_t s);
int gen_rmat_bounded(uint32_t n, uint64_t num_edges, double a, double b, double c, uint64_t seed, uint32_t *d_src,
                     uint32_t *d_dst, cudaStream_t s);
int gen_ba(uint32_t n, uint32_t d, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, cudaStream_t s);
int edges_offset(uint32_t *d_src, uint32_t *d_dst, uint64_t m, uint32_t off, cudaStream_t s);

}  // namespace kc

struct kc_graph : kc::Graph {};

namespace kc {
// An empty graph handle on `device` with its own stream (api.cu).
int graph_new(int device, kc_graph **out);
}  // namespace kc
