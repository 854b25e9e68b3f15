// Batched k-core decomposition of many independent graphs in one pass.
//
// The reference decomposes one graph per process (each driver's main()); a
// batch of graphs there is a loop of whole program runs.  Here a batch is a
// segmented CSR -- graph i owns vertices [vbase[i], vbase[i+1]) of one packed
// CSR and its rows reference only its own vertices -- decomposed by
// persistent kernels in which each CTA takes whole graphs from a work list
// (largest first) and peels them entirely on the SM:
//   * residual degrees and the claim bitmap of the graph live in shared memory
//     (uint16 degrees when the graph's maximum degree allows, else uint32);
//     graphs too large for shared memory use the same code on global memory;
//   * a level starts with one scan that claims every unclaimed vertex with
//     residual degree <= L (its core number is L) and queues its row in
//     chunk-sized items; warps then expand the queued rows (long items by the
//     whole warp, short ones concatenated through a shuffle-based owner
//     search) and decrement unclaimed neighbours with shared-memory atomics;
//     the decrement that takes a neighbour from L+1 to L claims it and queues
//     its row behind the current round, so cascades need no rescan; the
//     smallest residual degree left above L is the next level (empty levels
//     are skipped);
//   * CTA barriers (__syncthreads) replace the reference's host round trips.
// Graphs are split into size classes, each with its own kernel
// configuration, launched on forked streams; the sequence can be captured
// once as a CUDA graph and replayed.  kc_batch_autotune times a few
// configurations on the batch itself and keeps the fastest.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

constexpr unsigned BATCH_MIN_CHUNK = 128;
constexpr unsigned NO_LVL = 0xffffffffu;
constexpr int BATCH_U = 4;

struct BatchArgs {
    const int64_t *rowptr;
    const uint32_t *col;
    uint32_t *core;
    const uint32_t *vbase;
    const uint32_t *order;  // graph indices of this class, largest first
    uint32_t count;
    unsigned long long *F;            // row-chunk queue scratch (packed-graph sized)
    const unsigned long long *fbase;  // per-graph offset into F
    unsigned int *next;               // work counter of this class
    uint32_t *gdeg;                   // global-memory residual degrees (packed ids)
    uint8_t *gclaimed;                // global-memory claim flags (packed ids)
    uint32_t chunk;
    uint32_t smem_n;                  // vertex capacity of the shared-memory arrays
    unsigned long long *gtrace;       // per graph: start ns, end ns, SM id (or nullptr)
    uint32_t *alist;                  // two alive lists per graph (packed ids + packed n), or nullptr
    uint32_t alist_stride;            // packed vertex count: offset of the second list
};

// SMEM: degrees + claim bitmap in shared memory; otherwise global memory.
template <typename DegT, bool SMEM>
__device__ __forceinline__ bool is_claimed(const uint32_t *bits, const uint8_t *flags, uint32_t v) {
    return SMEM ? ((bits[v >> 5] >> (v & 31)) & 1u) != 0u : flags[v] != 0;
}

// Decrements unclaimed neighbour u.  Sets `claim` when this decrement moved u
// from L+1 to L (u is claimed here, at core L), and tracks the smallest
// residual degree left above L.
template <typename DegT, bool SMEM>
__device__ __forceinline__ void relax(DegT *deg, uint32_t *bits, uint8_t *flags, uint32_t u, unsigned L,
                                      unsigned &my_min, bool &claim) {
    claim = false;
    if (is_claimed<DegT, SMEM>(bits, flags, u)) return;
    unsigned old;
    if (sizeof(DegT) == 2) {
        const unsigned sh = (u & 1) * 16;
        old = (atomicSub(reinterpret_cast<unsigned int *>(deg) + (u >> 1), 1u << sh) >> sh) & 0xffffu;
    } else {
        old = atomicSub(reinterpret_cast<unsigned int *>(deg) + u, 1u);
    }
    if (old == L + 1) {
        claim = true;
        if (SMEM) atomicOr(&bits[u >> 5], 1u << (u & 31));
        else flags[u] = 1;
    } else if (old > L + 1) {
        my_min = min(my_min, old - 1);
    }
}

template <typename DegT, bool SMEM>
__global__ void batch_peel(BatchArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned int gi_sh, fcount, fhead, minnext, end_sh;
    __shared__ unsigned int list_len, kept_sh, use_list, cur_list, compact_sh;
    const unsigned tid = threadIdx.x, lane = tid & 31, nthreads = blockDim.x;
    for (;;) {
        if (tid == 0) gi_sh = atomicAdd(A.next, 1u);
        __syncthreads();
        const unsigned idx = gi_sh;
        __syncthreads();
        if (idx >= A.count) return;
        const uint32_t gi = A.order[idx];
        if (A.gtrace && tid == 0) {
            unsigned smid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            A.gtrace[3ull * gi] = global_ns();
            A.gtrace[3ull * gi + 2] = smid;
        }
        const uint32_t v0 = A.vbase[gi];
        const uint32_t n = A.vbase[gi + 1] - v0;
        const int64_t *rp = A.rowptr + v0;
        const uint32_t *colv = A.col;
        unsigned long long *F = A.F + A.fbase[gi];
        DegT *deg;
        uint32_t *bits = nullptr;
        uint8_t *flags = nullptr;
        if (SMEM) {
            deg = reinterpret_cast<DegT *>(smem);
            bits = reinterpret_cast<uint32_t *>(smem + ((A.smem_n * sizeof(DegT) + 15) & ~15u));
        } else {
            deg = reinterpret_cast<DegT *>(A.gdeg + v0);
            flags = A.gclaimed + v0;
        }
        for (uint32_t v = tid; v < n; v += nthreads) deg[v] = (DegT)(rp[v + 1] - rp[v]);
        if (SMEM) {
            for (uint32_t w = tid; w < (n + 31) / 32; w += nthreads) bits[w] = 0u;
        } else {
            for (uint32_t v = tid; v < n; v += nthreads) flags[v] = 0;
        }
        unsigned L = 0;
        if (tid == 0) {
            list_len = n;  // the first levels scan 0..n-1 directly
            use_list = 0;
            cur_list = 0;
            kept_sh = n;
        }
        __syncthreads();
        // Queues the row of claimed vertex v as chunk-sized items (warp-wide
        // call).  An item holds its row range itself -- start << 24 | length --
        // so expanding it needs no second read of the row offsets.
        auto enqueue = [&](bool take, uint32_t v) {
            uint32_t k = 0;
            int64_t r0 = 0, r1 = 0;
            if (take) {
                r0 = rp[v];
                r1 = rp[v + 1];
                k = (uint32_t)((r1 - r0 + A.chunk - 1) / A.chunk);
            }
            unsigned tot;
            const unsigned ex = warp_excl_scan(k, lane, tot);
            unsigned base = 0;
            if (lane == 0 && tot) base = atomicAdd(&fcount, tot);
            base = __shfl_sync(KC_FULL_MASK, base, 0);
            for (uint32_t j = 0; j < k; j++) {
                const int64_t s0 = r0 + (int64_t)j * A.chunk;
                const int64_t l = min((int64_t)A.chunk, r1 - s0);
                F[base + ex + j] = ((unsigned long long)s0 << 24) | (unsigned long long)l;
            }
        };
        for (;;) {  // levels
            if (tid == 0) {
                fcount = 0;
                minnext = NO_LVL;
                // rewrite the alive list once fewer than half of its entries
                // survived the last scan
                compact_sh = (A.alist != nullptr && kept_sh < list_len / 2) ? 1u : 0u;
                kept_sh = 0;
            }
            __syncthreads();
            unsigned my_min = NO_LVL;
            const unsigned len = list_len, compact = compact_sh;
            const uint32_t *lin = use_list ? A.alist + (size_t)cur_list * A.alist_stride + v0 : nullptr;
            uint32_t *lout = A.alist ? A.alist + (size_t)(cur_list ^ 1u) * A.alist_stride + v0 : nullptr;
            // ---- one scan per level over the alive list: claim every vertex
            // at or below L, count (or, when compacting, rewrite) the rest ----
            for (uint32_t b = 0; b < len; b += nthreads) {
                const uint32_t i = b + tid;
                const uint32_t v = i < len ? (lin ? lin[i] : i) : 0xffffffffu;
                bool take = false, keep = false;
                if (v != 0xffffffffu && !is_claimed<DegT, SMEM>(bits, flags, v)) {
                    const unsigned d = deg[v];
                    if (d <= L) {
                        take = true;
                        A.core[v0 + v] = L;
                        if (SMEM) atomicOr(&bits[v >> 5], 1u << (v & 31));
                        else flags[v] = 1;
                    } else {
                        keep = true;
                        my_min = min(my_min, d);
                    }
                }
                const unsigned km = __ballot_sync(KC_FULL_MASK, keep);
                unsigned kb = 0;
                if (lane == 0 && km) kb = atomicAdd(&kept_sh, (unsigned)__popc(km));
                if (compact) {
                    kb = __shfl_sync(KC_FULL_MASK, kb, 0);
                    if (keep) lout[kb + __popc(km & ((1u << lane) - 1u))] = v;
                }
                enqueue(take, v);
            }
            __syncthreads();
            if (tid == 0 && compact) {
                list_len = kept_sh;
                use_list = 1;
                cur_list ^= 1u;
            }
            // ---- expansion rounds: cascades land behind the current round ----
            unsigned start = 0;
            for (;;) {
                if (tid == 0) {
                    end_sh = fcount;
                    fhead = start;
                }
                __syncthreads();
                const unsigned end = end_sh;
                if (start >= end) break;
                for (;;) {
                    unsigned i0 = 0;
                    if (lane == 0) i0 = atomicAdd(&fhead, 32u);
                    i0 = __shfl_sync(KC_FULL_MASK, i0, 0);
                    if (i0 >= end) break;
                    const unsigned nit = min(32u, end - i0);
                    int64_t rs = 0;
                    uint32_t len = 0;
                    if (lane < nit) {
                        const unsigned long long it = F[i0 + lane];
                        rs = (int64_t)(it >> 24);
                        len = (uint32_t)(it & 0xffffffull);
                    }
                    // long items: the whole warp walks one row range, no search
                    unsigned bigm = __ballot_sync(KC_FULL_MASK, len >= 64);
                    while (bigm) {
                        const int j = __ffs(bigm) - 1;
                        bigm &= bigm - 1;
                        const int64_t rj = __shfl_sync(KC_FULL_MASK, rs, j);
                        const unsigned lj = __shfl_sync(KC_FULL_MASK, len, j);
                        for (unsigned e0 = 0; e0 < lj; e0 += 32 * BATCH_U) {
                            uint32_t u[BATCH_U];
#pragma unroll
                            for (int kk = 0; kk < BATCH_U; kk++) {
                                const unsigned e = e0 + kk * 32 + lane;
                                u[kk] = e < lj ? colv[rj + e] - v0 : 0xffffffffu;
                            }
#pragma unroll
                            for (int kk = 0; kk < BATCH_U; kk++) {
                                bool cl = false;
                                if (u[kk] != 0xffffffffu) relax<DegT, SMEM>(deg, bits, flags, u[kk], L, my_min, cl);
                                if (cl) A.core[v0 + u[kk]] = L;
                                enqueue(cl, u[kk]);
                            }
                        }
                    }
                    if (len >= 64) len = 0;
                    // short items: concatenated, each lane finds its owner item
                    unsigned total;
                    const unsigned off = warp_excl_scan(len, lane, total);
                    for (unsigned base = 0; base < total; base += 32) {
                        const unsigned e = base + lane;
                        unsigned j = 0;
#pragma unroll
                        for (unsigned step = 16; step > 0; step >>= 1) {
                            const unsigned cand = j + step;
                            const unsigned oc = __shfl_sync(KC_FULL_MASK, off, cand & 31);
                            if (cand < 32 && oc <= e) j = cand;
                        }
                        const int64_t rj = __shfl_sync(KC_FULL_MASK, rs, j);
                        const unsigned oj = __shfl_sync(KC_FULL_MASK, off, j);
                        bool cl = false;
                        uint32_t u = 0;
                        if (e < total) {
                            u = colv[rj + (e - oj)] - v0;
                            relax<DegT, SMEM>(deg, bits, flags, u, L, my_min, cl);
                            if (cl) A.core[v0 + u] = L;
                        }
                        enqueue(cl, u);
                    }
                }
                __syncthreads();
                start = end;
            }
            my_min = __reduce_min_sync(KC_FULL_MASK, my_min);
            if (lane == 0 && my_min != NO_LVL) atomicMin(&minnext, my_min);
            __syncthreads();
            const unsigned nx = minnext;
            __syncthreads();
            if (nx == NO_LVL) break;  // every vertex claimed
            L = nx;
        }
        if (A.gtrace && tid == 0) A.gtrace[3ull * gi + 1] = global_ns();
        __syncthreads();
    }
}

// Per-graph sizes: vertices, entries, largest degree (one warp per graph).
__global__ void batch_sizes(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ vbase, uint32_t G,
                            uint32_t *maxdeg, unsigned long long *fbase) {
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = warp; i < G; i += nw) {
        const uint32_t lo = vbase[i], hi = vbase[i + 1];
        uint32_t mx = 0;
        for (uint32_t v = lo + lane; v < hi; v += 32) mx = max(mx, (uint32_t)(rowptr[v + 1] - rowptr[v]));
        mx = __reduce_max_sync(KC_FULL_MASK, mx);
        if (lane == 0) {
            maxdeg[i] = mx;
            // graph i's chunk queue holds at most n_i + nnz_i / BATCH_MIN_CHUNK items
            fbase[i] = (unsigned long long)lo + (unsigned long long)rowptr[lo] / BATCH_MIN_CHUNK + i;
        }
    }
}

// Rows of graph i may only reference vertices of graph i.
__global__ void batch_check(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col,
                            const uint32_t *__restrict__ vbase, uint32_t G, unsigned long long *bad) {
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long b = 0;
    for (uint64_t i = warp; i < G; i += nw) {
        const uint32_t lo = vbase[i], hi = vbase[i + 1];
        for (int64_t e = rowptr[lo] + lane; e < rowptr[hi]; e += 32) {
            const uint32_t u = col[e];
            if (u < lo || u >= hi) b++;
        }
    }
    b = __reduce_add_sync(KC_FULL_MASK, (unsigned)b);
    if (lane == 0 && b) atomicAdd(bad, b);
}

struct BatchConfig {
    uint32_t small_n = 12288;   // graphs up to this many vertices: small-CTA class
    int small_threads = 256;
    int large_threads = 1024;
    uint32_t chunk = 256;
    int large_shared = 1;  // 0: graphs above small_n keep their degrees in global memory (more CTAs per SM)
};

struct BatchClass {
    int kind = 0;  // 0 small u16 smem, 1 large u16 smem, 2 u32 smem, 3 global
    std::vector<uint32_t> order;
    uint32_t smem_n = 0;
    uint32_t *d_order = nullptr;
    int threads = 256;
    int grid = 0;
    size_t smem_bytes = 0;
};

}  // namespace kc

struct kc_batch {
    kc_graph *g = nullptr;
    uint32_t G = 0;
    std::vector<uint32_t> vbase, maxdeg;
    std::vector<uint64_t> nnz;
    uint32_t *d_vbase = nullptr;
    unsigned long long *d_fbase = nullptr;
    unsigned long long *d_F = nullptr;
    uint64_t F_cap = 0;
    unsigned int *d_next = nullptr;  // one counter per class
    uint32_t *d_gdeg = nullptr;
    uint8_t *d_gclaimed = nullptr;
    uint32_t *d_alist = nullptr;  // two alive lists over the packed vertex ids
    kc::BatchConfig cfg;
    std::vector<kc::BatchClass> classes;
    bool planned = false;
    bool use_graph = true;
    bool trace = false;
    unsigned long long *d_gtrace = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t exec_stream = nullptr;
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t fork = nullptr, join[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0;
    ~kc_batch();
};

namespace kc {

static void free_classes(kc_batch *b) {
    for (auto &c : b->classes) dfree(c.d_order);
    b->classes.clear();
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    b->planned = false;
}

// Raises the dynamic shared-memory limit of batch_peel<DegT, SMEM> on the
// current device to the opt-in maximum, once per device.  The limit is never
// lowered afterwards, so a launch planned for one size stays valid whatever
// other launches of the same kernel (a later plan, the allocation-free entry
// point, another host thread) need.
template <typename DegT, bool SMEM>
static int batch_smem_limit() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    KC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(KC_ERR_INVALID, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(mu);
    if (done[dev]) return KC_OK;
    auto fn = batch_peel<DegT, SMEM>;
    int optin = 0;
    KC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    KC_CUDA(cudaFuncGetAttributes(&fa, fn));
    KC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
    done[dev] = true;
    return KC_OK;
}

template <typename DegT, bool SMEM>
static int class_grid(int threads, size_t smem, int sms, int *grid) {
    auto fn = batch_peel<DegT, SMEM>;
    if (smem > 48 * 1024) KC_TRY((batch_smem_limit<DegT, SMEM>()));
    int occ = 0;
    KC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem));
    if (occ < 1) return fail(KC_ERR_UNSUPPORTED, "batch kernel (%d threads, %zu B shared) cannot be resident", threads, smem);
    *grid = occ * sms;
    return KC_OK;
}

static int plan(kc_batch *b) {
    free_classes(b);
    int dev = b->g->device, smem_max = 0;
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t budget = (size_t)smem_max - 1024;  // static shared variables and alignment
    auto bytes_for = [](uint32_t n, size_t degsz) { return ((n * degsz + 15) & ~size_t(15)) + ((n + 31) / 32) * 4 + 16; };
    uint32_t large_u16 = 0, large_u32 = 0;
    while (bytes_for(large_u16 + 1024, 2) <= budget) large_u16 += 1024;
    while (bytes_for(large_u32 + 1024, 4) <= budget) large_u32 += 1024;
    const uint32_t small_n = std::min(b->cfg.small_n, large_u16);
    BatchClass cls[4];
    for (int k = 0; k < 4; k++) cls[k].kind = k;
    for (uint32_t i = 0; i < b->G; i++) {
        const uint32_t n = b->vbase[i + 1] - b->vbase[i];
        const bool fits16 = b->maxdeg[i] < 65535u;
        int k;
        if (fits16 && n <= small_n) k = 0;
        else if (!b->cfg.large_shared) k = 3;
        else if (fits16 && n <= large_u16) k = 1;
        else if (n <= large_u32) k = 2;
        else k = 3;
        cls[k].order.push_back(i);
    }
    cls[0].smem_n = small_n;
    cls[1].smem_n = large_u16;
    cls[2].smem_n = large_u32;
    for (int k = 0; k < 4; k++) {
        BatchClass &c = cls[k];
        if (c.order.empty()) continue;
        std::stable_sort(c.order.begin(), c.order.end(),
                         [&](uint32_t x, uint32_t y) { return b->nnz[x] > b->nnz[y]; });
        // shrink the shared arrays to the largest graph of the class
        uint32_t nmax = 0;
        for (uint32_t i : c.order) nmax = std::max(nmax, b->vbase[i + 1] - b->vbase[i]);
        if (k < 3) c.smem_n = std::max<uint32_t>(32, (nmax + 31) & ~31u);
        c.threads = k == 0 ? b->cfg.small_threads : b->cfg.large_threads;
        c.smem_bytes = k == 3 ? 0 : bytes_for(c.smem_n, k == 2 ? 4 : 2);
        int grid = 0;
        int rc;
        if (k <= 1) rc = class_grid<uint16_t, true>(c.threads, c.smem_bytes, b->g->sm_count, &grid);
        else if (k == 2) rc = class_grid<uint32_t, true>(c.threads, c.smem_bytes, b->g->sm_count, &grid);
        else rc = class_grid<uint32_t, false>(c.threads, 0, b->g->sm_count, &grid);
        if (rc) return rc;
        c.grid = (int)std::min<size_t>((size_t)grid, c.order.size());
        KC_TRY(dalloc(&c.d_order, c.order.size(), "batch class order"));
        KC_CUDA(cudaMemcpy(c.d_order, c.order.data(), c.order.size() * 4, cudaMemcpyHostToDevice));
        if (k == 3 && !b->d_gdeg) {
            KC_TRY(dalloc(&b->d_gdeg, (uint64_t)b->g->n + 1, "batch global degrees"));
            KC_TRY(dalloc(&b->d_gclaimed, (uint64_t)b->g->n + 1, "batch global flags"));
        }
        b->classes.push_back(std::move(c));
    }
    if (!b->d_alist) KC_TRY(dalloc(&b->d_alist, 2 * (uint64_t)b->g->n + 2, "batch alive lists"));
    b->planned = true;
    return KC_OK;
}

static int launch_all(kc_batch *b, cudaStream_t s) {
    Graph *g = b->g;
    const int nc = (int)b->classes.size();
    KC_CUDA(cudaMemsetAsync(b->d_next, 0, 4 * 4, s));
    KC_CUDA(cudaEventRecord(b->fork, s));
    for (int k = 0; k < nc; k++) {
        // the class of largest graphs first: its CTAs take the SMs before the
        // many small-graph CTAs fill them
        BatchClass &c = b->classes[nc - 1 - k];
        cudaStream_t cs = k == 0 ? s : b->side[k - 1];
        if (k > 0) KC_CUDA(cudaStreamWaitEvent(cs, b->fork, 0));
        BatchArgs A;
        A.rowptr = g->rowptr;
        A.col = g->col;
        A.core = g->core;
        A.vbase = b->d_vbase;
        A.order = c.d_order;
        A.count = (uint32_t)c.order.size();
        A.F = b->d_F;
        A.fbase = b->d_fbase;
        A.next = b->d_next + c.kind;
        A.gdeg = b->d_gdeg;
        A.gclaimed = b->d_gclaimed;
        A.chunk = b->cfg.chunk;
        A.smem_n = c.smem_n;
        A.gtrace = b->trace ? b->d_gtrace : nullptr;
        A.alist = b->d_alist;
        A.alist_stride = b->g->n;
        if (c.kind <= 1) batch_peel<uint16_t, true><<<c.grid, c.threads, c.smem_bytes, cs>>>(A);
        else if (c.kind == 2) batch_peel<uint32_t, true><<<c.grid, c.threads, c.smem_bytes, cs>>>(A);
        else batch_peel<uint32_t, false><<<c.grid, c.threads, 0, cs>>>(A);
        KC_CUDA(cudaGetLastError());
        if (k > 0) {
            KC_CUDA(cudaEventRecord(b->join[k - 1], cs));
            KC_CUDA(cudaStreamWaitEvent(s, b->join[k - 1], 0));
        }
    }
    return KC_OK;
}

static int run_batch(kc_batch *b, cudaStream_t s) {
    if (!b->planned) KC_TRY(plan(b));
    if (b->use_graph) {
        if (!b->exec || b->exec_stream != s) {
            if (b->exec) {
                cudaGraphExecDestroy(b->exec);
                b->exec = nullptr;
            }
            cudaGraph_t graph = nullptr;
            KC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            int rc = launch_all(b, s);
            cudaError_t e = cudaStreamEndCapture(s, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess) return fail(KC_ERR_CUDA, "batch capture: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&b->exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return fail(KC_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
            b->exec_stream = s;
        }
        KC_CUDA(cudaGraphLaunch(b->exec, s));
        return KC_OK;
    }
    return launch_all(b, s);
}

}  // namespace kc

kc_batch::~kc_batch() {
    int cur = 0;
    cudaGetDevice(&cur);
    if (g) cudaSetDevice(g->device);
    kc::free_classes(this);
    kc::dfree(d_vbase);
    kc::dfree(d_fbase);
    kc::dfree(d_F);
    kc::dfree(d_next);
    kc::dfree(d_gdeg);
    kc::dfree(d_gclaimed);
    kc::dfree(d_alist);
    kc::dfree(d_gtrace);
    for (int i = 0; i < 3; i++) {
        if (side[i]) {
            cudaStreamSynchronize(side[i]);
            kc::release_stream(g ? g->device : 0, side[i]);
        }
        kc::release_event(join[i]);
    }
    kc::release_event(fork);
    kc::release_event(ev0);
    kc::release_event(ev1);
    cudaSetDevice(cur);
}

using namespace kc;

extern "C" {

int kc_batch_create(kc_graph *g, const uint32_t *vbase, uint32_t num_graphs, kc_batch **out) {
    clear_error();
    if (!g || !vbase || !out || num_graphs == 0) return fail(KC_ERR_INVALID, "null argument or empty batch");
    *out = nullptr;
    if (vbase[0] != 0 || vbase[num_graphs] != g->n) return fail(KC_ERR_INVALID, "vbase must start at 0 and end at n");
    for (uint32_t i = 0; i < num_graphs; i++)
        if (vbase[i + 1] < vbase[i]) return fail(KC_ERR_INVALID, "vbase must be non-decreasing");
    KC_CUDA(cudaSetDevice(g->device));
    kc_batch *b = new (std::nothrow) kc_batch();
    if (!b) return fail(KC_ERR_NOMEM, "batch handle");
    b->g = g;
    b->G = num_graphs;
    b->vbase.assign(vbase, vbase + num_graphs + 1);
    int rc = dalloc(&b->d_vbase, num_graphs + 1, "batch vbase");
    if (!rc) rc = dalloc(&b->d_fbase, num_graphs, "batch queue offsets");
    if (!rc) rc = dalloc(&b->d_next, 4, "batch counters");
    uint32_t *d_maxdeg = nullptr;
    unsigned long long *d_bad = nullptr;
    if (!rc) rc = dalloc(&d_maxdeg, num_graphs, "batch max degrees");
    if (!rc) rc = dalloc(&d_bad, 1, "batch check");
    if (!rc && !g->core) rc = dalloc(&g->core, (uint64_t)g->n + 1, "core");
    if (rc) {
        dfree(d_maxdeg);
        dfree(d_bad);
        delete b;
        return rc;
    }
    cudaMemcpy(b->d_vbase, vbase, (num_graphs + 1) * 4ull, cudaMemcpyHostToDevice);
    cudaMemset(d_bad, 0, 8);
    const int blocks = std::max(1, std::min<int>(g->sm_count * 8, (int)((num_graphs * 32ull + 255) / 256)));
    batch_sizes<<<blocks, 256>>>(g->rowptr, b->d_vbase, num_graphs, d_maxdeg, b->d_fbase);
    batch_check<<<blocks, 256>>>(g->rowptr, g->col, b->d_vbase, num_graphs, d_bad);
    b->maxdeg.resize(num_graphs);
    unsigned long long bad = 0;
    std::vector<int64_t> rp(num_graphs + 1);
    cudaMemcpy(b->maxdeg.data(), d_maxdeg, num_graphs * 4ull, cudaMemcpyDeviceToHost);
    cudaMemcpy(&bad, d_bad, 8, cudaMemcpyDeviceToHost);
    // row offsets at the segment boundaries give each graph's entry count
    for (uint32_t i = 0; i <= num_graphs; i++) cudaMemcpy(&rp[i], g->rowptr + vbase[i], 8, cudaMemcpyDeviceToHost);
    cudaError_t e = cudaDeviceSynchronize();
    dfree(d_maxdeg);
    dfree(d_bad);
    if (e != cudaSuccess) {
        delete b;
        return fail(KC_ERR_CUDA, "batch setup: %s", cudaGetErrorString(e));
    }
    if (bad) {
        delete b;
        return fail(KC_ERR_INVALID, "%llu entries reference a vertex outside their graph", bad);
    }
    b->nnz.resize(num_graphs);
    for (uint32_t i = 0; i < num_graphs; i++) b->nnz[i] = (uint64_t)(rp[i + 1] - rp[i]);
    b->F_cap = (uint64_t)g->n + g->nnz / BATCH_MIN_CHUNK + num_graphs + 1;
    rc = dalloc(&b->d_F, b->F_cap, "batch row-chunk queue");
    if (!rc) {
        for (int i = 0; i < 3 && !rc; i++) {
            if (acquire_stream(g->device, &b->side[i]) != cudaSuccess ||
                acquire_event(&b->join[i]) != cudaSuccess)
                rc = fail(KC_ERR_CUDA, "batch streams");
        }
        if (!rc && (acquire_event(&b->fork) != cudaSuccess || acquire_event(&b->ev0) != cudaSuccess ||
                    acquire_event(&b->ev1) != cudaSuccess))
            rc = fail(KC_ERR_CUDA, "batch events");
    }
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return KC_OK;
}

int kc_batch_set_param(kc_batch *b, const char *name, int64_t value) {
    clear_error();
    if (!b || !name) return fail(KC_ERR_INVALID, "null argument");
    std::string k(name);
    if (k == "batch.small_n") {
        if (value < 32 || value > (1 << 20)) return fail(KC_ERR_INVALID, "batch.small_n: [32, 2^20]");
        b->cfg.small_n = (uint32_t)value;
    } else if (k == "batch.small_threads" || k == "batch.large_threads") {
        if (value < 64 || value > 1024 || (value & 31)) return fail(KC_ERR_INVALID, "%s: multiple of 32 in [64, 1024]", name);
        (k == "batch.small_threads" ? b->cfg.small_threads : b->cfg.large_threads) = (int)value;
    } else if (k == "batch.chunk") {
        if (value < BATCH_MIN_CHUNK || value > (1 << 16) || (value & (value - 1)))
            return fail(KC_ERR_INVALID, "batch.chunk: power of two in [%u, 2^16]", BATCH_MIN_CHUNK);
        b->cfg.chunk = (uint32_t)value;
    } else if (k == "batch.large_shared") {
        b->cfg.large_shared = value ? 1 : 0;
    } else if (k == "batch.cuda_graph") {
        b->use_graph = value != 0;
        return KC_OK;
    } else if (k == "trace") {
        b->trace = value != 0;
        if (b->trace && !b->d_gtrace) KC_TRY(dalloc(&b->d_gtrace, 3ull * b->G, "batch trace"));
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        return KC_OK;
    } else {
        return fail(KC_ERR_INVALID, "unknown parameter %s", name);
    }
    KC_CUDA(cudaSetDevice(b->g->device));
    free_classes(b);
    return KC_OK;
}

int kc_batch_get_param(const kc_batch *b, const char *name, int64_t *value) {
    clear_error();
    if (!b || !name || !value) return fail(KC_ERR_INVALID, "null argument");
    std::string k(name);
    if (k == "batch.small_n") *value = b->cfg.small_n;
    else if (k == "batch.small_threads") *value = b->cfg.small_threads;
    else if (k == "batch.large_threads") *value = b->cfg.large_threads;
    else if (k == "batch.chunk") *value = b->cfg.chunk;
    else if (k == "batch.large_shared") *value = b->cfg.large_shared;
    else if (k == "batch.cuda_graph") *value = b->use_graph ? 1 : 0;
    else return fail(KC_ERR_INVALID, "unknown parameter %s", name);
    return KC_OK;
}

int kc_batch_decompose(kc_batch *b, uint32_t *core_out, int out_on_device, kc_stats *stats, void *stream) {
    clear_error();
    NvtxRange nvtx_("kc_batch_decompose");
    if (!b) return fail(KC_ERR_INVALID, "null batch");
    Graph *g = b->g;
    KC_CUDA(cudaSetDevice(g->device));
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : g->stream;
    KC_CUDA(cudaEventRecord(b->ev0, s));
    if (int rc = run_batch(b, s)) {
        cudaStreamSynchronize(s);  // nothing launched may outlive a failed call
        return rc;
    }
    KC_CUDA(cudaEventRecord(b->ev1, s));
    if (core_out && g->n)
        KC_CUDA(cudaMemcpyAsync(core_out, g->core, (uint64_t)g->n * 4,
                                out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms;
    g->core_valid = true;
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->method = KC_PEELONE_DYN;
        stats->n = g->n;
        stats->nnz = g->nnz;
        stats->ms = ms;
        stats->build_ms = g->build_ms;
    }
    return KC_OK;
}

int kc_batch_autotune(kc_batch *b, double *best_ms) {
    clear_error();
    NvtxRange nvtx_("kc_batch_autotune");
    if (!b) return fail(KC_ERR_INVALID, "null batch");
    KC_CUDA(cudaSetDevice(b->g->device));
    const BatchConfig keep = b->cfg;
    BatchConfig best = keep;
    double best_t = 1e30;
    const uint32_t small_ns[] = {2048, 6144, 12288, 24576};
    const int small_threads[] = {128, 256, 512};
    const uint32_t chunks[] = {128, 256, 1024};
    for (uint32_t sn : small_ns)
        for (int st : small_threads)
            for (uint32_t ch : chunks) {
                b->cfg = keep;
                b->cfg.small_n = sn;
                b->cfg.small_threads = st;
                b->cfg.chunk = ch;
                free_classes(b);
                double t = 1e30;
                for (int rep = 0; rep < 2; rep++) {
                    int rc = kc_batch_decompose(b, nullptr, 0, nullptr, nullptr);
                    if (rc) {
                        b->cfg = keep;
                        free_classes(b);
                        return rc;
                    }
                    t = std::min(t, b->last_ms);
                }
                if (t < best_t) {
                    best_t = t;
                    best = b->cfg;
                }
            }
    b->cfg = best;
    free_classes(b);
    if (best_ms) *best_ms = best_t;
    return KC_OK;
}

int kc_batch_trace(const kc_batch *b, uint64_t *out, uint32_t cap) {
    clear_error();
    if (!b || !out) return fail(KC_ERR_INVALID, "null argument");
    if (!b->d_gtrace) return fail(KC_ERR_STATE, "batch trace not enabled");
    KC_CUDA(cudaSetDevice(b->g->device));
    KC_CUDA(cudaMemcpy(out, b->d_gtrace, 8ull * std::min<uint64_t>(cap, 3ull * b->G), cudaMemcpyDeviceToHost));
    return KC_OK;
}

int kc_batch_free(kc_batch *b) {
    clear_error();
    delete b;
    return KC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free decomposition of one small graph.
//
// For callers that cannot allocate device memory on this path: code running
// under a framework that owns all device memory through its own pool (so a
// cudaMalloc by this library would break its budget), latency-critical loops
// where cudaMalloc/cudaFree would synchronize the device, and code paths that
// must not create allocations at all.  The caller passes the graph and the
// output in device memory; the only scratch the batched kernel needs -- its
// row-chunk queue and a few control words -- lives in the fixed file-scope
// array below, which every GPU that loads this library holds until the
// process exits.  All calls share that array: calls whose work overlaps on
// the GPU (different streams, or different host threads) race on it and must
// be serialised by the caller.
namespace kc {

constexpr uint32_t NOALLOC_MAX_N = 50000;            // vertices
constexpr uint64_t NOALLOC_MAX_NNZ = 1ull << 22;     // directed CSR entries
constexpr uint64_t NOALLOC_CTRL_WORDS = 32;          // control block (256 bytes)
constexpr uint64_t NOALLOC_QUEUE = NOALLOC_MAX_N + NOALLOC_MAX_NNZ / BATCH_MIN_CHUNK + 2;
constexpr uint64_t NOALLOC_WORDS = NOALLOC_CTRL_WORDS + NOALLOC_QUEUE;  // 8-byte words, ~663 KB

static __device__ __align__(256) unsigned long long g_noalloc_scratch[NOALLOC_WORDS];

// Writes the one-graph work list into the control block: vbase = {0, n},
// order = {0}, fbase = {0}, work counter = 0, bad-entry count = 0.
__global__ void noalloc_prep(unsigned long long *scratch, uint32_t n) {
    uint32_t *w = reinterpret_cast<uint32_t *>(scratch);
    w[0] = 0;  // vbase[0]
    w[1] = n;  // vbase[1]
    w[2] = 0;  // order[0]
    w[4] = 0;  // next (work counter)
    scratch[3] = 0ull;  // fbase[0]
    w[8] = 0;  // entries that fail noalloc_check
}

// Counts, into control word 8, the row offsets that decrease (or a negative
// rowptr[0]) and the column ids >= n among col[0, nnz): the kernel indexes its
// shared-memory arrays by column id, so a caller's bad id must be turned into
// an error before it runs.
__global__ void noalloc_check(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col, uint32_t n,
                              uint64_t nnz, unsigned long long *scratch) {
    unsigned bad = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint64_t v = t0; v < n; v += stride) bad += (rowptr[v + 1] < rowptr[v]) ? 1u : 0u;
    if (t0 == 0 && rowptr[0] < 0) bad++;
    for (uint64_t e = t0; e < nnz; e += stride) bad += (col[e] >= n) ? 1u : 0u;
    bad = __reduce_add_sync(KC_FULL_MASK, bad);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(reinterpret_cast<uint32_t *>(scratch) + 8, bad);
}

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[64];

// Device address of the scratch array, looked up once per device with that
// device current (a host-side use of the symbol's name is not a device
// address).
static int noalloc_setup(int dev, unsigned long long **out) {
    if (dev < 0 || dev >= 64) return fail(KC_ERR_INVALID, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(KC_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
        KC_TRY((batch_smem_limit<uint32_t, true>()));
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<unsigned long long *>(g_noalloc_ptr[dev]);
    return KC_OK;
}

}  // namespace kc

extern "C" int kc_decompose_noalloc(const int64_t *d_rowptr, const uint32_t *d_col, uint32_t n, uint32_t *d_core,
                                    void *stream) {
    using namespace kc;
    clear_error();
    if (!d_rowptr || !d_core) return fail(KC_ERR_INVALID, "null argument");
    if (n > NOALLOC_MAX_N)
        return fail(KC_ERR_CAPACITY, "kc_decompose_noalloc: %u vertices exceed the limit of %u", n, NOALLOC_MAX_N);
    int dev = 0;
    KC_CUDA(cudaGetDevice(&dev));
    unsigned long long *scratch = nullptr;
    KC_TRY(noalloc_setup(dev, &scratch));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int64_t nnz = 0;
    KC_CUDA(cudaMemcpyAsync(&nnz, d_rowptr + n, sizeof(nnz), cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    if (nnz < 0 || (uint64_t)nnz > NOALLOC_MAX_NNZ)
        return fail(KC_ERR_CAPACITY, "kc_decompose_noalloc: %lld entries exceed the limit of %llu", (long long)nnz,
                    (unsigned long long)NOALLOC_MAX_NNZ);
    if (n == 0) return KC_OK;
    if (nnz > 0 && !d_col) return fail(KC_ERR_INVALID, "null column array with %lld entries", (long long)nnz);
    noalloc_prep<<<1, 1, 0, s>>>(scratch, n);
    {
        const uint64_t work = std::max<uint64_t>((uint64_t)nnz, n);
        const unsigned blocks = (unsigned)std::min<uint64_t>((work + 255) / 256, 1024);
        noalloc_check<<<blocks, 256, 0, s>>>(d_rowptr, d_col, n, (uint64_t)nnz, scratch);
        uint32_t bad = 0;
        KC_CUDA(cudaGetLastError());
        KC_CUDA(cudaMemcpyAsync(&bad, reinterpret_cast<uint32_t *>(scratch) + 8, sizeof(bad), cudaMemcpyDeviceToHost,
                                s));
        KC_CUDA(cudaStreamSynchronize(s));
        if (bad)
            return fail(KC_ERR_INVALID,
                        "kc_decompose_noalloc: %u row offsets or column ids invalid (ids must be < n = %u, "
                        "offsets non-decreasing from 0)", bad, n);
    }
    uint32_t *ctrl = reinterpret_cast<uint32_t *>(scratch);
    BatchArgs A;
    A.rowptr = d_rowptr;
    A.col = d_col;
    A.core = d_core;
    A.vbase = ctrl;
    A.order = ctrl + 2;
    A.count = 1;
    A.F = scratch + NOALLOC_CTRL_WORDS;
    A.fbase = scratch + 3;
    A.next = ctrl + 4;
    A.gdeg = nullptr;
    A.gclaimed = nullptr;
    A.chunk = 256;
    A.smem_n = (n + 31) & ~31u;
    A.gtrace = nullptr;
    A.alist = nullptr;  // scans the vertex range every level: no list storage
    A.alist_stride = 0;
    const size_t smem = ((A.smem_n * sizeof(uint32_t) + 15) & ~size_t(15)) + ((A.smem_n + 31) / 32) * 4 + 16;
    // the kernel's shared-memory limit was raised to the device maximum once,
    // in noalloc_setup, and is never lowered
    batch_peel<uint32_t, true><<<1, 1024, smem, s>>>(A);
    KC_CUDA(cudaGetLastError());
    KC_CUDA(cudaStreamSynchronize(s));
    return KC_OK;
}
