// C ABI of libkcore.so: graph handles, decomposition dispatch, generators.
// See include/kcore.h for the contract of each entry point.
#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

static thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

void clear_error() { g_last_error.clear(); }

// Device memory comes from the stream-ordered pool allocator: unlike
// cudaMalloc / cudaFree it does not synchronize the whole device, so work of
// independent graphs (server lanes) keeps overlapping.  Allocation is ordered
// on the legacy stream and waited for, so the memory is usable from any
// stream; every caller has finished its own stream's work on a buffer before
// freeing it.
//
// The pool keeps freed memory for reuse instead of returning it to the driver
// at every synchronisation (its default), so a graph built and freed per
// request or per step does not remap its buffers each time.  This is a
// property of this process's pool only.
static void keep_pool_memory() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    done[dev] = true;
}

// Free device memory of the current device, counting what this process's pool
// holds for reuse as free.
size_t device_free_bytes(size_t *total) {
    size_t f = 0, t = 0;
    cudaMemGetInfo(&f, &t);
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t reserved = 0, used = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
            f += (size_t)(reserved - used);
    }
    cudaGetLastError();
    if (total) *total = t;
    return f;
}

int dmalloc(void **p, size_t bytes, const char *what) {
    *p = nullptr;
    keep_pool_memory();
    cudaError_t e = cudaMallocAsync(p, bytes, cudaStreamLegacy);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamLegacy);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (*p) cudaFreeAsync(*p, cudaStreamLegacy);
        *p = nullptr;
        return fail(KC_ERR_NOMEM, "device allocation of %zu bytes for %s: %s", bytes, what, cudaGetErrorString(e));
    }
    return KC_OK;
}

void dfree(void *p) {
    if (p) cudaFreeAsync(p, cudaStreamLegacy);
}

// Graph handles take their stream from a per-process pool and give it back
// when freed: creating or destroying a stream can wait for a kernel that
// another thread runs (a cooperative decomposition holds every SM), which
// would serialise independent graphs built and freed while others decompose.
static std::mutex g_stream_mu;
static std::vector<std::pair<int, cudaStream_t>> g_stream_pool;

cudaError_t acquire_stream(int device, cudaStream_t *s) {
    {
        std::lock_guard<std::mutex> lock(g_stream_mu);
        for (size_t i = g_stream_pool.size(); i-- > 0;) {
            if (g_stream_pool[i].first == device) {
                *s = g_stream_pool[i].second;
                g_stream_pool.erase(g_stream_pool.begin() + (std::ptrdiff_t)i);
                return cudaSuccess;
            }
        }
    }
    return cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
}

void release_stream(int device, cudaStream_t s) {
    std::lock_guard<std::mutex> lock(g_stream_mu);
    if (g_stream_pool.size() < 256) g_stream_pool.emplace_back(device, s);
    else cudaStreamDestroy(s);
}

// Events likewise: destroying one waits, like a stream, for another thread's
// cooperative kernel.  Pooled events carry timing; they are handed back
// after their last use has completed.
static std::vector<std::pair<int, cudaEvent_t>> g_event_pool;

cudaError_t acquire_event(cudaEvent_t *e) {
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lock(g_stream_mu);
        for (size_t i = g_event_pool.size(); i-- > 0;) {
            if (g_event_pool[i].first == dev) {
                *e = g_event_pool[i].second;
                g_event_pool.erase(g_event_pool.begin() + (std::ptrdiff_t)i);
                return cudaSuccess;
            }
        }
    }
    return cudaEventCreate(e);
}

void release_event(cudaEvent_t e) {
    if (!e) return;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_stream_mu);
    if (g_event_pool.size() < 1024) g_event_pool.emplace_back(dev, e);
    else cudaEventDestroy(e);
}

Graph::~Graph() {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    dfree(rowptr);
    dfree(col);
    dfree(core);
    dfree(bitmap);
    dfree(alive);
    dfree(gq);
    dfree(peel_ctl);
    for (int i = 0; i < 2; i++) {
        dfree(list[i]);
        dfree(big[i]);
    }
    dfree(hctl);
    dfree(hx_bitmap);
    dfree(hx_ord);
    dfree(hx_lid);
    dfree(hx_pref);
    dfree(hx_bk);
    dfree(hx_vb);
    dfree(red);
    dfree(trace);
    dfree(mfront[0]);
    dfree(mfront[1]);
    dfree(mcand);
    dfree(mvisit);
    dfree(mcount);
    release_event(ev0);
    release_event(ev1);
    release_event(evk0);
    release_event(evk1);
    if (stream) release_stream(device, stream);  // idle: synchronised above
    cudaSetDevice(cur);
}

static int open_device(int device) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(KC_ERR_CUDA, "no CUDA device available (%s)", cudaGetErrorString(e));
    }
    if (device < 0 || device >= count) return fail(KC_ERR_INVALID, "device %d out of range (%d devices)", device, count);
    KC_CUDA(cudaSetDevice(device));
    return KC_OK;
}

static int new_graph(int device, kc_graph **out) {
    KC_TRY(open_device(device));
    kc_graph *g = new (std::nothrow) kc_graph();
    if (!g) return fail(KC_ERR_NOMEM, "host allocation of graph handle");
    g->device = device;
    cudaDeviceGetAttribute(&g->sm_count, cudaDevAttrMultiProcessorCount, device);
    cudaError_t e = acquire_stream(device, &g->stream);
    if (e != cudaSuccess) {
        g->stream = nullptr;
        delete g;
        return fail(KC_ERR_CUDA, "stream create: %s", cudaGetErrorString(e));
    }
    *out = g;
    return KC_OK;
}

int graph_new(int device, kc_graph **out) { return new_graph(device, out); }

__global__ void core_minmax(const uint32_t *__restrict__ c, uint32_t n, uint32_t *mm) {
    uint32_t mn = 0xffffffffu, mx = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = c[v];
        mn = min(mn, x);
        mx = max(mx, x);
    }
    mn = __reduce_min_sync(KC_FULL_MASK, mn);
    mx = __reduce_max_sync(KC_FULL_MASK, mx);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mm[0], mn);
        atomicMax(&mm[1], mx);
    }
}

}  // namespace kc

using namespace kc;

extern "C" {

int kc_abi_version(void) { return KC_ABI_VERSION; }

const char *kc_last_error(void) { return g_last_error.c_str(); }

int kc_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}

int kc_parse_mtx(const char *path, int mode, uint32_t *n, uint64_t *m, uint32_t **src, uint32_t **dst) {
    clear_error();
    return parse_mtx(path, mode, n, m, src, dst);
}

void kc_host_free_edges(uint32_t *src, uint32_t *dst) {
    free(src);
    free(dst);
}

int kc_graph_from_edges_device(const uint32_t *d_src, const uint32_t *d_dst, uint64_t m, uint32_t n, uint32_t flags,
                               int device, kc_graph **out) {
    clear_error();
    NvtxRange nvtx_("kc_graph_from_edges_device");
    if (!out || (m && (!d_src || !d_dst))) return fail(KC_ERR_INVALID, "null argument");
    *out = nullptr;
    kc_graph *g = nullptr;
    KC_TRY(new_graph(device, &g));
    cudaEvent_t a, b;
    acquire_event(&a);
    acquire_event(&b);
    cudaEventRecord(a, g->stream);
    int rc = build_csr_from_edges(g, d_src, d_dst, m, n, flags);
    cudaEventRecord(b, g->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    release_event(a);
    release_event(b);
    if (rc) {
        delete g;
        return rc;
    }
    if (g->max_deg >= 0x7fffffffu) {
        delete g;
        return fail(KC_ERR_UNSUPPORTED, "degree above 2^31-1");
    }
    g->build_ms = ms;
    *out = g;
    return KC_OK;
}

int kc_graph_from_edges(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n, uint32_t flags, int device,
                        kc_graph **out) {
    clear_error();
    if (!out || (m && (!src || !dst))) return fail(KC_ERR_INVALID, "null argument");
    *out = nullptr;
    KC_TRY(open_device(device));
    uint32_t *ds = nullptr, *dd = nullptr;
    KC_TRY(dalloc(&ds, std::max<uint64_t>(m, 1), "edge sources"));
    int rc = dalloc(&dd, std::max<uint64_t>(m, 1), "edge targets");
    if (rc) { dfree(ds); return rc; }
    if (m) {
        cudaError_t e1 = cudaMemcpy(ds, src, m * 4, cudaMemcpyHostToDevice);
        cudaError_t e2 = cudaMemcpy(dd, dst, m * 4, cudaMemcpyHostToDevice);
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            dfree(ds);
            dfree(dd);
            return fail(KC_ERR_CUDA, "edge upload: %s", cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
        }
    }
    rc = kc_graph_from_edges_device(ds, dd, m, n, flags, device, out);
    dfree(ds);
    dfree(dd);
    return rc;
}

int kc_graph_from_mtx(const char *path, int mode, int device, kc_graph **out) {
    clear_error();
    NvtxRange nvtx_("kc_graph_from_mtx");
    uint32_t n = 0, *src = nullptr, *dst = nullptr;
    uint64_t m = 0;
    KC_TRY(parse_mtx(path, mode, &n, &m, &src, &dst));
    int rc = kc_graph_from_edges(src, dst, m, n, mode == KC_LOAD_CSR_DEDUP ? KC_EDGES_DEDUP : 0u, device, out);
    free(src);
    free(dst);
    return rc;
}

// Largest degree and number of 32-wide virtual nodes of a CSR in host memory.
static int from_csr_common(const int64_t *rowptr, const uint32_t *col, uint32_t n, int device, kc_graph **out,
                           cudaMemcpyKind kind) {
    NvtxRange nvtx_("kc_graph_from_csr");
    if (!out || !rowptr) return fail(KC_ERR_INVALID, "null argument");
    *out = nullptr;
    kc_graph *g = nullptr;
    KC_TRY(new_graph(device, &g));
    int64_t nnz = 0;
    cudaError_t e = cudaSuccess;
    if (kind == cudaMemcpyHostToDevice) memcpy(&nnz, rowptr + n, 8);  // host memory: no driver call
    else e = cudaMemcpy(&nnz, rowptr + n, 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { delete g; return fail(KC_ERR_CUDA, "read rowptr[n]: %s", cudaGetErrorString(e)); }
    if (nnz < 0 || (nnz > 0 && !col)) { delete g; return fail(KC_ERR_INVALID, "bad rowptr[n] = %lld", (long long)nnz); }
    g->n = n;
    g->nnz = (uint64_t)nnz;
    int rc = dalloc(&g->rowptr, (uint64_t)n + 1, "row offsets");
    if (!rc) rc = dalloc(&g->col, g->nnz + 1, "column ids");
    if (rc) { delete g; return rc; }
    cudaEvent_t a, b;
    acquire_event(&a);
    acquire_event(&b);
    cudaEventRecord(a, g->stream);
    cudaMemcpyAsync(g->rowptr, rowptr, ((uint64_t)n + 1) * 8, kind, g->stream);
    if (nnz) cudaMemcpyAsync(g->col, col, g->nnz * 4, kind, g->stream);
    cudaEventRecord(b, g->stream);
    e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    release_event(a);
    release_event(b);
    if (e != cudaSuccess) { delete g; return fail(KC_ERR_CUDA, "CSR upload: %s", cudaGetErrorString(e)); }
    // degree statistics on the device: one pass over rowptr in HBM (about
    // 0.1 ms for 33.5 M rows) instead of host threads scanning the host CSR,
    // which compete with whatever else the host runs
    rc = graph_finish(g);
    if (rc) { delete g; return rc; }
    if (g->max_deg >= 0x7fffffffu) { delete g; return fail(KC_ERR_UNSUPPORTED, "degree above 2^31-1"); }
    g->build_ms = ms;
    *out = g;
    return KC_OK;
}

int kc_graph_from_csr(const int64_t *rowptr, const uint32_t *col, uint32_t n, int device, kc_graph **out) {
    clear_error();
    return from_csr_common(rowptr, col, n, device, out, cudaMemcpyHostToDevice);
}

int kc_graph_from_csr_device(const int64_t *d_rowptr, const uint32_t *d_col, uint32_t n, int device, kc_graph **out) {
    clear_error();
    return from_csr_common(d_rowptr, d_col, n, device, out, cudaMemcpyDeviceToDevice);
}

__global__ void segment_rebase(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col, uint32_t lo,
                               uint32_t n, int64_t *nrow, uint32_t *ncol) {
    const int64_t base = rowptr[lo];
    const int64_t nnz = rowptr[lo + n] - base;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v <= n; v += stride) nrow[v] = rowptr[lo + v] - base;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < (uint64_t)nnz; e += stride)
        ncol[e] = col[base + e] - lo;
}

int kc_graph_from_segment(const kc_graph *g, uint32_t lo, uint32_t hi, kc_graph **out) {
    clear_error();
    if (!g || !out || hi < lo || hi > g->n) return fail(KC_ERR_INVALID, "bad segment");
    *out = nullptr;
    kc_graph *h = nullptr;
    KC_TRY(new_graph(g->device, &h));
    h->n = hi - lo;
    int64_t r[2];
    cudaMemcpy(&r[0], g->rowptr + lo, 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(&r[1], g->rowptr + hi, 8, cudaMemcpyDeviceToHost);
    h->nnz = (uint64_t)(r[1] - r[0]);
    int rc = dalloc(&h->rowptr, (uint64_t)h->n + 1, "row offsets");
    if (!rc) rc = dalloc(&h->col, h->nnz + 1, "column ids");
    if (rc) { delete h; return rc; }
    const uint64_t items = std::max<uint64_t>(h->nnz, (uint64_t)h->n + 1);
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)h->sm_count * 8, (items + 255) / 256));
    segment_rebase<<<blocks, 256, 0, h->stream>>>(g->rowptr, g->col, lo, h->n, h->rowptr, h->col);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) { delete h; return fail(KC_ERR_CUDA, "segment: %s", cudaGetErrorString(e)); }
    rc = graph_finish(h);
    if (rc) { delete h; return rc; }
    *out = h;
    return KC_OK;
}

int kc_graph_validate(kc_graph *g, uint64_t *bad) {
    clear_error();
    if (!g || !bad) return fail(KC_ERR_INVALID, "null argument");
    KC_CUDA(cudaSetDevice(g->device));
    return graph_validate(g, bad);
}

int kc_graph_free(kc_graph *g) {
    clear_error();
    if (!g) return KC_OK;
    delete g;
    return KC_OK;
}

int kc_graph_info(const kc_graph *g, uint32_t *n, uint64_t *nnz, uint32_t *max_degree, uint64_t *num_vnodes) {
    clear_error();
    if (!g) return fail(KC_ERR_INVALID, "null graph");
    if (n) *n = g->n;
    if (nnz) *nnz = g->nnz;
    if (max_degree) *max_degree = g->max_deg;
    if (num_vnodes) *num_vnodes = g->num_vnodes;
    return KC_OK;
}

int kc_graph_device_csr(const kc_graph *g, const int64_t **d_rowptr, const uint32_t **d_col) {
    clear_error();
    if (!g) return fail(KC_ERR_INVALID, "null graph");
    if (d_rowptr) *d_rowptr = g->rowptr;
    if (d_col) *d_col = g->col;
    return KC_OK;
}

int kc_graph_copy_csr(const kc_graph *g, int64_t *rowptr, uint32_t *col) {
    clear_error();
    if (!g) return fail(KC_ERR_INVALID, "null graph");
    KC_CUDA(cudaSetDevice(g->device));
    if (rowptr) KC_CUDA(cudaMemcpy(rowptr, g->rowptr, ((uint64_t)g->n + 1) * 8, cudaMemcpyDeviceToHost));
    if (col && g->nnz) KC_CUDA(cudaMemcpy(col, g->col, g->nnz * 4, cudaMemcpyDeviceToHost));
    return KC_OK;
}

__global__ void degrees_kernel(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t *deg) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        deg[v] = (uint32_t)(rowptr[v + 1] - rowptr[v]);
}

int kc_graph_degrees(const kc_graph *g, uint32_t *deg) {
    clear_error();
    if (!g || !deg) return fail(KC_ERR_INVALID, "null argument");
    KC_CUDA(cudaSetDevice(g->device));
    if (!g->n) return KC_OK;
    uint32_t *d = nullptr;
    KC_TRY(dalloc(&d, g->n, "degrees"));
    degrees_kernel<<<std::max(1, std::min<int>(g->sm_count * 8, (int)((g->n + 255) / 256))), 256, 0, g->stream>>>(
        g->rowptr, g->n, d);
    cudaError_t e = cudaMemcpyAsync(deg, d, (uint64_t)g->n * 4, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    dfree(d);
    if (e != cudaSuccess) return fail(KC_ERR_CUDA, "degrees: %s", cudaGetErrorString(e));
    return KC_OK;
}

int kc_graph_virtual_layout(kc_graph *g, uint32_t part_size, uint32_t *node_pointer, uint32_t *edge_list,
                            uint32_t *parts, uint64_t *num_parts) {
    clear_error();
    if (!g || !num_parts) return fail(KC_ERR_INVALID, "null argument");
    KC_CUDA(cudaSetDevice(g->device));
    return virtual_layout(g, part_size, node_pointer, edge_list, parts, num_parts);
}

namespace kc {

// One decomposition by `method` (no stats, result stays on the device).
static int run_method(Graph *g, int method, cudaStream_t s) {
    if (g->n == 0) return KC_OK;
    if (method == KC_HISTO || method == KC_CNT || method == KC_NBR) return hindex_run(g, s, nullptr);
    return peel_run(g, s, method == KC_GPP, nullptr);
}

// The autotuner behind KC_AUTO: times the candidates on this graph -- the
// bucket peel with its default tunables, the peel with the other row-chunk
// size, the peel keeping more cascade items per CTA before it publishes them
// to the shared queues, and the h-index iteration -- each
// once to warm up and then twice, keeps the fastest (its method and peel
// tunables) in the graph and restores nothing else.
static int autotune_graph(Graph *g, cudaStream_t s) {
    struct Cand {
        int method;
        int chunk;
        int spill;
    };
    const Tuning base = g->tune;
    const int other_chunk = (g->nnz >= (1ull << 29)) ? 1024 : 2048;
    const Cand cands[] = {{KC_PEELONE_DYN, base.peel_chunk, base.peel_spill},
                          {KC_PEELONE_DYN, other_chunk, base.peel_spill},
                          {KC_PEELONE_DYN, base.peel_chunk, 2 * base.peel_spill + 16},
                          {KC_NBR, base.peel_chunk, base.peel_spill}};
    double best = 1e300;
    Cand pick = cands[0];
    for (const Cand &c : cands) {
        g->tune.peel_chunk = c.chunk;
        g->tune.peel_spill = c.spill;
        double t = 1e300;
        for (int rep = 0; rep < 3; rep++) {
            KC_TRY(run_method(g, c.method, s));
            if (rep > 0) t = std::min(t, g->last_ms);
        }
        if (t < best) {
            best = t;
            pick = c;
        }
    }
    g->tune.peel_chunk = pick.chunk;
    g->tune.peel_spill = pick.spill;
    g->auto_method = pick.method;
    g->auto_ms = best;
    return KC_OK;
}

}  // namespace kc

int kc_graph_autotune(kc_graph *g, int *method, double *best_ms) {
    clear_error();
    NvtxRange nvtx_("kc_graph_autotune");
    if (!g) return fail(KC_ERR_INVALID, "null graph");
    KC_CUDA(cudaSetDevice(g->device));
    KC_TRY(autotune_graph(g, g->stream));
    if (method) *method = g->auto_method;
    if (best_ms) *best_ms = g->auto_ms;
    return KC_OK;
}

int kc_decompose(kc_graph *g, int method, uint32_t *core_out, int out_on_device, kc_stats *stats, void *stream) {
    clear_error();
    NvtxRange nvtx_("kc_decompose");
    if (!g) return fail(KC_ERR_INVALID, "null graph");
    if (method < KC_HISTO || method > KC_AUTO) return fail(KC_ERR_INVALID, "unknown method %d", method);
    KC_CUDA(cudaSetDevice(g->device));
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : g->stream;
    kc_stats st;
    memset(&st, 0, sizeof(st));
    if (method == KC_AUTO && g->auto_method < 0 && g->n) KC_TRY(autotune_graph(g, s));
    int run = method == KC_AUTO ? (g->auto_method < 0 ? KC_PEELONE_DYN : g->auto_method) : method;
    st.method = (uint32_t)run;
    st.n = g->n;
    st.nnz = g->nnz;
    st.build_ms = g->build_ms;
    int rc;
    if (g->n == 0) {
        rc = KC_OK;
        if (!g->core) KC_TRY(dalloc(&g->core, 1, "core"));
        g->core_valid = true;
    } else if (run == KC_HISTO || run == KC_CNT || run == KC_NBR) {
        rc = hindex_run(g, s, &st);
    } else {
        rc = peel_run(g, s, run == KC_GPP, &st);
    }
    if (rc) return rc;
    if (stats) {
        // Max K / Min K as utility::PrintMaxMin reports them (util.cpp:6-22):
        // the minimum starts at 10, so it never exceeds 10.
        if (!g->red) KC_TRY(dalloc(&g->red, 2, "reduction"));
        uint32_t init[2] = {10u, 0u};
        KC_CUDA(cudaMemcpyAsync(g->red, init, 8, cudaMemcpyHostToDevice, s));
        if (g->n)
            core_minmax<<<std::max(1, std::min<int>(g->sm_count * 4, (int)((g->n + 255) / 256))), 256, 0, s>>>(
                g->core, g->n, g->red);
        uint32_t mm[2];
        KC_CUDA(cudaMemcpyAsync(mm, g->red, 8, cudaMemcpyDeviceToHost, s));
        KC_CUDA(cudaStreamSynchronize(s));
        st.kmin = mm[0];
        st.kmax = mm[1];
        *stats = st;
    }
    if (core_out && g->n) {
        KC_CUDA(cudaMemcpyAsync(core_out, g->core, (uint64_t)g->n * 4,
                                out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
        KC_CUDA(cudaStreamSynchronize(s));
    }
    return KC_OK;
}

int kc_graph_set_param(kc_graph *g, const char *name, int64_t value) {
    clear_error();
    if (!g || !name) return fail(KC_ERR_INVALID, "null argument");
    std::string k(name);
    Tuning &t = g->tune;
    if (k == "peel.chunk") {
        if (value != 0 && (value < 256 || value > (1 << 20) || (value & (value - 1))))
            return fail(KC_ERR_INVALID, "peel.chunk: 0 (by graph size) or a power of two in [256, 2^20]");
        t.peel_chunk = (int)value;
    } else if (k == "peel.spill") {
        if (value < 0 || value > 3072) return fail(KC_ERR_INVALID, "peel.spill: [0, 3072]");
        t.peel_spill = (int)value;
    } else if (k == "peel.steal") {
        if (value < 1 || value > 64) return fail(KC_ERR_INVALID, "peel.steal: [1, 64]");
        t.peel_steal = (int)value;
    } else if (k == "peel.queues") {
        if (value < 1 || value > PEEL_MAX_QUEUES) return fail(KC_ERR_INVALID, "peel.queues: [1, %d]", PEEL_MAX_QUEUES);
        t.peel_queues = (int)value;
    } else if (k == "peel.ctas_per_sm") {
        if (value < 0 || value > 32) return fail(KC_ERR_INVALID, "peel.ctas_per_sm: [0, 32]");
        t.peel_ctas_per_sm = (int)value;
    } else if (k == "peel.unroll") {
        if (value != 4 && value != 8) return fail(KC_ERR_INVALID, "peel.unroll: 4 or 8");
        t.peel_unroll = (int)value;
    } else if (k == "peel.threads") {
        if (value != 256 && value != 512) return fail(KC_ERR_INVALID, "peel.threads: 256 or 512");
        t.peel_threads = (int)value;
    } else if (k == "peel.balanced") {
        t.peel_balanced = value ? 1 : 0;
    } else if (k == "peel.round_entries") {
        if (value < 256 || value > (1 << 24)) return fail(KC_ERR_INVALID, "peel.round_entries: [256, 2^24]");
        t.peel_round_entries = (int)value;
    } else if (k == "peel.aggregate") {
        t.peel_aggregate = value ? 1 : 0;
    } else if (k == "peel.scan_unroll") {
        if (value != 4 && value != 8) return fail(KC_ERR_INVALID, "peel.scan_unroll: 4 or 8");
        t.peel_scan_unroll = (int)value;
    } else if (k == "hindex.warp_rows") {
        if (value < 512 || value > (int64_t)1 << 30) return fail(KC_ERR_INVALID, "hindex.warp_rows: [512, 2^30]");
        t.hindex_warp_rows = value;
    } else if (k == "hindex.order") {
        t.hindex_order = value ? 1 : 0;
    } else if (k == "hindex.order_min") {
        if (value < 128 || value > (int64_t)1 << 30) return fail(KC_ERR_INVALID, "hindex.order_min: [128, 2^30]");
        t.hindex_order_min = value;
    } else if (k == "trace") {
        t.trace = value ? 1 : 0;
    } else if (k == "update.incremental_max") {
        if (value < 0) return fail(KC_ERR_INVALID, "update.incremental_max: >= 0");
        t.update_incremental_max = value;
    } else if (k == "update.deletion_incremental_max") {
        if (value < 0) return fail(KC_ERR_INVALID, "update.deletion_incremental_max: >= 0");
        t.update_deletion_incremental_max = value;
    } else if (k == "wait.timeout_us") {
        if (value < 1000 || value > 600000000) return fail(KC_ERR_INVALID, "wait.timeout_us: [1000, 6e8]");
        t.wait_timeout_us = value;
    } else if (k == "test.withhold") {
        t.withhold = value ? 1 : 0;
    } else {
        return fail(KC_ERR_INVALID, "unknown parameter %s", name);
    }
    return KC_OK;
}

int kc_graph_trace(const kc_graph *g, kc_level_trace *out, uint32_t cap, uint32_t *count) {
    clear_error();
    if (!g || !count) return fail(KC_ERR_INVALID, "null argument");
    static_assert(sizeof(kc_level_trace) == sizeof(PeelTrace), "trace layout");
    uint32_t c = g->trace_count;
    *count = c;
    if (out && cap && c) {
        KC_CUDA(cudaSetDevice(g->device));
        KC_CUDA(cudaMemcpy(out, g->trace, sizeof(PeelTrace) * std::min(c, cap), cudaMemcpyDeviceToHost));
    }
    return KC_OK;
}

int kc_graph_last_timing(const kc_graph *g, double *total_ms, double *kernel_ms) {
    clear_error();
    if (!g) return fail(KC_ERR_INVALID, "null graph");
    if (total_ms) *total_ms = g->last_ms;
    if (kernel_ms) *kernel_ms = g->last_kernel_ms;
    return KC_OK;
}

int kc_graph_update(kc_graph *g, const uint32_t *ins_src, const uint32_t *ins_dst, uint64_t n_ins,
                    const uint32_t *del_src, const uint32_t *del_dst, uint64_t n_del, uint32_t *core_out,
                    int out_on_device, kc_update_stats *stats) {
    clear_error();
    NvtxRange nvtx_("kc_graph_update");
    if (!g || (n_ins && (!ins_src || !ins_dst)) || (n_del && (!del_src || !del_dst)))
        return fail(KC_ERR_INVALID, "null argument");
    KC_CUDA(cudaSetDevice(g->device));
    int rc = graph_update(g, ins_src, ins_dst, n_ins, del_src, del_dst, n_del, stats);
    if (rc) {
        g->core_valid = false;
        return rc;
    }
    if (core_out && g->n) {
        KC_CUDA(cudaMemcpyAsync(core_out, g->core, (uint64_t)g->n * 4,
                                out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, g->stream));
        KC_CUDA(cudaStreamSynchronize(g->stream));
    }
    return KC_OK;
}

int kc_graph_device_core(const kc_graph *g, const uint32_t **d_core) {
    clear_error();
    if (!g || !d_core) return fail(KC_ERR_INVALID, "null argument");
    if (!g->core_valid) return fail(KC_ERR_STATE, "no decomposition has completed on this graph");
    *d_core = g->core;
    return KC_OK;
}

int kc_host_alloc(void **p, size_t bytes) {
    clear_error();
    if (!p) return fail(KC_ERR_INVALID, "null argument");
    cudaError_t e = cudaMallocHost(p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(KC_ERR_NOMEM, "cudaMallocHost(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return KC_OK;
}

int kc_host_free(void *p) {
    clear_error();
    if (p) KC_CUDA(cudaFreeHost(p));
    return KC_OK;
}

int kc_device_alloc(void **p, size_t bytes, int device) {
    clear_error();
    if (!p) return fail(KC_ERR_INVALID, "null argument");
    KC_TRY(open_device(device));
    return dmalloc(p, bytes ? bytes : 1, "kc_device_alloc");
}

int kc_device_free(void *p) {
    clear_error();
    // ordered after earlier work on the legacy stream (e.g. a device-to-device
    // kc_memcpy), like every free of pool memory in this library
    if (p) {
        KC_CUDA(cudaFreeAsync(p, cudaStreamLegacy));
        KC_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
    }
    return KC_OK;
}

int kc_memcpy(void *dst, const void *src, size_t bytes, int kind) {
    clear_error();
    if (!bytes) return KC_OK;
    if (!dst || !src) return fail(KC_ERR_INVALID, "null argument");
    cudaMemcpyKind k = kind == 1 ? cudaMemcpyHostToDevice
                                 : (kind == 2 ? cudaMemcpyDeviceToHost : (kind == 3 ? cudaMemcpyDeviceToDevice : cudaMemcpyDefault));
    if (kind < 1 || kind > 3) return fail(KC_ERR_INVALID, "copy kind %d", kind);
    KC_CUDA(cudaMemcpy(dst, src, bytes, k));
    // a device-to-device cudaMemcpy may return before the copy is done
    if (kind == 3) KC_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
    return KC_OK;
}

int kc_device_synchronize(int device) {
    clear_error();
    KC_TRY(open_device(device));
    KC_CUDA(cudaDeviceSynchronize());
    return KC_OK;
}

int kc_gen_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c, uint64_t seed, uint32_t *d_src,
                uint32_t *d_dst, void *stream) {
    clear_error();
    return gen_rmat(scale, num_edges, a, b, c, seed, d_src, d_dst, static_cast<cudaStream_t>(stream));
}

int kc_gen_er(uint32_t n, uint64_t m, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, void *stream) {
    clear_error();
    return gen_er(n, m, seed, d_src, d_dst, static_cast<cudaStream_t>(stream));
}

int kc_gen_planted(uint32_t n, uint32_t k, double p, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, uint64_t cap,
                   uint64_t *m, void *stream) {
    clear_error();
    if (!m) return fail(KC_ERR_INVALID, "null argument");
    return gen_planted(n, k, p, seed, d_src, d_dst, cap, m, static_cast<cudaStream_t>(stream));
}

int kc_gen_rmat_bounded(uint32_t n, uint64_t num_edges, double a, double b, double c, uint64_t seed, uint32_t *d_src,
                        uint32_t *d_dst, void *stream) {
    clear_error();
    return gen_rmat_bounded(n, num_edges, a, b, c, seed, d_src, d_dst, static_cast<cudaStream_t>(stream));
}

int kc_gen_ba(uint32_t n, uint32_t d, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, void *stream) {
    clear_error();
    return gen_ba(n, d, seed, d_src, d_dst, static_cast<cudaStream_t>(stream));
}

int kc_edges_offset(uint32_t *d_src, uint32_t *d_dst, uint64_t m, uint32_t offset, void *stream) {
    clear_error();
    return edges_offset(d_src, d_dst, m, offset, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
