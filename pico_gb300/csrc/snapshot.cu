// Graph files and result extraction around the decomposition:
//   * a binary snapshot of a graph and its core numbers, checked by a content
//     hash on load (the reference's only cache is a text CSR keyed by the
//     input's basename, peel/src/graph.cpp:9-54,151, which silently reuses a
//     stale file when a different graph has the same name);
//   * binary edge-list input read through mmap (the fast input path for
//     graphs whose MatrixMarket text would take minutes to parse);
//   * the induced k-core subgraph of a decomposed graph, built on the device.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

namespace {

constexpr char SNAP_MAGIC[8] = {'K', 'C', 'S', 'N', 'A', 'P', '0', '1'};
constexpr uint32_t SNAP_VERSION = 1;
constexpr uint32_t SNAP_HAS_CORE = 1u;

struct SnapHeader {
    char magic[8];
    uint32_t version;
    uint32_t flags;
    uint64_t n;
    uint64_t nnz;
    uint64_t hash;  // of the payload bytes after the header
    uint64_t reserved[3];
};
static_assert(sizeof(SnapHeader) == 64, "snapshot header is 64 bytes");

// 64-bit hash of a byte range, one multiply-xor step per 8-byte word (the
// FNV-1a recurrence widened to words), computed over 64 MB blocks in parallel
// and folded in block order, so the result does not depend on the thread count.
uint64_t hash_words(const unsigned char *p, uint64_t len) {
    uint64_t h = 0xcbf29ce484222325ull;
    uint64_t i = 0;
    for (; i + 8 <= len; i += 8) {
        uint64_t w;
        std::memcpy(&w, p + i, 8);
        h = (h ^ w) * 0x100000001b3ull;
    }
    if (i < len) {
        uint64_t w = 0;
        std::memcpy(&w, p + i, len - i);
        h = (h ^ w) * 0x100000001b3ull;
    }
    return h ^ (h >> 29);
}

uint64_t content_hash(const std::vector<std::pair<const void *, uint64_t>> &parts) {
    constexpr uint64_t BLOCK = 64ull << 20;
    struct Piece {
        const unsigned char *p;
        uint64_t len;
    };
    std::vector<Piece> pieces;
    for (auto &pt : parts)
        for (uint64_t off = 0; off < pt.second; off += BLOCK)
            pieces.push_back({(const unsigned char *)pt.first + off, std::min(BLOCK, pt.second - off)});
    std::vector<uint64_t> hs(pieces.size());
    const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++)
        th.emplace_back([&, t] {
            for (size_t i = t; i < pieces.size(); i += nt) hs[i] = hash_words(pieces[i].p, pieces[i].len);
        });
    for (auto &x : th) x.join();
    uint64_t h = 0x84222325cbf29ce4ull;
    for (uint64_t x : hs) h = (h ^ x) * 0x100000001b3ull;
    return h;
}

struct Mapping {
    void *p = MAP_FAILED;
    size_t len = 0;
    int fd = -1;
    ~Mapping() {
        if (p != MAP_FAILED) munmap(p, len);
        if (fd >= 0) close(fd);
    }
};

int map_file(const char *path, Mapping &m) {
    m.fd = open(path, O_RDONLY);
    if (m.fd < 0) return fail(KC_ERR_IO, "cannot open %s", path);
    struct stat st;
    if (fstat(m.fd, &st) != 0) return fail(KC_ERR_IO, "cannot stat %s", path);
    m.len = (size_t)st.st_size;
    if (m.len == 0) return KC_OK;
    m.p = mmap(nullptr, m.len, PROT_READ, MAP_PRIVATE, m.fd, 0);
    if (m.p == MAP_FAILED) return fail(KC_ERR_IO, "cannot map %s", path);
    madvise(m.p, m.len, MADV_SEQUENTIAL);
    return KC_OK;
}

// ---- induced k-core subgraph --------------------------------------------

__global__ void kcore_flags(const uint32_t *__restrict__ core, uint32_t n, uint32_t k, uint32_t *keep) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        keep[v] = core[v] >= k ? 1u : 0u;
}

// one warp per kept vertex: its number of kept neighbours, and its old id
__global__ void kcore_count(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col,
                            const uint32_t *__restrict__ core, const int64_t *__restrict__ pos, uint32_t n, uint32_t k,
                            uint32_t *cnt, uint32_t *map) {
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t v = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        if (core[v] < k) continue;
        uint32_t c = 0;
        for (int64_t e = rowptr[v] + lane; e < rowptr[v + 1]; e += 32) c += core[col[e]] >= k ? 1u : 0u;
        c = __reduce_add_sync(KC_FULL_MASK, c);
        if (lane == 0) {
            cnt[pos[v]] = c;
            if (map) map[pos[v]] = (uint32_t)v;
        }
    }
}

// one warp per kept vertex: kept neighbours, renumbered, in row order
__global__ void kcore_write(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col,
                            const uint32_t *__restrict__ core, const int64_t *__restrict__ pos, uint32_t n, uint32_t k,
                            const int64_t *__restrict__ nrow, uint32_t *ncol) {
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t v = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        if (core[v] < k) continue;
        int64_t out = nrow[pos[v]];
        const int64_t r0 = rowptr[v], r1 = rowptr[v + 1];
        for (int64_t b = r0; b < r1; b += 32) {
            const int64_t e = b + lane;
            uint32_t u = 0;
            bool keepu = false;
            if (e < r1) {
                u = col[e];
                keepu = core[u] >= k;
            }
            const unsigned m = __ballot_sync(KC_FULL_MASK, keepu);
            if (keepu) ncol[out + __popc(m & ((1u << lane) - 1u))] = (uint32_t)pos[u];
            out += __popc(m);
        }
    }
}

}  // namespace

}  // namespace kc

using namespace kc;

extern "C" {

int kc_graph_save(const kc_graph *g, const char *path) {
    clear_error();
    NvtxRange nvtx_("kc_graph_save");
    if (!g || !path) return fail(KC_ERR_INVALID, "null argument");
    KC_CUDA(cudaSetDevice(g->device));
    KC_CUDA(cudaStreamSynchronize(g->stream));
    const uint64_t n = g->n, nnz = g->nnz;
    const bool with_core = g->core_valid && g->core;
    const uint64_t b_row = (n + 1) * 8, b_col = nnz * 4, pad = (8 - (b_col & 7)) & 7, b_core = with_core ? n * 4 : 0;
    // The file is sized first and mapped: the device copies land in its
    // pages directly (no zero-filled staging buffer, no second copy by a
    // write call), and the hash is taken from them.
    const uint64_t payload = b_row + b_col + pad + b_core;
    const uint64_t total = sizeof(SnapHeader) + payload;
    const int fd = open(path, O_RDWR | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return fail(KC_ERR_IO, "cannot create %s", path);
    if (ftruncate(fd, (off_t)total) != 0) {
        close(fd);
        return fail(KC_ERR_IO, "cannot size %s to %llu bytes", path, (unsigned long long)total);
    }
    void *map = mmap(nullptr, total, PROT_READ | PROT_WRITE, MAP_SHARED, fd, 0);
    if (map == MAP_FAILED) {
        close(fd);
        return fail(KC_ERR_IO, "cannot map %s for writing", path);
    }
    unsigned char *base = (unsigned char *)map + sizeof(SnapHeader);
    cudaError_t e = cudaMemcpy(base, g->rowptr, b_row, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && b_col) e = cudaMemcpy(base + b_row, g->col, b_col, cudaMemcpyDeviceToHost);
    if (pad) std::memset(base + b_row + b_col, 0, pad);
    if (e == cudaSuccess && b_core) e = cudaMemcpy(base + b_row + b_col + pad, g->core, b_core, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        munmap(map, total);
        close(fd);
        return fail(KC_ERR_CUDA, "snapshot download: %s", cudaGetErrorString(e));
    }
    SnapHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, SNAP_MAGIC, 8);
    h.version = SNAP_VERSION;
    h.flags = with_core ? SNAP_HAS_CORE : 0u;
    h.n = n;
    h.nnz = nnz;
    h.hash = content_hash({{base, payload}});
    std::memcpy(map, &h, sizeof(h));
    const bool ok = munmap(map, total) == 0;
    if (close(fd) != 0 || !ok) return fail(KC_ERR_IO, "write failed: %s", path);
    return KC_OK;
}

int kc_graph_load(const char *path, int device, kc_graph **out) {
    clear_error();
    NvtxRange nvtx_("kc_graph_load");
    if (!path || !out) return fail(KC_ERR_INVALID, "null argument");
    *out = nullptr;
    Mapping m;
    KC_TRY(map_file(path, m));
    if (m.len < sizeof(SnapHeader)) return fail(KC_ERR_IO, "%s: too short for a snapshot", path);
    SnapHeader h;
    std::memcpy(&h, m.p, sizeof(h));
    if (std::memcmp(h.magic, SNAP_MAGIC, 8) != 0) return fail(KC_ERR_IO, "%s: not a graph snapshot", path);
    if (h.version != SNAP_VERSION) return fail(KC_ERR_UNSUPPORTED, "%s: snapshot version %u", path, h.version);
    if (h.n >= 0xffffffffull) return fail(KC_ERR_IO, "%s: vertex count %llu", path, (unsigned long long)h.n);
    const uint64_t b_row = (h.n + 1) * 8, b_col = h.nnz * 4, pad = (8 - (b_col & 7)) & 7;
    const uint64_t b_core = (h.flags & SNAP_HAS_CORE) ? h.n * 4 : 0;
    const uint64_t payload = b_row + b_col + pad + b_core;
    if (m.len != sizeof(SnapHeader) + payload) return fail(KC_ERR_IO, "%s: size does not match its header", path);
    const unsigned char *base = (const unsigned char *)m.p + sizeof(SnapHeader);
    if (content_hash({{base, payload}}) != h.hash) return fail(KC_ERR_IO, "%s: content hash mismatch", path);
    const int64_t *rowptr = (const int64_t *)base;
    if (rowptr[0] != 0 || rowptr[h.n] != (int64_t)h.nnz) return fail(KC_ERR_IO, "%s: row offsets inconsistent", path);
    kc_graph *g = nullptr;
    KC_TRY(kc_graph_from_csr(rowptr, (const uint32_t *)(base + b_row), (uint32_t)h.n, device, &g));
    if (b_core) {
        int rc = dalloc(&g->core, h.n + 1, "core");
        if (!rc) {
            cudaError_t e = cudaMemcpy(g->core, base + b_row + b_col + pad, b_core, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) rc = fail(KC_ERR_CUDA, "core upload: %s", cudaGetErrorString(e));
        }
        if (rc) {
            delete g;
            return rc;
        }
        g->core_valid = true;
    }
    *out = g;
    return KC_OK;
}

int kc_graph_from_edge_file(const char *path, uint32_t flags, int device, kc_graph **out) {
    clear_error();
    NvtxRange nvtx_("kc_graph_from_edge_file");
    if (!path || !out) return fail(KC_ERR_INVALID, "null argument");
    *out = nullptr;
    Mapping m;
    KC_TRY(map_file(path, m));
    if (m.len % 8) return fail(KC_ERR_IO, "%s: size %zu is not a whole number of 8-byte edges", path, m.len);
    const uint64_t edges = m.len / 8;
    const uint32_t *pairs = edges ? (const uint32_t *)m.p : nullptr;
    // split into endpoint arrays and find the largest id, in parallel
    std::vector<uint32_t> src, dst;
    try {
        src.resize(std::max<uint64_t>(edges, 1));
        dst.resize(std::max<uint64_t>(edges, 1));
    } catch (...) {
        return fail(KC_ERR_NOMEM, "host endpoint arrays");
    }
    const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
    std::vector<uint32_t> mx(nt, 0);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++)
        th.emplace_back([&, t] {
            const uint64_t lo = edges * t / nt, hi = edges * (t + 1) / nt;
            uint32_t x = 0;
            for (uint64_t i = lo; i < hi; i++) {
                const uint32_t a = pairs[2 * i], b = pairs[2 * i + 1];
                src[i] = a;
                dst[i] = b;
                x = std::max(x, std::max(a, b));
            }
            mx[t] = x;
        });
    for (auto &x : th) x.join();
    const uint32_t maxid = *std::max_element(mx.begin(), mx.end());
    if (edges && maxid == 0xffffffffu) return fail(KC_ERR_UNSUPPORTED, "%s: id 2^32-1", path);
    const uint32_t n = edges ? maxid + 1 : 0;
    return kc_graph_from_edges(src.data(), dst.data(), edges, n, flags, device, out);
}

int kc_graph_kcore_subgraph(const kc_graph *g, uint32_t k, kc_graph **out, uint32_t *map_out, int map_on_device) {
    clear_error();
    NvtxRange nvtx_("kc_graph_kcore_subgraph");
    if (!g || !out) return fail(KC_ERR_INVALID, "null argument");
    *out = nullptr;
    if (!g->core_valid) return fail(KC_ERR_STATE, "no decomposition has completed on this graph");
    KC_CUDA(cudaSetDevice(g->device));
    cudaStream_t s = g->stream;
    const uint32_t n = g->n;
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g->sm_count * 8, (n + 255) / 256));
    uint32_t *keep = nullptr;
    int64_t *pos = nullptr;
    KC_TRY(dalloc(&keep, (uint64_t)n + 1, "k-core flags"));
    int rc = dalloc(&pos, (uint64_t)n + 1, "k-core positions");
    if (rc) {
        dfree(keep);
        return rc;
    }
    kcore_flags<<<blocks, 256, 0, s>>>(g->core, n, k, keep);
    rc = exclusive_scan_u32_i64(keep, pos, n, s);
    int64_t nk = 0;
    if (!rc) {
        cudaMemcpyAsync(&nk, pos + n, 8, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(KC_ERR_CUDA, "k-core scan: %s", cudaGetErrorString(e));
    }
    kc_graph *h = nullptr;
    if (!rc) rc = [&]() -> int {
        KC_TRY(graph_new(g->device, &h));
        h->n = (uint32_t)nk;
        uint32_t *map = nullptr;
        KC_TRY(dalloc(&h->rowptr, (uint64_t)nk + 1, "row offsets"));
        // the per-vertex counts go into the keep array (no longer needed)
        if (map_out) KC_TRY(dalloc(&map, (uint64_t)nk + 1, "k-core map"));
        KC_CUDA(cudaMemsetAsync(keep, 0, ((uint64_t)nk + 1) * 4, s));
        const int wblocks =
            (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g->sm_count * 16, ((uint64_t)n * 32 + 255) / 256));
        kcore_count<<<wblocks, 256, 0, s>>>(g->rowptr, g->col, g->core, pos, n, k, keep, map);
        int r2 = exclusive_scan_u32_i64(keep, h->rowptr, (uint64_t)nk, s);
        if (r2) {
            cudaStreamSynchronize(s);
            dfree(map);
            return r2;
        }
        int64_t nnz = 0;
        cudaMemcpyAsync(&nnz, h->rowptr + nk, 8, cudaMemcpyDeviceToHost, s);
        KC_CUDA(cudaStreamSynchronize(s));
        h->nnz = (uint64_t)nnz;
        r2 = dalloc(&h->col, h->nnz + 1, "column ids");
        if (r2) {
            cudaStreamSynchronize(s);
            dfree(map);
            return r2;
        }
        kcore_write<<<wblocks, 256, 0, s>>>(g->rowptr, g->col, g->core, pos, n, k, h->rowptr, h->col);
        if (map_out && nk)
            cudaMemcpyAsync(map_out, map, (uint64_t)nk * 4, map_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            s);
        cudaError_t e = cudaStreamSynchronize(s);
        dfree(map);
        if (e != cudaSuccess) return fail(KC_ERR_CUDA, "k-core extraction: %s", cudaGetErrorString(e));
        return graph_finish(h);
    }();
    cudaStreamSynchronize(s);  // nothing of this call may still use the scratch arrays
    dfree(keep);
    dfree(pos);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return KC_OK;
}

}  // extern "C"
