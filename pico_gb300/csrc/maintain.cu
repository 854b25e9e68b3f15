// Exact core maintenance for batches of edge insertions and deletions.
//
// The reference has no edge-update path (its "dyn" drivers only use dynamic
// work queues); this subsystem is new.  Core numbers stay exact:
//   * the CSR is rewritten in one streaming pass per change set: every row
//     keeps its entries minus the deleted ones plus the inserted ones, sorted
//     (binary searches in the small per-row change lists give every entry's
//     output position directly);
//   * deletions: cores only decrease, so the old cores are upper bounds; the
//     h-index iteration restarts from them with the endpoints of the deleted
//     edges active and converges to the new cores (only vertices whose
//     neighbourhood changed are revisited);
//   * insertions are split into matchings (greedy edge colouring on the
//     host).  Inserting a matching M raises a core by at most one: the
//     (k+1)-core of G+M minus M has minimum degree >= k, so it lies in the
//     k-core of G.  A vertex can rise only if it is reachable from a
//     lower-core endpoint of an edge of M through vertices of its own old core
//     (otherwise its component together with the (k+1)-core of G would already
//     be a (k+1)-core of G).  Those vertices are found by a BFS, raised to
//     min(core + 1, degree), and the h-index iteration settles them;
//   * batches above a size threshold (a larger one for batches of deletions
//     only) are applied in one rewrite and followed by a full decomposition,
//     which is cheaper than many rounds.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

static int grid_of(const Graph *g, uint64_t items) {
    uint64_t b = (items + 255) / 256;
    uint64_t cap = (uint64_t)std::max(g->sm_count, 1) * 16;
    return (int)std::max<uint64_t>(1, std::min(b, cap));
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *a, uint32_t len, uint32_t x) {
    uint32_t lo = 0, hi = len;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Every row: new length = old length, no changes yet; flags the rows that
// the change lists touch.
__global__ void mark_changed(const int64_t *__restrict__ rowptr, uint32_t n, const int64_t *__restrict__ drp,
                             const int64_t *__restrict__ irp, uint32_t *dcnt, uint32_t *icnt, uint32_t *newlen,
                             uint32_t *flag) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        newlen[v] = (uint32_t)(rowptr[v + 1] - rowptr[v]);
        if (dcnt) dcnt[v] = 0;
        if (icnt) icnt[v] = 0;
        const bool ch = (drp && drp[v + 1] != drp[v]) || (irp && irp[v + 1] != irp[v]);
        flag[v] = ch ? 1u : 0u;
    }
}

__global__ void list_changed(const uint32_t *__restrict__ flag, const int64_t *__restrict__ pos, uint32_t n,
                             uint32_t *changed) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        if (flag[v]) changed[pos[v]] = (uint32_t)v;
}

// Plans the changed rows (one warp per listed row): positions of deleted
// entries, inserted values not already present, new row lengths.
__global__ void merge_plan(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col,
                           const uint32_t *__restrict__ changed, uint32_t nchanged,
                           const int64_t *__restrict__ drp, const uint32_t *__restrict__ dcol,
                           const int64_t *__restrict__ irp, const uint32_t *__restrict__ icol, uint32_t *dpos,
                           uint32_t *dcnt, uint32_t *ival, uint32_t *icnt, uint32_t *newlen,
                           unsigned long long *applied) {
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long nd = 0, ni = 0;
    for (uint64_t ci = warp; ci < nchanged; ci += nw) {
        const uint32_t v = changed[ci];
        const int64_t r0 = rowptr[v];
        const uint32_t len = (uint32_t)(rowptr[v + 1] - r0);
        const int64_t d0 = drp ? drp[v] : 0, i0 = irp ? irp[v] : 0;
        const uint32_t dl = drp ? (uint32_t)(drp[v + 1] - d0) : 0u;
        const uint32_t il = irp ? (uint32_t)(irp[v + 1] - i0) : 0u;
        if (dl == 0 && il == 0) {
            if (lane == 0) {
                newlen[v] = len;
                if (dcnt) dcnt[v] = 0;
                if (icnt) icnt[v] = 0;
            }
            continue;
        }
        const uint32_t *row = col + r0;
        uint32_t wd = 0, wi = 0;
        for (uint32_t b = 0; b < dl; b += 32) {
            const uint32_t j = b + lane;
            bool del = false;
            uint32_t p = 0;
            if (j < dl) {
                const uint32_t x = dcol[d0 + j];
                p = lower_bound_u32(row, len, x);
                del = p < len && row[p] == x;
                if (del && il) {
                    const uint32_t q = lower_bound_u32(icol + i0, il, x);
                    if (q < il && icol[i0 + q] == x) del = false;  // deleted and re-inserted: keep
                }
            }
            const unsigned m = __ballot_sync(KC_FULL_MASK, del);
            if (del) dpos[d0 + wd + __popc(m & ((1u << lane) - 1u))] = p;
            wd += __popc(m);
        }
        for (uint32_t b = 0; b < il; b += 32) {
            const uint32_t j = b + lane;
            bool ins = false;
            uint32_t x = 0;
            if (j < il) {
                x = icol[i0 + j];
                const uint32_t p = lower_bound_u32(row, len, x);
                ins = !(p < len && row[p] == x);
            }
            const unsigned m = __ballot_sync(KC_FULL_MASK, ins);
            if (ins) ival[i0 + wi + __popc(m & ((1u << lane) - 1u))] = x;
            wi += __popc(m);
        }
        if (lane == 0) {
            if (dcnt) dcnt[v] = wd;
            if (icnt) icnt[v] = wi;
            newlen[v] = len - wd + wi;
        }
        nd += wd;
        ni += wi;
    }
    if (lane == 0 && (nd || ni)) {
        atomicAdd(&applied[0], nd);
        atomicAdd(&applied[1], ni);
    }
}

// Phase 2, one warp per row: write the merged, sorted row.
// Runs of unchanged rows between consecutive changed rows: run j covers
// rows changed[j-1]+1 .. changed[j]-1 (changed[-1] = -1, changed[R] = n);
// its old entries [ra, rb) move by rd.
__global__ void make_runs(const int64_t *__restrict__ rowptr, const int64_t *__restrict__ nrow,
                          const uint32_t *__restrict__ changed, uint32_t R, uint32_t n, int64_t *ra, int64_t *rb,
                          int64_t *rd) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j <= R; j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t first = j ? changed[j - 1] + 1 : 0u;
        const uint32_t end = j < R ? changed[j] : n;
        ra[j] = rowptr[first];
        rb[j] = rowptr[end > first ? end : first];
        rd[j] = nrow[first] - rowptr[first];
    }
}

// Bulk move of the unchanged rows: each CTA copies one tile of the old column
// array, run by run (runs are ordered and usually span many tiles).
constexpr uint64_t RUN_TILE = 8192;
__global__ void copy_runs(const uint32_t *__restrict__ col, uint64_t nnz_old, const int64_t *__restrict__ ra,
                          const int64_t *__restrict__ rb, const int64_t *__restrict__ rd, uint32_t R,
                          uint32_t *ncol) {
    for (uint64_t t0 = blockIdx.x * RUN_TILE; t0 < nnz_old; t0 += (uint64_t)gridDim.x * RUN_TILE) {
        const uint64_t t1 = t0 + RUN_TILE < nnz_old ? t0 + RUN_TILE : nnz_old;
        // first run ending after t0
        uint32_t lo = 0, hi = R + 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if ((uint64_t)rb[mid] <= t0) lo = mid + 1;
            else hi = mid;
        }
        for (uint32_t j = lo; j <= R && (uint64_t)ra[j] < t1; j++) {
            const uint64_t a = (uint64_t)ra[j] > t0 ? (uint64_t)ra[j] : t0;
            const uint64_t b = (uint64_t)rb[j] < t1 ? (uint64_t)rb[j] : t1;
            const int64_t d = rd[j];
            for (uint64_t e = a + threadIdx.x; e < b; e += blockDim.x) ncol[(int64_t)e + d] = col[e];
        }
    }
}

// The changed rows are written in chunks of MERGE_CHUNK old entries, one warp
// per chunk, so a long row (deletions drawn from the edge set land on hub
// rows of 10^5 entries) spreads over many warps instead of holding one warp
// for the whole update.  nchunks[i] = chunks of changed row i (at least one,
// so that a row that only gains entries still writes them).
constexpr uint32_t MERGE_CHUNK = 1024;
__global__ void merge_chunk_counts(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ changed,
                                   uint32_t nchanged, uint32_t *nchunks) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nchanged;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = changed[i];
        const uint64_t len = (uint64_t)(rowptr[v + 1] - rowptr[v]);
        const uint64_t k = (len + MERGE_CHUNK - 1) / MERGE_CHUNK;
        nchunks[i] = (uint32_t)(k > 0 ? k : 1);
    }
}

// Chunk ci of the concatenated chunk lists (cstart: exclusive prefix of
// nchunks, cstart[nchanged] = total): kept old entries p of its range move to
// w0 + p - (deleted entries before p) + (inserted values below row[p]); the
// row's inserted values are shared out over its chunks.
__global__ void merge_write_chunks(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col,
                                   const uint32_t *__restrict__ changed, uint32_t nchanged,
                                   const int64_t *__restrict__ cstart, uint64_t nch,
                                   const int64_t *__restrict__ drp, const uint32_t *__restrict__ dpos,
                                   const uint32_t *__restrict__ dcnt, const int64_t *__restrict__ irp,
                                   const uint32_t *__restrict__ ival, const uint32_t *__restrict__ icnt,
                                   const int64_t *__restrict__ nrow, uint32_t *ncol) {
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t ci = warp; ci < nch; ci += nw) {
        // changed row of this chunk: the last i with cstart[i] <= ci
        uint32_t lo = 0, hi = nchanged;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if ((uint64_t)cstart[mid] <= ci) lo = mid;
            else hi = mid;
        }
        const uint32_t v = changed[lo];
        const uint32_t c = (uint32_t)(ci - (uint64_t)cstart[lo]);
        const uint32_t nc = (uint32_t)(cstart[lo + 1] - cstart[lo]);
        const int64_t r0 = rowptr[v];
        const uint32_t len = (uint32_t)(rowptr[v + 1] - r0);
        const int64_t w0 = nrow[v];
        const uint32_t dc = dcnt ? dcnt[v] : 0u, ic = icnt ? icnt[v] : 0u;
        const uint32_t *dp = dc ? dpos + drp[v] : nullptr;
        const uint32_t *iv = ic ? ival + irp[v] : nullptr;
        const uint32_t *row = col + r0;
        const uint32_t p_end = min(len, (c + 1) * MERGE_CHUNK);
        for (uint32_t p = c * MERGE_CHUNK + lane; p < p_end; p += 32) {
            const uint32_t x = row[p];
            const uint32_t before_d = dc ? lower_bound_u32(dp, dc, p) : 0u;
            if (before_d < dc && dp[before_d] == p) continue;  // deleted
            const uint32_t before_i = ic ? lower_bound_u32(iv, ic, x) : 0u;
            ncol[w0 + p - before_d + before_i] = x;
        }
        for (uint32_t j = c * 32 + lane; j < ic; j += nc * 32) {
            const uint32_t y = iv[j];
            const uint32_t lb = lower_bound_u32(row, len, y);
            const uint32_t before_d = dc ? lower_bound_u32(dp, dc, lb) : 0u;
            ncol[w0 + lb - before_d + j] = y;
        }
    }
}

// Rows sorted and without repeated neighbours (required by the merge).
// Counts entries that are not strictly above their predecessor in the same
// row.  Each CTA checks one tile of entries; the row starts falling in the
// tile are marked in shared memory first, so hub rows split over many CTAs.
constexpr uint64_t CHECK_TILE = 8192;
__global__ void rows_simple(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col, uint32_t n,
                            uint64_t nnz, unsigned long long *bad) {
    __shared__ uint32_t starts[CHECK_TILE / 32];
    __shared__ uint32_t first_row;
    unsigned long long b = 0;
    for (uint64_t t0 = blockIdx.x * CHECK_TILE; t0 < nnz; t0 += (uint64_t)gridDim.x * CHECK_TILE) {
        const uint64_t t1 = t0 + CHECK_TILE < nnz ? t0 + CHECK_TILE : nnz;
        for (unsigned i = threadIdx.x; i < CHECK_TILE / 32; i += blockDim.x) starts[i] = 0;
        if (threadIdx.x == 0) {
            // the last row starting at or before t0
            uint32_t lo = 0, hi = n;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if ((uint64_t)rowptr[mid] <= t0) lo = mid;
                else hi = mid - 1;
            }
            first_row = lo;
        }
        __syncthreads();
        for (uint64_t v = first_row + threadIdx.x; v < n && (uint64_t)rowptr[v] < t1; v += blockDim.x) {
            const uint64_t r = (uint64_t)rowptr[v];
            if (r >= t0) atomicOr(&starts[(r - t0) >> 5], 1u << ((r - t0) & 31));
        }
        __syncthreads();
        for (uint64_t e = t0 + threadIdx.x; e < t1; e += blockDim.x) {
            const uint64_t o = e - t0;
            const bool is_start = (starts[o >> 5] >> (o & 31)) & 1u;
            if (!is_start && e > 0) b += col[e] <= col[e - 1];
        }
        __syncthreads();
    }
    if (b) atomicAdd(bad, b);
}

// Roots of a matching: the endpoint(s) with the smaller old core.
__global__ void matching_roots(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t m,
                               const uint32_t *__restrict__ core, uint32_t *visited, uint32_t *out,
                               unsigned long long *out_len) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = src[i], b = dst[i];
        const uint32_t ca = core[a], cb = core[b];
        const uint32_t k = min(ca, cb);
        const uint32_t ends[2] = {a, b};
        const uint32_t cs[2] = {ca, cb};
        for (int t = 0; t < 2; t++) {
            if (cs[t] != k) continue;
            const uint32_t v = ends[t];
            const unsigned bit = 1u << (v & 31);
            if (atomicOr(&visited[v >> 5], bit) & bit) continue;
            out[atomicAdd(out_len, 1ull)] = v;
        }
    }
}

// One BFS level over edges joining vertices of equal old core; newly reached
// vertices go to the next frontier and to the candidate list.
__global__ void subcore_bfs(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col,
                            const uint32_t *__restrict__ core, const uint32_t *__restrict__ front, uint64_t flen,
                            uint32_t *visited, uint32_t *next, unsigned long long *next_len, uint32_t *cand,
                            unsigned long long *cand_len) {
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = warp; i < flen; i += nw) {
        const uint32_t v = front[i];
        const uint32_t k = core[v];
        for (int64_t e = rowptr[v] + lane; e < rowptr[v + 1]; e += 32) {
            const uint32_t u = col[e];
            if (core[u] != k) continue;
            const unsigned bit = 1u << (u & 31);
            if (__ldcg(&visited[u >> 5]) & bit) continue;
            if (atomicOr(&visited[u >> 5], bit) & bit) continue;
            next[atomicAdd(next_len, 1ull)] = u;
            cand[atomicAdd(cand_len, 1ull)] = u;
        }
    }
}

// Raise candidates by one (at most to their degree): new upper bounds.
__global__ void raise_bounds(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ list, uint64_t len,
                             uint32_t *core) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = list[i];
        const uint32_t d = (uint32_t)(rowptr[v + 1] - rowptr[v]);
        core[v] = min(core[v] + 1u, d);
    }
}

// Endpoints of an edge list as a vertex list (duplicates allowed).
__global__ void endpoints(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t m,
                          uint32_t *out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        out[2 * i] = src[i];
        out[2 * i + 1] = dst[i];
    }
}

// Temporary device arrays freed on scope exit.
// Scratch arrays of one call, freed when the call returns (after the call's
// stream has finished with them, so an early error return cannot free memory
// that a launched kernel still uses).
struct Scratch {
    cudaStream_t stream = nullptr;
    std::vector<void *> ptrs;
    template <class T>
    int get(T **p, uint64_t count, const char *what) {
        int rc = dalloc(p, std::max<uint64_t>(count, 1), what);
        if (!rc) ptrs.push_back(*p);
        return rc;
    }
    ~Scratch() {
        if (stream && !ptrs.empty()) cudaStreamSynchronize(stream);
        for (void *p : ptrs) dfree(p);
    }
};

// Rewrites g's CSR: minus the edges of `del`, plus the edges of `ins` (both
// undirected edge lists on the device; either may be empty).  Counts the
// undirected edges actually deleted / inserted.
static int apply_changes(Graph *g, const uint32_t *d_isrc, const uint32_t *d_idst, uint64_t mi, const uint32_t *d_dsrc,
                         const uint32_t *d_ddst, uint64_t md, uint64_t *n_del, uint64_t *n_ins) {
    cudaStream_t s = g->stream;
    const uint32_t n = g->n;
    Graph dg, ig;  // per-row change lists, built like any graph
    dg.device = ig.device = g->device;
    dg.sm_count = ig.sm_count = g->sm_count;
    // the temporaries borrow g's stream only while they are built (their
    // destructor would otherwise destroy it)
    if (md) {
        dg.stream = s;
        const int rc = build_csr_from_edges(&dg, d_dsrc, d_ddst, md, n, KC_EDGES_DEDUP);
        dg.stream = nullptr;
        if (rc) return rc;
    }
    if (mi) {
        ig.stream = s;
        const int rc = build_csr_from_edges(&ig, d_isrc, d_idst, mi, n, KC_EDGES_DEDUP);
        ig.stream = nullptr;
        if (rc) return rc;
    }
    Scratch sc;
    sc.stream = s;
    uint32_t *dpos = nullptr, *dcnt = nullptr, *ival = nullptr, *icnt = nullptr, *newlen = nullptr;
    unsigned long long *applied = nullptr;
    if (md) {
        KC_TRY(sc.get(&dpos, dg.nnz, "deleted positions"));
        KC_TRY(sc.get(&dcnt, n, "deleted counts"));
    }
    if (mi) {
        KC_TRY(sc.get(&ival, ig.nnz, "inserted values"));
        KC_TRY(sc.get(&icnt, n, "inserted counts"));
    }
    KC_TRY(sc.get(&newlen, n, "new row lengths"));
    KC_TRY(sc.get(&applied, 2, "applied counts"));
    uint32_t *flag = nullptr;
    int64_t *cpos = nullptr;
    KC_TRY(sc.get(&flag, n, "changed-row flags"));
    KC_TRY(sc.get(&cpos, (uint64_t)n + 1, "changed-row positions"));
    KC_CUDA(cudaMemsetAsync(applied, 0, 16, s));
    const int64_t *drp = md ? dg.rowptr : nullptr, *irp = mi ? ig.rowptr : nullptr;
    // only the rows that the change lists touch are planned and rewritten
    // row by row; the others move as whole runs
    mark_changed<<<grid_of(g, n), 256, 0, s>>>(g->rowptr, n, drp, irp, dcnt, icnt, newlen, flag);
    KC_TRY(exclusive_scan_u32_i64(flag, cpos, n, s));
    int64_t R64 = 0;
    KC_CUDA(cudaMemcpyAsync(&R64, cpos + n, 8, cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    const uint32_t R = (uint32_t)R64;
    uint32_t *changed = nullptr;
    int64_t *ra = nullptr, *rb = nullptr, *rd = nullptr;
    KC_TRY(sc.get(&changed, (uint64_t)R + 1, "changed rows"));
    KC_TRY(sc.get(&ra, (uint64_t)R + 1, "run starts"));
    KC_TRY(sc.get(&rb, (uint64_t)R + 1, "run ends"));
    KC_TRY(sc.get(&rd, (uint64_t)R + 1, "run shifts"));
    list_changed<<<grid_of(g, n), 256, 0, s>>>(flag, cpos, n, changed);
    const int gw = grid_of(g, (uint64_t)std::max<uint32_t>(R, 1) * 32);
    if (R)
        merge_plan<<<gw, 256, 0, s>>>(g->rowptr, g->col, changed, R, drp, md ? dg.col : nullptr, irp,
                                      mi ? ig.col : nullptr, dpos, dcnt, ival, icnt, newlen, applied);
    // chunks of the changed rows for the merge
    uint32_t *nchunks = nullptr;
    int64_t *cstart = nullptr;
    KC_TRY(sc.get(&nchunks, (uint64_t)R + 1, "merge chunk counts"));
    KC_TRY(sc.get(&cstart, (uint64_t)R + 1, "merge chunk starts"));
    if (R) {
        merge_chunk_counts<<<grid_of(g, R), 256, 0, s>>>(g->rowptr, changed, R, nchunks);
        KC_TRY(exclusive_scan_u32_i64(nchunks, cstart, R, s));
    }
    int64_t *rp_new = nullptr;
    KC_TRY(dalloc(&rp_new, (uint64_t)n + 1, "row offsets"));
    int rc = exclusive_scan_u32_i64(newlen, rp_new, n, s);
    int64_t nnz_new = 0, nch = 0;
    if (!rc) {
        cudaMemcpyAsync(&nnz_new, rp_new + n, 8, cudaMemcpyDeviceToHost, s);
        if (R) cudaMemcpyAsync(&nch, cstart + R, 8, cudaMemcpyDeviceToHost, s);
        cudaError_t e0 = cudaStreamSynchronize(s);
        if (e0 != cudaSuccess) rc = fail(KC_ERR_CUDA, "CSR merge plan: %s", cudaGetErrorString(e0));
    }
    if (!rc) {
        uint32_t *col_new = nullptr;
        rc = dalloc(&col_new, (uint64_t)nnz_new + 1, "column ids");
        if (!rc) {
            make_runs<<<grid_of(g, (uint64_t)R + 1), 256, 0, s>>>(g->rowptr, rp_new, changed, R, n, ra, rb, rd);
            if (g->nnz) {
                const uint64_t tiles = (g->nnz + RUN_TILE - 1) / RUN_TILE;
                const int cb = (int)std::min<uint64_t>(tiles, (uint64_t)g->sm_count * 16);
                copy_runs<<<cb, 256, 0, s>>>(g->col, g->nnz, ra, rb, rd, R, col_new);
            }
            if (R && nch > 0)
                merge_write_chunks<<<grid_of(g, (uint64_t)nch * 32), 256, 0, s>>>(
                    g->rowptr, g->col, changed, R, cstart, (uint64_t)nch, drp, dpos, dcnt, irp, ival, icnt, rp_new,
                    col_new);
            unsigned long long h[2];
            cudaMemcpyAsync(h, applied, 16, cudaMemcpyDeviceToHost, s);
            cudaError_t e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                dfree(col_new);
                rc = fail(KC_ERR_CUDA, "CSR merge: %s", cudaGetErrorString(e));
            } else {
                dfree(g->rowptr);
                dfree(g->col);
                g->rowptr = rp_new;
                g->col = col_new;
                g->nnz = (uint64_t)nnz_new;
                rp_new = nullptr;
                *n_del = h[0] / 2;
                *n_ins = h[1] / 2;
            }
        }
    }
    dfree(rp_new);
    if (rc) return rc;
    return graph_finish(g);
}

static int ensure_maint(Graph *g) {
    if (!g->mfront[0]) {
        const uint64_t n = g->n;
        KC_TRY(dalloc(&g->mfront[0], n + 1, "bfs frontier"));
        KC_TRY(dalloc(&g->mfront[1], n + 1, "bfs frontier"));
        KC_TRY(dalloc(&g->mcand, n + 1, "candidates"));
        KC_TRY(dalloc(&g->mvisit, (n + 31) / 32 + 1, "bfs visited"));
        KC_TRY(dalloc(&g->mcount, 4, "bfs counters"));
    }
    return KC_OK;
}

// Subcore candidates of one inserted matching (already in the CSR); returns
// their number, the list in g->mcand.
static int subcore_candidates(Graph *g, const uint32_t *d_src, const uint32_t *d_dst, uint64_t m, uint64_t *count) {
    cudaStream_t s = g->stream;
    KC_TRY(ensure_maint(g));
    unsigned long long *lens = g->mcount;  // [0] frontier a, [1] frontier b, [2] candidates
    KC_CUDA(cudaMemsetAsync(g->mvisit, 0, (((uint64_t)g->n + 31) / 32) * 4, s));
    KC_CUDA(cudaMemsetAsync(lens, 0, 32, s));
    matching_roots<<<grid_of(g, m), 256, 0, s>>>(d_src, d_dst, m, g->core, g->mvisit, g->mfront[0], &lens[0]);
    unsigned long long flen = 0;
    KC_CUDA(cudaMemcpyAsync(&flen, &lens[0], 8, cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    // the roots are candidates too
    KC_CUDA(cudaMemcpyAsync(g->mcand, g->mfront[0], flen * 4, cudaMemcpyDeviceToDevice, s));
    unsigned long long total = flen;
    KC_CUDA(cudaMemcpyAsync(&lens[2], &total, 8, cudaMemcpyHostToDevice, s));
    int cur = 0;
    for (uint32_t level = 0; flen > 0; level++) {
        if (level > g->n) return fail(KC_ERR_CAPACITY, "subcore search did not terminate");
        const int nxt = cur ^ 1;
        KC_CUDA(cudaMemsetAsync(&lens[nxt], 0, 8, s));
        subcore_bfs<<<grid_of(g, flen * 32), 256, 0, s>>>(g->rowptr, g->col, g->core, g->mfront[cur], flen, g->mvisit,
                                                          g->mfront[nxt], &lens[nxt], g->mcand, &lens[2]);
        KC_CUDA(cudaMemcpyAsync(&flen, &lens[nxt], 8, cudaMemcpyDeviceToHost, s));
        KC_CUDA(cudaStreamSynchronize(s));
        cur = nxt;
    }
    KC_CUDA(cudaMemcpyAsync(&total, &lens[2], 8, cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    *count = total;
    return KC_OK;
}

int graph_update(Graph *g, const uint32_t *ins_src, const uint32_t *ins_dst, uint64_t n_ins, const uint32_t *del_src,
                 const uint32_t *del_dst, uint64_t n_del, kc_update_stats *st) {
    cudaStream_t s = g->stream;
    const auto t0 = std::chrono::steady_clock::now();
    kc_update_stats out;
    memset(&out, 0, sizeof(out));
    const uint32_t n = g->n;
    // deletions alone need no matching rounds: the h-index iteration from the
    // old cores beats a full decomposition up to a few hundred thousand edges
    // (R-MAT 22: 10^3 2.0 vs 8.4 ms, 10^5 6.3 vs 8.9 ms, 10^6 11.2 vs 10.6 ms)
    const bool incremental = n_ins + n_del <= (uint64_t)g->tune.update_incremental_max ||
                             (n_ins == 0 && n_del <= (uint64_t)g->tune.update_deletion_incremental_max);
    // The incremental path applies the deletions before it colours the
    // insertions on the host (which indexes per-vertex arrays), so it checks
    // every id first; the full path builds both change lists on the device,
    // which rejects ids >= n before the graph is rewritten.
    if (incremental) {
        for (uint64_t i = 0; i < n_ins; i++)
            if (ins_src[i] >= n || ins_dst[i] >= n) return fail(KC_ERR_INVALID, "inserted edge endpoint >= n");
        for (uint64_t i = 0; i < n_del; i++)
            if (del_src[i] >= n || del_dst[i] >= n) return fail(KC_ERR_INVALID, "deleted edge endpoint >= n");
    }
    if (!g->simple_checked) {
        unsigned long long *bad = nullptr;
        KC_TRY(dalloc(&bad, 1, "row check"));
        cudaMemsetAsync(bad, 0, 8, s);
        if (n && g->nnz) {
            const uint64_t tiles = (g->nnz + CHECK_TILE - 1) / CHECK_TILE;
            rows_simple<<<(int)std::min<uint64_t>(tiles, (uint64_t)g->sm_count * 16), 256, 0, s>>>(g->rowptr, g->col, n,
                                                                                                   g->nnz, bad);
        }
        unsigned long long hb = 0;
        cudaMemcpyAsync(&hb, bad, 8, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        dfree(bad);
        if (e != cudaSuccess) return fail(KC_ERR_CUDA, "row check: %s", cudaGetErrorString(e));
        if (hb) return fail(KC_ERR_UNSUPPORTED, "updates need sorted rows without parallel edges (build with KC_EDGES_DEDUP)");
        g->simple_checked = true;
    }
    if (!g->core_valid) KC_TRY(peel_run(g, s, false, nullptr));
    Scratch sc;
    sc.stream = s;
    uint32_t *d_del_s = nullptr, *d_del_d = nullptr;
    if (n_del) {
        KC_TRY(sc.get(&d_del_s, n_del, "deleted edges"));
        KC_TRY(sc.get(&d_del_d, n_del, "deleted edges"));
        KC_CUDA(cudaMemcpyAsync(d_del_s, del_src, n_del * 4, cudaMemcpyHostToDevice, s));
        KC_CUDA(cudaMemcpyAsync(d_del_d, del_dst, n_del * 4, cudaMemcpyHostToDevice, s));
    }
    if (!incremental) {
        uint32_t *d_is = nullptr, *d_id = nullptr;
        if (n_ins) {
            KC_TRY(sc.get(&d_is, n_ins, "inserted edges"));
            KC_TRY(sc.get(&d_id, n_ins, "inserted edges"));
            KC_CUDA(cudaMemcpyAsync(d_is, ins_src, n_ins * 4, cudaMemcpyHostToDevice, s));
            KC_CUDA(cudaMemcpyAsync(d_id, ins_dst, n_ins * 4, cudaMemcpyHostToDevice, s));
        }
        uint64_t nd = 0, ni = 0;
        KC_TRY(apply_changes(g, d_is, d_id, n_ins, d_del_s, d_del_d, n_del, &nd, &ni));
        KC_TRY(peel_run(g, s, false, nullptr));
        out.deleted = nd;
        out.inserted = ni;
        out.recomputed = 1;
    } else {
        if (n_del) {
            uint64_t nd = 0, ni = 0;
            KC_TRY(apply_changes(g, nullptr, nullptr, 0, d_del_s, d_del_d, n_del, &nd, &ni));
            out.deleted = nd;
            if (nd) {
                uint32_t *ends = nullptr;
                KC_TRY(sc.get(&ends, 2 * n_del, "deleted endpoints"));
                endpoints<<<grid_of(g, n_del), 256, 0, s>>>(d_del_s, d_del_d, n_del, ends);
                kc_stats hs;
                memset(&hs, 0, sizeof(hs));
                KC_TRY(hindex_run_from(g, ends, 2 * n_del, s, &hs));
                out.sweeps += hs.iterations;
            }
        }
        if (n_ins) {
            // greedy edge colouring: every colour class is a matching
            std::vector<uint32_t> color(n_ins), used;
            if (g->color_count.size() != n) g->color_count.assign(n, 0);
            uint32_t rounds = 0;
            for (uint64_t i = 0; i < n_ins; i++) {
                const uint32_t a = ins_src[i], b = ins_dst[i];
                if (a == b) {
                    color[i] = 0xffffffffu;
                    continue;
                }
                const uint32_t c = std::max(g->color_count[a], g->color_count[b]);
                color[i] = c;
                if (!g->color_count[a]) used.push_back(a);
                if (!g->color_count[b]) used.push_back(b);
                g->color_count[a] = g->color_count[b] = c + 1;
                rounds = std::max(rounds, c + 1);
            }
            for (uint32_t v : used) g->color_count[v] = 0;
            std::vector<uint64_t> cstart(rounds + 1, 0);
            for (uint64_t i = 0; i < n_ins; i++)
                if (color[i] != 0xffffffffu) cstart[color[i] + 1]++;
            for (uint32_t r = 0; r < rounds; r++) cstart[r + 1] += cstart[r];
            std::vector<uint32_t> hs_(cstart[rounds]), hd_(cstart[rounds]);
            std::vector<uint64_t> fill(cstart.begin(), cstart.end() - 1);
            for (uint64_t i = 0; i < n_ins; i++) {
                if (color[i] == 0xffffffffu) continue;
                const uint64_t p = fill[color[i]]++;
                hs_[p] = ins_src[i];
                hd_[p] = ins_dst[i];
            }
            uint32_t *d_is = nullptr, *d_id = nullptr;
            KC_TRY(sc.get(&d_is, hs_.size(), "inserted edges"));
            KC_TRY(sc.get(&d_id, hd_.size(), "inserted edges"));
            if (!hs_.empty()) {
                KC_CUDA(cudaMemcpyAsync(d_is, hs_.data(), hs_.size() * 4, cudaMemcpyHostToDevice, s));
                KC_CUDA(cudaMemcpyAsync(d_id, hd_.data(), hd_.size() * 4, cudaMemcpyHostToDevice, s));
            }
            for (uint32_t r = 0; r < rounds; r++) {
                const uint64_t m = cstart[r + 1] - cstart[r];
                if (!m) continue;
                uint64_t nd = 0, ni = 0;
                KC_TRY(apply_changes(g, d_is + cstart[r], d_id + cstart[r], m, nullptr, nullptr, 0, &nd, &ni));
                out.inserted += ni;
                out.rounds++;
                if (!ni) continue;
                uint64_t cands = 0;
                KC_TRY(subcore_candidates(g, d_is + cstart[r], d_id + cstart[r], m, &cands));
                out.candidates += cands;
                if (!cands) continue;
                raise_bounds<<<grid_of(g, cands), 256, 0, s>>>(g->rowptr, g->mcand, cands, g->core);
                kc_stats hs;
                memset(&hs, 0, sizeof(hs));
                KC_TRY(hindex_run_from(g, g->mcand, cands, s, &hs));
                out.sweeps += hs.iterations;
            }
        }
    }
    KC_CUDA(cudaStreamSynchronize(s));
    g->core_valid = true;
    out.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (st) *st = out;
    return KC_OK;
}

}  // namespace kc
