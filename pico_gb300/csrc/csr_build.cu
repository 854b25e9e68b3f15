// Device CSR / virtual-graph builder.
//
// Replaces the reference's serial host builders: VirtualGraph::VirtualGraph +
// MakeUGraph (index2core/shared/virtual_graph.cpp:12-45, 96-192) and the
// std::set adjacency of Graph::readFile (peel/src/graph.cpp:103-131).  Steps,
// all on the GPU:
//   1. degree count (atomicAdd per endpoint; self-loops dropped, ids checked),
//   2. exclusive scan of degrees into int64 row offsets,
//   3. scatter of both directions of every edge into its row,
//   4. segmented row sort -- by neighbour id (dedup / sorted rows) or by the
//      entry's position in the edge list (the row order MakeUGraph produces),
//      with three size classes: <=32 entries (one warp, register bitonic),
//      <=4096 (one CTA, shared-memory bitonic), larger (one CTA, stable LSD
//      radix through a global staging buffer),
//   5. optional unique per row, rescan and compaction.
#include <algorithm>
#include <vector>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

static int grid_for(uint64_t items, int threads, int sm_count) {
    uint64_t g = (items + threads - 1) / threads;
    uint64_t cap = (uint64_t)std::max(sm_count, 1) * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

static int current_sms() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

// ---------------------------------------------------------------- scan ----
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ unsigned long long block_excl_scan_u64(unsigned long long x,
                                                                  unsigned long long *warp_sums,
                                                                  unsigned long long &total) {
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long v = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        unsigned long long y = __shfl_up_sync(KC_FULL_MASK, v, d);
        if (lane >= (unsigned)d) v += y;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0ull;
        unsigned long long iv = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            unsigned long long y = __shfl_up_sync(KC_FULL_MASK, iv, d);
            if (lane >= (unsigned)d) iv += y;
        }
        if (lane < (blockDim.x >> 5)) warp_sums[lane] = iv - w;
        if (lane == 31) warp_sums[32] = iv;
    }
    __syncthreads();
    unsigned long long r = warp_sums[warp] + v - x;
    total = warp_sums[32];
    __syncthreads();
    return r;
}

__global__ void scan_tile_sums(const uint32_t *__restrict__ in, uint64_t n, unsigned long long *sums) {
    __shared__ unsigned long long ws[33];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    unsigned long long s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        uint64_t j = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        if (j < n) s += in[j];
    }
    unsigned long long tot;
    block_excl_scan_u64(s, ws, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void scan_sums_single(unsigned long long *sums, uint64_t count) {
    __shared__ unsigned long long ws[33];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < count; base += blockDim.x) {
        uint64_t j = base + threadIdx.x;
        unsigned long long x = j < count ? sums[j] : 0ull;
        unsigned long long tot;
        unsigned long long ex = block_excl_scan_u64(x, ws, tot);
        if (j < count) sums[j] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[count] = carry;
}

__global__ void scan_tile_apply(const uint32_t *__restrict__ in, int64_t *__restrict__ out, uint64_t n,
                                const unsigned long long *sums) {
    __shared__ unsigned long long ws[33];
    __shared__ uint32_t tile[SCAN_TILE];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
        uint64_t j = base + i;
        tile[i] = j < n ? in[j] : 0u;
    }
    __syncthreads();
    unsigned long long loc[SCAN_ITEMS];
    unsigned long long s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        loc[i] = s;
        s += tile[threadIdx.x * SCAN_ITEMS + i];
    }
    unsigned long long tot;
    unsigned long long ex = block_excl_scan_u64(s, ws, tot);
    unsigned long long off = sums[blockIdx.x] + ex;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        uint64_t j = base + (uint64_t)threadIdx.x * SCAN_ITEMS + i;
        if (j < n) out[j] = (int64_t)(off + loc[i]);
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        uint64_t tiles = gridDim.x;
        out[n] = (int64_t)sums[tiles];
    }
}

// out[0..n] = exclusive prefix of in[0..n), out[n] = total.
int exclusive_scan_u32_i64(const uint32_t *d_in, int64_t *d_out, uint64_t n, cudaStream_t s) {
    uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 0) {
        KC_CUDA(cudaMemsetAsync(d_out, 0, sizeof(int64_t), s));
        return KC_OK;
    }
    unsigned long long *sums = nullptr;
    KC_TRY(dalloc(&sums, tiles + 1, "scan sums"));
    scan_tile_sums<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(d_in, n, sums);
    scan_sums_single<<<1, 1024, 0, s>>>(sums, tiles);
    scan_tile_apply<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(d_in, d_out, n, sums);
    cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(s);
    dfree(sums);
    if (e != cudaSuccess) return fail(KC_ERR_CUDA, "scan launch: %s", cudaGetErrorString(e));
    return KC_OK;
}

// ------------------------------------------------------- count/scatter ----
__global__ void count_degrees(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t m,
                              uint32_t n, uint32_t *deg, unsigned int *err) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t a = src[i], b = dst[i];
        if (a >= n || b >= n) {
            atomicCAS(err, 0u, 1u);
            continue;
        }
        if (a == b) continue;
        atomicAdd(&deg[a], 1u);
        atomicAdd(&deg[b], 1u);
    }
}

// cur: 64-bit row cursors preset to the row offsets, so one atomic gives an
// entry's position with no row-offset read (random 8-byte reads of rowptr
// were a third of this kernel's gathers: 8% of the C3 build measured).
__global__ void scatter_edges(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t m,
                              uint32_t n, unsigned long long *cur, uint32_t *col, uint32_t *key) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t a = src[i], b = dst[i];
        if (a >= n || b >= n || a == b) continue;
        const unsigned long long pa = atomicAdd(&cur[a], 1ull);
        const unsigned long long pb = atomicAdd(&cur[b], 1ull);
        col[pa] = b;
        col[pb] = a;
        if (key) {
            key[pa] = (uint32_t)(2 * i);
            key[pb] = (uint32_t)(2 * i + 1);
        }
    }
}

// ------------------------------------------------------ segmented sort ----
// Rows are sorted by size class: up to 32 entries one warp per row (shuffle
// bitonic network); 33..4096 entries padded to P = 2^k (k = 6..12) and sorted
// SORT_PACK / P rows at a time per CTA in shared memory (one bitonic network,
// so short rows share the barriers instead of occupying a CTA each); longer
// rows one CTA per row with an LSD radix sort.
constexpr uint32_t CLASS_A_MAX = 32;
constexpr uint32_t CLASS_B_MAX = 4096;
constexpr int SORT_BUCKETS = 9;  // 0: <= 32; 1..7: P = 64..4096; 8: > 4096
constexpr uint32_t SORT_PACK = 1024;

__device__ __forceinline__ int sort_bucket(int64_t len) {
    if (len < 2) return -1;
    if (len <= (int64_t)CLASS_A_MAX) return 0;
    if (len > (int64_t)CLASS_B_MAX) return SORT_BUCKETS - 1;
    int k = 6;
    while (((int64_t)1 << k) < len) k++;
    return k - 5;  // 64 -> 1, ..., 4096 -> 7
}

// Pass 1 (cursor == nullptr): rows per bucket into counts.  Pass 2: each row
// id goes to list[cursor[bucket]++] (cursors start at the buckets' offsets).
__global__ void classify_rows(const int64_t *__restrict__ rowptr, uint32_t n, unsigned long long *counts,
                              unsigned long long *cursor, uint32_t *list) {
    const unsigned lane = threadIdx.x & 31;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < n; base += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v = base + threadIdx.x;
        const int cls = v < n ? sort_bucket(rowptr[v + 1] - rowptr[v]) : -1;
        for (int c = 0; c < SORT_BUCKETS; c++) {
            const unsigned b = __ballot_sync(KC_FULL_MASK, cls == c);
            if (!b) continue;
            unsigned long long pos = 0;
            if (lane == 0) pos = atomicAdd(cursor ? &cursor[c] : &counts[c], (unsigned long long)__popc(b));
            pos = __shfl_sync(KC_FULL_MASK, pos, 0);
            if (cursor && cls == c) list[pos + __popc(b & ((1u << lane) - 1))] = (uint32_t)v;
        }
    }
}

// (k, v) lexicographic compare; v is ignored when HAS_VAL is false.
template <bool HAS_VAL>
__device__ __forceinline__ bool kv_less(uint32_t ka, uint32_t va, uint32_t kb, uint32_t vb) {
    if (HAS_VAL) return ka < kb || (ka == kb && va < vb);
    return ka < kb;
}

// Class A: one warp per row of <= 32 entries, bitonic network over shuffles.
template <bool HAS_VAL>
__global__ void sort_rows_warp(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ rows,
                               uint64_t nrows, uint32_t *key, uint32_t *val) {
    const unsigned lane = threadIdx.x & 31;
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = warp; r < nrows; r += nwarps) {
        uint32_t v = rows[r];
        int64_t start = rowptr[v];
        uint32_t len = (uint32_t)(rowptr[v + 1] - start);
        uint32_t k = lane < len ? key[start + lane] : 0xffffffffu;
        uint32_t x = (HAS_VAL && lane < len) ? val[start + lane] : 0xffffffffu;
#pragma unroll
        for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                uint32_t pk = __shfl_xor_sync(KC_FULL_MASK, k, stride);
                uint32_t px = HAS_VAL ? __shfl_xor_sync(KC_FULL_MASK, x, stride) : 0u;
                bool asc = (lane & size) == 0 || size == 32;
                bool lower = (lane & stride) == 0;
                bool p_less = kv_less<HAS_VAL>(pk, px, k, x);
                bool p_greater = kv_less<HAS_VAL>(k, x, pk, px);
                bool take = (lower == asc) ? p_less : p_greater;
                if (take) {
                    k = pk;
                    x = px;
                }
            }
        }
        if (lane < len) {
            key[start + lane] = k;
            if (HAS_VAL) val[start + lane] = x;
        }
    }
}

// Class B: rows of P/2 < len <= P entries (P = 2^LOGP, 64..4096), padded to
// P with the largest key, SORT_PACK / P rows per CTA (one row for P > 1024).
template <bool HAS_VAL, int LOGP>
__global__ void __launch_bounds__(256) sort_rows_pack(const int64_t *__restrict__ rowptr,
                                                      const uint32_t *__restrict__ rows, uint64_t nrows,
                                                      uint32_t *key, uint32_t *val) {
    constexpr uint32_t P = 1u << LOGP;
    constexpr uint32_t E = P > SORT_PACK ? P : SORT_PACK;  // elements per CTA
    constexpr uint32_t RPC = E / P;                          // rows per CTA
    __shared__ uint32_t sk[E];
    __shared__ uint32_t sv[HAS_VAL ? E : 1];
    __shared__ int64_t rstart[RPC];
    __shared__ uint32_t rlen[RPC];
    for (uint64_t grp = blockIdx.x; grp * RPC < nrows; grp += gridDim.x) {
        if (threadIdx.x < RPC) {
            const uint64_t r = grp * RPC + threadIdx.x;
            if (r < nrows) {
                const uint32_t v = rows[r];
                rstart[threadIdx.x] = rowptr[v];
                rlen[threadIdx.x] = (uint32_t)(rowptr[v + 1] - rowptr[v]);
            } else {
                rstart[threadIdx.x] = 0;
                rlen[threadIdx.x] = 0;
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < E; i += blockDim.x) {
            const uint32_t j = i / P, o = i % P;
            const bool in = o < rlen[j];
            sk[i] = in ? key[rstart[j] + o] : 0xffffffffu;
            if (HAS_VAL) sv[i] = in ? val[rstart[j] + o] : 0xffffffffu;
        }
        __syncthreads();
        for (uint32_t size = 2; size <= P; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (uint32_t q = threadIdx.x; q < E / 2; q += blockDim.x) {
                    const uint32_t i = 2 * stride * (q / stride) + (q % stride);
                    const uint32_t j = i + stride;
                    const bool asc = ((i & (P - 1)) & size) == 0;
                    const uint32_t ki = sk[i], kj = sk[j];
                    const uint32_t vi = HAS_VAL ? sv[i] : 0u, vj = HAS_VAL ? sv[j] : 0u;
                    const bool sw = asc ? kv_less<HAS_VAL>(kj, vj, ki, vi) : kv_less<HAS_VAL>(ki, vi, kj, vj);
                    if (sw) {
                        sk[i] = kj;
                        sk[j] = ki;
                        if (HAS_VAL) {
                            sv[i] = vj;
                            sv[j] = vi;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t i = threadIdx.x; i < E; i += blockDim.x) {
            const uint32_t j = i / P, o = i % P;
            if (o < rlen[j]) {
                key[rstart[j] + o] = sk[i];
                if (HAS_VAL) val[rstart[j] + o] = sv[i];
            }
        }
        __syncthreads();
    }
}

// Class C: one CTA per long row, stable LSD radix sort with 8-bit digits.
// Ping-pongs between the row and the same range of the staging arrays
// (tk, tv), one pass per digit, and copies back after an odd pass count.
constexpr int RADIX_THREADS = 256;
constexpr int RADIX_WARPS = RADIX_THREADS / 32;

template <bool HAS_VAL>
__global__ void __launch_bounds__(RADIX_THREADS) sort_rows_radix(const int64_t *__restrict__ rowptr,
                                                                 const uint32_t *__restrict__ rows, uint64_t nrows,
                                                                 uint32_t *key, uint32_t *val, uint32_t *tk,
                                                                 uint32_t *tv, int passes) {
    __shared__ uint32_t hist[256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[RADIX_WARPS][256];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t r = blockIdx.x; r < nrows; r += gridDim.x) {
        uint32_t v = rows[r];
        int64_t start = rowptr[v];
        uint32_t len = (uint32_t)(rowptr[v + 1] - start);
        uint32_t *ik = key + start, *iv = HAS_VAL ? val + start : nullptr;
        uint32_t *ok = tk + start, *ov = HAS_VAL ? tv + start : nullptr;
        for (int pass = 0; pass < passes; pass++) {
            int shift = 8 * pass;
            for (int i = threadIdx.x; i < 256; i += RADIX_THREADS) hist[i] = 0;
            __syncthreads();
            for (uint32_t j = threadIdx.x; j < len; j += RADIX_THREADS) atomicAdd(&hist[(ik[j] >> shift) & 255u], 1u);
            __syncthreads();
            if (warp == 0) {
                uint32_t loc[8];
                uint32_t s = 0;
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    loc[i] = s;
                    s += hist[lane * 8 + i];
                }
                uint32_t tot;
                uint32_t ex = warp_excl_scan(s, lane, tot);
#pragma unroll
                for (int i = 0; i < 8; i++) base[lane * 8 + i] = ex + loc[i];
            }
            __syncthreads();
            for (uint32_t tile = 0; tile < len; tile += RADIX_THREADS) {
                for (int i = threadIdx.x; i < RADIX_WARPS * 256; i += RADIX_THREADS) (&wcnt[0][0])[i] = 0;
                __syncthreads();
                uint32_t j = tile + threadIdx.x;
                bool valid = j < len;
                uint32_t kk = valid ? ik[j] : 0u;
                uint32_t vv = (HAS_VAL && valid) ? iv[j] : 0u;
                uint32_t d = valid ? ((kk >> shift) & 255u) : 256u;
                unsigned int peers = __match_any_sync(KC_FULL_MASK, d);
                uint32_t rank = __popc(peers & ((1u << lane) - 1u));
                if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
                __syncthreads();
                if (valid) {
                    uint32_t before = 0;
                    for (unsigned w = 0; w < warp; w++) before += wcnt[w][d];
                    uint32_t dest = base[d] + before + rank;
                    ok[dest] = kk;
                    if (HAS_VAL) ov[dest] = vv;
                }
                __syncthreads();
                for (int dd = threadIdx.x; dd < 256; dd += RADIX_THREADS) {
                    uint32_t t = 0;
                    for (int w = 0; w < RADIX_WARPS; w++) t += wcnt[w][dd];
                    base[dd] += t;
                }
                __syncthreads();
            }
            uint32_t *t0 = ik; ik = ok; ok = t0;
            if (HAS_VAL) { uint32_t *t1 = iv; iv = ov; ov = t1; }
            __syncthreads();
        }
        if (passes & 1) {
            // result sits in the staging range: copy back into the row
            for (uint32_t j = threadIdx.x; j < len; j += RADIX_THREADS) {
                key[start + j] = tk[start + j];
                if (HAS_VAL) val[start + j] = tv[start + j];
            }
        }
        __syncthreads();
    }
}

template <bool HAS_VAL>
static void launch_pack(int logp, const int64_t *rowptr, const uint32_t *rows, uint64_t nrows, uint32_t *key,
                        uint32_t *val, int sms, cudaStream_t s) {
    const uint64_t rpc = logp >= 10 ? 1 : (SORT_PACK >> logp);
    const int gr = (int)std::max<uint64_t>(1, std::min<uint64_t>((nrows + rpc - 1) / rpc, (uint64_t)sms * 8));
    switch (logp) {
    case 6: sort_rows_pack<HAS_VAL, 6><<<gr, 256, 0, s>>>(rowptr, rows, nrows, key, val); break;
    case 7: sort_rows_pack<HAS_VAL, 7><<<gr, 256, 0, s>>>(rowptr, rows, nrows, key, val); break;
    case 8: sort_rows_pack<HAS_VAL, 8><<<gr, 256, 0, s>>>(rowptr, rows, nrows, key, val); break;
    case 9: sort_rows_pack<HAS_VAL, 9><<<gr, 256, 0, s>>>(rowptr, rows, nrows, key, val); break;
    case 10: sort_rows_pack<HAS_VAL, 10><<<gr, 256, 0, s>>>(rowptr, rows, nrows, key, val); break;
    case 11: sort_rows_pack<HAS_VAL, 11><<<gr, 256, 0, s>>>(rowptr, rows, nrows, key, val); break;
    default: sort_rows_pack<HAS_VAL, 12><<<gr, 256, 0, s>>>(rowptr, rows, nrows, key, val); break;
    }
}

static int sort_rows(Graph *g, uint32_t *key, uint32_t *val, uint32_t max_key, cudaStream_t s) {
    const uint32_t n = g->n;
    if (n == 0 || g->nnz == 0) return KC_OK;
    const int sms = current_sms();
    uint32_t *list = nullptr;
    unsigned long long *counts = nullptr;
    KC_TRY(dalloc(&list, (uint64_t)n, "row class list"));
    if (dalloc(&counts, 2 * SORT_BUCKETS, "row class counts") != KC_OK) { dfree(list); return KC_ERR_NOMEM; }
    unsigned long long *cursor = counts + SORT_BUCKETS;
    cudaMemsetAsync(counts, 0, SORT_BUCKETS * sizeof(unsigned long long), s);
    classify_rows<<<grid_for(n, 256, sms), 256, 0, s>>>(g->rowptr, n, counts, nullptr, nullptr);
    unsigned long long h[SORT_BUCKETS], off[SORT_BUCKETS + 1];
    cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { dfree(list); dfree(counts); return fail(KC_ERR_CUDA, "classify: %s", cudaGetErrorString(e)); }
    off[0] = 0;
    for (int c = 0; c < SORT_BUCKETS; c++) off[c + 1] = off[c] + h[c];
    cudaMemcpyAsync(cursor, off, SORT_BUCKETS * sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
    classify_rows<<<grid_for(n, 256, sms), 256, 0, s>>>(g->rowptr, n, nullptr, cursor, list);
    const bool hv = val != nullptr;
    if (h[0]) {
        int gr = grid_for(h[0] * 32, 256, sms);
        if (hv) sort_rows_warp<true><<<gr, 256, 0, s>>>(g->rowptr, list, h[0], key, val);
        else sort_rows_warp<false><<<gr, 256, 0, s>>>(g->rowptr, list, h[0], key, val);
    }
    for (int c = 1; c < SORT_BUCKETS - 1; c++) {
        if (!h[c]) continue;
        if (hv) launch_pack<true>(c + 5, g->rowptr, list + off[c], h[c], key, val, sms, s);
        else launch_pack<false>(c + 5, g->rowptr, list + off[c], h[c], key, val, sms, s);
    }
    uint32_t *tk = nullptr, *tv = nullptr;
    int rc = KC_OK;
    const unsigned long long hc = h[SORT_BUCKETS - 1];
    if (hc) {
        int bits = 1;
        while (bits < 32 && (max_key >> bits) != 0) bits++;
        int passes = (bits + 7) / 8;
        rc = dalloc(&tk, g->nnz, "radix staging keys");
        if (rc == KC_OK && hv) rc = dalloc(&tv, g->nnz, "radix staging values");
        if (rc == KC_OK) {
            const uint32_t *lc = list + off[SORT_BUCKETS - 1];
            int gr = (int)std::min<unsigned long long>(hc, (unsigned long long)sms * 4);
            if (hv) sort_rows_radix<true><<<gr, RADIX_THREADS, 0, s>>>(g->rowptr, lc, hc, key, val, tk, tv, passes);
            else sort_rows_radix<false><<<gr, RADIX_THREADS, 0, s>>>(g->rowptr, lc, hc, key, val, tk, tv, passes);
        }
    }
    e = cudaGetLastError();
    cudaError_t e2 = cudaStreamSynchronize(s);
    dfree(tk);
    dfree(tv);
    dfree(list);
    dfree(counts);
    if (rc != KC_OK) return rc;
    if (e != cudaSuccess || e2 != cudaSuccess)
        return fail(KC_ERR_CUDA, "row sort: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    return KC_OK;
}

// ----------------------------------------------------------- unique -------
// De-duplication of sorted rows, entry-parallel: an entry is kept when it
// starts its row or differs from its predecessor.  Row starts are first set
// in a bitmap over the entries (one thread per row), so a tile of UQ_TILE
// entries (UQ_PER consecutive entries per thread) reads them with its entries
// whatever the number of rows, empty ones included, that start in it.  Pass 1
// counts the kept entries of each tile; a scan gives each tile its output
// offset; pass 2 writes the kept entries and saves, per thread, its kept mask
// and the kept count before it in the tile; a pass over the rows then gives
// each row its new offset from those.
constexpr unsigned UQ_THREADS = 256;
constexpr unsigned UQ_PER = 16;
constexpr unsigned UQ_TILE = UQ_THREADS * UQ_PER;

__global__ void mark_row_starts(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t *startbits) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const int64_t r = rowptr[v];
        if (rowptr[v + 1] > r) atomicOr(&startbits[r >> 5], 1u << (r & 31));
    }
}

// Kept mask of this thread's UQ_PER entries of tile [t0, t0 + len) (bit i:
// entry t0 + threadIdx.x * UQ_PER + i).
__device__ __forceinline__ unsigned uq_mask(const uint32_t *__restrict__ col, const uint32_t *__restrict__ startbits,
                                            uint64_t t0, unsigned len) {
    unsigned mask = 0;
    const unsigned o0 = threadIdx.x * UQ_PER;
    if (o0 < len) {
        const uint64_t e0 = t0 + o0;  // a multiple of UQ_PER: the bits lie in one word
        const unsigned sb = (startbits[e0 >> 5] >> (e0 & 31)) & ((1u << UQ_PER) - 1u);
        uint32_t prev = e0 > 0 ? col[e0 - 1] : 0u;
#pragma unroll
        for (unsigned i = 0; i < UQ_PER; i++) {
            if (o0 + i < len) {
                const uint32_t x = col[e0 + i];
                if (((sb >> i) & 1u) || x != prev) mask |= 1u << i;
                prev = x;
            }
        }
    }
    return mask;
}

__global__ void __launch_bounds__(UQ_THREADS) unique_tiles_count(const uint32_t *__restrict__ col,
                                                                  const uint32_t *__restrict__ startbits, uint64_t nnz,
                                                                  uint32_t *tile_cnt) {
    __shared__ uint32_t wsum[UQ_THREADS / 32];
    const uint64_t tiles = (nnz + UQ_TILE - 1) / UQ_TILE;
    for (uint64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const uint64_t t0 = t * UQ_TILE;
        const unsigned len = (unsigned)(nnz - t0 < (uint64_t)UQ_TILE ? nnz - t0 : (uint64_t)UQ_TILE);
        const unsigned c = __reduce_add_sync(KC_FULL_MASK, (unsigned)__popc(uq_mask(col, startbits, t0, len)));
        if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned tot = 0;
            for (unsigned w = 0; w < UQ_THREADS / 32; w++) tot += wsum[w];
            tile_cnt[t] = tot;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(UQ_THREADS) unique_tiles_write(const uint32_t *__restrict__ col,
                                                                  const uint32_t *__restrict__ startbits, uint64_t nnz,
                                                                  const int64_t *__restrict__ tile_off, uint32_t *ncol,
                                                                  uint16_t *tmask, uint16_t *tpre) {
    __shared__ uint32_t wsum[UQ_THREADS / 32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t tiles = (nnz + UQ_TILE - 1) / UQ_TILE;
    for (uint64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const uint64_t t0 = t * UQ_TILE;
        const unsigned len = (unsigned)(nnz - t0 < (uint64_t)UQ_TILE ? nnz - t0 : (uint64_t)UQ_TILE);
        const unsigned mask = uq_mask(col, startbits, t0, len);
        unsigned wt;
        const unsigned ex = warp_excl_scan((unsigned)__popc(mask), lane, wt);
        if (lane == 0) wsum[warp] = wt;
        __syncthreads();
        unsigned before = 0;
        for (unsigned w = 0; w < warp; w++) before += wsum[w];
        const int64_t base = tile_off[t] + before + ex;
        tmask[t * UQ_THREADS + threadIdx.x] = (uint16_t)mask;
        tpre[t * UQ_THREADS + threadIdx.x] = (uint16_t)(before + ex);
        const uint64_t e0 = t0 + threadIdx.x * UQ_PER;
        unsigned k = 0;
#pragma unroll
        for (unsigned i = 0; i < UQ_PER; i++)
            if ((mask >> i) & 1u) ncol[base + k++] = col[e0 + i];
        __syncthreads();
    }
}

// New offset of every row: the kept entries before its old start.
__global__ void unique_rows(const int64_t *__restrict__ rowptr, uint32_t n, uint64_t nnz,
                            const int64_t *__restrict__ tile_off, const uint16_t *__restrict__ tmask,
                            const uint16_t *__restrict__ tpre, int64_t *nrow) {
    const uint64_t tiles = (nnz + UQ_TILE - 1) / UQ_TILE;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v <= n; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = (uint64_t)rowptr[v];
        if (r >= nnz) {
            nrow[v] = tile_off[tiles];
            continue;
        }
        const uint64_t t = r / UQ_TILE;
        const unsigned o = (unsigned)(r % UQ_TILE);
        const uint64_t th = t * UQ_THREADS + o / UQ_PER;
        nrow[v] = tile_off[t] + tpre[th] + __popc((unsigned)tmask[th] & ((1u << (o % UQ_PER)) - 1u));
    }
}

// ------------------------------------------------------- graph stats ------
__global__ void degree_stats(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t *maxdeg,
                             unsigned long long *vnodes) {
    uint32_t mx = 0;
    unsigned long long vn = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t d = (uint64_t)(rowptr[v + 1] - rowptr[v]);
        mx = max(mx, (uint32_t)d);
        vn += (d + 31) / 32;
    }
    mx = __reduce_max_sync(KC_FULL_MASK, mx);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vn += __shfl_xor_sync(KC_FULL_MASK, vn, o);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(maxdeg, mx);
        atomicAdd(vnodes, vn);
    }
}

int graph_finish(Graph *g) {
    cudaStream_t s = g->stream;
    uint32_t *md = nullptr;
    KC_TRY(dalloc(&md, 4, "graph stats"));
    unsigned long long *vn = reinterpret_cast<unsigned long long *>(md + 2);
    cudaMemsetAsync(md, 0, 16, s);
    if (g->n) degree_stats<<<grid_for(g->n, 256, g->sm_count), 256, 0, s>>>(g->rowptr, g->n, md, vn);
    uint32_t h[4];
    cudaMemcpyAsync(h, md, 16, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    dfree(md);
    if (e != cudaSuccess) return fail(KC_ERR_CUDA, "graph stats: %s", cudaGetErrorString(e));
    g->max_deg = h[0];
    unsigned long long vv;
    memcpy(&vv, &h[2], 8);
    g->num_vnodes = vv;
    return KC_OK;
}

// ------------------------------------------------------------ build -------
int build_csr_from_edges(Graph *g, const uint32_t *d_src, const uint32_t *d_dst, uint64_t m, uint32_t n,
                         uint32_t flags) {
    cudaStream_t s = g->stream;
    const int sms = g->sm_count;
    const bool keep_order = (flags & (KC_EDGES_DEDUP | KC_EDGES_SORT_ROWS)) == 0;
    if (keep_order && 2 * m > 0xffffffffull)
        return fail(KC_ERR_UNSUPPORTED, "edge-list row order needs 2*m < 2^32 (m=%llu); pass KC_EDGES_SORT_ROWS",
                    (unsigned long long)m);
    g->n = n;
    uint32_t *deg = nullptr, *err = nullptr;
    KC_TRY(dalloc(&deg, (uint64_t)n + 1, "degrees"));
    int rc = dalloc(&err, 1, "error flag");
    if (rc) { dfree(deg); return rc; }
    rc = dalloc(&g->rowptr, (uint64_t)n + 1, "row offsets");
    if (rc) { dfree(deg); dfree(err); return rc; }
    cudaMemsetAsync(deg, 0, ((uint64_t)n + 1) * 4, s);
    cudaMemsetAsync(err, 0, 4, s);
    if (m) count_degrees<<<grid_for(m, 256, sms), 256, 0, s>>>(d_src, d_dst, m, n, deg, err);
    uint32_t herr = 0;
    cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { dfree(deg); dfree(err); return fail(KC_ERR_CUDA, "degree count: %s", cudaGetErrorString(e)); }
    if (herr) { dfree(deg); dfree(err); return fail(KC_ERR_INVALID, "edge endpoint >= n (%u)", n); }
    rc = exclusive_scan_u32_i64(deg, g->rowptr, n, s);
    if (rc) { dfree(deg); dfree(err); return rc; }
    int64_t nnz = 0;
    cudaMemcpy(&nnz, g->rowptr + n, 8, cudaMemcpyDeviceToHost);
    g->nnz = (uint64_t)nnz;
    uint32_t *key = nullptr;
    rc = dalloc(&g->col, g->nnz + 1, "column ids");
    if (rc == KC_OK && keep_order) rc = dalloc(&key, g->nnz + 1, "edge order keys");
    if (rc) { dfree(deg); dfree(err); dfree(key); return rc; }
    unsigned long long *cur = nullptr;  // row fill cursors, starting at the row offsets
    if (m) {
        rc = dalloc(&cur, (uint64_t)n + 1, "row cursors");
        if (rc) { dfree(deg); dfree(err); dfree(key); return rc; }
        cudaMemcpyAsync(cur, g->rowptr, ((uint64_t)n + 1) * 8, cudaMemcpyDeviceToDevice, s);
        scatter_edges<<<grid_for(m, 256, sms), 256, 0, s>>>(d_src, d_dst, m, n, cur, g->col, key);
    }
    e = cudaStreamSynchronize(s);
    dfree(cur);
    if (e != cudaSuccess) { dfree(deg); dfree(err); dfree(key); return fail(KC_ERR_CUDA, "scatter: %s", cudaGetErrorString(e)); }
    if (keep_order) {
        rc = sort_rows(g, key, g->col, (uint32_t)(2 * m), s);
    } else {
        rc = sort_rows(g, g->col, nullptr, n, s);
    }
    dfree(key);
    if (rc) { dfree(deg); dfree(err); return rc; }
    if ((flags & KC_EDGES_DEDUP) && g->nnz) {
        int64_t *nrow = nullptr, *toff = nullptr;
        uint32_t *ncol = nullptr, *tcnt = nullptr, *sbits = nullptr;
        uint16_t *tmask = nullptr, *tpre = nullptr;
        const uint64_t tiles = (g->nnz + UQ_TILE - 1) / UQ_TILE;
        auto release = [&]() {
            dfree(tcnt);
            dfree(toff);
            dfree(sbits);
            dfree(tmask);
            dfree(tpre);
        };
        rc = dalloc(&nrow, (uint64_t)n + 1, "dedup row offsets");
        if (rc == KC_OK) rc = dalloc(&tcnt, tiles, "dedup tile counts");
        if (rc == KC_OK) rc = dalloc(&toff, tiles + 1, "dedup tile offsets");
        if (rc == KC_OK) rc = dalloc(&sbits, tiles * (UQ_TILE / 32), "row-start bitmap");
        if (rc == KC_OK) rc = dalloc(&tmask, tiles * UQ_THREADS, "dedup masks");
        if (rc == KC_OK) rc = dalloc(&tpre, tiles * UQ_THREADS, "dedup prefixes");
        if (rc) { release(); dfree(nrow); dfree(deg); dfree(err); return rc; }
        cudaMemsetAsync(sbits, 0, tiles * (UQ_TILE / 32) * sizeof(uint32_t), s);
        mark_row_starts<<<grid_for(n, 256, sms), 256, 0, s>>>(g->rowptr, n, sbits);
        const int ug = (int)std::min<uint64_t>(tiles, (uint64_t)sms * 8);
        unique_tiles_count<<<ug, UQ_THREADS, 0, s>>>(g->col, sbits, g->nnz, tcnt);
        rc = exclusive_scan_u32_i64(tcnt, toff, tiles, s);
        int64_t nn = 0;
        if (rc == KC_OK) {
            cudaMemcpy(&nn, toff + tiles, 8, cudaMemcpyDeviceToHost);
            rc = dalloc(&ncol, (uint64_t)nn + 1, "dedup column ids");
        }
        if (rc) { release(); dfree(nrow); dfree(deg); dfree(err); return rc; }
        unique_tiles_write<<<ug, UQ_THREADS, 0, s>>>(g->col, sbits, g->nnz, toff, ncol, tmask, tpre);
        unique_rows<<<grid_for((uint64_t)n + 1, 256, sms), 256, 0, s>>>(g->rowptr, n, g->nnz, toff, tmask, tpre, nrow);
        e = cudaStreamSynchronize(s);
        release();
        dfree(g->rowptr);
        dfree(g->col);
        g->rowptr = nrow;
        g->col = ncol;
        g->nnz = (uint64_t)nn;
        if (e != cudaSuccess) { dfree(deg); dfree(err); return fail(KC_ERR_CUDA, "unique: %s", cudaGetErrorString(e)); }
    }
    dfree(deg);
    dfree(err);
    return graph_finish(g);
}

// ---------------------------------------------------------- validate ------
__device__ __forceinline__ unsigned long long pair_hash(uint32_t a, uint32_t b) {
    unsigned long long z = ((unsigned long long)a << 32 | b) + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Symmetry as multiset equality of {(min,max)} over entries above and below
// the diagonal: counts and a commutative hash sum must agree.
__global__ void validate_kernel(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col, uint32_t n,
                                unsigned long long *acc) {
    const unsigned lane = threadIdx.x & 31;
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long bad = 0, hlo = 0, hhi = 0, clo = 0, chi = 0;
    for (uint64_t v = warp; v < n; v += nwarps) {
        for (int64_t j = rowptr[v] + lane; j < rowptr[v + 1]; j += 32) {
            uint32_t u = col[j];
            if (u >= n || u == v) { bad++; continue; }
            if (u > v) { hlo += pair_hash((uint32_t)v, u); clo++; }
            else { hhi += pair_hash(u, (uint32_t)v); chi++; }
        }
    }
    atomicAdd(&acc[0], bad);
    atomicAdd(&acc[1], hlo);
    atomicAdd(&acc[2], hhi);
    atomicAdd(&acc[3], clo);
    atomicAdd(&acc[4], chi);
}

int graph_validate(Graph *g, uint64_t *bad) {
    unsigned long long *acc = nullptr;
    KC_TRY(dalloc(&acc, 5, "validate"));
    cudaMemsetAsync(acc, 0, 40, g->stream);
    if (g->n) validate_kernel<<<grid_for((uint64_t)g->n * 32, 256, g->sm_count), 256, 0, g->stream>>>(g->rowptr, g->col, g->n, acc);
    unsigned long long h[5];
    cudaMemcpyAsync(h, acc, 40, cudaMemcpyDeviceToHost, g->stream);
    cudaError_t e = cudaStreamSynchronize(g->stream);
    dfree(acc);
    if (e != cudaSuccess) return fail(KC_ERR_CUDA, "validate: %s", cudaGetErrorString(e));
    uint64_t b = h[0];
    b += h[3] > h[4] ? h[3] - h[4] : h[4] - h[3];
    if (h[3] == h[4] && h[1] != h[2]) b += 1;
    *bad = b;
    return KC_OK;
}

// ---------------------------------------------------- virtual layout ------
__global__ void vlayout_kernel(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ col, uint32_t n,
                               uint32_t *node_pointer, uint32_t *edge_list) {
    const unsigned lane = threadIdx.x & 31;
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t v = warp; v < n; v += nwarps) {
        int64_t s = rowptr[v], e = rowptr[v + 1];
        uint64_t slot = (uint64_t)s + v;
        if (lane == 0) {
            node_pointer[v] = (uint32_t)slot;
            edge_list[slot] = (uint32_t)(e - s);
        }
        for (int64_t j = s + lane; j < e; j += 32) edge_list[slot + 1 + (j - s)] = col[j];
    }
}

__global__ void vparts_count(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t part_size, uint32_t *k) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        k[v] = (uint32_t)(((uint64_t)(rowptr[v + 1] - rowptr[v]) + part_size - 1) / part_size);
}

__global__ void vparts_fill(const int64_t *__restrict__ pstart, const uint32_t *__restrict__ k, uint32_t n,
                            uint32_t *parts) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        int64_t p = pstart[v];
        for (uint32_t j = 0; j < k[v]; j++) {
            parts[2 * (p + j)] = (uint32_t)v;
            parts[2 * (p + j) + 1] = j;
        }
    }
}

int virtual_layout(Graph *g, uint32_t part_size, uint32_t *h_node_pointer, uint32_t *h_edge_list,
                   uint32_t *h_parts, uint64_t *num_parts) {
    if (part_size == 0) return fail(KC_ERR_INVALID, "part_size must be > 0");
    cudaStream_t s = g->stream;
    const uint32_t n = g->n;
    uint32_t *k = nullptr;
    int64_t *pstart = nullptr;
    KC_TRY(dalloc(&k, (uint64_t)n + 1, "vnode counts"));
    int rc = dalloc(&pstart, (uint64_t)n + 1, "vnode offsets");
    if (rc) { dfree(k); return rc; }
    if (n) vparts_count<<<grid_for(n, 256, g->sm_count), 256, 0, s>>>(g->rowptr, n, part_size, k);
    rc = exclusive_scan_u32_i64(k, pstart, n, s);
    int64_t np = 0;
    if (rc == KC_OK) cudaMemcpy(&np, pstart + n, 8, cudaMemcpyDeviceToHost);
    *num_parts = (uint64_t)np;
    if (rc || (!h_parts && !h_node_pointer && !h_edge_list)) { dfree(k); dfree(pstart); return rc; }
    if (g->nnz + n > 0xffffffffull) { dfree(k); dfree(pstart); return fail(KC_ERR_UNSUPPORTED, "layout offsets exceed uint32"); }
    uint32_t *dnp = nullptr, *del = nullptr, *dparts = nullptr;
    rc = dalloc(&dnp, (uint64_t)n + 1, "nodePointer");
    if (!rc) rc = dalloc(&del, g->nnz + n + 1, "edgeList");
    if (!rc) rc = dalloc(&dparts, 2ull * (uint64_t)np + 2, "partNodePointer");
    if (!rc) {
        if (n) {
            vlayout_kernel<<<grid_for((uint64_t)n * 32, 256, g->sm_count), 256, 0, s>>>(g->rowptr, g->col, n, dnp, del);
            vparts_fill<<<grid_for(n, 256, g->sm_count), 256, 0, s>>>(pstart, k, n, dparts);
        }
        if (h_node_pointer) cudaMemcpyAsync(h_node_pointer, dnp, (uint64_t)n * 4, cudaMemcpyDeviceToHost, s);
        if (h_edge_list) cudaMemcpyAsync(h_edge_list, del, (g->nnz + n) * 4, cudaMemcpyDeviceToHost, s);
        if (h_parts) cudaMemcpyAsync(h_parts, dparts, 2ull * np * 4, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(KC_ERR_CUDA, "virtual layout: %s", cudaGetErrorString(e));
    }
    dfree(dnp);
    dfree(del);
    dfree(dparts);
    dfree(k);
    dfree(pstart);
    return rc;
}

}  // namespace kc
