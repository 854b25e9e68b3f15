// h-index iteration: the k-core path of HistoCore / CntCore / NbrCore
// (index2core/HistoCore.cu:15-202,292-341; CntCore.cu:17-264,344-417;
// NbrCore.cu:12-167,244-297) as one cooperative launch.
//
// Every vertex starts at its degree; a sweep replaces the estimate c[v] of each
// active vertex by the h-index of its neighbours' estimates (the largest k
// with at least k neighbours at >= k), which never exceeds c[v].  Estimates
// stay upper bounds of the core numbers and the iteration stops at the
// largest fixpoint, which is the core vector.  The reference runs three
// trigger schemes for the same operator (persistent per-vertex histograms,
// support counters, neighbour flags), each as several launches plus a
// blocking flag copy per iteration.  Here:
//   * a vertex is re-examined only when a neighbour's estimate dropped from
//     at or above its own to below it (the neighbour stopped supporting it;
//     notifications are deduplicated by one bitmap per sweep parity), or
//     after its own estimate dropped, so settled vertices read nothing;
//   * the support test "at least c[v] neighbours at >= c[v]" runs first,
//     stops as soon as it holds and settles most re-examined vertices (the
//     support counter of CntCore.cu:258-261 / the top bin of
//     HistoCore.cu:184-198); when it fails, the same pass has built the
//     histogram;
//   * otherwise the h-index comes from a degree-capped histogram built in
//     shared memory and a suffix scan: 8 lanes per vertex for rows of at
//     most 32 entries, one warp per vertex for rows of at most 8,192 entries
//     (512 in sweep 0, where estimates are still degrees, unless the rows are
//     ordered: see below), with a window of 512 values below the estimate;
//     otherwise one CTA,
//     which narrows the value range with 4096-bin passes until bins are one
//     value wide;
//   * rows above 128 entries are read from a copy made at the start of the
//     decomposition in which the neighbours come in descending buckets of
//     floor(log2(degree)), with the length of every bucket prefix.  An
//     estimate never exceeds the degree, so each pass reads only the prefix
//     that can hold the values it needs: the support test the neighbours of
//     degree >= c[v], the notification those of degree > the new estimate,
//     and the histogram grows one bucket at a time until the h-index is
//     pinned (count(>= k) is exact for every k at or above the last bucket
//     read).  The prefix lengths alone also bound the h-index (no k above
//     P[floor(log2 k)] qualifies); when the bound is below the estimate the
//     support test is skipped and the histogram window is put under the
//     bound, so sweep 0 gives rows up to 8,192 entries to warps.  On R-MAT
//     graphs this reads about 40% fewer row entries;
//   * updates are visible at once within a sweep (Gauss-Seidel), which only
//     shortens the trajectory; sweeps are separated by a grid barrier with a
//     bounded wait.
#include <algorithm>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

constexpr int HX_THREADS = 512;
constexpr int HX_WARPS = HX_THREADS / 32;
constexpr uint32_t HX_WARP_MAX = 512;   // rows up to this length: one warp
constexpr uint32_t HX_BINS = 4096;      // CTA histogram bins
constexpr unsigned HX_GRAB = 8;         // short-row vertices a warp takes per cursor step
constexpr int HX_CACHE = 4;             // row entries per lane kept in registers (rows up to 32 * HX_CACHE)
constexpr uint32_t HX_ORD_MIN = 32 * HX_CACHE;  // the shortest rows that can get an ordered copy are longer
constexpr uint32_t HX_ORD_WARP = 8192;  // the copy of a row up to this length is made by one warp

struct HxArgs {
    const int64_t *rowptr;
    const uint32_t *col;
    // ordered copies of the rows above ord_min entries (nullptr: read col)
    uint32_t ord_min;      // >= HX_ORD_MIN
    const uint32_t *ord;   // same positions as col
    const uint32_t *lid;   // vertex -> long-row index
    const uint32_t *pref;  // 32 per long row: entries in degree buckets >= b
    uint32_t n;
    uint32_t *c;
    uint32_t *inlist[2];  // bitmaps: vertex queued for the sweep of that parity
    uint32_t *list[2];
    uint32_t *big[2];
    HindexCtl *ctl;
    unsigned long long timeout_ns;
    uint32_t max_sweeps;
    uint32_t first_all;  // sweep 0 covers every vertex (else list[0] / big[0])
    uint32_t withhold;   // CTA 0 never arrives at the first barrier (failure-detection hook)
    uint32_t warp_rows;  // rows up to this length are re-examined by one warp
    uint32_t sweep0_rows;  // in sweep 0: HX_WARP_MAX, or warp_rows when long rows are ordered
    PeelTrace *trace;    // per-sweep trace or nullptr
    uint32_t trace_cap;
};

__device__ __forceinline__ unsigned hx_bucket(uint32_t x) { return x ? 31u - __clz(x) : 0u; }

// Estimates start at the degrees; rows above sweep0_rows entries are queued
// for the CTAs of sweep 0.  With ord_rows, the rows above ord_min entries
// are listed for the ordered copy: up to HX_ORD_WARP entries from the front
// of ord_rows (long-row index p), longer ones from its far end (index
// max_long - 1 - q), each with its index in lid, and vb holds every
// vertex's degree bucket (one byte: the copies gather these, not degrees).
__global__ void hindex_init(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t *c, uint32_t *inlist0,
                            uint32_t *inlist1, uint32_t *big0, uint32_t sweep0_rows, uint32_t *ord_rows,
                            uint32_t *lid, uint8_t *vb, uint32_t ord_min, uint64_t max_long, HindexCtl *ctl) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < n; base += stride) {
        uint64_t v = base + threadIdx.x;
        bool bigv = false, midl = false, hugel = false;
        if (v < n) {
            uint32_t d = (uint32_t)(rowptr[v + 1] - rowptr[v]);
            c[v] = d;
            if (vb) vb[v] = (uint8_t)hx_bucket(d);
            bigv = d > sweep0_rows;
            midl = ord_rows && d > ord_min && d <= HX_ORD_WARP;
            hugel = ord_rows && d > ord_min && d > HX_ORD_WARP;
        }
        unsigned b = __ballot_sync(KC_FULL_MASK, bigv);
        if (b) {
            unsigned long long p = 0;
            if (lane == 0) p = atomicAdd(&ctl->big_len[0], (unsigned long long)__popc(b));
            p = __shfl_sync(KC_FULL_MASK, p, 0);
            if (bigv) big0[p + __popc(b & lt)] = (uint32_t)v;
        }
        const unsigned bm = __ballot_sync(KC_FULL_MASK, midl);
        if (bm) {
            unsigned long long p = 0;
            if (lane == 0) p = atomicAdd(&ctl->ord_len, (unsigned long long)__popc(bm));
            p = __shfl_sync(KC_FULL_MASK, p, 0) + __popc(bm & lt);
            if (midl) {
                ord_rows[p] = (uint32_t)v;
                lid[v] = (uint32_t)p;
            }
        }
        const unsigned bh = __ballot_sync(KC_FULL_MASK, hugel);
        if (bh) {
            unsigned long long q = 0;
            if (lane == 0) q = atomicAdd(&ctl->ord_huge, (unsigned long long)__popc(bh));
            q = __shfl_sync(KC_FULL_MASK, q, 0) + __popc(bh & lt);
            if (hugel) {
                ord_rows[n - 1 - q] = (uint32_t)v;
                lid[v] = (uint32_t)(max_long - 1 - q);
            }
        }
    }
    uint64_t words = ((uint64_t)n + 31) / 32;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < words; w += stride) {
        inlist0[w] = 0u;
        inlist1[w] = 0u;
    }
}

// The ordered copy of the row s..e, made by NW warps sharing `bins` (32
// words): count the neighbours per bucket of floor(log2(degree)) and keep
// each entry's bucket in bk (one byte per entry, so the degrees are gathered
// once), turn the counts into prefix lengths (bucket 31 first), then place
// every neighbour at its bucket's cursor.  Lanes with the same bucket make
// one shared-memory atomic.  Neighbours within a bucket keep no particular
// order.
template <int NW>
__device__ __forceinline__ void hx_order_count(const uint32_t *__restrict__ col, const uint8_t *__restrict__ vb,
                                               uint8_t *bk, int64_t s, int64_t e, uint32_t *bins, unsigned w,
                                               unsigned lane) {
    for (int64_t jw = s + (int64_t)w * 128; jw < e; jw += (int64_t)NW * 128) {
        uint32_t u[4], b[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int64_t j = jw + k * 32 + lane;
            u[k] = j < e ? col[j] : 0xffffffffu;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) b[k] = u[k] != 0xffffffffu ? (uint32_t)__ldg(&vb[u[k]]) : 32u;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (b[k] < 32u) bk[jw + k * 32 + lane] = (uint8_t)b[k];
            const unsigned peers = __match_any_sync(KC_FULL_MASK, b[k]);
            if (b[k] < 32u && (int)lane == __ffs(peers) - 1) atomicAdd(&bins[b[k]], (unsigned)__popc(peers));
        }
    }
}

template <int NW>
__device__ __forceinline__ void hx_order_place(const uint32_t *__restrict__ col, const uint8_t *bk, int64_t s,
                                               int64_t e, uint32_t *cursor, uint32_t *ord, unsigned w,
                                               unsigned lane) {
    const unsigned lt = (1u << lane) - 1u;
    for (int64_t jw = s + (int64_t)w * 128; jw < e; jw += (int64_t)NW * 128) {
        uint32_t u[4], b[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int64_t j = jw + k * 32 + lane;
            u[k] = j < e ? col[j] : 0xffffffffu;
            b[k] = j < e ? (uint32_t)bk[j] : 32u;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const unsigned peers = __match_any_sync(KC_FULL_MASK, b[k]);
            const int leader = __ffs(peers) - 1;
            unsigned base = 0;
            if (b[k] < 32u && (int)lane == leader) base = atomicAdd(&cursor[b[k]], (unsigned)__popc(peers));
            base = __shfl_sync(KC_FULL_MASK, base, leader);
            if (b[k] < 32u) ord[s + base + __popc(peers & lt)] = u[k];
        }
    }
}

// bins[lane] = count of bucket lane -> pref_row[lane] = entries in buckets >=
// lane, bins[lane] = entries in buckets > lane (the bucket's first slot)
__device__ __forceinline__ void hx_order_prefix(uint32_t *bins, uint32_t *pref_row, unsigned lane) {
    const uint32_t own = bins[lane];
    uint32_t x = own;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_down_sync(KC_FULL_MASK, x, d);
        if (lane + d < 32) x += y;
    }
    pref_row[lane] = x;
    __syncwarp();
    bins[lane] = x - own;
}

// Ordered copies of every listed row in one launch of 512-thread CTAs: each
// CTA first takes rows above HX_ORD_WARP entries (listed from the far end of
// `rows`, n entries) one at a time with all its warps, then its warps take
// the shorter rows (listed from the front) one each, both from shared
// cursors, so the long rows' tail overlaps the short rows.  vb: the degree
// bucket of every vertex.
constexpr int HX_ORD_THREADS = 512;
__global__ void __launch_bounds__(HX_ORD_THREADS) hx_order_rows(const int64_t *__restrict__ rowptr,
                                                                const uint32_t *__restrict__ col,
                                                                const uint8_t *__restrict__ vb, const uint32_t *rows,
                                                                uint32_t n, HindexCtl *ctl, uint32_t *ord,
                                                                uint32_t *pref, uint8_t *bk, uint64_t max_long) {
    constexpr int NW = HX_ORD_THREADS / 32;
    __shared__ uint32_t cbins[32];
    __shared__ uint32_t wbins[NW][32];
    __shared__ unsigned long long item_sh;
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned long long nh = ctl->ord_huge, nrows = ctl->ord_len;
    for (;;) {
        if (threadIdx.x == 0) item_sh = atomicAdd(&ctl->ord_huge_cursor, 1ull);
        if (threadIdx.x < 32) cbins[threadIdx.x] = 0;
        __syncthreads();
        const unsigned long long q = item_sh;
        if (q >= nh) break;  // uniform: read after the barrier
        const uint32_t v = rows[n - 1 - q];
        const int64_t s = rowptr[v], e = rowptr[v + 1];
        hx_order_count<NW>(col, vb, bk, s, e, cbins, w, lane);
        __syncthreads();
        if (w == 0) hx_order_prefix(cbins, pref + (max_long - 1 - q) * 32, lane);
        __syncthreads();
        hx_order_place<NW>(col, bk, s, e, cbins, ord, w, lane);
        __syncthreads();
    }
    uint32_t *bins = wbins[w];
    for (;;) {
        unsigned long long i = 0;
        if (lane == 0) i = atomicAdd(&ctl->ord_cursor, 1ull);
        i = __shfl_sync(KC_FULL_MASK, i, 0);
        if (i >= nrows) break;
        const uint32_t v = rows[i];
        const int64_t s = rowptr[v], e = rowptr[v + 1];
        bins[lane] = 0;
        __syncwarp();
        hx_order_count<1>(col, vb, bk, s, e, bins, 0, lane);
        __syncwarp();
        hx_order_prefix(bins, pref + i * 32, lane);
        __syncwarp();
        hx_order_place<1>(col, bk, s, e, bins, ord, 0, lane);
        __syncwarp();
    }
}

// Queue u for the next sweep (list and bitmap of parity nxt) unless it is
// queued already.  Vertices pending in the current sweep are queued again: a
// notification never relies on an evaluation still to come in this sweep,
// which could read the neighbour's estimate before its update is visible.
// Rows up to A.warp_rows entries (tunable "hindex.warp_rows") go to the warp list: one warp streams
// such a row with fewer synchronisations than a CTA.  Rows above
// HX_WARP_MAX entries are kept apart and handed out first, one per warp, so
// that the short rows even out the end of the sweep.
__device__ __forceinline__ void hx_activate(const HxArgs &A, uint32_t u, unsigned nxt) {
    unsigned bit = 1u << (u & 31);
    if (__ldcg(&A.inlist[nxt][u >> 5]) & bit) return;
    unsigned old = atomicOr(&A.inlist[nxt][u >> 5], bit);
    if (old & bit) return;
    uint32_t d = (uint32_t)(A.rowptr[u + 1] - A.rowptr[u]);
    if (d > A.warp_rows) {
        unsigned long long p = atomicAdd(&A.ctl->big_len[nxt], 1ull);
        A.big[nxt][p] = u;
    } else if (d > HX_WARP_MAX) {
        // medium rows fill the list from its far end (a vertex is listed
        // once, so both ends together hold at most n entries)
        unsigned long long p = atomicAdd(&A.ctl->mid_len[nxt], 1ull);
        A.list[nxt][A.n - p] = u;
    } else {
        unsigned long long p = atomicAdd(&A.ctl->list_len[nxt], 1ull);
        A.list[nxt][p] = u;
    }
}

// hx_activate for K candidates per lane (u[k] where cand[k]), warp-wide:
// every lane calls it.  The pending-bit reads, the claiming atomicOr, the
// row-length reads and the list appends of all K candidates are each in
// flight together, and the appends to each list take one atomicAdd per warp.
template <int K>
__device__ __forceinline__ void hx_activate_all(const HxArgs &A, const uint32_t (&u)[K], const bool (&cand)[K],
                                                unsigned nxt, unsigned lane) {
    bool anyc = false;
#pragma unroll
    for (int k = 0; k < K; k++) anyc |= cand[k];
    if (!__any_sync(KC_FULL_MASK, anyc)) return;
    bool need[K];
#pragma unroll
    for (int k = 0; k < K; k++)
        need[k] = cand[k] && !(__ldcg(&A.inlist[nxt][u[k] >> 5]) & (1u << (u[k] & 31)));
    unsigned old[K];
#pragma unroll
    for (int k = 0; k < K; k++) old[k] = need[k] ? atomicOr(&A.inlist[nxt][u[k] >> 5], 1u << (u[k] & 31)) : ~0u;
    int kind[K];  // -1: nothing to queue; 0 short, 1 medium, 2 long row
#pragma unroll
    for (int k = 0; k < K; k++) {
        kind[k] = -1;
        if (!(old[k] & (1u << (u[k] & 31)))) {
            const int64_t d = A.rowptr[u[k] + 1] - A.rowptr[u[k]];
            kind[k] = d > (int64_t)A.warp_rows ? 2 : d > (int64_t)HX_WARP_MAX ? 1 : 0;
        }
    }
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < K; k++) {
        if (!__any_sync(KC_FULL_MASK, kind[k] >= 0)) continue;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const unsigned m = __ballot_sync(KC_FULL_MASK, kind[k] == q);
            if (!m) continue;
            unsigned long long base = 0;
            if (lane == __ffs(m) - 1)
                base = atomicAdd(q == 2 ? &A.ctl->big_len[nxt] : q == 1 ? &A.ctl->mid_len[nxt] : &A.ctl->list_len[nxt],
                                 (unsigned long long)__popc(m));
            base = __shfl_sync(KC_FULL_MASK, base, __ffs(m) - 1);
            if (kind[k] == q) {
                const unsigned long long p = base + __popc(m & lt);
                if (q == 2) A.big[nxt][p] = u[k];
                else if (q == 1) A.list[nxt][A.n - p] = u[k];
                else A.list[nxt][p] = u[k];
            }
        }
    }
}

// The largest k in [kmin, top] with count(>= k) >= k, where count(>= k) is
// carry (on entry: the count above top) plus the bins hist[k' - lo] for
// k <= k' <= top; -1 if none qualifies, and then carry = count(>= kmin).
__device__ __forceinline__ int64_t hx_warp_scan_from(const uint32_t *hist, uint32_t lo, int64_t top, int64_t kmin,
                                                     unsigned lane, uint32_t &carry) {
    for (; top >= kmin; top -= 32) {
        const int64_t k = top - lane;
        uint32_t incl = k >= kmin ? hist[k - lo] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(KC_FULL_MASK, incl, d);
            if (lane >= (unsigned)d) incl += y;
        }
        const bool ok = k >= kmin && carry + incl >= (uint32_t)k;
        const unsigned bb = __ballot_sync(KC_FULL_MASK, ok);
        if (bb) return top - (__ffs(bb) - 1);
        carry += __shfl_sync(KC_FULL_MASK, incl, 31);
    }
    return -1;
}

// The largest k in [max(lo, 1), hi] with count(>= k) >= k, from the window
// hist[k - lo] whose top bin hi - lo counts every value at or above hi; -1 if
// none qualifies, and then carry = count(>= max(lo, 1)).
__device__ __forceinline__ int64_t hx_warp_scan(const uint32_t *hist, uint32_t lo, uint32_t hi, unsigned lane,
                                                uint32_t &carry) {
    carry = 0;
    return hx_warp_scan_from(hist, lo, (int64_t)hi, lo > 1 ? (int64_t)lo : 1, lane, carry);
}

// Row storage of a warp's vertex: the ordered copy (pf: on lane b, the
// entries in degree buckets >= b) or col.  end(t) is the end of the part of
// the row that holds every neighbour of degree >= t: the prefix of buckets
// >= floor(log2(t)) of an ordered row, the whole row otherwise.
struct HxRow {
    const uint32_t *r;
    int64_t s, e;
    uint32_t pf;
    bool ordered;
    __device__ __forceinline__ int64_t end(uint32_t t) const {
        const uint32_t p = __shfl_sync(KC_FULL_MASK, pf, t ? 31 - __clz(t) : 0);
        return ordered && t ? s + (int64_t)p : e;
    }
    // An upper bound of the h-index from the prefix lengths alone (ordered
    // rows): count(>= k) <= P[floor(log2 k)], so no k in a bucket b with
    // P[b] < 2^b qualifies, and k <= P[b] for the highest bucket b that can.
    __device__ __forceinline__ uint32_t hbound() const {
        const unsigned lane = threadIdx.x & 31;
        const unsigned ok = __ballot_sync(KC_FULL_MASK, pf >= (1u << lane));
        if (!ok) return 0;
        const unsigned b = 31 - __clz(ok);
        const uint32_t pb = __shfl_sync(KC_FULL_MASK, pf, b);
        return b >= 31 ? pb : min(pb, (2u << b) - 1u);
    }
};

// The h-index lies below lo (above = count(>= lo)): windows of HX_WARP_MAX
// values further down, each built from another pass over the part of the
// row that can hold values in the window.
__device__ __forceinline__ uint32_t hx_warp_lower(const HxRow &R, const uint32_t *c, uint32_t *hist, uint32_t lo,
                                                  uint32_t above, unsigned lane) {
    for (;;) {
        if (lo <= 1) return 0;  // no k >= 1 qualified
        const uint32_t hi = lo;
        lo = hi > HX_WARP_MAX ? hi - HX_WARP_MAX : 0u;
        __syncwarp();
        for (uint32_t b = lane; b < hi - lo; b += 32) hist[b] = 0;
        if (lane == 0) hist[hi - lo] = above;
        __syncwarp();
        const int64_t ee = R.end(lo);
        for (int64_t j = R.s + lane; j < ee; j += 32) {
            const uint32_t x = __ldcg(&c[R.r[j]]);
            if (x < hi && x >= lo) atomicAdd(&hist[x - lo], 1u);
        }
        __syncwarp();
        uint32_t carry;
        const int64_t k = hx_warp_scan(hist, lo, hi, lane, carry);
        if (k >= 0) return (uint32_t)k;
        above = carry;
    }
}

constexpr int HX_STREAM = 4;  // row entries in flight per lane when a warp streams a long row (8: slower, spills)

// Add the estimates of row entries [j0, j1) to the window [lo, cap) of
// hist (bin x - lo) and count those at or above cap, starting from cnt.
// Stops early once the count reaches stop (stop = 0: the whole range).
__device__ __forceinline__ uint32_t hx_warp_gather(const uint32_t *row, const uint32_t *c, int64_t j0, int64_t j1,
                                                   uint32_t *hist, uint32_t lo, uint32_t cap, uint32_t cnt,
                                                   uint32_t stop, unsigned lane) {
    for (; j0 < j1 && (stop == 0 || cnt < stop); j0 += 32 * HX_STREAM) {
        uint32_t uu[HX_STREAM], c1 = 0;
#pragma unroll
        for (int k = 0; k < HX_STREAM; k++) {
            const int64_t j = j0 + k * 32 + lane;
            uu[k] = j < j1 ? row[j] : 0xffffffffu;
        }
        uint32_t xx[HX_STREAM];
#pragma unroll
        for (int k = 0; k < HX_STREAM; k++) xx[k] = uu[k] != 0xffffffffu ? __ldcg(&c[uu[k]]) : 0u;
#pragma unroll
        for (int k = 0; k < HX_STREAM; k++)
            if (uu[k] != 0xffffffffu) {
                if (xx[k] >= cap) c1++;
                else if (xx[k] >= lo) atomicAdd(&hist[xx[k] - lo], 1u);
            }
        cnt += __reduce_add_sync(KC_FULL_MASK, c1);
    }
    return cnt;
}

// One warp: recompute vertex v (any row length; long rows are streamed).
// hist: this warp's HX_WARP_MAX+1 shared bins.  Returns true if c[v] dropped.
// Rows of at most HX_CACHE * 32 entries keep their neighbour ids and
// estimates in registers: one gather pass serves the support test, the
// histogram and the neighbour notification.  Longer rows run the support
// test in chunks of HX_CACHE * 32 entries and stop once it holds.
__device__ bool hx_warp_vertex(const HxArgs &A, uint32_t v, unsigned cur, bool clear, uint32_t *hist,
                               unsigned lane) {
    const unsigned nxt = cur ^ 1u;
    const int64_t s = A.rowptr[v], e = A.rowptr[v + 1];
    // this sweep's bitmap is cleared as its vertices are examined, so it is
    // empty when it becomes the next sweep's
    if (clear && lane == 0) atomicAnd(&A.inlist[cur][v >> 5], ~(1u << (v & 31)));
    const uint32_t cap = __ldcg(&A.c[v]);
    if (cap == 0) return false;
    const bool cached = e - s <= 32 * HX_CACHE;
    HxRow R;
    R.s = s;
    R.e = e;
    R.ordered = A.ord != nullptr && e - s > (int64_t)A.ord_min;  // never a cached row
    R.r = R.ordered ? A.ord : A.col;
    R.pf = R.ordered ? A.pref[(size_t)A.lid[v] * 32 + lane] : 0u;
    uint32_t cu[HX_CACHE], cv[HX_CACHE];
    uint32_t cnt = 0;
    uint32_t lo = 0;      // lowest value the histogram window covers
    uint32_t capw = cap;  // its top bin counts the values at or above capw
    if (cached) {
#pragma unroll
        for (int k = 0; k < HX_CACHE; k++) {
            const int64_t j = s + k * 32 + lane;
            cu[k] = j < e ? A.col[j] : 0xffffffffu;
        }
#pragma unroll
        for (int k = 0; k < HX_CACHE; k++) cv[k] = cu[k] != 0xffffffffu ? __ldcg(&A.c[cu[k]]) : 0u;
#pragma unroll
        for (int k = 0; k < HX_CACHE; k++) cnt += (cu[k] != 0xffffffffu && cv[k] >= cap) ? 1u : 0u;
        cnt = __reduce_add_sync(KC_FULL_MASK, cnt);
        if (cnt >= cap) return false;  // support intact: estimate stands
        // histogram of min(c[u], capw) over bins [0, capw], capw = min(cap,
        // row length) <= 128: the h-index is at most the row length, and an
        // estimate above it (an old core number after deletions) still
        // decides the notification window below
        capw = min(cap, (uint32_t)(e - s));
        for (uint32_t b = lane; b <= capw; b += 32) hist[b] = 0;
        __syncwarp();
#pragma unroll
        for (int k = 0; k < HX_CACHE; k++)
            if (cu[k] != 0xffffffffu) atomicAdd(&hist[cv[k] < capw ? cv[k] : capw], 1u);
    } else {
        // One pass counts the values at or above capw and builds the
        // histogram of those in the window [lo, capw) of at most HX_WARP_MAX
        // values (bin x - lo); it stops early once the support test holds.
        // An ordered row is read only as far as the neighbours of degree >=
        // capw, and capw is lowered to one above the row's h-index bound:
        // below cap, the support test cannot hold (the common case in sweep 0,
        // where estimates are still degrees).
        if (R.ordered) {
            const uint32_t hb = R.hbound();
            if (hb < cap) capw = hb + 1;
        }
        lo = capw > HX_WARP_MAX ? capw - HX_WARP_MAX : 0u;
        for (uint32_t b = lane; b < capw - lo; b += 32) hist[b] = 0;
        __syncwarp();
        cnt = hx_warp_gather(R.r, A.c, s, R.end(capw), hist, lo, capw, 0u, capw == cap ? cap : 0u, lane);
        if (capw == cap && cnt >= cap) return false;  // support intact: estimate stands
        if (lane == 0) hist[capw - lo] = cnt;
    }
    __syncwarp();
    // Suffix scan of the window from its top bin: the largest k with
    // count(>= k) >= k.  Estimates fall by little per sweep, so the h-index
    // is nearly always in the first window.
    uint32_t carry = 0;
    int64_t hk;
    if (!R.ordered) {
        hk = hx_warp_scan(hist, lo, capw, lane, carry);
    } else {
        // all buckets >= b are in the histogram, so count(>= k) is exact for
        // k >= 2^b: scan down to there, then add the next bucket
        unsigned b = hx_bucket(capw);
        int64_t top = capw, jr = R.end(capw);
        for (;;) {
            const uint32_t kmin = max(max(1u << b, lo), 1u);
            hk = hx_warp_scan_from(hist, lo, top, kmin, lane, carry);
            if (hk >= 0 || (1u << b) <= lo || b == 0) break;
            top = (int64_t)kmin - 1;
            b--;
            const int64_t j1 = R.end(1u << b);
            hx_warp_gather(R.r, A.c, jr, j1, hist, lo, capw, 0u, 0u, lane);
            jr = j1;
            __syncwarp();
        }
    }
    const uint32_t h = hk >= 0 ? (uint32_t)hk : hx_warp_lower(R, A.c, hist, lo, carry, lane);
    __syncwarp();
    if (h >= cap) return false;
    if (lane == 0) A.c[v] = h;
    __syncwarp();
    // v stopped supporting exactly the neighbours u with h < c[u] <= cap.
    // An estimate read earlier in this call is at least the current one; it
    // can differ only if u was lowered concurrently in this sweep, and such a
    // u re-examines itself in the next sweep (below), after this write.
    if (cached) {
        bool cand[HX_CACHE];
#pragma unroll
        for (int k = 0; k < HX_CACHE; k++) cand[k] = cu[k] != 0xffffffffu && cv[k] > h && cv[k] <= cap;
        hx_activate_all(A, cu, cand, nxt, lane);
    } else {
        // candidates have degree > h: an ordered row is read that far
        const int64_t en = R.end(h + 1);
        for (int64_t jw = s; jw < en; jw += 32 * HX_STREAM) {  // warp-uniform trip count
            uint32_t uu[HX_STREAM], xx[HX_STREAM];
#pragma unroll
            for (int k = 0; k < HX_STREAM; k++) {
                const int64_t j = jw + k * 32 + lane;
                uu[k] = j < en ? R.r[j] : 0xffffffffu;
            }
#pragma unroll
            for (int k = 0; k < HX_STREAM; k++) xx[k] = uu[k] != 0xffffffffu ? __ldcg(&A.c[uu[k]]) : 0u;
            bool cand[HX_STREAM];
#pragma unroll
            for (int k = 0; k < HX_STREAM; k++) cand[k] = uu[k] != 0xffffffffu && xx[k] > h && xx[k] <= cap;
            hx_activate_all(A, uu, cand, nxt, lane);
        }
    }
    // A neighbour lowered in this sweep may have read c[v] before this write
    // and skipped v (its window test saw the old, higher value) while this
    // call counted it at its old estimate: v re-examines itself next sweep.
    if (lane == 0) hx_activate(A, v, nxt);
    return true;
}

// Four vertices per warp, one per group of 8 lanes, for rows of at most
// HX_TINY entries (4 per lane): the same steps as hx_warp_vertex (pending
// bit, support test, histogram of min(c[u], cap) over [0, cap] in the
// group's HX_TINY + 1 bins, suffix scan, notification window, self-requeue)
// with group-wide shuffles.  vg / valid: the vertex of this lane's group.
// Returns the number of estimates lowered (the same on every lane).
constexpr uint32_t HX_TINY = 32;

__device__ unsigned hx_warp_tiny(const HxArgs &A, uint32_t vg, bool valid, unsigned cur, bool clear,
                                 uint32_t *hist, unsigned lane) {
    const unsigned nxt = cur ^ 1u;
    const unsigned gi = lane >> 3, gl = lane & 7;
    int64_t s = 0, e = 0;
    uint32_t cap = 0;
    if (valid) {
        s = A.rowptr[vg];
        e = A.rowptr[vg + 1];
        if (clear && gl == 0) atomicAnd(&A.inlist[cur][vg >> 5], ~(1u << (vg & 31)));
        cap = __ldcg(&A.c[vg]);
    }
    uint32_t cu[4], cv[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int64_t j = s + gl + 8 * k;
        cu[k] = valid && j < e ? A.col[j] : 0xffffffffu;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) cv[k] = cu[k] != 0xffffffffu ? __ldcg(&A.c[cu[k]]) : 0u;
    uint32_t cnt = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) cnt += (cu[k] != 0xffffffffu && cv[k] >= cap) ? 1u : 0u;
    cnt += __shfl_xor_sync(KC_FULL_MASK, cnt, 1);
    cnt += __shfl_xor_sync(KC_FULL_MASK, cnt, 2);
    cnt += __shfl_xor_sync(KC_FULL_MASK, cnt, 4);
    const bool act = valid && cap > 0 && cnt < cap;  // the same on the group's lanes
    // bins [0, capt], capt = min(cap, row length) <= HX_TINY (see hx_warp_vertex)
    const uint32_t capt = min(cap, (uint32_t)(e - s));
    uint32_t *hb = hist + gi * (HX_TINY + 1);
    if (act)
        for (uint32_t b = gl; b <= capt; b += 8) hb[b] = 0;
    __syncwarp();
    if (act) {
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (cu[k] != 0xffffffffu) atomicAdd(&hb[cv[k] < capt ? cv[k] : capt], 1u);
    }
    __syncwarp();
    // lane gl holds bins capt - 4 gl - t (t = 0..3, from the top): suffix
    // counts from the bins of the lanes before it, then its own
    uint32_t loc[4], lsum = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const int k = (int)capt - 4 * (int)gl - t;
        loc[t] = act && k >= 1 ? hb[k] : 0u;
        lsum += loc[t];
    }
    uint32_t run = lsum;
#pragma unroll
    for (int d = 1; d < 8; d <<= 1) {
        const uint32_t y = __shfl_up_sync(KC_FULL_MASK, run, d, 8);
        if (gl >= (unsigned)d) run += y;
    }
    run -= lsum;
    int best = 0;  // the largest k with count(>= k) >= k (0 if none)
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const int k = (int)capt - 4 * (int)gl - t;
        run += loc[t];
        if (act && k >= 1 && run >= (uint32_t)k && best == 0) best = k;
    }
    best = max(best, __shfl_xor_sync(KC_FULL_MASK, best, 1));
    best = max(best, __shfl_xor_sync(KC_FULL_MASK, best, 2));
    best = max(best, __shfl_xor_sync(KC_FULL_MASK, best, 4));
    const uint32_t h = (uint32_t)best;
    const bool low = act && h < cap;
    if (low && gl == 0) A.c[vg] = h;
    __syncwarp();
    // notification window and self-requeue as in hx_warp_vertex
    bool cand[4];
#pragma unroll
    for (int k = 0; k < 4; k++) cand[k] = low && cu[k] != 0xffffffffu && cv[k] > h && cv[k] <= cap;
    hx_activate_all(A, cu, cand, nxt, lane);
    if (low && gl == 0) hx_activate(A, vg, nxt);
    return (unsigned)__popc(__ballot_sync(KC_FULL_MASK, low && gl == 0));
}

// Block-wide helpers for the CTA path.
__device__ __forceinline__ uint32_t block_sum(uint32_t x, uint32_t *red) {
    x = __reduce_add_sync(KC_FULL_MASK, x);
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = x;
    __syncthreads();
    uint32_t t = 0;
    for (int w = 0; w < HX_WARPS; w++) t += red[w];
    __syncthreads();
    return t;
}

// Bins b in [0, nb) cover values [base + b*w, base + (b+1)*w); `above` counts
// values beyond the last bin.  Returns the highest b whose suffix count
// above + sum_{b' >= b} hist[b'] reaches base + b*w (the h-index lies in that
// bin), or -1 if none does.
__device__ int hx_block_suffix_find(const uint32_t *hist, int nb, uint64_t base, uint64_t w, uint64_t above,
                                    uint32_t *red) {
    // each thread owns HX_BINS / HX_THREADS consecutive bins
    constexpr int PER = HX_BINS / HX_THREADS;
    const int t = threadIdx.x;
    // suffix sums: thread t covers bins [t*PER, t*PER+PER); we need, for each
    // bin, the count of bins above it -> scan in reverse thread order
    uint32_t local[PER];
    uint32_t sum = 0;
#pragma unroll
    for (int i = PER - 1; i >= 0; i--) {
        int b = t * PER + i;
        local[i] = b < nb ? hist[b] : 0u;
        sum += local[i];
    }
    // exclusive scan over threads in reverse order (threads above t)
    const unsigned lane = t & 31, warp = t >> 5;
    uint32_t v = sum;
    // reverse within warp: use shfl_down to accumulate lanes above
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_down_sync(KC_FULL_MASK, v, d);
        if (lane + d < 32) v += y;
    }
    // v = inclusive suffix within warp (this lane and above)
    __shared__ uint32_t wsum[HX_WARPS];
    __shared__ int best;
    if (lane == 0) wsum[warp] = v;
    if (t == 0) best = -1;
    __syncthreads();
    uint32_t warps_above = 0;
    for (int w2 = warp + 1; w2 < HX_WARPS; w2++) warps_above += wsum[w2];
    uint64_t suffix = (uint64_t)(v - sum) + warps_above + above;  // bins above this thread's range
    int mybest = -1;
#pragma unroll
    for (int i = PER - 1; i >= 0; i--) {
        int b = t * PER + i;
        suffix += local[i];
        if (b < nb && suffix >= base + (uint64_t)b * w && mybest < 0) mybest = b;
    }
    if (mybest >= 0) atomicMax(&best, mybest);
    __syncthreads();
    int r = best;
    __syncthreads();
    (void)red;
    return r;
}

// One CTA: recompute vertex v with a long row.
__device__ bool hx_block_vertex(const HxArgs &A, uint32_t v, unsigned nxt, uint32_t *hist, uint32_t *red) {
    const int64_t s = A.rowptr[v], e = A.rowptr[v + 1];
    __shared__ uint32_t cap_sh;
    __shared__ uint32_t pref_sh[32];  // ordered row: entries in degree buckets >= b
    const bool ordered = A.ord != nullptr && e - s > (int64_t)A.ord_min;
    const uint32_t *row = ordered ? A.ord : A.col;
    if (threadIdx.x == 0) cap_sh = __ldcg(&A.c[v]);
    if (ordered && threadIdx.x < 32) pref_sh[threadIdx.x] = A.pref[(size_t)A.lid[v] * 32 + threadIdx.x];
    __syncthreads();
    // end of the part of the row that holds every neighbour of degree >= t
    auto upto = [&](uint32_t t) -> int64_t { return ordered && t ? s + (int64_t)pref_sh[hx_bucket(t)] : e; };
    const uint32_t cap = cap_sh;
    if (cap == 0) return false;
    // capw: one above the h-index bound of an ordered row (see HxRow::hbound),
    // if that is below cap (then the support test cannot hold), else cap
    uint32_t capw = cap;
    if (ordered) {
        int b = 31;
        while (b > 0 && pref_sh[b] < (1u << b)) b--;
        const uint32_t hb = b >= 31 ? pref_sh[b] : min(pref_sh[b], (2u << b) - 1u);
        if (hb < cap) capw = hb + 1;
    }
    // Support test in chunks that double from 2,048 entries; it stops as
    // soon as cap neighbours at >= cap have been seen.  For capw <= HX_BINS
    // the same pass builds the histogram of the values below capw.
    const bool onepass = capw <= HX_BINS;
    if (onepass) {
        for (uint32_t b = threadIdx.x; b < capw; b += HX_THREADS) hist[b] = 0;
        __syncthreads();
    }
    uint32_t cnt = 0;  // values at or above capw
    int64_t span = 4 * HX_THREADS;
    const int64_t e1 = upto(capw);
    const uint32_t stop = capw == cap ? cap : 0xffffffffu;
    for (int64_t j0 = s; j0 < e1 && cnt < stop; span *= 2) {
        const int64_t j1 = e1 - j0 < span ? e1 : j0 + span;
        uint32_t c1 = 0;
        for (int64_t jb = j0 + threadIdx.x; jb < j1; jb += HX_CACHE * HX_THREADS) {
            uint32_t uu[HX_CACHE], xx[HX_CACHE];
#pragma unroll
            for (int k = 0; k < HX_CACHE; k++) {
                const int64_t j = jb + k * HX_THREADS;
                uu[k] = j < j1 ? row[j] : 0xffffffffu;
            }
#pragma unroll
            for (int k = 0; k < HX_CACHE; k++) xx[k] = uu[k] != 0xffffffffu ? __ldcg(&A.c[uu[k]]) : 0u;
#pragma unroll
            for (int k = 0; k < HX_CACHE; k++)
                if (uu[k] != 0xffffffffu) {
                    if (xx[k] >= capw) c1++;
                    else if (onepass) atomicAdd(&hist[xx[k]], 1u);
                }
        }
        cnt += block_sum(c1, red);
        j0 = j1;
    }
    if (capw == cap && cnt >= cap) return false;
    uint32_t h = 0;
    if (onepass && !ordered) {
        const int b = hx_block_suffix_find(hist, (int)capw, 0, 1, cnt, red);
        h = b < 0 ? 0u : (uint32_t)b;
    } else if (onepass) {
        // every bucket >= b is in the histogram, so count(>= k) is exact for
        // k >= 2^b: look for the h-index there, else add the next bucket
        unsigned b = hx_bucket(capw);
        int64_t jr = e1;
        for (;;) {
            const uint32_t kmin = 1u << b;
            const int r = hx_block_suffix_find(hist + kmin, (int)(capw - kmin), kmin, 1, cnt, red);
            if (r >= 0) {
                h = kmin + (uint32_t)r;
                break;
            }
            if (b == 0) break;  // no k >= 1 qualifies: h = 0
            b--;
            const int64_t j1 = upto(1u << b);
            for (int64_t jb = jr + threadIdx.x; jb < j1; jb += HX_CACHE * HX_THREADS) {
                uint32_t uu[HX_CACHE], xx[HX_CACHE];
#pragma unroll
                for (int k = 0; k < HX_CACHE; k++) {
                    const int64_t j = jb + k * HX_THREADS;
                    uu[k] = j < j1 ? row[j] : 0xffffffffu;
                }
#pragma unroll
                for (int k = 0; k < HX_CACHE; k++) xx[k] = uu[k] != 0xffffffffu ? __ldcg(&A.c[uu[k]]) : 0u;
#pragma unroll
                for (int k = 0; k < HX_CACHE; k++)
                    if (uu[k] != 0xffffffffu && xx[k] < capw) atomicAdd(&hist[xx[k]], 1u);
            }
            jr = j1;
            __syncthreads();
        }
    } else {
        // narrow [lo, hi) -- known to contain h -- with 4096-bin passes until
        // the bins are one value wide; `above` counts neighbours at >= hi.
        // A pass reads the part of the row that can hold values >= lo.
        uint64_t lo = 0, hi = capw;
        for (;;) {
            const uint64_t w = (hi - lo + HX_BINS - 1) / HX_BINS;
            const int nb = (int)((hi - lo + w - 1) / w);
            for (int b = threadIdx.x; b < (int)HX_BINS; b += HX_THREADS) hist[b] = 0;
            __syncthreads();
            uint32_t above = 0;
            const int64_t ee = upto((uint32_t)lo);
            for (int64_t j = s + threadIdx.x; j < ee; j += HX_THREADS) {
                uint32_t x = __ldcg(&A.c[row[j]]);
                if (x >= hi) above++;
                else if (x >= lo) atomicAdd(&hist[(x - lo) / w], 1u);
            }
            above = block_sum(above, red);
            int b = hx_block_suffix_find(hist, nb, lo, w, above, red);
            // The previous pass found count(>= lo) >= lo.  If estimates fell
            // since, none of the bins qualifies: the h-index of the current
            // estimates is below lo, so lo (bin 0) is still an upper bound of
            // the core number, and v re-examines itself in the next sweep.
            if (b < 0) b = 0;
            if (w == 1) {
                h = (uint32_t)(lo + b);
                break;
            }
            const uint64_t nlo = lo + (uint64_t)b * w;
            hi = nlo + w < hi ? nlo + w : hi;
            lo = nlo;
        }
    }
    if (h >= cap) return false;
    if (threadIdx.x == 0) A.c[v] = h;
    __syncthreads();
    // notification window and self-requeue as in hx_warp_vertex; candidates
    // have degree > h
    {
        const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int64_t en = upto(h + 1);
        // warp-uniform blocks of 32 * HX_CACHE entries
        for (int64_t jw = s + (int64_t)warp * 32 * HX_CACHE; jw < en; jw += (int64_t)HX_THREADS * HX_CACHE) {
            uint32_t uu[HX_CACHE], xx[HX_CACHE];
#pragma unroll
            for (int k = 0; k < HX_CACHE; k++) {
                const int64_t j = jw + k * 32 + lane;
                uu[k] = j < en ? row[j] : 0xffffffffu;
            }
#pragma unroll
            for (int k = 0; k < HX_CACHE; k++) xx[k] = uu[k] != 0xffffffffu ? __ldcg(&A.c[uu[k]]) : 0u;
            bool cand[HX_CACHE];
#pragma unroll
            for (int k = 0; k < HX_CACHE; k++) cand[k] = uu[k] != 0xffffffffu && xx[k] > h && xx[k] <= cap;
            hx_activate_all(A, uu, cand, nxt, lane);
        }
    }
    if (threadIdx.x == 0) hx_activate(A, v, nxt);
    __syncthreads();
    return true;
}

constexpr uint32_t HX_SMEM_WORDS =
    HX_WARPS * (HX_WARP_MAX + 1) > HX_BINS ? HX_WARPS * (HX_WARP_MAX + 1) : HX_BINS;

__global__ void __launch_bounds__(HX_THREADS, 2) hindex_kernel(HxArgs A) {
    __shared__ uint32_t hist[HX_SMEM_WORDS];
    __shared__ uint32_t red[HX_WARPS];
    __shared__ unsigned int changed_sh;  // estimates this CTA lowered in the sweep
    __shared__ unsigned long long item_sh;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    HindexCtl *ctl = A.ctl;
    const unsigned G = gridDim.x;
    if (A.withhold && blockIdx.x == 0) {
        // The barrier count never reaches the grid size: the other CTAs' waits
        // run into their limit.  This CTA waits (bounded) for their verdict.
        if (threadIdx.x == 0) {
            const unsigned long long t0 = global_ns();
            while (ld_relaxed(&ctl->err) == 0u) {
                if (global_ns() - t0 > A.timeout_ns) {
                    atomicCAS(&ctl->err, 0u, (unsigned)KC_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(1000);
            }
        }
        return;
    }
    for (uint32_t sweep = 0;; sweep++) {
        const unsigned cur = sweep & 1, nxt = cur ^ 1;
        if (threadIdx.x == 0) changed_sh = 0;
        __syncthreads();
        const bool tr = A.trace != nullptr && sweep < A.trace_cap;
        const unsigned long long t_sweep = tr ? global_ns() : 0ull;
        const bool all = sweep == 0 && A.first_all;
        const unsigned long long nsmall = all ? (unsigned long long)A.n : ld_relaxed64(&ctl->list_len[cur]);
        const unsigned long long nmid = all ? 0ull : ld_relaxed64(&ctl->mid_len[cur]);
        const unsigned long long nbig = ld_relaxed64(&ctl->big_len[cur]);
        if (tr && blockIdx.x == 0 && threadIdx.x == 0) {
            A.trace[sweep].t_start_ns = t_sweep;
            A.trace[sweep].level = sweep;
            A.trace[sweep].scan_len = (unsigned)(nsmall + nmid);
            A.trace[sweep].spilled = (unsigned)nbig;
        }
        // long rows: one CTA each, taken dynamically
        for (;;) {
            if (threadIdx.x == 0) item_sh = atomicAdd(&ctl->big_cursor, 1ull);
            __syncthreads();
            unsigned long long i = item_sh;
            __syncthreads();
            if (i >= nbig) break;
            uint32_t v = A.big[cur][i];
            if (!all && threadIdx.x == 0) atomicAnd(&A.inlist[cur][v >> 5], ~(1u << (v & 31)));
            __syncthreads();
            const bool low = hx_block_vertex(A, v, nxt, hist, red);
            if (low && threadIdx.x == 0) changed_sh++;
            if (tr && threadIdx.x == 0) {
                const int64_t len = A.rowptr[v + 1] - A.rowptr[v];
                atomicMax(&A.trace[sweep].max_steal, len > 0xffffffffll ? 0xffffffffu : (unsigned)len);
                if (low) atomicAdd(&A.trace[sweep].steals, 1u);
            }
            __syncthreads();
        }
        const unsigned long long t_big = tr ? global_ns() : 0ull;
        // medium rows, one per warp, then short rows, HX_GRAB consecutive
        // entries at a time, each taken from a shared cursor; sweep 0 covers
        // every short row
        uint32_t *wh = hist + warp * (HX_WARP_MAX + 1);
        unsigned wchanged = 0;
        while (nmid) {
            unsigned long long i = 0;
            if (lane == 0) i = atomicAdd(&ctl->mid_cursor, 1ull);
            i = __shfl_sync(KC_FULL_MASK, i, 0);
            if (i >= nmid) break;
            wchanged += hx_warp_vertex(A, A.list[cur][A.n - i], cur, true, wh, lane) ? 1u : 0u;
        }
        for (;;) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&ctl->cursor, (unsigned long long)HX_GRAB);
            base = __shfl_sync(KC_FULL_MASK, base, 0);
            if (base >= nsmall) break;
            const unsigned cntv = (unsigned)(nsmall - base < HX_GRAB ? nsmall - base : HX_GRAB);
            // the grab's vertices and row lengths on lanes 0..cntv-1; rows
            // of at most HX_TINY entries go four at a time, the others one
            // per warp (sweep 0 leaves rows above A.sweep0_rows to the CTAs)
            uint32_t vi = 0;
            int64_t di = 0;
            if (lane < cntv) {
                vi = all ? (uint32_t)(base + lane) : A.list[cur][base + lane];
                di = A.rowptr[vi + 1] - A.rowptr[vi];
            }
            const bool in = lane < cntv && !(all && di > (int64_t)A.sweep0_rows);
            unsigned tinym = __ballot_sync(KC_FULL_MASK, in && di <= (int64_t)HX_TINY);
            unsigned restm = __ballot_sync(KC_FULL_MASK, in && di > (int64_t)HX_TINY);
            while (tinym) {
                int pick = -1;  // this lane's group takes the (lane / 8)-th remaining tiny vertex
#pragma unroll
                for (unsigned g2 = 0; g2 < 4; g2++) {
                    const int p = tinym ? __ffs(tinym) - 1 : -1;
                    if (g2 == (lane >> 3)) pick = p;
                    tinym &= tinym - 1u;
                }
                const uint32_t vg = __shfl_sync(KC_FULL_MASK, vi, pick < 0 ? 0 : pick);
                wchanged += hx_warp_tiny(A, vg, pick >= 0, cur, !all, wh, lane);
            }
            while (restm) {
                const int p = __ffs(restm) - 1;
                restm &= restm - 1u;
                const uint32_t v = __shfl_sync(KC_FULL_MASK, vi, p);
                wchanged += hx_warp_vertex(A, v, cur, !all, wh, lane) ? 1u : 0u;
            }
        }
        if (lane == 0 && wchanged) atomicAdd(&changed_sh, wchanged);
        __syncthreads();
        if (threadIdx.x == 0 && changed_sh) atomicOr(&ctl->changed, 1u);
        const unsigned long long t_small = tr ? global_ns() : 0ull;
        if (tr && threadIdx.x == 0) {
            if (changed_sh) atomicAdd(&A.trace[sweep].claimed, changed_sh);
            atomicAdd(&A.trace[sweep].cta_ns[0], t_big - t_sweep);
            atomicAdd(&A.trace[sweep].cta_ns[1], t_small - t_big);
            atomicMax(&A.trace[sweep].t_work_end_ns, t_small);
        }
        if (!grid_barrier(&ctl->bar_count, &ctl->bar_gen, G, &ctl->err, KC_ERR_TIMEOUT, A.timeout_ns)) return;
        // one CTA resets the consumed lists; everyone reads the verdict after a second barrier
        __shared__ unsigned int go_on;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctl->list_len[cur] = 0;
            ctl->mid_len[cur] = 0;
            ctl->big_len[cur] = 0;
            ctl->big_cursor = 0;
            ctl->mid_cursor = 0;
            ctl->cursor = 0;
            ctl->sweeps = sweep + 1;
            ctl->changed = 0;
            // a sweep that lowered nothing queued nothing
            unsigned long long pend = ctl->list_len[nxt] + ctl->mid_len[nxt] + ctl->big_len[nxt];
            ctl->go_on = pend > 0 ? 1u : 0u;
            if (sweep + 1 >= A.max_sweeps && pend > 0) atomicCAS(&ctl->err, 0u, (unsigned)KC_ERR_CAPACITY);
            __threadfence();
        }
        if (!grid_barrier(&ctl->bar_count, &ctl->bar_gen, G, &ctl->err, KC_ERR_TIMEOUT, A.timeout_ns)) return;
        // CTA 0 rewrites the flag only after the next sweep's first barrier,
        // by which time every CTA has read it
        if (threadIdx.x == 0) go_on = ld_relaxed(&ctl->go_on);
        if (tr && threadIdx.x == 0) atomicAdd(&A.trace[sweep].cta_ns[2], global_ns() - t_small);
        __syncthreads();
        if (!go_on) return;
    }
}

static int ensure_hx_buffers(Graph *g) {
    const uint64_t n = g->n;
    if (!g->core) KC_TRY(dalloc(&g->core, n + 1, "core"));
    if (!g->bitmap) KC_TRY(dalloc(&g->bitmap, (n + 31) / 32 + 1, "active bitmap"));
    if (!g->hx_bitmap) KC_TRY(dalloc(&g->hx_bitmap, (n + 31) / 32 + 1, "active bitmap (odd sweeps)"));
    for (int i = 0; i < 2; i++) {
        if (!g->list[i]) KC_TRY(dalloc(&g->list[i], n + 1, "active list"));
        if (!g->big[i]) KC_TRY(dalloc(&g->big[i], n + 1, "active list (long rows)"));
    }
    if (!g->hctl) KC_TRY(dalloc(&g->hctl, 1, "h-index control"));
    // one trace record per sweep; sweeps beyond the capacity are not recorded
    const uint32_t tcap = (uint32_t)std::min<uint64_t>(n + 3, 65536);
    if (g->tune.trace && (!g->trace || g->trace_cap < tcap)) {
        dfree(g->trace);
        g->trace = nullptr;
        g->trace_cap = tcap;
        KC_TRY(dalloc(&g->trace, g->trace_cap, "h-index trace"));
    }
    return KC_OK;
}

// Rows above ord_min entries number at most nnz / (ord_min + 1).
static uint32_t order_min(const Graph *g) {
    return (uint32_t)std::max<int64_t>(HX_ORD_MIN, std::min<int64_t>(g->tune.hindex_order_min, 0x7fffffff));
}
static uint64_t max_long_rows(const Graph *g) { return g->nnz / ((uint64_t)order_min(g) + 1) + 1; }

// Rows up to this length are evaluated by one warp in sweep 0, where the
// estimates are still degrees: a warp's 512-value window below the estimate
// misses the h-index of a longer row unless the row is ordered (its prefix
// lengths bound the h-index, and the window is put below that bound).
static uint32_t sweep0_rows(const Graph *g, bool ordered) {
    return ordered && order_min(g) <= HX_WARP_MAX ? (uint32_t)g->tune.hindex_warp_rows : HX_WARP_MAX;
}

static void free_hx_order(Graph *g) {
    dfree(g->hx_ord);
    dfree(g->hx_bk);
    dfree(g->hx_lid);
    dfree(g->hx_vb);
    dfree(g->hx_pref);
    g->hx_ord = g->hx_lid = g->hx_pref = nullptr;
    g->hx_bk = g->hx_vb = nullptr;
    g->hx_ord_cap = g->hx_lid_cap = g->hx_pref_rows = 0;
}

// The buffers of the ordered copy, kept for later decompositions of the same
// graph (regrown when an update enlarged it); on a failed allocation all are
// released, so that a decomposition without the copy has the memory.
static int ensure_hx_order(Graph *g) {
    const uint64_t rows = max_long_rows(g);
    if (g->hx_ord && g->hx_bk && g->hx_ord_cap >= g->nnz && g->hx_lid && g->hx_vb && g->hx_lid_cap >= g->n &&
        g->hx_pref && g->hx_pref_rows >= rows)
        return KC_OK;
    free_hx_order(g);
    int rc = dalloc(&g->hx_ord, g->nnz + 1, "h-index ordered rows");
    if (!rc) rc = dalloc(&g->hx_bk, g->nnz + 1, "h-index entry buckets");
    if (!rc) rc = dalloc(&g->hx_lid, (uint64_t)g->n + 1, "h-index long-row index");
    if (!rc) rc = dalloc(&g->hx_vb, (uint64_t)g->n + 1, "h-index degree buckets");
    if (!rc) rc = dalloc(&g->hx_pref, rows * 32, "h-index bucket prefixes");
    if (rc) {
        free_hx_order(g);
        return rc;
    }
    g->hx_ord_cap = g->nnz;
    g->hx_lid_cap = g->n;
    g->hx_pref_rows = rows;
    return KC_OK;
}

static int hindex_launch(Graph *g, cudaStream_t s, kc_stats *st, bool first_all, bool ordered) {
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device);
    if (!coop) return fail(KC_ERR_UNSUPPORTED, "device lacks cooperative launch");
    int occ = 0;
    KC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, hindex_kernel, HX_THREADS, 0));
    if (occ < 1) return fail(KC_ERR_UNSUPPORTED, "h-index kernel cannot be resident");
    const int grid = occ * g->sm_count;
    HxArgs A;
    A.rowptr = g->rowptr;
    A.col = g->col;
    A.ord = ordered ? g->hx_ord : nullptr;
    A.lid = ordered ? g->hx_lid : nullptr;
    A.pref = ordered ? g->hx_pref : nullptr;
    A.ord_min = order_min(g);
    A.n = g->n;
    A.c = g->core;
    A.inlist[0] = g->bitmap;
    A.inlist[1] = g->hx_bitmap;
    A.list[0] = g->list[0];
    A.list[1] = g->list[1];
    A.big[0] = g->big[0];
    A.big[1] = g->big[1];
    A.ctl = g->hctl;
    A.timeout_ns = (unsigned long long)g->tune.wait_timeout_us * 1000ull;
    A.withhold = (unsigned)g->tune.withhold;
    // runaway guard only: every sweep but the one after a sweep without
    // change lowers an estimate, so sweeps <= 2 * (nnz + 1)
    A.max_sweeps = (uint32_t)std::min<uint64_t>(2 * ((uint64_t)g->nnz + 1) + 4, 0xffffffffull);
    A.first_all = first_all ? 1u : 0u;
    A.warp_rows = (uint32_t)g->tune.hindex_warp_rows;
    A.sweep0_rows = sweep0_rows(g, ordered);
    A.trace = g->tune.trace ? g->trace : nullptr;
    A.trace_cap = g->tune.trace ? g->trace_cap : 0;
    if (A.trace) KC_CUDA(cudaMemsetAsync(g->trace, 0, sizeof(PeelTrace) * g->trace_cap, s));
    void *args[] = {&A};
    KC_CUDA(cudaEventRecord(g->evk0, s));
    KC_CUDA(cudaLaunchCooperativeKernel((const void *)hindex_kernel, dim3(grid), dim3(HX_THREADS), args, 0, s));
    KC_CUDA(cudaEventRecord(g->evk1, s));
    KC_CUDA(cudaEventRecord(g->ev1, s));
    HindexCtl h;
    KC_CUDA(cudaMemcpyAsync(&h, g->hctl, sizeof(h), cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f, kms = 0.f;
    cudaEventElapsedTime(&ms, g->ev0, g->ev1);
    cudaEventElapsedTime(&kms, g->evk0, g->evk1);
    g->last_ms = ms;
    g->last_kernel_ms = kms;
    g->trace_count = A.trace ? std::min<uint32_t>(h.sweeps, g->trace_cap) : 0;
    if (h.err) {
        g->core_valid = false;
        return fail((int)h.err, "h-index kernel raised error %u", h.err);
    }
    g->core_valid = true;
    if (st) {
        st->iterations = h.sweeps;
        st->levels = 0;
        st->ms = ms;
    }
    return KC_OK;
}

static int ensure_events(Graph *g) {
    if (!g->ev0) {
        KC_CUDA(acquire_event(&g->ev0));
        KC_CUDA(acquire_event(&g->ev1));
        KC_CUDA(acquire_event(&g->evk0));
        KC_CUDA(acquire_event(&g->evk1));
    }
    return KC_OK;
}

int hindex_run(Graph *g, cudaStream_t s, kc_stats *st) {
    KC_TRY(ensure_hx_buffers(g));
    KC_TRY(ensure_events(g));
    bool ordered = g->tune.hindex_order && g->nnz > 0;
    if (ordered) {
        // without room for the copy (5 bytes per entry and a table), the
        // iteration reads the rows as they are
        const int rc = ensure_hx_order(g);
        if (rc == KC_ERR_NOMEM) {
            clear_error();
            ordered = false;
        } else if (rc) {
            return rc;
        }
    }
    KC_CUDA(cudaEventRecord(g->ev0, s));
    KC_CUDA(cudaMemsetAsync(g->hctl, 0, sizeof(HindexCtl), s));
    const int ig = std::max(1, std::min<int>(g->sm_count * 8, (int)((g->n + 255) / 256)));
    // the ordered copies of the long rows (part of every decomposition's
    // time); list[1] holds the rows to copy until sweep 0 queues vertices there
    hindex_init<<<ig, 256, 0, s>>>(g->rowptr, g->n, g->core, g->bitmap, g->hx_bitmap, g->big[0],
                                   sweep0_rows(g, ordered), ordered ? g->list[1] : nullptr, g->hx_lid,
                                   ordered ? g->hx_vb : nullptr, order_min(g), max_long_rows(g), g->hctl);
    if (ordered)
        hx_order_rows<<<g->sm_count * 4, HX_ORD_THREADS, 0, s>>>(g->rowptr, g->col, g->hx_vb, g->list[1], g->n,
                                                                 g->hctl, g->hx_ord, g->hx_pref, g->hx_bk,
                                                                 max_long_rows(g));
    return hindex_launch(g, s, st, true, ordered);
}

// Queue the vertices of `list` for sweep 0 (long rows to big[0]); the bitmap
// must be clear.
__global__ void hindex_seed(const int64_t *__restrict__ rowptr, const uint32_t *__restrict__ list, uint64_t len,
                            uint32_t *inlist, uint32_t *small0, uint32_t *big0, HindexCtl *ctl) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = list[i];
        const unsigned bit = 1u << (v & 31);
        if (atomicOr(&inlist[v >> 5], bit) & bit) continue;  // listed twice
        if (rowptr[v + 1] - rowptr[v] > (int64_t)HX_WARP_MAX) big0[atomicAdd(&ctl->big_len[0], 1ull)] = v;
        else small0[atomicAdd(&ctl->list_len[0], 1ull)] = v;
    }
}

// h-index iteration from the current contents of g->core (which must be
// upper bounds of the core numbers; after deletions they can exceed a
// vertex's degree), starting with the vertices of d_list active.  Used by the
// maintenance of dynamic graphs.
int hindex_run_from(Graph *g, const uint32_t *d_list, uint64_t len, cudaStream_t s, kc_stats *st) {
    KC_TRY(ensure_hx_buffers(g));
    KC_TRY(ensure_events(g));
    KC_CUDA(cudaEventRecord(g->ev0, s));
    KC_CUDA(cudaMemsetAsync(g->hctl, 0, sizeof(HindexCtl), s));
    KC_CUDA(cudaMemsetAsync(g->bitmap, 0, ((uint64_t)g->n + 31) / 32 * 4, s));
    KC_CUDA(cudaMemsetAsync(g->hx_bitmap, 0, ((uint64_t)g->n + 31) / 32 * 4, s));
    if (len) {
        const int ig = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)g->sm_count * 8, (len + 255) / 256));
        hindex_seed<<<ig, 256, 0, s>>>(g->rowptr, d_list, len, g->bitmap, g->list[0], g->big[0], g->hctl);
    }
    return hindex_launch(g, s, st, false, false);
}

}  // namespace kc
