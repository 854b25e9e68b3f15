// Persistent bucket peel: the k-core path of peelone / gppeel / peelone_dyn /
// peel_dyn (peel/peelone.cu:14-91,157-186; peel/gppeel.cu:12-104,186-228;
// peel/src/peelone-dyn.cc:2-117,141-158; peel/src/peel-dyn.cc:2-131,155-171)
// as ONE cooperative launch per decomposition instead of one host round trip
// per (sub)level.
//
// State per vertex: deg[v] (residual degree; equals the core number when the
// kernel returns) and one bit in `claimed` (v has been peeled).  Per level L:
//   * scan: CTA b takes tiles b, b + G, b + 2G, ... (threads x SCAN_U
//     entries each) of the list of still-alive vertices, claims those with
//     deg <= L (atomicOr on the claim bit decides a unique owner), appends
//     the survivors to the next level's list and the claims to its queue
//     (one reservation per warp) and records min(deg) of the survivors;
//   * process: balanced rounds spread the row entries of the queued items
//     (up to round_e of them) over all threads of the CTA; rows above CHUNK
//     entries are split into chunk items that any CTA may take, and the
//     claims made while relaxing carry their row range in the item.  Each
//     unclaimed neighbour u gets atomicSub(deg[u]); the thread that moves u
//     from L+1 to L claims it and queues it, so sub-level cascades run inside
//     the level without grid synchronisation (the reference repeats the level
//     from the host, or uses a block-local queue guarded by a device assert).
//     A decrement that finds deg <= L is undone (the reference's clamp,
//     peelone.cu:80-86 / peelone-dyn.cc:95-98); values above L feed the
//     next-level minimum.  Each CTA keeps at most SPILL_T queued items in
//     shared memory; the rest go to a global queue that idle CTAs steal from.
//   * level skipping: the next level is the smallest residual degree seen,
//     not L+1, so empty levels cost nothing.
// Work accounting instead of a grid barrier: every level has a counter of
// outstanding credits (one per CTA until it finds no scan tile left and its
// queue drained, plus every item put on the global queue).  A level ends when
// the counter is zero.  All waits are bounded by a wall-clock limit and report
// KC_ERR_TIMEOUT instead of hanging.
#include <algorithm>
#include <cstddef>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

// Work items (64 bits): (v << 32) | c is chunk c of the row of vertex v
// (c < 2^31); a range item, bit 31 set, carries the row entries
// [r0, r0 + len) themselves (r0 < 2^40, len < 2^23), so that the CTA taking
// it needs no load of the row offsets.  Claims made while relaxing a row and
// the chunks of long rows are range items.
constexpr uint32_t RANGE_FLAG = 0x80000000u;
constexpr uint32_t RANGE_LEN = (1u << 23) - 1u;
__device__ __forceinline__ unsigned long long range_item(int64_t r0, uint32_t len) {
    return ((unsigned long long)((uint64_t)r0 >> 8) << 32) | RANGE_FLAG | ((uint32_t)(r0 & 0xff) << 23) | len;
}
__device__ __forceinline__ bool range_fits(int64_t r0, int64_t r1) {
    return r1 - r0 <= (int64_t)RANGE_LEN && r1 < ((int64_t)1 << 40) - 1;  // never the all-ones sentinel
}
constexpr unsigned LOW_WATER = 1024;  // take a new scan tile only below this queue size
constexpr unsigned MIN_CHUNK = 256;   // smallest row chunk (sizes the shared queues)
constexpr unsigned long long SENT = ~0ull;
constexpr unsigned int NO_LEVEL = 0xffffffffu;

enum : int { M_SCAN = 1, M_PROC = 2, M_STEAL = 3, M_SPIN = 4, M_DONE = 5, M_EXIT = 6 };

struct PeelArgs {
    const int64_t *rowptr;
    const uint32_t *col;
    uint32_t n;
    uint32_t *deg;
    uint32_t *claimed;
    uint32_t *alive;  // two lists of n entries
    unsigned long long *gq;      // 3 level slots x nq queues of gq_cap items
    unsigned long long gq_cap;
    PeelCtl *ctl;
    PeelTrace *trace;            // per-level trace or nullptr
    unsigned trace_cap;
    unsigned long long timeout_ns;
    uint32_t max_level_indices;
    unsigned chunk;              // row entries per work item
    unsigned spill_t;            // cascade items a CTA keeps locally
    unsigned steal_max;          // items per steal
    unsigned nq;                 // shared queues in use
    unsigned round_e;            // balanced rounds: row entries a CTA takes per round
    unsigned withhold;           // CTA 0 keeps one credit of level index 1 (failure-detection hook)
    unsigned aggregate;          // lanes of a warp decrementing the same vertex issue one atomicSub
};

// Initialisation and level 0 in one streaming pass: residual degrees from the
// row offsets; degree-0 vertices are peeled at level 0 (their claim bits are
// written whole, one warp ballot per 32-vertex word); every other vertex is
// appended to the alive list that level index 1 scans, and the smallest
// degree among them becomes level index 1's level.
__global__ void peel_init(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t *deg, uint32_t *claimed,
                          uint32_t *alive1, PeelCtl *ctl, unsigned int grid) {
    __shared__ unsigned int wcnt[32];
    __shared__ unsigned long long base_sh;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned dmin = 0xffffffffu;
    bool any_zero = false;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b0 = (uint64_t)blockIdx.x * blockDim.x; b0 < n; b0 += stride) {
        const uint64_t v = b0 + threadIdx.x;  // b0 is a multiple of 32: a warp covers one bitmap word
        uint32_t d = 0;
        const bool inr = v < n;
        if (inr) {
            d = (uint32_t)(rowptr[v + 1] - rowptr[v]);
            deg[v] = d;
        }
        const unsigned zero = __ballot_sync(KC_FULL_MASK, inr && d == 0);
        if (lane == 0 && v < n) claimed[v >> 5] = zero;
        any_zero |= zero != 0u;
        const bool keep = inr && d != 0;
        if (keep) dmin = min(dmin, d);
        const unsigned kb = __ballot_sync(KC_FULL_MASK, keep);
        if (lane == 0) wcnt[warp] = __popc(kb);
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned tot = 0;
            for (unsigned w = 0; w < nw; w++) {
                unsigned c = wcnt[w];
                wcnt[w] = tot;
                tot += c;
            }
            base_sh = tot ? atomicAdd(&ctl->out_len[0], (unsigned long long)tot) : 0ull;
        }
        __syncthreads();
        if (keep) alive1[base_sh + wcnt[warp] + __popc(kb & ((1u << lane) - 1u))] = (uint32_t)v;
        __syncthreads();
    }
    dmin = __reduce_min_sync(KC_FULL_MASK, dmin);
    if (lane == 0 && dmin != 0xffffffffu) atomicMin(&ctl->next_min[0], dmin);
    if (__any_sync(KC_FULL_MASK, any_zero) && lane == 0) atomicExch(&ctl->nonempty[0], 1u);
}

// Resets the control block before peel_init runs.
__global__ void peel_ctl_reset(PeelCtl *ctl, unsigned int grid) {
    for (int i = 0; i < 3; i++) {
        ctl->pending[i] = grid;
        ctl->scan_cursor[i] = 0;
        ctl->out_len[i] = 0;
        ctl->next_min[i] = NO_LEVEL;
        ctl->nonempty[i] = 0;
    }
    for (int sl = 0; sl < 3; sl++)
        for (int i = 0; i < PEEL_MAX_QUEUES; i++) {
            ctl->q[sl][i].head = 0;
            ctl->q[sl][i].tail = 0;
        }
    ctl->err = 0;
    ctl->err_info = 0;
    ctl->level_indices = 0;
    ctl->levels = 0;
    ctl->kmax = 0;
}

// Degree-0 vertices get core 1 in GPP mode (gppeel.cu:35-39: its first
// level is 1 and every vertex with residual degree <= level is deleted).
__global__ void gpp_zero_to_one(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t *core) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        if (rowptr[v + 1] == rowptr[v]) core[v] = 1u;
}

__device__ __forceinline__ void set_err(PeelCtl *ctl, unsigned code, unsigned info) {
    if (atomicCAS(&ctl->err, 0u, code) == 0u) ctl->err_info = info;
}

// PEEL_U: row entries each lane keeps in flight while walking rows; NT:
// threads per CTA (two CTAs of 512 or four of 256 per SM, 64 registers each);
// BAL: balanced processing rounds; SCAN_U: alive-list entries per thread per
// scan tile.
template <int PEEL_U, int NT, bool BAL, int SCAN_U>
__global__ void __launch_bounds__(NT, 1024 / NT) peel_kernel(PeelArgs A) {
    constexpr unsigned QCAP = 4096u;  // shared-memory queue capacity (items)
    // a scan tile is taken only while the queue has room for all its claims
    constexpr unsigned SCAN_BELOW = LOW_WATER < QCAP - NT * SCAN_U + 1 ? LOW_WATER : QCAP - NT * SCAN_U + 1;
    constexpr int PEEL_THREADS = NT;
    constexpr int PEEL_WARPS = NT / 32;
    constexpr unsigned TILE = NT * SCAN_U;
    __shared__ unsigned long long q[QCAP];
    __shared__ unsigned int q_head, q_tail;
    __shared__ unsigned int q_res;  // scan: queue slots reserved so far in this tile
    __shared__ int mode;
    __shared__ unsigned int b_base, b_per_warp, b_take;
    __shared__ unsigned long long tile_base, scan_len;
    __shared__ unsigned int scan_done;
    __shared__ unsigned long long credit;
    __shared__ unsigned int min_sh, claimed_any;
    __shared__ unsigned long long res_base, res_mask;  // reserved queue slots still expected
    __shared__ unsigned int steal_cnt, probe, claims_sh, spill_rr;
    __shared__ unsigned int level_sh, li_sh;
    __shared__ unsigned long long wait_t0;
    __shared__ unsigned long long next_tile;
    __shared__ unsigned int withheld;
    __shared__ unsigned int rounds_sh;
    __shared__ unsigned long long mode_ns[4], mode_t0;  // trace: time per mode in this level
    __shared__ int prev_mode;
    __shared__ unsigned int bal_off[BAL ? NT + 1 : 1];  // balanced rounds: item offsets,
    __shared__ int64_t bal_rs[BAL ? NT : 1];            // row starts,
    __shared__ unsigned int bal_wsum[NT / 32];          // per-warp sums

    const unsigned tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned G = gridDim.x;
    PeelCtl *ctl = A.ctl;
    const uint32_t n = A.n;

    if (tid == 0) {
        // level index 0 (the degree-0 vertices) was done by peel_init
        q_head = q_tail = 0;
        level_sh = ld_acquire(&ctl->next_min[0]);
        li_sh = 1;
        scan_len = ld_relaxed64(&ctl->out_len[0]);
        probe = blockIdx.x;
        spill_rr = blockIdx.x;
        res_mask = 0;
        steal_cnt = 0;
        withheld = 0;
    }
    __syncthreads();
    if (level_sh == NO_LEVEL) {  // every vertex had degree 0
        if (blockIdx.x == 0 && tid == 0) {
            ctl->level_indices = 1;
            ctl->levels = ld_relaxed(&ctl->nonempty[0]) ? 1u : 0u;
        }
        return;
    }
    if (blockIdx.x == 0 && tid == 0) {
        if (ld_relaxed(&ctl->nonempty[0])) ctl->levels = 1;
        if (A.trace && A.trace_cap) {
            A.trace[0].t_start_ns = global_ns();
            A.trace[0].level = 0;
            A.trace[0].scan_len = n;
            A.trace[0].claimed = n - (unsigned)scan_len;
        }
    }

    for (;;) {  // level loop
        const unsigned li = li_sh;
        const unsigned L = level_sh;
        const unsigned s = li % 3;
        const uint32_t *src = A.alive + (size_t)(li & 1) * n;
        uint32_t *dst = A.alive + (size_t)((li + 1) & 1) * n;
        if (tid == 0) {
            if (blockIdx.x == 0) {
                unsigned s1 = (li + 1) % 3;
                ctl->pending[s1] = G;
                ctl->scan_cursor[s1] = 0;
                ctl->out_len[s1] = 0;
                ctl->next_min[s1] = NO_LEVEL;
                ctl->nonempty[s1] = 0;
                for (unsigned i = 0; i < A.nq; i++) {
                    ctl->q[s1][i].head = 0;
                    ctl->q[s1][i].tail = 0;
                }
                __threadfence();
            }
            if (A.trace && blockIdx.x == 0 && li < A.trace_cap) {
                A.trace[li].t_start_ns = global_ns();
                A.trace[li].level = L;
                A.trace[li].scan_len = (unsigned)scan_len;
            }
            claims_sh = 0;
            next_tile = blockIdx.x;  // tiles blockIdx.x, +G, +2G, ... of the alive list
            scan_done = (scan_len == 0);
            credit = 1;  // this CTA's token for the level
            min_sh = NO_LEVEL;
            claimed_any = 0;
            wait_t0 = 0;
            rounds_sh = 0;
            if (A.trace) {
                mode_ns[0] = mode_ns[1] = mode_ns[2] = mode_ns[3] = 0;
                mode_t0 = global_ns();
                prev_mode = M_SPIN;
            }
        }
        __syncthreads();

        for (;;) {  // work loop of one level
            if (tid == 0) {
                int md = 0;
                unsigned qsize = q_tail - q_head;
                // the error flag is read only when this CTA has no work at
                // hand: a busy CTA finishes its local work first, and
                // reading the flag every step would put one more round trip
                // on the path of every scan tile and processing round
                if (!scan_done && qsize < SCAN_BELOW) {
                    unsigned long long t = next_tile * TILE;
                    if (t < scan_len) {
                        tile_base = t;
                        next_tile += G;
                        q_res = q_tail;
                        md = M_SCAN;
                    } else {
                        scan_done = 1;
                    }
                }
                if (!md && qsize > 0) {
                    if constexpr (BAL) {
                        // candidates; the round itself decides how many it takes
                        b_base = q_head;
                        b_take = min(qsize, (unsigned)NT);
                    } else {
                        unsigned per = (qsize + PEEL_WARPS - 1) / PEEL_WARPS;
                        if (per > 32) per = 32;
                        unsigned take = min(qsize, per * PEEL_WARPS);
                        b_base = q_head;
                        b_per_warp = per;
                        b_take = take;
                        q_head += take;
                    }
                    md = M_PROC;
                    rounds_sh++;
                }
                if (!md && ld_relaxed(&ctl->err) != 0) md = M_EXIT;
                if (!md) {
                    // idle: hand back the credits held, after publishing this
                    // CTA's level minimum and claim flag
                    if (credit > 0) {
                        if (A.trace && li < A.trace_cap) {
                            if (claims_sh) atomicAdd(&A.trace[li].claimed, claims_sh);
                            claims_sh = 0;
                            atomicMax(&A.trace[li].rounds, rounds_sh);
                            atomicMax(&A.trace[li].t_work_end_ns, global_ns());
                        }
                        if (min_sh != NO_LEVEL) atomicMin(&ctl->next_min[s], min_sh);
                        if (claimed_any) {
                            ctl->nonempty[s] = 1u;
                            atomicMax(&ctl->kmax, L);
                        }
                        __threadfence();
                        unsigned long long give = credit;
                        if (A.withhold && blockIdx.x == 0 && li == 1 && !withheld) {
                            // the level's count can no longer reach zero: every
                            // CTA's wait runs into its limit
                            give -= 1;
                            withheld = 1;
                        }
                        atomicAdd(&ctl->pending[s], (unsigned long long)(0ull - give));
                        credit = 0;
                    }
                    // Shared queues: a CTA reserves up to steal_max slots with one
                    // atomicAdd on the queue head (never fails) and takes the
                    // items as producers fill them.  Slots still empty when the
                    // level's credit count reaches zero will never be filled
                    // (producers push only while holding credit) and are dropped.
                    md = M_SPIN;
                    if (res_mask == 0) {
                        for (unsigned k = 0; k < A.nq; k++) {
                            const unsigned qi = (probe + k) % A.nq;
                            unsigned long long h = ld_relaxed64(&ctl->q[s][qi].head);
                            unsigned long long t = ld_relaxed64(&ctl->q[s][qi].tail);
                            if (t > A.gq_cap) t = A.gq_cap;  // an overflow was flagged; never read past the end
                            if (h >= t) continue;
                            unsigned long long want = (t - h + 3) / 4;
                            if (want > A.steal_max) want = A.steal_max;
                            unsigned long long r = atomicAdd(&ctl->q[s][qi].head, want);
                            if (r < A.gq_cap) {
                                if (r + want > A.gq_cap) want = A.gq_cap - r;
                                res_base = ((unsigned long long)s * A.nq + qi) * A.gq_cap + r;
                                res_mask = want >= 64 ? ~0ull : ((1ull << want) - 1);
                                if (A.trace && li < A.trace_cap) {
                                    atomicAdd(&A.trace[li].steals, 1u);
                                    atomicMax(&A.trace[li].max_steal, (unsigned)want);
                                }
                            }
                            probe = qi;
                            break;
                        }
                    }
                    if (res_mask != 0) {
                        const unsigned j0 = __ffsll((long long)res_mask) - 1;
                        if (ld_relaxed64(&A.gq[res_base + j0]) != SENT) {
                            md = M_STEAL;
                            wait_t0 = 0;
                        } else if (A.trace && li < A.trace_cap) {
                            atomicAdd(&A.trace[li].steal_fail, 1u);
                        }
                    }
                    if (md == M_SPIN) {
                        if (ld_acquire64(&ctl->pending[s]) == 0ull) {
                            res_mask = 0;  // the level is over: nothing more will arrive
                            md = M_DONE;
                        } else {
                            unsigned long long now = global_ns();
                            if (wait_t0 == 0) wait_t0 = now;
                            else if (now - wait_t0 > A.timeout_ns) {
                                set_err(ctl, KC_ERR_TIMEOUT, 1);
                                md = M_EXIT;
                            }
                        }
                    }
                }
                mode = md;
                if (A.trace) {
                    const unsigned long long now = global_ns();
                    const int pm = prev_mode;
                    const int slot = pm == M_SCAN ? 0 : pm == M_PROC ? 1 : pm == M_STEAL ? 2 : 3;
                    mode_ns[slot] += now - mode_t0;
                    mode_t0 = now;
                    prev_mode = md;
                }
            }
            __syncthreads();
            const int md = mode;
            if (md == M_DONE || md == M_EXIT) break;

            if (md == M_SPIN) {
                if (tid == 0) __nanosleep(100);
                __syncthreads();
                continue;
            }

            if (md == M_STEAL) {
                // take every filled slot of the reservation into the CTA queue
                const unsigned long long mask = res_mask;
                const unsigned qt = q_tail;
                if (tid < 64 && ((mask >> tid) & 1ull)) {
                    unsigned long long *slot = &A.gq[res_base + tid];
                    unsigned long long it = ld_relaxed64(slot);
                    if (it != SENT) {
                        st_relaxed64(slot, SENT);
                        unsigned pos = atomicAdd(&steal_cnt, 1u);
                        q[(qt + pos) % QCAP] = it;
                        atomicAnd(&res_mask, ~(1ull << tid));
                    }
                }
                __syncthreads();
                if (tid == 0) {
                    q_tail = qt + steal_cnt;
                    credit += steal_cnt;
                    steal_cnt = 0;
                }
                __syncthreads();
                continue;
            }

            if (md == M_SCAN) {
                // ---- scan one tile (SCAN_U entries per thread) of the alive list
                uint32_t v[SCAN_U];
                unsigned d[SCAN_U];
                bool inr[SCAN_U], keep[SCAN_U];
#pragma unroll
                for (int k = 0; k < SCAN_U; k++) {
                    const unsigned long long pos = tile_base + (unsigned)k * PEEL_THREADS + tid;
                    inr[k] = pos < scan_len;
                    v[k] = inr[k] ? src[pos] : 0u;
                }
                // The residual degree alone sorts the entries: a vertex peeled
                // at an earlier level holds its level (< L); one peeled at this
                // level holds L, or less while a clamped decrement is being
                // undone; a survivor holds more than L.  So no claim-bit read is
                // needed: entries at or below L try to claim, and the atomicOr
                // that claims returns whether someone (a relaxer, or this scan
                // at an earlier level) already had.
#pragma unroll
                for (int k = 0; k < SCAN_U; k++) d[k] = inr[k] ? __ldcg(&A.deg[v[k]]) : 0u;
                unsigned dkeep = NO_LEVEL;
                // claims: lanes whose vertices share a bitmap word set their
                // bits with one atomicOr by the lowest such lane; all the
                // atomics are issued before any result is used
                unsigned oldw[SCAN_U];
                int leader[SCAN_U];
                unsigned kb[SCAN_U];
                unsigned kcnt = 0;
#pragma unroll
                for (int k = 0; k < SCAN_U; k++) {
                    keep[k] = inr[k] && (int)d[k] > (int)L;
                    if (keep[k]) dkeep = min(dkeep, d[k]);
                    const bool want = inr[k] && !keep[k];
                    const unsigned word = want ? (v[k] >> 5) : 0xffffffffu;
                    const unsigned bit = want ? (1u << (v[k] & 31)) : 0u;
                    const unsigned peers = __match_any_sync(KC_FULL_MASK, word);
                    const unsigned bits = __reduce_or_sync(peers, bit);
                    leader[k] = __ffs(peers) - 1;
                    oldw[k] = 0;
                    if (want && (int)lane == leader[k]) oldw[k] = atomicOr(&A.claimed[word], bits);
                    kb[k] = __ballot_sync(KC_FULL_MASK, keep[k]);
                    kcnt += __popc(kb[k]);
                }
                // survivors: each warp reserves its run of the next alive list
                // with one atomicAdd, in flight with the claim atomics
                unsigned long long wbase = 0;
                if (lane == 0 && kcnt) wbase = atomicAdd(&ctl->out_len[s], (unsigned long long)kcnt);
                dkeep = __reduce_min_sync(KC_FULL_MASK, dkeep);
                if (lane == 0 && dkeep != NO_LEVEL) atomicMin(&min_sh, dkeep);
                unsigned cb[SCAN_U];
                unsigned ccnt = 0;
#pragma unroll
                for (int k = 0; k < SCAN_U; k++) {
                    const unsigned old = __shfl_sync(KC_FULL_MASK, oldw[k], leader[k]);
                    const bool take = inr[k] && !keep[k] && !(old & (1u << (v[k] & 31)));
                    // listed vertices have non-empty rows (the degree-0 ones
                    // are peeled by peel_init), so every claim is queued
                    cb[k] = __ballot_sync(KC_FULL_MASK, take);
                    ccnt += __popc(cb[k]);
                }
                // claims: each warp reserves queue slots in shared memory (the
                // tile was taken only while the queue had room for all of them)
                unsigned qb = 0;
                if (lane == 0 && ccnt) qb = atomicAdd(&q_res, ccnt);
                if (lane == 0 && ccnt) {
                    claimed_any = 1;
                    if (A.trace) atomicAdd(&claims_sh, ccnt);
                }
                wbase = __shfl_sync(KC_FULL_MASK, wbase, 0);
                qb = __shfl_sync(KC_FULL_MASK, qb, 0);
                const unsigned lt = (1u << lane) - 1u;
                unsigned ko = 0, co = 0;
#pragma unroll
                for (int k = 0; k < SCAN_U; k++) {
                    if (keep[k]) dst[wbase + ko + __popc(kb[k] & lt)] = v[k];
                    if (cb[k] & (1u << lane)) q[(qb + co + __popc(cb[k] & lt)) % QCAP] = ((unsigned long long)v[k] << 32);
                    ko += __popc(kb[k]);
                    co += __popc(cb[k]);
                }
                __syncthreads();
                if (tid == 0) q_tail = q_res;
                continue;
            }

            // ---- M_PROC ------------------------------------------------------
            // Unbalanced form: each warp expands the concatenated rows of its
            // own share of the queued items.  Balanced form (BAL): the CTA
            // takes queued items up to a budget of A.round_e row entries and
            // spreads those entries evenly over all its threads, so a round
            // never outlasts a few dependent memory round trips and a claim
            // made in it is picked up in the next round.
            {
                // the CTA queue's head once this round's items are taken (the
                // spill threshold counts the items queued behind it)
                unsigned round_head = q_head;
                unsigned bal_n = 0;  // balanced rounds: items taken
                unsigned long long item = SENT;
                unsigned nit;
                if constexpr (BAL) {
                    nit = tid < b_take ? 1u : 0u;
                    if (nit) item = q[(b_base + tid) % QCAP];
                } else {
                    const unsigned my_lo = b_base + warp * b_per_warp;
                    const unsigned my_hi = min(my_lo + b_per_warp, b_base + b_take);
                    nit = my_hi > my_lo ? my_hi - my_lo : 0u;
                    if (lane < nit) item = q[(my_lo + lane) % QCAP];
                }
                int64_t rs = 0, r0 = 0, r1 = 0;
                uint32_t len = 0;
                bool hub = false;
                if (item != SENT) {
                    const uint32_t lo = (uint32_t)item;
                    uint32_t c = 0;
                    if (lo & RANGE_FLAG) {
                        r0 = (int64_t)(((item >> 32) << 8) | ((lo >> 23) & 0xffu));
                        r1 = r0 + (lo & RANGE_LEN);
                    } else {
                        const uint32_t v = (uint32_t)(item >> 32);
                        c = lo;
                        r0 = A.rowptr[v];
                        r1 = A.rowptr[v + 1];
                    }
                    rs = r0 + (int64_t)c * A.chunk;
                    int64_t re = min(r1, rs + (int64_t)A.chunk);
                    len = re > rs ? (uint32_t)(re - rs) : 0u;
                    hub = (c == 0 && r1 - r0 > (int64_t)A.chunk);
                }
                unsigned total;
                unsigned off = warp_excl_scan(len, lane, total);
                if constexpr (BAL) {
                    // CTA-wide exclusive scan of the item lengths
                    if (lane == 0) bal_wsum[warp] = total;
                    __syncthreads();
                    unsigned wbase = 0, ctot = 0;
#pragma unroll
                    for (int w2 = 0; w2 < PEEL_WARPS; w2++) {
                        const unsigned x = bal_wsum[w2];
                        wbase += (w2 < (int)warp) ? x : 0u;
                        ctot += x;
                    }
                    off += wbase;
                    // the items that start within the budget (a prefix); each
                    // writes its start and, at the next index, its end (the
                    // next item's start: the same value), so the barrier that
                    // counts them also publishes the offsets
                    const bool inb = nit && off < A.round_e;
                    if (inb) {
                        bal_off[tid] = off;
                        bal_off[tid + 1] = off + len;
                        bal_rs[tid] = rs;
                    }
                    const unsigned take = (unsigned)__syncthreads_count(inb);
                    bal_n = take;
                    round_head = b_base + take;  // the rest stays queued
                    if (tid == 0) q_head = round_head;
                    hub = hub && inb;
                    (void)ctot;
                    total = bal_off[take];
                }
                // split hub rows: chunk items 1..k-1 go to the global queue
                unsigned hubs = __ballot_sync(KC_FULL_MASK, hub);
                while (hubs) {
                    const int srcl = __ffs(hubs) - 1;
                    hubs &= hubs - 1;
                    const int64_t h0 = __shfl_sync(KC_FULL_MASK, r0, srcl);
                    const int64_t h1 = __shfl_sync(KC_FULL_MASK, r1, srcl);
                    const int64_t d = h1 - h0;
                    unsigned k = (unsigned)((d + A.chunk - 1) / A.chunk);
                    unsigned extra = k - 1;
                    // spread the chunks over the shared queues, 32 per queue
                    for (unsigned c0 = 0; c0 < extra; c0 += 32) {
                        const unsigned cnt = min(32u, extra - c0);
                        unsigned qi = 0;
                        if (lane == 0) qi = atomicAdd(&spill_rr, 1u) % A.nq;
                        qi = __shfl_sync(KC_FULL_MASK, qi, 0);
                        unsigned long long pos = 0;
                        if (lane == 0) {
                            atomicAdd(&ctl->pending[s], (unsigned long long)cnt);
                            __threadfence();
                            pos = atomicAdd(&ctl->q[s][qi].tail, (unsigned long long)cnt);
                            if (pos + cnt > A.gq_cap) set_err(ctl, KC_ERR_CAPACITY, 3);
                            if (A.trace && li < A.trace_cap) atomicAdd(&A.trace[li].spilled, cnt);
                        }
                        pos = __shfl_sync(KC_FULL_MASK, pos, 0);
                        if (lane < cnt && pos + cnt <= A.gq_cap) {
                            // chunk c0 + lane + 1 as a range item
                            const int64_t cs = h0 + (int64_t)(c0 + lane + 1) * A.chunk;
                            const int64_t ce = min(h1, cs + (int64_t)A.chunk);
                            st_relaxed64(&A.gq[((unsigned long long)s * A.nq + qi) * A.gq_cap + pos + lane],
                                         range_item(cs, (uint32_t)(ce - cs)));
                        }
                    }
                }
                // expand the rows; each thread keeps PEEL_U entries in flight
                // (loads, then bitmap probes, then decrements) so the round
                // trips overlap
                constexpr unsigned SPAN = BAL ? (unsigned)NT : 32u;  // threads sharing the rows
                const unsigned me = BAL ? tid : lane;
                const bool single = !BAL && __ballot_sync(KC_FULL_MASK, len != 0) == 1u;  // one item, in lane 0
                unsigned local_min = NO_LEVEL;
                unsigned wclaims = 0;
                for (unsigned base = 0; base < total; base += SPAN * PEEL_U) {
                    uint32_t u[PEEL_U];
                    unsigned a[PEEL_U];
                    bool live[PEEL_U];
#pragma unroll
                    for (int k = 0; k < PEEL_U; k++) {
                        const unsigned e = base + k * SPAN + me;
                        int64_t rj;
                        unsigned oj;
                        live[k] = e < total;
                        if constexpr (BAL) {
                            // owner item: the last j with bal_off[j] <= e
                            unsigned lo = 0, hi2 = bal_n;
                            if (live[k]) {
                                while (hi2 - lo > 1) {
                                    const unsigned mid = (lo + hi2) >> 1;
                                    if (bal_off[mid] <= e) lo = mid;
                                    else hi2 = mid;
                                }
                            }
                            rj = bal_rs[lo];
                            oj = bal_off[lo];
                        } else if (single) {
                            rj = __shfl_sync(KC_FULL_MASK, rs, 0);
                            oj = 0;
                        } else {
                            // owner = last lane j with off_j <= e
                            unsigned j = 0;
#pragma unroll
                            for (unsigned step = 16; step > 0; step >>= 1) {
                                unsigned cand = j + step;
                                unsigned oc = __shfl_sync(KC_FULL_MASK, off, cand & 31);
                                if (cand < 32 && oc <= e) j = cand;
                            }
                            rj = __shfl_sync(KC_FULL_MASK, rs, j);
                            oj = __shfl_sync(KC_FULL_MASK, off, j);
                        }
                        u[k] = live[k] ? __ldcs(&A.col[rj + (e - oj)]) : 0u;
                    }
#pragma unroll
                    for (int k = 0; k < PEEL_U; k++) {
                        if (live[k]) {
                            unsigned w = __ldcg(&A.claimed[u[k] >> 5]);
                            live[k] = !(w & (1u << (u[k] & 31)));
                        }
                    }
                    // Warp-aggregated decrements: lanes holding the same
                    // vertex (hubs shared by many short rows) form a group
                    // whose lowest lane subtracts the group's size once.
                    unsigned cnt[PEEL_U];
#pragma unroll
                    for (int k = 0; k < PEEL_U; k++) {
                        cnt[k] = 1u;
                        if (A.aggregate) {
                            const unsigned peers = __match_any_sync(KC_FULL_MASK, live[k] ? u[k] : 0xffffffffu);
                            cnt[k] = __popc(peers);
                            if ((int)lane != __ffs(peers) - 1) live[k] = false;
                        }
                    }
#pragma unroll
                    for (int k = 0; k < PEEL_U; k++) a[k] = live[k] ? atomicSub(&A.deg[u[k]], cnt[k]) : 0u;
                    // The decrement (or group) that moved u from above L to L
                    // or below claims it and lifts it back to exactly L; a
                    // decrement that found u at or below L is undone (the
                    // reference's clamp).  A residual degree never falls below
                    // zero: it has lost at most one decrement per entry of its
                    // row.  The claim atomics of all PEEL_U entries are in
                    // flight together (with the row offsets of each candidate,
                    // so that its row can be queued as a range item).
                    unsigned oldc[PEEL_U];
                    int64_t cr0[PEEL_U], cr1[PEEL_U];
#pragma unroll
                    for (int k = 0; k < PEEL_U; k++) {
                        oldc[k] = ~0u;
                        cr0[k] = cr1[k] = 0;
                        if (live[k]) {
                            const unsigned nv = a[k] - cnt[k];
                            if ((int)a[k] <= (int)L) {
                                atomicAdd(&A.deg[u[k]], cnt[k]);
                            } else if (nv <= L) {
                                oldc[k] = atomicOr(&A.claimed[u[k] >> 5], 1u << (u[k] & 31));
                                cr0[k] = A.rowptr[u[k]];
                                cr1[k] = A.rowptr[u[k] + 1];
                                if (nv < L) atomicAdd(&A.deg[u[k]], L - nv);
                            } else {
                                local_min = min(local_min, nv);
                            }
                        }
                    }
#pragma unroll
                    for (int k = 0; k < PEEL_U; k++) {
                        const bool push = !(oldc[k] & (1u << (u[k] & 31)));
                        unsigned pb = __ballot_sync(KC_FULL_MASK, push);
                        wclaims += __popc(pb);
                        if (pb) {
                            // claimed neighbours: append to the CTA queue while it
                            // holds fewer than spill_t items (and the ring would not
                            // overwrite this step's batch, which starts at b_base);
                            // otherwise publish them on a shared queue
                            const unsigned cnt = __popc(pb);
                            unsigned slot_lo = 0, slot_hi = 0;
                            int spill = 0;
                            if (lane == 0) {
                                unsigned t = q_tail;
                                for (;;) {
                                    if (t + cnt - b_base > QCAP || t + cnt - round_head > A.spill_t) { spill = 1; break; }
                                    unsigned old = atomicCAS(&q_tail, t, t + cnt);
                                    if (old == t) break;
                                    t = old;
                                }
                                unsigned long long p = t;
                                if (spill) {
                                    const unsigned qi = atomicAdd(&spill_rr, 1u) % A.nq;
                                    atomicAdd(&ctl->pending[s], (unsigned long long)cnt);
                                    __threadfence();
                                    p = atomicAdd(&ctl->q[s][qi].tail, (unsigned long long)cnt);
                                    if (p + cnt > A.gq_cap) { set_err(ctl, KC_ERR_CAPACITY, 4); spill = 2; }
                                    p += ((unsigned long long)s * A.nq + qi) * A.gq_cap;
                                    if (A.trace && li < A.trace_cap) atomicAdd(&A.trace[li].spilled, cnt);
                                }
                                slot_lo = (unsigned)p;
                                slot_hi = (unsigned)(p >> 32);
                            }
                            spill = __shfl_sync(KC_FULL_MASK, spill, 0);
                            slot_lo = __shfl_sync(KC_FULL_MASK, slot_lo, 0);
                            slot_hi = __shfl_sync(KC_FULL_MASK, slot_hi, 0);
                            const unsigned r = __popc(pb & ((1u << lane) - 1u));
                            if (push) {
                                const unsigned long long itm = range_fits(cr0[k], cr1[k])
                                                                   ? range_item(cr0[k], (uint32_t)(cr1[k] - cr0[k]))
                                                                   : (unsigned long long)u[k] << 32;
                                if (spill == 0)
                                    q[(slot_lo + r) % QCAP] = itm;
                                else if (spill == 1)
                                    st_relaxed64(&A.gq[(((unsigned long long)slot_hi << 32) | slot_lo) + r], itm);
                            }
                        }
                    }
                }
                local_min = __reduce_min_sync(KC_FULL_MASK, local_min);
                if (lane == 0 && local_min != NO_LEVEL) atomicMin(&min_sh, local_min);
                if (lane == 0 && nit) claimed_any = 1;
                if (A.trace && lane == 0 && wclaims) atomicAdd(&claims_sh, wclaims);
            }
            __syncthreads();
        }

        // ---- level boundary (all CTAs saw the level's credits reach zero) ----
        __syncthreads();
        if (tid == 0 && A.trace && li < A.trace_cap) {
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (mode_ns[i]) atomicAdd(&A.trace[li].cta_ns[i], mode_ns[i]);
        }
        if (tid == 0) {
            unsigned nxt = NO_LEVEL;
            if (mode == M_DONE) {
                // pending reached zero (read with acquire) after every CTA's
                // last update of this slot: both values are final and are
                // fetched together
                __threadfence();
                nxt = ld_relaxed(&ctl->next_min[s]);
                scan_len = ld_relaxed64(&ctl->out_len[s]);
                if (blockIdx.x == 0) {
                    ctl->level_indices = li + 1;
                    if (ld_relaxed(&ctl->nonempty[s])) ctl->levels += 1;
                }
                if (nxt != NO_LEVEL && li + 1 >= A.max_level_indices) {
                    set_err(ctl, KC_ERR_CAPACITY, 5);
                    nxt = NO_LEVEL;
                }
            }
            level_sh = nxt;
            li_sh = li + 1;
        }
        __syncthreads();
        if (mode != M_DONE || level_sh == NO_LEVEL) break;
    }
}

// ------------------------------------------------------------ host -------
static int ensure_peel_buffers(Graph *g) {
    const uint64_t n = g->n;
    if (!g->core) KC_TRY(dalloc(&g->core, n + 1, "core"));
    if (!g->bitmap) KC_TRY(dalloc(&g->bitmap, (n + 31) / 32 + 1, "claim bitmap"));
    if (!g->alive) KC_TRY(dalloc(&g->alive, 2 * n + 2, "alive lists"));
    const unsigned nq = (unsigned)g->tune.peel_queues;
    const unsigned long long items = n + g->nnz / MIN_CHUNK + 64;
    if (!g->gq || g->gq_nq != nq || g->gq_items < items) {
        // Pushes per level <= n (each vertex is claimed once) + nnz/MIN_CHUNK
        // (row chunks).  Every CTA rotates over the queues one push (<= 32
        // items) at a time, so a queue receives at most total/nq + 32 items
        // per CTA.  Each level slot (3) has its own queues, restarted at 0
        // when the slot is recycled; consumed entries are reset to SENT.
        dfree(g->gq);
        g->gq = nullptr;
        const unsigned long long total = items + items / 4;  // room for the graph to grow
        const unsigned long long ctas = (unsigned long long)g->sm_count * 4;
        g->gq_cap = total / nq + 32 * ctas + 8192;
        g->gq_items = total;
        KC_TRY(dalloc(&g->gq, 3 * g->gq_cap * nq, "spill queues"));
        g->gq_nq = nq;
        g->gq_clean = false;
    }
    if (g->tune.trace && (!g->trace || g->trace_cap < g->max_deg + 3)) {
        dfree(g->trace);
        g->trace = nullptr;
        g->trace_cap = g->max_deg + 3;
        KC_TRY(dalloc(&g->trace, g->trace_cap, "peel trace"));
    }
    if (!g->peel_ctl) KC_TRY(dalloc(&g->peel_ctl, 1, "peel control"));
    return KC_OK;
}

// The kernel variant selected by the tunables, and its thread count.
template <int U, int NT, bool B>
static const void *peel_variant_su(int scan_u) {
    return scan_u == 8 ? (const void *)peel_kernel<U, NT, B, 8> : (const void *)peel_kernel<U, NT, B, 4>;
}

template <int U, int NT>
static const void *peel_variant_b(const Tuning &t) {
    return t.peel_balanced ? peel_variant_su<U, NT, true>(t.peel_scan_unroll) : peel_variant_su<U, NT, false>(t.peel_scan_unroll);
}

template <int NT>
static const void *peel_variant_u(const Tuning &t) {
    return t.peel_unroll == 8 ? peel_variant_b<8, NT>(t) : peel_variant_b<4, NT>(t);
}

static const void *peel_variant(const Tuning &t, int *threads) {
    *threads = t.peel_threads;
    return t.peel_threads == 256 ? peel_variant_u<256>(t) : peel_variant_u<512>(t);
}

static int peel_grid(const void *kern, int threads, int sm_count, int ctas_per_sm, int *grid) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, 0);
    if (e != cudaSuccess) return fail(KC_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
    if (occ < 1) return fail(KC_ERR_UNSUPPORTED, "peel kernel cannot be resident");
    if (ctas_per_sm > 0 && ctas_per_sm < occ) occ = ctas_per_sm;
    *grid = occ * sm_count;
    return KC_OK;
}

static unsigned nq_of(const Graph *g) { return g->gq_nq; }

int peel_run(Graph *g, cudaStream_t s, bool gpp_zero_to_one_flag, kc_stats *st) {
    KC_TRY(ensure_peel_buffers(g));
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device);
    if (!coop) return fail(KC_ERR_UNSUPPORTED, "device lacks cooperative launch");
    int grid = 0;
    int threads = 0;
    const void *kern = peel_variant(g->tune, &threads);
    KC_TRY(peel_grid(kern, threads, g->sm_count, g->tune.peel_ctas_per_sm, &grid));
    if (!g->gq_clean) {
        KC_CUDA(cudaMemsetAsync(g->gq, 0xff, 3 * g->gq_cap * g->gq_nq * sizeof(unsigned long long), s));
        g->gq_clean = true;
    }
    if (!g->ev0) {
        KC_CUDA(acquire_event(&g->ev0));
        KC_CUDA(acquire_event(&g->ev1));
        KC_CUDA(acquire_event(&g->evk0));
        KC_CUDA(acquire_event(&g->evk1));
    }
    PeelArgs A;
    A.rowptr = g->rowptr;
    A.col = g->col;
    A.n = g->n;
    A.deg = g->core;
    A.claimed = g->bitmap;
    A.alive = g->alive;
    A.gq = g->gq;
    A.gq_cap = g->gq_cap;
    A.ctl = g->peel_ctl;
    A.trace = g->tune.trace ? g->trace : nullptr;
    A.trace_cap = g->tune.trace ? g->trace_cap : 0;
    A.timeout_ns = (unsigned long long)g->tune.wait_timeout_us * 1000ull;
    A.withhold = (unsigned)g->tune.withhold;
    A.max_level_indices = g->max_deg + 3;
    // measured: 1024-entry chunks on R-MAT scale 22 (128 M entries), 2048 on
    // R-MAT scale 25 (1.07 B entries, 4% faster than 1024)
    A.chunk = g->tune.peel_chunk ? (unsigned)g->tune.peel_chunk : (g->nnz >= (1ull << 29) ? 2048u : 1024u);
    A.spill_t = (unsigned)g->tune.peel_spill;
    A.steal_max = (unsigned)g->tune.peel_steal;
    A.nq = nq_of(g);
    A.round_e = (unsigned)g->tune.peel_round_entries;
    A.aggregate = (unsigned)g->tune.peel_aggregate;
    KC_CUDA(cudaEventRecord(g->ev0, s));
    if (A.trace) KC_CUDA(cudaMemsetAsync(g->trace, 0, sizeof(PeelTrace) * g->trace_cap, s));
    const int ig = std::max(1, std::min<int>(g->sm_count * 8, (int)((g->n + 255) / 256)));
    peel_ctl_reset<<<1, 1, 0, s>>>(g->peel_ctl, (unsigned)grid);
    peel_init<<<ig, 256, 0, s>>>(g->rowptr, g->n, g->core, g->bitmap, g->alive + g->n, g->peel_ctl, (unsigned)grid);
    void *args[] = {&A};
    KC_CUDA(cudaEventRecord(g->evk0, s));
    KC_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(threads), args, 0, s));
    KC_CUDA(cudaEventRecord(g->evk1, s));
    if (gpp_zero_to_one_flag && g->n)
        gpp_zero_to_one<<<ig, 256, 0, s>>>(g->rowptr, g->n, g->core);
    KC_CUDA(cudaEventRecord(g->ev1, s));
    PeelCtl h;
    KC_CUDA(cudaMemcpyAsync(&h, g->peel_ctl, offsetof(PeelCtl, q), cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f, kms = 0.f;
    cudaEventElapsedTime(&ms, g->ev0, g->ev1);
    cudaEventElapsedTime(&kms, g->evk0, g->evk1);
    g->last_ms = ms;
    g->last_kernel_ms = kms;
    if (h.err) {
        g->gq_clean = false;
        g->core_valid = false;
        return fail((int)h.err, "peel kernel raised error %u at site %u", h.err, h.err_info);
    }
    g->core_valid = true;
    g->trace_count = A.trace ? std::min<uint32_t>(h.level_indices, g->trace_cap) : 0;
    if (st) {
        st->iterations = h.level_indices;
        st->levels = h.levels;
        st->kmax = h.kmax;
        st->ms = ms;
    }
    return KC_OK;
}

}  // namespace kc
