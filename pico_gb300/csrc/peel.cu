// Persistent bucket peel: the k-core path of peelone / gppeel / peelone_dyn /
// peel_dyn (peel/peelone.cu:14-91,157-186; peel/gppeel.cu:12-104,398-440;
// peel/src/peelone-dyn.cc:2-117,141-158; peel/src/peel-dyn.cc:2-131,323-341)
// as ONE cooperative launch per decomposition instead of one host round trip
// per (sub)level.
//
// State per vertex: deg[v] (residual degree; equals the core number when the
// kernel returns) and one bit in `claimed` (v has been peeled).  Per level L:
//   * scan: every CTA walks its private segment of still-alive vertices,
//     claims those with deg <= L (atomicOr on the claim bit decides a unique
//     owner), compacts the survivors in place and records min(deg) of them;
//   * process: a claimed vertex's row is walked by one warp (rows above CHUNK
//     entries are split into chunk items that any CTA may take).  Each
//     unclaimed neighbour u gets atomicSub(deg[u]); the thread that moves u
//     from L+1 to L claims it and pushes it onto the CTA's shared-memory
//     queue, so sub-level cascades run inside the level without any grid
//     synchronisation (the reference repeats the level from the host or
//     relies on a block-local queue with a 1e6-entry device assert).  A
//     decrement that finds deg <= L is undone (the reference's clamp,
//     peelone.cu:80-86 / peelone-dyn.cc:95-98); values above L feed the
//     next-level minimum.
//   * level skipping: the next level is the smallest residual degree seen,
//     not L+1, so empty levels cost nothing.
// Work accounting instead of a grid barrier: every level has a counter of
// outstanding credits (one per CTA until its scan and queue are drained, plus
// every item spilled to the global queue).  A level ends when the counter is
// zero; idle CTAs steal spilled items meanwhile.  All waits are bounded by a
// wall-clock limit and report KC_ERR_TIMEOUT instead of hanging.
#include <algorithm>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

constexpr int PEEL_THREADS = 512;
constexpr int PEEL_WARPS = PEEL_THREADS / 32;
constexpr unsigned QCAP = 4096;       // shared-memory queue capacity (items)
constexpr unsigned LOW_WATER = 1024;  // scan a new tile only below this queue size
constexpr unsigned CHUNK = 2048;      // row entries per work item
constexpr unsigned long long SENT = ~0ull;
constexpr unsigned int NO_LEVEL = 0xffffffffu;

enum : int { M_SCAN = 1, M_PROC = 2, M_STEAL = 3, M_SPIN = 4, M_DONE = 5, M_EXIT = 6 };

struct PeelArgs {
    const int64_t *rowptr;
    const uint32_t *col;
    uint32_t n;
    uint32_t *deg;
    uint32_t *claimed;
    uint32_t *alive;
    unsigned long long *gq;
    unsigned long long gq_cap;
    PeelCtl *ctl;
    unsigned long long timeout_ns;
    uint32_t max_level_indices;
};

__global__ void peel_init(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t *deg, uint32_t *claimed,
                          PeelCtl *ctl, unsigned int grid) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += stride)
        deg[v] = (uint32_t)(rowptr[v + 1] - rowptr[v]);
    uint64_t words = ((uint64_t)n + 31) / 32;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < words; w += stride) claimed[w] = 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int i = 0; i < 3; i++) {
            ctl->pending[i] = grid;
            ctl->next_min[i] = NO_LEVEL;
            ctl->nonempty[i] = 0;
        }
        ctl->gq_head = 0;
        ctl->gq_tail = 0;
        ctl->err = 0;
        ctl->err_info = 0;
        ctl->level_indices = 0;
        ctl->levels = 0;
        ctl->kmax = 0;
    }
}

// Degree-0 vertices get core 1 in GPP mode (gppeel.cu:247-252: its first
// level is 1 and every vertex with residual degree <= level is deleted).
__global__ void gpp_zero_to_one(const int64_t *__restrict__ rowptr, uint32_t n, uint32_t *core) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        if (rowptr[v + 1] == rowptr[v]) core[v] = 1u;
}

__device__ __forceinline__ void set_err(PeelCtl *ctl, unsigned code, unsigned info) {
    if (atomicCAS(&ctl->err, 0u, code) == 0u) ctl->err_info = info;
}

__global__ void __launch_bounds__(PEEL_THREADS, 2) peel_kernel(PeelArgs A) {
    __shared__ unsigned long long q[QCAP];
    __shared__ unsigned int q_head, q_tail;
    __shared__ int mode;
    __shared__ unsigned int b_base, b_per_warp, b_take;
    __shared__ unsigned int scan_pos, scan_len, write_pos, scan_done;
    __shared__ unsigned long long credit;
    __shared__ unsigned int min_sh, claimed_any;
    __shared__ unsigned long long steal_base;
    __shared__ unsigned int steal_n;
    __shared__ unsigned int level_sh, li_sh;
    __shared__ unsigned long long wait_t0;
    __shared__ unsigned int warp_cnt[PEEL_WARPS];

    const unsigned tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned G = gridDim.x;
    PeelCtl *ctl = A.ctl;
    const uint32_t n = A.n;
    const uint32_t seg = (uint32_t)(((uint64_t)n + G - 1) / G);
    const uint64_t lo64 = (uint64_t)blockIdx.x * seg, hi64 = lo64 + seg;
    const uint32_t seg_lo = (uint32_t)(lo64 < n ? lo64 : n);
    const uint32_t seg_hi = (uint32_t)(hi64 < n ? hi64 : n);

    if (tid == 0) {
        q_head = q_tail = 0;
        level_sh = 0;
        li_sh = 0;
        scan_len = seg_hi - seg_lo;
    }
    __syncthreads();

    for (;;) {  // level loop
        const unsigned li = li_sh;
        const unsigned L = level_sh;
        const unsigned s = li % 3;
        if (tid == 0) {
            if (blockIdx.x == 0 && li >= 1) {
                unsigned s1 = (li + 1) % 3;
                ctl->pending[s1] = G;
                ctl->next_min[s1] = NO_LEVEL;
                ctl->nonempty[s1] = 0;
                __threadfence();
            }
            scan_pos = 0;
            write_pos = 0;
            scan_done = (scan_len == 0);
            credit = 1;  // this CTA's token for the level
            min_sh = NO_LEVEL;
            claimed_any = 0;
            wait_t0 = 0;
        }
        __syncthreads();

        for (;;) {  // work loop of one level
            if (tid == 0) {
                int md;
                unsigned qsize = q_tail - q_head;
                if (ld_relaxed(&ctl->err) != 0) {
                    md = M_EXIT;
                } else if (!scan_done && qsize < LOW_WATER) {
                    md = M_SCAN;
                } else if (qsize > 0) {
                    unsigned per = (qsize + PEEL_WARPS - 1) / PEEL_WARPS;
                    if (per > 32) per = 32;
                    unsigned take = min(qsize, per * PEEL_WARPS);
                    b_base = q_head;
                    b_per_warp = per;
                    b_take = take;
                    q_head += take;
                    md = M_PROC;
                } else {
                    // idle: hand back the credits held, after publishing this
                    // CTA's level minimum and claim flag
                    if (credit > 0) {
                        if (min_sh != NO_LEVEL) atomicMin(&ctl->next_min[s], min_sh);
                        if (claimed_any) {
                            ctl->nonempty[s] = 1u;
                            atomicMax(&ctl->kmax, L);
                        }
                        __threadfence();
                        atomicAdd(&ctl->pending[s], (unsigned long long)(0ull - credit));
                        credit = 0;
                    }
                    unsigned long long h = ld_relaxed64(&ctl->gq_head);
                    unsigned long long t = ld_relaxed64(&ctl->gq_tail);
                    if (t > A.gq_cap) t = A.gq_cap;  // an overflow was flagged; never read past the end
                    md = M_SPIN;
                    if (h < t) {
                        unsigned long long take = t - h;
                        if (take > QCAP / 2) take = QCAP / 2;
                        if (atomicCAS(&ctl->gq_head, h, h + take) == h) {
                            steal_base = h;
                            steal_n = (unsigned)take;
                            credit += take;
                            md = M_STEAL;
                            wait_t0 = 0;
                        }
                    } else if (ld_acquire64(&ctl->pending[s]) == 0ull) {
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
                mode = md;
            }
            __syncthreads();
            const int md = mode;
            if (md == M_DONE || md == M_EXIT) break;

            if (md == M_SPIN) {
                if (tid == 0) __nanosleep(200);
                __syncthreads();
                continue;
            }

            if (md == M_STEAL) {
                const unsigned long long base = steal_base;
                const unsigned cnt = steal_n;
                const unsigned qt = q_tail;
                for (unsigned j = tid; j < cnt; j += PEEL_THREADS) {
                    unsigned long long *slot = &A.gq[base + j];
                    unsigned long long it = ld_relaxed64(slot);
                    unsigned long long t0 = 0;
                    unsigned spins = 0;
                    while (it == SENT) {
                        if (ld_relaxed(&ctl->err) != 0) break;
                        if ((++spins & 255u) == 0) {
                            unsigned long long now = global_ns();
                            if (t0 == 0) t0 = now;
                            else if (now - t0 > A.timeout_ns) { set_err(ctl, KC_ERR_TIMEOUT, 2); break; }
                        }
                        __nanosleep(20);
                        it = ld_relaxed64(slot);
                    }
                    st_relaxed64(slot, SENT);
                    q[(qt + j) % QCAP] = it;
                }
                __syncthreads();
                if (tid == 0) q_tail = qt + cnt;
                __syncthreads();
                continue;
            }

            if (md == M_SCAN) {
                // ---- scan one tile of this CTA's alive segment ------------
                const unsigned pos = scan_pos + tid;
                const bool inr = pos < scan_len;
                uint32_t v = 0;
                bool keep = false, take = false;
                unsigned dkeep = NO_LEVEL;
                if (inr) {
                    v = (li == 0) ? seg_lo + pos : A.alive[seg_lo + pos];
                    unsigned w = __ldcg(&A.claimed[v >> 5]);
                    unsigned bit = 1u << (v & 31);
                    if (!(w & bit)) {
                        unsigned d = __ldcg(&A.deg[v]);
                        if ((int)d <= (int)L) {
                            unsigned old = atomicOr(&A.claimed[v >> 5], bit);
                            take = !(old & bit);
                        } else {
                            keep = true;
                            dkeep = d;
                        }
                    }
                }
                dkeep = __reduce_min_sync(KC_FULL_MASK, dkeep);
                if (lane == 0 && dkeep != NO_LEVEL) atomicMin(&min_sh, dkeep);
                // a claimed vertex with an empty row needs no processing
                const bool push = take && (A.rowptr[v + 1] != A.rowptr[v]);
                // survivors: in-place compaction (write index <= read index)
                unsigned kb = __ballot_sync(KC_FULL_MASK, keep);
                unsigned cb = __ballot_sync(KC_FULL_MASK, push);
                const unsigned tb = __ballot_sync(KC_FULL_MASK, take);
                if (lane == 0 && tb != 0u) claimed_any = 1;
                if (lane == 0) warp_cnt[warp] = __popc(kb) | (__popc(cb) << 16);
                __syncthreads();
                unsigned kofs = 0, cofs = 0, ktot = 0, ctot = 0;
                for (unsigned w2 = 0; w2 < PEEL_WARPS; w2++) {
                    unsigned x = warp_cnt[w2];
                    if (w2 < warp) {
                        kofs += x & 0xffffu;
                        cofs += x >> 16;
                    }
                    ktot += x & 0xffffu;
                    ctot += x >> 16;
                }
                const unsigned lt = (1u << lane) - 1u;
                if (keep) A.alive[seg_lo + write_pos + kofs + __popc(kb & lt)] = v;
                if (push) q[(q_tail + cofs + __popc(cb & lt)) % QCAP] = ((unsigned long long)v << 32);
                __syncthreads();
                if (tid == 0) {
                    write_pos += ktot;
                    q_tail += ctot;
                    scan_pos += PEEL_THREADS;
                    if (scan_pos >= scan_len) scan_done = 1;
                }
                __syncthreads();
                continue;
            }

            // ---- M_PROC: each warp expands its share of the queue ----------
            {
                const unsigned my_lo = b_base + warp * b_per_warp;
                const unsigned my_hi = min(my_lo + b_per_warp, b_base + b_take);
                const unsigned nit = my_hi > my_lo ? my_hi - my_lo : 0u;
                unsigned long long item = SENT;
                if (lane < nit) item = q[(my_lo + lane) % QCAP];
                int64_t rs = 0;
                uint32_t len = 0;
                if (item != SENT) {
                    uint32_t v = (uint32_t)(item >> 32);
                    uint32_t c = (uint32_t)item;
                    int64_t r0 = A.rowptr[v], r1 = A.rowptr[v + 1];
                    rs = r0 + (int64_t)c * CHUNK;
                    int64_t re = min(r1, rs + (int64_t)CHUNK);
                    len = re > rs ? (uint32_t)(re - rs) : 0u;
                    if (c == 0 && r1 - r0 > (int64_t)CHUNK) item |= 1ull << 31;  // mark: split needed
                }
                // split hub rows: chunk items 1..k-1 go to the global queue
                unsigned hubs = __ballot_sync(KC_FULL_MASK, item != SENT && (item & (1ull << 31)));
                while (hubs) {
                    const int src = __ffs(hubs) - 1;
                    hubs &= hubs - 1;
                    unsigned long long hi = __shfl_sync(KC_FULL_MASK, item, src);
                    uint32_t v = (uint32_t)(hi >> 32);
                    int64_t d = A.rowptr[v + 1] - A.rowptr[v];
                    unsigned k = (unsigned)((d + CHUNK - 1) / CHUNK);
                    unsigned extra = k - 1;
                    unsigned long long pos = 0;
                    if (lane == 0) {
                        atomicAdd(&ctl->pending[s], (unsigned long long)extra);
                        __threadfence();
                        pos = atomicAdd(&ctl->gq_tail, (unsigned long long)extra);
                        if (pos + extra > A.gq_cap) set_err(ctl, KC_ERR_CAPACITY, 3);
                    }
                    pos = __shfl_sync(KC_FULL_MASK, pos, 0);
                    if (pos + extra <= A.gq_cap)
                        for (unsigned j = lane; j < extra; j += 32)
                            st_relaxed64(&A.gq[pos + j], ((unsigned long long)v << 32) | (j + 1));
                }
                // expand the concatenated rows of this warp's items
                unsigned total;
                unsigned off = warp_excl_scan(len, lane, total);
                unsigned local_min = NO_LEVEL;
                for (unsigned base = 0; base < total; base += 32) {
                    const unsigned e = base + lane;
                    bool push = false;
                    uint32_t u = 0;
                    // owner = last lane j with off_j <= e
                    unsigned j = 0;
#pragma unroll
                    for (unsigned step = 16; step > 0; step >>= 1) {
                        unsigned cand = j + step;
                        unsigned oc = __shfl_sync(KC_FULL_MASK, off, cand & 31);
                        if (cand < 32 && oc <= e) j = cand;
                    }
                    int64_t rj = __shfl_sync(KC_FULL_MASK, rs, j);
                    unsigned oj = __shfl_sync(KC_FULL_MASK, off, j);
                    if (e < total) {
                        u = __ldcs(&A.col[rj + (e - oj)]);
                        const unsigned bit = 1u << (u & 31);
                        unsigned w = __ldcg(&A.claimed[u >> 5]);
                        if (!(w & bit)) {
                            unsigned a = atomicSub(&A.deg[u], 1u);
                            if (a == L + 1) {
                                unsigned old = atomicOr(&A.claimed[u >> 5], bit);
                                push = !(old & bit);
                            } else if ((int)a <= (int)L) {
                                atomicAdd(&A.deg[u], 1u);
                            } else {
                                local_min = min(local_min, a - 1);
                            }
                        }
                    }
                    unsigned pb = __ballot_sync(KC_FULL_MASK, push);
                    if (pb) {
                        // claimed neighbours: append to the CTA queue, or spill
                        // to the global queue when the ring would overwrite
                        // items of this step's batch (which starts at b_base)
                        const unsigned cnt = __popc(pb);
                        unsigned slot_lo = 0, slot_hi = 0;
                        int spill = 0;
                        if (lane == 0) {
                            unsigned t = q_tail;
                            for (;;) {
                                if (t + cnt - b_base > QCAP) { spill = 1; break; }
                                unsigned old = atomicCAS(&q_tail, t, t + cnt);
                                if (old == t) break;
                                t = old;
                            }
                            unsigned long long p = t;
                            if (spill) {
                                atomicAdd(&ctl->pending[s], (unsigned long long)cnt);
                                __threadfence();
                                p = atomicAdd(&ctl->gq_tail, (unsigned long long)cnt);
                                if (p + cnt > A.gq_cap) { set_err(ctl, KC_ERR_CAPACITY, 4); spill = 2; }
                            }
                            slot_lo = (unsigned)p;
                            slot_hi = (unsigned)(p >> 32);
                        }
                        spill = __shfl_sync(KC_FULL_MASK, spill, 0);
                        slot_lo = __shfl_sync(KC_FULL_MASK, slot_lo, 0);
                        slot_hi = __shfl_sync(KC_FULL_MASK, slot_hi, 0);
                        const unsigned r = __popc(pb & ((1u << lane) - 1u));
                        if (push) {
                            const unsigned long long itm = (unsigned long long)u << 32;
                            if (spill == 0)
                                q[(slot_lo + r) % QCAP] = itm;
                            else if (spill == 1)
                                st_relaxed64(&A.gq[(((unsigned long long)slot_hi << 32) | slot_lo) + r], itm);
                        }
                    }
                }
                local_min = __reduce_min_sync(KC_FULL_MASK, local_min);
                if (lane == 0 && local_min != NO_LEVEL) atomicMin(&min_sh, local_min);
                if (lane == 0 && nit) claimed_any = 1;
            }
            __syncthreads();
        }

        // ---- level boundary (all CTAs saw the level's credits reach zero) ----
        __syncthreads();
        if (tid == 0) {
            unsigned nxt = NO_LEVEL;
            if (mode == M_DONE) {
                __threadfence();
                nxt = ld_acquire(&ctl->next_min[s]);
                if (blockIdx.x == 0) {
                    ctl->level_indices = li + 1;
                    if (ld_relaxed(&ctl->nonempty[s])) ctl->levels += 1;
                }
                if (nxt != NO_LEVEL && li + 1 >= A.max_level_indices) {
                    set_err(ctl, KC_ERR_CAPACITY, 5);
                    nxt = NO_LEVEL;
                }
            }
            scan_len = write_pos;
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
    if (!g->alive) KC_TRY(dalloc(&g->alive, n + 1, "alive lists"));
    if (!g->gq) {
        g->gq_cap = 2 * n + g->nnz / CHUNK + 4096;
        KC_TRY(dalloc(&g->gq, g->gq_cap, "spill queue"));
        g->gq_clean = false;
    }
    if (!g->peel_ctl) KC_TRY(dalloc(&g->peel_ctl, 1, "peel control"));
    return KC_OK;
}

static int peel_grid(int sm_count, int *grid) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, peel_kernel, PEEL_THREADS, 0);
    if (e != cudaSuccess) return fail(KC_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
    if (occ < 1) return fail(KC_ERR_UNSUPPORTED, "peel kernel cannot be resident");
    *grid = occ * sm_count;
    return KC_OK;
}

int peel_run(Graph *g, cudaStream_t s, bool gpp_zero_to_one_flag, kc_stats *st) {
    KC_TRY(ensure_peel_buffers(g));
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device);
    if (!coop) return fail(KC_ERR_UNSUPPORTED, "device lacks cooperative launch");
    int grid = 0;
    KC_TRY(peel_grid(g->sm_count, &grid));
    if (!g->gq_clean) {
        KC_CUDA(cudaMemsetAsync(g->gq, 0xff, g->gq_cap * sizeof(unsigned long long), s));
        g->gq_clean = true;
    }
    if (!g->ev0) {
        KC_CUDA(cudaEventCreate(&g->ev0));
        KC_CUDA(cudaEventCreate(&g->ev1));
        KC_CUDA(cudaEventCreate(&g->evk0));
        KC_CUDA(cudaEventCreate(&g->evk1));
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
    A.timeout_ns = 20ull * 1000 * 1000 * 1000;
    A.max_level_indices = g->max_deg + 3;
    KC_CUDA(cudaEventRecord(g->ev0, s));
    const int ig = std::max(1, std::min<int>(g->sm_count * 8, (int)((g->n + 255) / 256)));
    peel_init<<<ig, 256, 0, s>>>(g->rowptr, g->n, g->core, g->bitmap, g->peel_ctl, (unsigned)grid);
    void *args[] = {&A};
    KC_CUDA(cudaEventRecord(g->evk0, s));
    KC_CUDA(cudaLaunchCooperativeKernel((const void *)peel_kernel, dim3(grid), dim3(PEEL_THREADS), args, 0, s));
    KC_CUDA(cudaEventRecord(g->evk1, s));
    if (gpp_zero_to_one_flag && g->n)
        gpp_zero_to_one<<<ig, 256, 0, s>>>(g->rowptr, g->n, g->core);
    KC_CUDA(cudaEventRecord(g->ev1, s));
    PeelCtl h;
    KC_CUDA(cudaMemcpyAsync(&h, g->peel_ctl, sizeof(h), cudaMemcpyDeviceToHost, s));
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
    if (st) {
        st->iterations = h.level_indices;
        st->levels = h.levels;
        st->kmax = h.kmax;
        st->ms = ms;
    }
    return KC_OK;
}

}  // namespace kc
