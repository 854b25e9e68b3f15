// Request server: continuous batching of k-core requests on one GPU.
//
// The reference has no serving path (each decomposition is a program run).
// A kc_server keeps one graph resident on the device and serves two kinds of
// requests concurrently:
//   * update: an edge batch applied to the resident graph with exact core
//     maintenance (kc_graph_update); updates run one after another in
//     submission order on their own lane;
//   * decompose: the core numbers of a graph sent with the request.  Waiting
//     requests are admitted as decomposition lanes free up and as device
//     memory allows (free device memory plus what this process's allocator
//     pool holds for reuse, minus a reserve and minus what admitted
//     requests may still allocate); a lane packs every admissible waiting
//     request (up to a graph count and byte budget) into one segmented CSR
//     and decomposes them in one batched launch, so requests arriving while
//     others run join the next launch.
// Each lane has its own CUDA stream, so updates and decompositions overlap on
// the device.  Latency is measured from submission to the result being on
// the host; the server reports p50 / p99 per request kind.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "kc_device.cuh"
#include "kc_internal.h"

namespace kc {

__host__ __device__ __forceinline__ uint64_t digest_mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Digest of a core array: sum over v of core[v] * mix(v + 1), mod 2^64, and
// the largest core.  Order-independent, so it can be reduced in parallel.
__global__ void core_digest(const uint32_t *__restrict__ core, uint32_t n, unsigned long long *out) {
    unsigned long long s = 0;
    uint32_t mx = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        s += (unsigned long long)core[v] * digest_mix(v + 1);
        mx = max(mx, core[v]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(KC_FULL_MASK, s, o);
    mx = __reduce_max_sync(KC_FULL_MASK, mx);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], s);
        atomicMax(&out[1], (unsigned long long)mx);
    }
}

uint64_t host_digest(const uint32_t *core, uint32_t n, uint32_t *kmax) {
    uint64_t s = 0;
    uint32_t mx = 0;
    for (uint32_t v = 0; v < n; v++) {
        s += (uint64_t)core[v] * digest_mix((uint64_t)v + 1);
        mx = std::max(mx, core[v]);
    }
    if (kmax) *kmax = mx;
    return s;
}

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    int kind = 0;  // 0 update, 1 decompose
    std::vector<uint32_t> is, id, ds, dd;
    bool want_core = false;
    std::vector<int64_t> rowptr;
    std::vector<uint32_t> col;
    uint32_t n = 0;
    uint64_t need = 0;  // device bytes estimate
    Clock::time_point t_submit, t_start, t_end;
    int status = KC_OK;
    std::string err;
    std::vector<uint32_t> core;
    uint32_t kmax = 0;
    uint64_t digest = 0;
    kc_update_stats ust{};
    bool done = false;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace kc

struct kc_server {
    kc_graph *g = nullptr;
    kc_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<kc::Request *> upd_q, dec_q;
    std::unordered_map<uint64_t, kc::Request *> reqs;
    std::vector<std::thread> workers;
    bool stop = false;
    uint64_t next_ticket = 1;
    uint64_t admitted_need = 0;  // device bytes of admitted, unfinished decompositions
    uint32_t running = 0, max_running = 0;
    // statistics
    std::vector<double> lat_upd, lat_dec;
    uint64_t n_upd = 0, n_dec = 0, n_rej = 0, edges_dec = 0, edges_upd = 0, launches = 0;
    bool started = false;
    kc::Clock::time_point t_first, t_last;
    unsigned long long *d_digest = nullptr;
};

namespace kc {

static void finish(kc_server *S, Request *r) {
    r->t_end = Clock::now();
    std::lock_guard<std::mutex> lk(S->mu);
    r->done = true;
    const double lat = ms_between(r->t_submit, r->t_end);
    if (r->status == KC_OK) {
        if (r->kind == 0) {
            S->lat_upd.push_back(lat);
            S->n_upd++;
            S->edges_upd += r->is.size() + r->ds.size();
        } else {
            S->lat_dec.push_back(lat);
            S->n_dec++;
            S->edges_dec += r->col.size() / 2;
        }
    } else {
        S->n_rej++;
    }
    S->t_last = r->t_end;
    S->cv_done.notify_all();
}

static void update_worker(kc_server *S) {
    cudaSetDevice(S->g->device);
    for (;;) {
        Request *r;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->upd_q.empty(); });
            if (S->upd_q.empty()) return;
            r = S->upd_q.front();
            S->upd_q.pop_front();
            S->running++;
            S->max_running = std::max(S->max_running, S->running);
        }
        r->t_start = Clock::now();
        Graph *g = S->g;
        NvtxRange nvtx_("server update request");
        int rc = graph_update(g, r->is.data(), r->id.data(), r->is.size(), r->ds.data(), r->dd.data(), r->ds.size(),
                              &r->ust);
        if (rc == KC_OK) {
            cudaMemsetAsync(S->d_digest, 0, 16, g->stream);
            if (g->n)
                core_digest<<<std::max(1, std::min<int>(g->sm_count * 4, (int)((g->n + 255) / 256))), 256, 0,
                              g->stream>>>(g->core, g->n, S->d_digest);
            unsigned long long h[2] = {0, 0};
            cudaMemcpyAsync(h, S->d_digest, 16, cudaMemcpyDeviceToHost, g->stream);
            if (r->want_core) {
                r->core.resize(g->n);
                if (g->n) cudaMemcpyAsync(r->core.data(), g->core, (uint64_t)g->n * 4, cudaMemcpyDeviceToHost, g->stream);
            }
            cudaError_t e = cudaStreamSynchronize(g->stream);
            if (e != cudaSuccess) {
                rc = fail(KC_ERR_CUDA, "update digest: %s", cudaGetErrorString(e));
            } else {
                r->digest = h[0];
                r->kmax = (uint32_t)h[1];
                r->n = g->n;
            }
        }
        if (rc) {
            r->status = rc;
            r->err = kc_last_error();
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->running--;
        }
        finish(S, r);
    }
}

// Decomposes one packed group of requests.
static int run_group(kc_server *S, std::vector<Request *> &grp) {
    const int dev = S->g->device;
    uint64_t n_tot = 0, nnz_tot = 0;
    for (Request *r : grp) {
        n_tot += r->n;
        nnz_tot += r->col.size();
    }
    if (n_tot >= 0xffffffffull) return fail(KC_ERR_CAPACITY, "packed batch exceeds uint32 vertex ids");
    kc_graph *pg = nullptr;
    if (grp.size() == 1) {
        Request *r = grp[0];
        KC_TRY(kc_graph_from_csr(r->rowptr.data(), r->col.data(), r->n, dev, &pg));
    } else {
        std::vector<int64_t> rp(n_tot + 1);
        std::vector<uint32_t> col(nnz_tot);
        uint64_t v = 0, e = 0;
        for (Request *r : grp) {
            for (uint32_t i = 0; i < r->n; i++) rp[v + i] = (int64_t)e + r->rowptr[i];
            for (size_t j = 0; j < r->col.size(); j++) col[e + j] = r->col[j] + (uint32_t)v;
            v += r->n;
            e += r->col.size();
        }
        rp[n_tot] = (int64_t)e;
        KC_TRY(kc_graph_from_csr(rp.data(), col.data(), (uint32_t)n_tot, dev, &pg));
    }
    std::vector<uint32_t> vbase(grp.size() + 1, 0);
    for (size_t i = 0; i < grp.size(); i++) vbase[i + 1] = vbase[i] + grp[i]->n;
    std::vector<uint32_t> core(std::max<uint64_t>(n_tot, 1));
    int rc;
    const uint32_t batch_limit = 200000;  // larger graphs: grid-wide peel
    if (grp.size() == 1 && grp[0]->n > batch_limit) {
        rc = kc_decompose(pg, KC_PEELONE_DYN, core.data(), 0, nullptr, nullptr);
    } else {
        kc_batch *b = nullptr;
        rc = kc_batch_create(pg, vbase.data(), (uint32_t)grp.size(), &b);
        if (!rc) {
            kc_batch_set_param(b, "batch.cuda_graph", 0);
            rc = kc_batch_decompose(b, core.data(), 0, nullptr, nullptr);
        }
        kc_batch_free(b);
    }
    kc_graph_free(pg);
    if (rc) return rc;
    for (size_t i = 0; i < grp.size(); i++) {
        Request *r = grp[i];
        r->core.assign(core.begin() + vbase[i], core.begin() + vbase[i + 1]);
        r->digest = host_digest(r->core.data(), r->n, &r->kmax);
    }
    return KC_OK;
}

static void decompose_worker(kc_server *S) {
    cudaSetDevice(S->g->device);
    for (;;) {
        std::vector<Request *> grp;
        uint64_t need = 0;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            for (;;) {
                if (S->stop && S->dec_q.empty()) return;
                if (!S->dec_q.empty()) {
                    size_t total_b = 0;
                    const size_t free_b = device_free_bytes(&total_b);
                    const uint64_t avail = free_b > S->cfg.hbm_reserve_bytes + S->admitted_need
                                               ? free_b - S->cfg.hbm_reserve_bytes - S->admitted_need
                                               : 0;
                    Request *head = S->dec_q.front();
                    if (head->need + S->cfg.hbm_reserve_bytes > total_b) {  // can never be admitted: reject
                        S->dec_q.pop_front();
                        head->status = KC_ERR_NOMEM;
                        head->err = "not admitted: request needs more device memory than the GPU keeps available";
                        lk.unlock();
                        finish(S, head);
                        lk.lock();
                        continue;
                    }
                    uint64_t bytes = 0;
                    while (!S->dec_q.empty() && grp.size() < S->cfg.max_batch_graphs) {
                        Request *r = S->dec_q.front();
                        if (need + r->need > avail) break;
                        if (!grp.empty() && bytes + r->need > S->cfg.max_batch_bytes) break;
                        if (!grp.empty() && r->n > 200000) break;  // large graphs run alone
                        grp.push_back(r);
                        need += r->need;
                        bytes += r->need;
                        S->dec_q.pop_front();
                        if (r->n > 200000) break;
                    }
                    if (!grp.empty()) {
                        S->admitted_need += need;
                        S->running++;
                        S->max_running = std::max(S->max_running, S->running);
                        S->launches++;
                        break;
                    }
                    // not admissible yet: wait for memory to free up
                    S->cv_work.wait_for(lk, std::chrono::milliseconds(1));
                    continue;
                }
                S->cv_work.wait(lk);
            }
        }
        const auto ts = Clock::now();
        for (Request *r : grp) r->t_start = ts;
        int rc;
        {
            NvtxRange nvtx_("server decomposition group");
            rc = run_group(S, grp);
        }
        std::string msg = rc ? std::string(kc_last_error()) : std::string();
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->admitted_need -= need;
            S->running--;
        }
        S->cv_work.notify_all();
        for (Request *r : grp) {
            if (rc) {
                r->status = rc;
                r->err = msg;
            }
            finish(S, r);
        }
    }
}

static double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

static uint64_t submit(kc_server *S, Request *r) {
    std::lock_guard<std::mutex> lk(S->mu);
    r->ticket = S->next_ticket++;
    r->t_submit = Clock::now();
    if (!S->started) {
        S->started = true;
        S->t_first = r->t_submit;
    }
    S->reqs[r->ticket] = r;
    (r->kind == 0 ? S->upd_q : S->dec_q).push_back(r);
    S->cv_work.notify_all();
    return r->ticket;
}

}  // namespace kc

using namespace kc;

extern "C" {

int kc_server_create(kc_graph *resident, const kc_server_config *cfg, kc_server **out) {
    clear_error();
    if (!resident || !out) return fail(KC_ERR_INVALID, "null argument");
    *out = nullptr;
    KC_CUDA(cudaSetDevice(resident->device));
    kc_server *S = new (std::nothrow) kc_server();
    if (!S) return fail(KC_ERR_NOMEM, "server handle");
    S->g = resident;
    S->cfg.decompose_slots = 2;
    S->cfg.max_batch_graphs = 64;
    S->cfg.max_batch_bytes = 256ull << 20;
    S->cfg.hbm_reserve_bytes = 1ull << 30;
    if (cfg) {
        if (cfg->decompose_slots) S->cfg.decompose_slots = std::min<uint32_t>(cfg->decompose_slots, 16);
        if (cfg->max_batch_graphs) S->cfg.max_batch_graphs = cfg->max_batch_graphs;
        if (cfg->max_batch_bytes) S->cfg.max_batch_bytes = cfg->max_batch_bytes;
        S->cfg.hbm_reserve_bytes = cfg->hbm_reserve_bytes;
    }
    int rc = dalloc(&S->d_digest, 2, "digest");
    if (rc) {
        delete S;
        return rc;
    }
    if (!resident->core_valid) {
        rc = peel_run(resident, resident->stream, false, nullptr);
        if (rc) {
            dfree(S->d_digest);
            delete S;
            return rc;
        }
    }
    S->workers.emplace_back(update_worker, S);
    for (uint32_t i = 0; i < S->cfg.decompose_slots; i++) S->workers.emplace_back(decompose_worker, S);
    *out = S;
    return KC_OK;
}

int kc_server_submit_update(kc_server *S, const uint32_t *ins_src, const uint32_t *ins_dst, uint64_t n_ins,
                            const uint32_t *del_src, const uint32_t *del_dst, uint64_t n_del, int want_core,
                            uint64_t *ticket) {
    clear_error();
    if (!S || !ticket || (n_ins && (!ins_src || !ins_dst)) || (n_del && (!del_src || !del_dst)))
        return fail(KC_ERR_INVALID, "null argument");
    Request *r = new (std::nothrow) Request();
    if (!r) return fail(KC_ERR_NOMEM, "request");
    r->kind = 0;
    r->is.assign(ins_src, ins_src + n_ins);
    r->id.assign(ins_dst, ins_dst + n_ins);
    r->ds.assign(del_src, del_src + n_del);
    r->dd.assign(del_dst, del_dst + n_del);
    r->want_core = want_core != 0;
    *ticket = submit(S, r);
    return KC_OK;
}

int kc_server_submit_decompose(kc_server *S, const int64_t *rowptr, const uint32_t *col, uint32_t n,
                               uint64_t *ticket) {
    clear_error();
    if (!S || !ticket || !rowptr) return fail(KC_ERR_INVALID, "null argument");
    const int64_t nnz = rowptr[n];
    if (nnz < 0 || (nnz && !col)) return fail(KC_ERR_INVALID, "bad CSR");
    Request *r = new (std::nothrow) Request();
    if (!r) return fail(KC_ERR_NOMEM, "request");
    r->kind = 1;
    r->n = n;
    r->rowptr.assign(rowptr, rowptr + n + 1);
    r->col.assign(col, col + nnz);
    // device footprint: CSR, core, batch queues, degrees and alive lists,
    // with headroom
    r->need = 3 * (8ull * (n + 1) + 4ull * nnz) + 24ull * n + (1ull << 20);
    *ticket = submit(S, r);
    return KC_OK;
}

int kc_server_wait(kc_server *S, uint64_t ticket, kc_request_result *res, uint32_t *core_out, uint64_t core_cap) {
    clear_error();
    if (!S) return fail(KC_ERR_INVALID, "null server");
    Request *r;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->reqs.find(ticket);
        if (it == S->reqs.end()) return fail(KC_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
        r = it->second;
        S->cv_done.wait(lk, [&] { return r->done; });
        S->reqs.erase(it);
    }
    int rc = r->status;
    if (res) {
        memset(res, 0, sizeof(*res));
        res->status = r->status;
        res->kind = (uint32_t)r->kind;
        res->n = r->n;
        res->kmax = r->kmax;
        res->digest = r->digest;
        res->latency_ms = ms_between(r->t_submit, r->t_end);
        res->queue_ms = ms_between(r->t_submit, r->t_start);
        res->update = r->ust;
        res->has_core = r->core.empty() ? 0u : 1u;
    }
    if (core_out && !r->core.empty()) {
        if (core_cap < r->core.size()) rc = rc ? rc : fail(KC_ERR_CAPACITY, "core buffer too small");
        else memcpy(core_out, r->core.data(), r->core.size() * 4);
    }
    if (r->status) fail(r->status, "%s", r->err.c_str());
    delete r;
    return rc;
}

int kc_server_get_stats(kc_server *S, kc_server_stats *st) {
    clear_error();
    if (!S || !st) return fail(KC_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    memset(st, 0, sizeof(*st));
    st->completed_updates = S->n_upd;
    st->completed_decompositions = S->n_dec;
    st->failed = S->n_rej;
    st->p50_update_ms = percentile(S->lat_upd, 0.50);
    st->p99_update_ms = percentile(S->lat_upd, 0.99);
    st->p50_decompose_ms = percentile(S->lat_dec, 0.50);
    st->p99_decompose_ms = percentile(S->lat_dec, 0.99);
    st->elapsed_ms = S->started ? ms_between(S->t_first, S->t_last) : 0.0;
    st->edges_decomposed = S->edges_dec;
    st->edges_updated = S->edges_upd;
    st->decompose_launches = S->launches;
    st->max_inflight = S->max_running;
    return KC_OK;
}

int kc_server_free(kc_server *S) {
    clear_error();
    if (!S) return KC_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (auto &t : S->workers) t.join();
    for (auto &kv : S->reqs) delete kv.second;
    cudaSetDevice(S->g->device);
    dfree(S->d_digest);
    delete S;
    return KC_OK;
}

}  // extern "C"
