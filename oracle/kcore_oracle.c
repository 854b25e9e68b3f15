/*
 * kcore_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of chriszhao13/pico's k-core algorithms, used as the parity
 * checker for the CUDA engine in pico_gb300.  Only the tests, the smoke check
 * and bench.py's CPU-baseline leg load this file; the product never does.
 *
 * Contents
 *   orc_bz            serial Batagelj-Zaversnik bucket peel (Batagelj &
 *                     Zaversnik, "An O(m) Algorithm for Cores Decomposition of
 *                     Networks", 2003).  The reference has no CPU k-core code,
 *                     so this is the primary oracle, written from the paper.
 *   orc_hindex_jacobi synchronous h-index iteration restating the common
 *                     trajectory of index2core/NbrCore.cu:78-113,244-297,
 *                     index2core/CntCore.cu:82-130,344-417 and
 *                     index2core/HistoCore.cu:77-128,292-341 (all three apply
 *                     the h-index operator to every vertex whose neighbourhood
 *                     changed, from core = degree).
 *   orc_peel_rounds   level-synchronous peel restating peel/peelone.cu:14-91,
 *                     157-186 with one round per kernel launch.
 *   orc_gpp           two-phase scan/scatter peel restating
 *                     peel/gppeel.cu:12-104,186-228, including its core = 1
 *                     for degree-0 vertices.
 *   orc_peel_dyn      per-level select + queue peel restating
 *                     peel/src/peelone-dyn.cc:2-117,120-168.
 *   orc_make_ugraph   inline-degree CSR + virtual nodes restating
 *                     index2core/shared/virtual_graph.cpp:96-192.
 *   orc_csr_dedup     sorted, de-duplicated CSR restating
 *                     peel/src/graph.cpp:103-131.
 *   orc_check_local   per-vertex fixpoint test of a core vector.
 *   orc_gen_rmat_mt / orc_csr_dedup_mt  the host R-MAT generator and the
 *                     de-duplicating CSR build on several threads (the
 *                     CPU arm of the benchmark builds billion-entry graphs).
 *
 * Parity is pinned by the reference's own known answer (example.txt: every
 * core is 2) and by golden files produced with the reference's own loader and
 * virtual-graph code compiled from its sources (see oracle/build_ref.sh and
 * tests/golden/make_golden.py).
 *
 * Graph input convention for the decomposition routines: CSR with int64 row
 * offsets rowptr[n+1] and uint32 column ids col[rowptr[n]], both directions of
 * every undirected edge present, no self-loops.  Parallel entries (the
 * reference's COO loader keeps duplicate lines) count with multiplicity.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_ENOMEM 4

/* ------------------------------------------------------------------------ */
/* Batagelj-Zaversnik (2003), Algorithm 1 of the paper: bin-sort vertices by
 * degree, then repeatedly take the vertex of least residual degree and move
 * each neighbour with a larger residual degree one bin down. O(n + m).      */
int64_t orc_bz(uint32_t n, const int64_t *rowptr, const uint32_t *col, uint32_t *core)
{
    if (n == 0) return 0;
    uint32_t md = 0;
    for (uint32_t v = 0; v < n; v++) {
        uint64_t d = (uint64_t)(rowptr[v + 1] - rowptr[v]);
        core[v] = (uint32_t)d;
        if (core[v] > md) md = core[v];
    }
    uint64_t *bin = (uint64_t *)calloc((size_t)md + 1, sizeof(uint64_t));
    uint32_t *vert = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    uint32_t *pos = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    if (!bin || !vert || !pos) { free(bin); free(vert); free(pos); return -ORC_ENOMEM; }
    for (uint32_t v = 0; v < n; v++) bin[core[v]]++;
    uint64_t start = 0;
    for (uint32_t d = 0; d <= md; d++) { uint64_t num = bin[d]; bin[d] = start; start += num; }
    for (uint32_t v = 0; v < n; v++) { pos[v] = (uint32_t)bin[core[v]]; vert[pos[v]] = v; bin[core[v]]++; }
    for (uint32_t d = md; d >= 1; d--) bin[d] = bin[d - 1];
    bin[0] = 0;
    uint32_t kmax = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t v = vert[i];
        uint32_t cv = core[v];
        if (cv > kmax) kmax = cv;
        for (int64_t e = rowptr[v]; e < rowptr[v + 1]; e++) {
            uint32_t u = col[e];
            if (core[u] > cv) {
                uint32_t du = core[u];
                uint32_t pu = pos[u];
                uint32_t pw = (uint32_t)bin[du];
                uint32_t w = vert[pw];
                if (u != w) { pos[u] = pw; vert[pu] = w; pos[w] = pu; vert[pw] = u; }
                bin[du]++;
                core[u]--;
            }
        }
    }
    free(bin); free(vert); free(pos);
    return kmax;
}

/* ------------------------------------------------------------------------ */
/* h-index of the multiset {min(cap, c[u]) : u in N(v)}: the largest k <= cap
 * with at least k neighbours of value >= k.  `hist` has cap+1 zeroed slots and
 * is left zeroed.  This is the suffix-sum scan of NbrCore.cu:97-104.        */
static uint32_t hindex_of(const int64_t *rowptr, const uint32_t *col, const uint32_t *c,
                          uint32_t v, uint32_t cap, uint32_t *hist)
{
    for (int64_t e = rowptr[v]; e < rowptr[v + 1]; e++) {
        uint32_t x = c[col[e]];
        hist[x < cap ? x : cap]++;
    }
    uint64_t sum = 0;
    uint32_t k;
    for (k = cap; k >= 1; k--) {
        sum += hist[k];
        if (sum >= k) break;
    }
    for (int64_t e = rowptr[v]; e < rowptr[v + 1]; e++) {
        uint32_t x = c[col[e]];
        hist[x < cap ? x : cap] = 0;
    }
    hist[0] = 0;
    return k;
}

/* Synchronous (Jacobi) h-index iteration from core = degree.  Each sweep
 * recomputes every vertex flagged by a neighbour's change in the previous
 * sweep (all vertices in the first), reading the previous sweep's values, as
 * the separate histogram / count / notify launches of NbrCore.cu:253-296 do.
 * *iters receives the number of sweeps including the final sweep that changes
 * nothing, i.e. the reference's "Number of iterations".                    */
int orc_hindex_jacobi(uint32_t n, const int64_t *rowptr, const uint32_t *col, uint32_t *core,
                      uint32_t *iters)
{
    uint32_t md = 0;
    uint32_t *prev = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 4);
    uint8_t *flag = (uint8_t *)malloc((size_t)n + 1);
    uint8_t *next = (uint8_t *)malloc((size_t)n + 1);
    for (uint32_t v = 0; v < n; v++) {
        core[v] = (uint32_t)(rowptr[v + 1] - rowptr[v]);
        if (core[v] > md) md = core[v];
    }
    uint32_t *hist = (uint32_t *)calloc((size_t)md + 2, sizeof(uint32_t));
    if (!prev || !flag || !next || !hist) { free(prev); free(flag); free(next); free(hist); return ORC_ENOMEM; }
    memset(flag, 1, n);
    uint32_t it = 0;
    for (;;) {
        it++;
        memcpy(prev, core, (size_t)n * sizeof(uint32_t));
        memset(next, 0, n);
        int changed = 0;
        for (uint32_t v = 0; v < n; v++) {
            if (!flag[v] || prev[v] == 0) continue;
            uint32_t k = hindex_of(rowptr, col, prev, v, prev[v], hist);
            if (k != prev[v]) {
                core[v] = k;
                changed = 1;
                for (int64_t e = rowptr[v]; e < rowptr[v + 1]; e++) next[col[e]] = 1;
            }
        }
        if (!changed) break;
        uint8_t *t = flag; flag = next; next = t;
    }
    *iters = it;
    free(prev); free(flag); free(next); free(hist);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Level-synchronous peel of peelone.cu:157-186: `level` rises by one after a
 * round that removed nothing, otherwise the same level is repeated (a
 * sub-level round).  A round removes every live vertex whose residual degree
 * equals the level at the start of the round and decrements each neighbour
 * above the level (peelone.cu:48-87).  Degree-0 vertices have no virtual
 * node, are never visited, and keep core 0.  *rounds = kernel launches of
 * the reference driver, including the last one that finds nothing live.   */
int orc_peel_rounds(uint32_t n, const int64_t *rowptr, const uint32_t *col, uint32_t *dist,
                    uint32_t *rounds, uint32_t *kmax)
{
    uint8_t *done = (uint8_t *)calloc((size_t)n + 1, 1);
    uint32_t *front = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 4);
    if (!done || !front) { free(done); free(front); return ORC_ENOMEM; }
    uint64_t live = 0;
    for (uint32_t v = 0; v < n; v++) {
        dist[v] = (uint32_t)(rowptr[v + 1] - rowptr[v]);
        if (dist[v] == 0) done[v] = 1; else live++;
    }
    uint32_t level = 0, r = 0, km = 0;
    int plus = 1;
    for (;;) {
        r++;
        if (plus) level++; else plus = 1;
        if (live == 0) break;
        uint32_t nf = 0;
        for (uint32_t v = 0; v < n; v++)
            if (!done[v] && dist[v] == level) front[nf++] = v;
        for (uint32_t i = 0; i < nf; i++) {
            uint32_t v = front[i];
            done[v] = 1; live--; plus = 0;
            if (level > km) km = level;
            for (int64_t e = rowptr[v]; e < rowptr[v + 1]; e++) {
                uint32_t u = col[e];
                if (dist[u] > level) dist[u]--;
            }
        }
    }
    *rounds = r;
    *kmax = km;
    free(done); free(front);
    return ORC_OK;
}

/* GPP peel of gppeel.cu:186-228: per round, scan_nodes deletes every live
 * vertex with residual degree <= level and records final_core = level, then
 * scatter_edges decrements each live neighbour without clamping.  Because
 * the first level is 1, degree-0 vertices get core 1 (gppeel.cu:35-39).  */
int orc_gpp(uint32_t n, const int64_t *rowptr, const uint32_t *col, uint32_t *final_core,
            uint32_t *rounds)
{
    uint32_t *core = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 4);
    uint8_t *del = (uint8_t *)calloc((size_t)n + 1, 1);
    uint32_t *front = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 4);
    if (!core || !del || !front) { free(core); free(del); free(front); return ORC_ENOMEM; }
    for (uint32_t v = 0; v < n; v++) { core[v] = (uint32_t)(rowptr[v + 1] - rowptr[v]); final_core[v] = 0; }
    uint64_t live = n;
    uint32_t level = 0, r = 0;
    int plus = 1;
    for (;;) {
        r++;
        if (plus) level++; else plus = 1;
        if (live == 0) break;
        uint32_t nf = 0;
        for (uint32_t v = 0; v < n; v++) {
            if (del[v]) continue;
            if (core[v] <= level) { del[v] = 1; final_core[v] = level; front[nf++] = v; plus = 0; live--; }
        }
        for (uint32_t i = 0; i < nf; i++) {
            uint32_t v = front[i];
            for (int64_t e = rowptr[v]; e < rowptr[v + 1]; e++)
                if (!del[col[e]]) core[col[e]]--;
        }
    }
    *rounds = r;
    free(core); free(del); free(front);
    return ORC_OK;
}

/* peelone_dyn of peelone-dyn.cc:141-158: for level = 0, 1, ... select the
 * vertices whose residual degree equals the level, then drain a queue: each
 * neighbour above the level is decremented and, if it lands on the level, is
 * appended to the queue (the sub-levels run inside one launch).  Residual
 * degrees end as core numbers; *levels = number of select/process launches
 * (kmax + 1).                                                              */
int orc_peel_dyn(uint32_t n, const int64_t *rowptr, const uint32_t *col, uint32_t *deg,
                 uint32_t *levels)
{
    uint32_t *q = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 4);
    if (!q) return ORC_ENOMEM;
    for (uint32_t v = 0; v < n; v++) deg[v] = (uint32_t)(rowptr[v + 1] - rowptr[v]);
    uint64_t count = 0;
    uint32_t level = 0;
    while (count < n) {
        uint64_t head = 0, tail = 0;
        for (uint32_t v = 0; v < n; v++)
            if (deg[v] == level) q[tail++] = v;
        while (head < tail) {
            uint32_t v = q[head++];
            for (int64_t e = rowptr[v]; e < rowptr[v + 1]; e++) {
                uint32_t u = col[e];
                if (deg[u] > level) {
                    if (--deg[u] == level) q[tail++] = u;
                }
            }
        }
        count += tail;
        level++;
    }
    *levels = level;
    free(q);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Inline-degree CSR with virtual nodes, as MakeUGraph builds it
 * (virtual_graph.cpp:96-192): nodePointer[v] indexes a slot holding deg(v),
 * followed by v's neighbours in edge-list order; each undirected edge i is
 * scattered source->end then end->source.  Vertex v owns ceil(deg/part_size)
 * virtual nodes {v, j}.  `parts` receives 2*numParts words (node, part).
 * Degrees are computed here as in VirtualGraph::VirtualGraph (:28-44).     */
int orc_make_ugraph(uint32_t n, uint64_t m, const uint32_t *src, const uint32_t *dst,
                    uint32_t part_size, uint32_t *nodePointer, uint32_t *edgeList,
                    uint32_t *parts, uint64_t *numParts)
{
    uint32_t *deg = (uint32_t *)calloc((size_t)n + 1, sizeof(uint32_t));
    uint32_t *fill = (uint32_t *)calloc((size_t)n + 1, sizeof(uint32_t));
    if (!deg || !fill) { free(deg); free(fill); return ORC_ENOMEM; }
    for (uint64_t i = 0; i < m; i++) { deg[src[i]]++; deg[dst[i]]++; }
    uint64_t counter = 0, np = 0;
    for (uint32_t v = 0; v < n; v++) {
        nodePointer[v] = (uint32_t)counter;
        edgeList[counter] = deg[v];
        np += (deg[v] + part_size - 1) / part_size;
        counter += (uint64_t)deg[v] + 1;
    }
    for (uint64_t i = 0; i < m; i++) {
        uint32_t s = src[i], t = dst[i];
        edgeList[(uint64_t)nodePointer[s] + fill[s] + 1] = t; fill[s]++;
        edgeList[(uint64_t)nodePointer[t] + fill[t] + 1] = s; fill[t]++;
    }
    if (parts) {
        uint64_t c = 0;
        for (uint32_t v = 0; v < n; v++) {
            uint32_t k = (deg[v] + part_size - 1) / part_size;
            for (uint32_t j = 0; j < k; j++) { parts[2 * c] = v; parts[2 * c + 1] = j; c++; }
        }
    }
    *numParts = np;
    free(deg); free(fill);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
static int cmp_u32(const void *a, const void *b)
{
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

/* In-place LSD radix sort of a short array through `tmp` (same length). */
static void radix_u32(uint32_t *a, uint32_t *tmp, uint64_t len)
{
    uint64_t cnt[256];
    uint32_t *src = a, *dst = tmp;
    for (int shift = 0; shift < 32; shift += 8) {
        memset(cnt, 0, sizeof(cnt));
        for (uint64_t i = 0; i < len; i++) cnt[(src[i] >> shift) & 255u]++;
        uint64_t s = 0;
        for (int d = 0; d < 256; d++) { uint64_t c = cnt[d]; cnt[d] = s; s += c; }
        for (uint64_t i = 0; i < len; i++) dst[cnt[(src[i] >> shift) & 255u]++] = src[i];
        uint32_t *t = src; src = dst; dst = t;
    }
}

/* De-duplicated, sorted CSR of peel/src/graph.cpp:103-131 (a std::set per
 * vertex): both directions of every non-self-loop edge, each neighbour once,
 * ascending.  rowptr must hold n+1 entries; col must hold 2*m entries.
 * Counting sort by row, then each row sorted and made unique.
 * Returns the number of CSR entries, or -1 on allocation failure.         */
int64_t orc_csr_dedup(uint32_t n, uint64_t m, const uint32_t *src, const uint32_t *dst,
                      int64_t *rowptr, uint32_t *col)
{
    int64_t *start = (int64_t *)calloc((size_t)n + 2, sizeof(int64_t));
    uint32_t *tmp = NULL;
    if (!start) return -1;
    for (uint64_t i = 0; i < m; i++) {
        if (src[i] == dst[i]) continue;
        start[src[i] + 1]++;
        start[dst[i] + 1]++;
    }
    for (uint32_t v = 0; v < n; v++) start[v + 1] += start[v];
    int64_t total = start[n];
    int64_t *fill = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
    if (!fill) { free(start); return -1; }
    memcpy(fill, start, ((size_t)n + 1) * sizeof(int64_t));
    for (uint64_t i = 0; i < m; i++) {
        if (src[i] == dst[i]) continue;
        col[fill[src[i]]++] = dst[i];
        col[fill[dst[i]]++] = src[i];
    }
    free(fill);
    uint64_t maxlen = 0;
    for (uint32_t v = 0; v < n; v++) {
        uint64_t l = (uint64_t)(start[v + 1] - start[v]);
        if (l > maxlen) maxlen = l;
    }
    if (maxlen > 256) tmp = (uint32_t *)malloc((size_t)maxlen * sizeof(uint32_t));
    int64_t w = 0;
    rowptr[0] = 0;
    for (uint32_t v = 0; v < n; v++) {
        uint32_t *row = col + start[v];
        uint64_t l = (uint64_t)(start[v + 1] - start[v]);
        if (l > 256 && tmp) radix_u32(row, tmp, l);
        else qsort(row, (size_t)l, sizeof(uint32_t), cmp_u32);
        for (uint64_t j = 0; j < l; j++)
            if (j == 0 || row[j] != row[j - 1]) col[w++] = row[j];
        rowptr[v + 1] = w;
    }
    (void)total;
    free(tmp);
    free(start);
    return w;
}

/* ------------------------------------------------------------------------ */
/* Local fixpoint test: for every v, at least c[v] neighbours have c >= c[v]
 * and at most c[v] neighbours have c >= c[v]+1.  Every core vector passes;
 * it is a cheap necessary condition used beside the BZ comparison.  Returns
 * the number of failing vertices.                                          */
uint64_t orc_check_local(uint32_t n, const int64_t *rowptr, const uint32_t *col, const uint32_t *c)
{
    uint64_t bad = 0;
    for (uint32_t v = 0; v < n; v++) {
        uint64_t ge = 0, gt = 0;
        for (int64_t e = rowptr[v]; e < rowptr[v + 1]; e++) {
            uint32_t x = c[col[e]];
            if (x >= c[v]) ge++;
            if (x >= c[v] + 1) gt++;
        }
        if (ge < c[v] || gt > c[v]) bad++;
    }
    return bad;
}

/* ------------------------------------------------------------------------ */
/* Host restatement of the device R-MAT generator (pico_gb300/csrc/gen.cu):
 * edge i draws its quadrants from the splitmix64 finaliser of a counter, so
 * the same (scale, m, seed, thresholds) give the same edge list.            */
static uint64_t orc_mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void orc_gen_rmat(uint32_t scale, uint64_t m, uint64_t ta, uint64_t tab, uint64_t tabc, uint64_t seed,
                  uint32_t *src, uint32_t *dst)
{
    for (uint64_t i = 0; i < m; i++) {
        uint64_t base = orc_mix64(seed * 0xD1B54A32D192ED03ull + i);
        uint32_t u = 0, v = 0;
        uint64_t word = 0;
        for (uint32_t b = 0; b < scale; b++) {
            if ((b & 1) == 0) word = orc_mix64(base ^ ((uint64_t)((b >> 1) + 1) * 0xA24BAED4963EE407ull));
            uint32_t r = (uint32_t)(word >> (32 * (b & 1)));
            uint32_t q = r < ta ? 0u : (r < tab ? 1u : (r < tabc ? 2u : 3u));
            u = (u << 1) | (q >> 1);
            v = (v << 1) | (q & 1u);
        }
        src[i] = u;
        dst[i] = v;
    }
}

/* ------------------------------------------------------------------------ */
/* Multi-threaded forms of the two host builders above, for graphs of a
 * billion entries (R-MAT scale 25: the serial forms take minutes).  Same
 * output bit for bit: the generator is counter-based, and every CSR row is
 * sorted and made unique after its entries are placed, so the order in which
 * threads place them does not matter.                                      */

typedef void (*orc_range_fn)(void *ctx, uint64_t lo, uint64_t hi);
typedef struct { orc_range_fn fn; void *ctx; uint64_t lo, hi; } orc_job;

static void *orc_job_run(void *p)
{
    orc_job *j = (orc_job *)p;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

/* Runs fn over [0, total) split into `threads` contiguous ranges. */
static void orc_parallel(int threads, uint64_t total, orc_range_fn fn, void *ctx)
{
    enum { MAXT = 128 };
    pthread_t th[MAXT];
    orc_job jobs[MAXT];
    int started[MAXT];
    if (threads < 1) threads = 1;
    if (threads > MAXT) threads = MAXT;
    for (int t = 0; t < threads; t++) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].lo = total * (uint64_t)t / (uint64_t)threads;
        jobs[t].hi = total * (uint64_t)(t + 1) / (uint64_t)threads;
        started[t] = t > 0 && pthread_create(&th[t], NULL, orc_job_run, &jobs[t]) == 0;
    }
    orc_job_run(&jobs[0]);
    for (int t = 1; t < threads; t++) {
        if (started[t]) pthread_join(th[t], NULL);
        else orc_job_run(&jobs[t]);
    }
}

typedef struct {
    uint32_t scale;
    uint64_t ta, tab, tabc, seed;
    uint32_t *src, *dst;
} orc_rmat_ctx;

static void orc_rmat_range(void *p, uint64_t lo, uint64_t hi)
{
    orc_rmat_ctx *c = (orc_rmat_ctx *)p;
    for (uint64_t i = lo; i < hi; i++) {
        uint64_t base = orc_mix64(c->seed * 0xD1B54A32D192ED03ull + i);
        uint32_t u = 0, v = 0;
        uint64_t word = 0;
        for (uint32_t b = 0; b < c->scale; b++) {
            if ((b & 1) == 0) word = orc_mix64(base ^ ((uint64_t)((b >> 1) + 1) * 0xA24BAED4963EE407ull));
            uint32_t r = (uint32_t)(word >> (32 * (b & 1)));
            uint32_t q = r < c->ta ? 0u : (r < c->tab ? 1u : (r < c->tabc ? 2u : 3u));
            u = (u << 1) | (q >> 1);
            v = (v << 1) | (q & 1u);
        }
        c->src[i] = u;
        c->dst[i] = v;
    }
}

/* orc_gen_rmat on `threads` threads. */
void orc_gen_rmat_mt(uint32_t scale, uint64_t m, uint64_t ta, uint64_t tab, uint64_t tabc, uint64_t seed,
                     uint32_t *src, uint32_t *dst, int threads)
{
    orc_rmat_ctx c = {scale, ta, tab, tabc, seed, src, dst};
    orc_parallel(threads, m, orc_rmat_range, &c);
}

typedef struct {
    uint64_t m;
    const uint32_t *src, *dst;
    int64_t *cnt;     /* row sizes, then row fill cursors */
    uint32_t *col;    /* scatter target */
    uint32_t *ulen;   /* unique entries per row */
    const int64_t *start;
} orc_csr_ctx;

static void orc_csr_count(void *p, uint64_t lo, uint64_t hi)
{
    orc_csr_ctx *c = (orc_csr_ctx *)p;
    for (uint64_t i = lo; i < hi; i++) {
        if (c->src[i] == c->dst[i]) continue;
        __atomic_fetch_add(&c->cnt[c->src[i]], 1, __ATOMIC_RELAXED);
        __atomic_fetch_add(&c->cnt[c->dst[i]], 1, __ATOMIC_RELAXED);
    }
}

static void orc_csr_scatter(void *p, uint64_t lo, uint64_t hi)
{
    orc_csr_ctx *c = (orc_csr_ctx *)p;
    for (uint64_t i = lo; i < hi; i++) {
        uint32_t s = c->src[i], d = c->dst[i];
        if (s == d) continue;
        c->col[__atomic_fetch_add(&c->cnt[s], 1, __ATOMIC_RELAXED)] = d;
        c->col[__atomic_fetch_add(&c->cnt[d], 1, __ATOMIC_RELAXED)] = s;
    }
}

static void orc_csr_rows(void *p, uint64_t lo, uint64_t hi)
{
    orc_csr_ctx *c = (orc_csr_ctx *)p;
    uint64_t maxlen = 0;
    for (uint64_t v = lo; v < hi; v++) {
        uint64_t l = (uint64_t)(c->start[v + 1] - c->start[v]);
        if (l > maxlen) maxlen = l;
    }
    uint32_t *tmp = maxlen > 32 ? (uint32_t *)malloc((size_t)maxlen * sizeof(uint32_t)) : NULL;
    for (uint64_t v = lo; v < hi; v++) {
        uint32_t *row = c->col + c->start[v];
        uint64_t l = (uint64_t)(c->start[v + 1] - c->start[v]);
        if (l > 32 && tmp) {
            radix_u32(row, tmp, l);
        } else {
            for (uint64_t a = 1; a < l; a++) {  /* insertion sort of a short row */
                uint32_t x = row[a];
                uint64_t b = a;
                while (b > 0 && row[b - 1] > x) { row[b] = row[b - 1]; b--; }
                row[b] = x;
            }
        }
        uint64_t w = 0;
        for (uint64_t j = 0; j < l; j++)
            if (j == 0 || row[j] != row[j - 1]) row[w++] = row[j];
        c->ulen[v] = (uint32_t)w;
    }
    free(tmp);
}

/* orc_csr_dedup on `threads` threads (same arguments and result). */
int64_t orc_csr_dedup_mt(uint32_t n, uint64_t m, const uint32_t *src, const uint32_t *dst,
                         int64_t *rowptr, uint32_t *col, int threads)
{
    int64_t *start = (int64_t *)calloc((size_t)n + 2, sizeof(int64_t));
    uint32_t *ulen = (uint32_t *)malloc(((size_t)n + 1) * sizeof(uint32_t));
    if (!start || !ulen) { free(start); free(ulen); return -1; }
    orc_csr_ctx c = {m, src, dst, start + 1, col, ulen, start};
    orc_parallel(threads, m, orc_csr_count, &c);
    for (uint32_t v = 0; v < n; v++) start[v + 1] += start[v];
    int64_t *fill = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
    if (!fill) { free(start); free(ulen); return -1; }
    memcpy(fill, start, ((size_t)n + 1) * sizeof(int64_t));
    c.cnt = fill;
    orc_parallel(threads, m, orc_csr_scatter, &c);
    free(fill);
    orc_parallel(threads, n, orc_csr_rows, &c);
    /* compaction: rows move down (never up), in increasing row order */
    int64_t w = 0;
    rowptr[0] = 0;
    for (uint32_t v = 0; v < n; v++) {
        if (w != start[v]) memmove(col + w, col + start[v], (size_t)ulen[v] * sizeof(uint32_t));
        w += ulen[v];
        rowptr[v + 1] = w;
    }
    free(start);
    free(ulen);
    return w;
}
