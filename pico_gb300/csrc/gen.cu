// Seeded graph generators on the device.  Every random draw is a pure function
// of (seed, item index) through the splitmix64 finaliser (Steele, Lea and
// Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014), so
// the output does not depend on the launch shape and a host restatement
// reproduces it exactly.  Used to make the synthetic inputs the reference's
// SuiteSparse/KONECT files stand in for.
#include <cmath>

#include "kc_internal.h"

namespace kc {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------- R-MAT --
// Edge i: base = mix64(seed * K1 + i); level b takes the 32-bit half
// (b & 1) of mix64(base ^ ((b >> 1) + 1) * K2) and picks quadrant
// a | b | c | d by integer thresholds; ids are built most significant bit first.
__global__ void rmat_kernel(uint32_t scale, uint64_t m, uint64_t ta, uint64_t tab, uint64_t tabc, uint64_t seed,
                            uint32_t *src, uint32_t *dst) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t base = mix64(seed * 0xD1B54A32D192ED03ull + i);
        uint32_t u = 0, v = 0;
        uint64_t word = 0;
        for (uint32_t b = 0; b < scale; b++) {
            if ((b & 1) == 0) word = mix64(base ^ ((uint64_t)((b >> 1) + 1) * 0xA24BAED4963EE407ull));
            uint32_t r = (uint32_t)(word >> (32 * (b & 1)));
            uint32_t q = r < ta ? 0u : (r < tab ? 1u : (r < tabc ? 2u : 3u));
            u = (u << 1) | (q >> 1);
            v = (v << 1) | (q & 1u);
        }
        src[i] = u;
        dst[i] = v;
    }
}

static uint64_t prob_threshold(double p) {
    double t = std::floor(p * 4294967296.0);
    if (t < 0) t = 0;
    if (t > 4294967296.0) t = 4294967296.0;
    return (uint64_t)t;
}

int gen_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c, uint64_t seed, uint32_t *d_src,
             uint32_t *d_dst, cudaStream_t s) {
    if (scale == 0 || scale > 32) return fail(KC_ERR_INVALID, "R-MAT scale must be in [1, 32]");
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return fail(KC_ERR_INVALID, "R-MAT probabilities invalid");
    if (!num_edges) return KC_OK;
    uint64_t ta = prob_threshold(a), tab = prob_threshold(a + b), tabc = prob_threshold(a + b + c);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t blocks = (num_edges + 255) / 256;
    if (blocks > (uint64_t)sms * 32) blocks = (uint64_t)sms * 32;
    rmat_kernel<<<(unsigned)blocks, 256, 0, s>>>(scale, num_edges, ta, tab, tabc, seed, d_src, d_dst);
    KC_CUDA(cudaGetLastError());
    return KC_OK;
}

// ----------------------------------------------------- keyed permutation --
// Balanced 4-round Feistel network on 2h bits with cycle walking: a bijection
// of [0, N) for any N <= 2^(2h).
struct Feistel {
    uint32_t half;  // h
    uint64_t mask;  // 2^h - 1
    uint64_t N;
    uint64_t key[4];
};

__host__ __device__ __forceinline__ uint64_t feistel_once(const Feistel &f, uint64_t x) {
    uint64_t L = x >> f.half, R = x & f.mask;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        uint64_t F = mix64(f.key[r] ^ R) & f.mask;
        uint64_t nl = R;
        R = L ^ F;
        L = nl;
    }
    return (L << f.half) | R;
}

__host__ __device__ __forceinline__ uint64_t feistel_perm(const Feistel &f, uint64_t i) {
    uint64_t x = i;
    do {
        x = feistel_once(f, x);
    } while (x >= f.N);
    return x;
}

static Feistel make_feistel(uint64_t N, uint64_t seed) {
    Feistel f;
    uint32_t bits = 2;
    while (bits < 64 && (1ull << bits) < N) bits += 2;
    f.half = bits / 2;
    f.mask = (1ull << f.half) - 1;
    f.N = N;
    for (int r = 0; r < 4; r++) f.key[r] = mix64(seed * 0x9E6C63D0676A9A99ull + (uint64_t)r + 1);
    return f;
}

// Pair index p in [0, k(k-1)/2) -> (a, b), a < b, upper triangle row-major.
__host__ __device__ __forceinline__ void tri_unrank(uint64_t k, uint64_t p, uint64_t &a, uint64_t &b) {
    double kk = (double)(2 * k - 1);
    double disc = kk * kk - 8.0 * (double)p;
    double ad = (kk - sqrt(disc > 0 ? disc : 0)) / 2.0;
    uint64_t r = ad > 0 ? (uint64_t)ad : 0;
    if (r > k - 2) r = k - 2;
    // T(r) = r*k - r(r+1)/2 pairs precede row r
    while (r > 0 && r * k - r * (r + 1) / 2 > p) r--;
    while (r + 1 <= k - 2 && (r + 1) * k - (r + 1) * (r + 2) / 2 <= p) r++;
    a = r;
    b = p - (r * k - r * (r + 1) / 2) + r + 1;
}

__global__ void er_kernel(uint32_t n, uint64_t m, Feistel f, uint32_t *src, uint32_t *dst) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p = feistel_perm(f, i);
        uint64_t a, b;
        tri_unrank(n, p, a, b);
        src[i] = (uint32_t)a;
        dst[i] = (uint32_t)b;
    }
}

int gen_er(uint32_t n, uint64_t m, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, cudaStream_t s) {
    if (n < 2 || n >= (1u << 31)) return fail(KC_ERR_INVALID, "G(n,m) needs 2 <= n < 2^31");
    uint64_t N = (uint64_t)n * (n - 1) / 2;
    if (m > N) return fail(KC_ERR_INVALID, "G(n,m): m exceeds n(n-1)/2");
    if (!m) return KC_OK;
    Feistel f = make_feistel(N, seed);
    uint64_t blocks = (m + 255) / 256;
    if (blocks > 65535ull * 16) blocks = 65535ull * 16;
    er_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, m, f, d_src, d_dst);
    KC_CUDA(cudaGetLastError());
    return KC_OK;
}

// ------------------------------------------------------- planted subgraph --
constexpr uint64_t PLANT_CHUNK = 1024;  // pairs per counting slot

__global__ void planted_members(uint32_t k, Feistel f, uint32_t *members) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < k; i += (uint64_t)gridDim.x * blockDim.x)
        members[i] = (uint32_t)feistel_perm(f, i);
}

__device__ __forceinline__ bool planted_edge(uint64_t seed, uint64_t p, uint64_t thr) {
    return (mix64(seed * 0xC2B2AE3D27D4EB4Full + p) & 0xffffffffull) < thr;
}

__global__ void planted_count(uint64_t npairs, uint64_t seed, uint64_t thr, uint32_t *cnt) {
    uint64_t slots = (npairs + PLANT_CHUNK - 1) / PLANT_CHUNK;
    for (uint64_t sl = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; sl < slots; sl += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t lo = sl * PLANT_CHUNK, hi = lo + PLANT_CHUNK < npairs ? lo + PLANT_CHUNK : npairs;
        uint32_t c = 0;
        for (uint64_t p = lo; p < hi; p++) c += planted_edge(seed, p, thr) ? 1u : 0u;
        cnt[sl] = c;
    }
}

__global__ void planted_write(uint64_t npairs, uint32_t k, uint64_t seed, uint64_t thr, const int64_t *off,
                              const uint32_t *members, uint32_t *src, uint32_t *dst, uint64_t cap) {
    uint64_t slots = (npairs + PLANT_CHUNK - 1) / PLANT_CHUNK;
    for (uint64_t sl = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; sl < slots; sl += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t lo = sl * PLANT_CHUNK, hi = lo + PLANT_CHUNK < npairs ? lo + PLANT_CHUNK : npairs;
        uint64_t w = (uint64_t)off[sl];
        for (uint64_t p = lo; p < hi; p++) {
            if (!planted_edge(seed, p, thr)) continue;
            uint64_t a, b;
            tri_unrank(k, p, a, b);
            if (w < cap) {
                src[w] = members[a];
                dst[w] = members[b];
            }
            w++;
        }
    }
}

int gen_planted(uint32_t n, uint32_t k, double p, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, uint64_t cap,
                uint64_t *m, cudaStream_t s) {
    if (k < 2 || k > n) return fail(KC_ERR_INVALID, "planted subgraph needs 2 <= k <= n");
    uint64_t npairs = (uint64_t)k * (k - 1) / 2;
    uint64_t slots = (npairs + PLANT_CHUNK - 1) / PLANT_CHUNK;
    uint64_t thr = prob_threshold(p);
    uint32_t *members = nullptr, *cnt = nullptr;
    int64_t *off = nullptr;
    KC_TRY(dalloc(&members, k, "planted members"));
    int rc = dalloc(&cnt, slots + 1, "planted counts");
    if (!rc) rc = dalloc(&off, slots + 1, "planted offsets");
    if (rc) { dfree(members); dfree(cnt); dfree(off); return rc; }
    Feistel f = make_feistel(n, seed ^ 0x5851F42D4C957F2Dull);
    planted_members<<<(k + 255) / 256, 256, 0, s>>>(k, f, members);
    unsigned blocks = (unsigned)((slots + 255) / 256);
    planted_count<<<blocks, 256, 0, s>>>(npairs, seed, thr, cnt);
    rc = exclusive_scan_u32_i64(cnt, off, slots, s);
    int64_t total = 0;
    if (!rc) {
        cudaMemcpy(&total, off + slots, 8, cudaMemcpyDeviceToHost);
        planted_write<<<blocks, 256, 0, s>>>(npairs, k, seed, thr, off, members, d_src, d_dst, cap);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(KC_ERR_CUDA, "planted: %s", cudaGetErrorString(e));
    }
    dfree(members);
    dfree(cnt);
    dfree(off);
    if (rc) return rc;
    *m = (uint64_t)total;
    if ((uint64_t)total > cap) return fail(KC_ERR_CAPACITY, "planted subgraph has %lld edges, capacity %llu",
                                          (long long)total, (unsigned long long)cap);
    return KC_OK;
}

}  // namespace kc

namespace kc {

// ------------------------------------------------ bounded R-MAT / offsets --
// R-MAT over 2^ceil(log2 n) ids with draws outside [0, n) rejected: a
// rejected draw is written as the self-loop (0, 0), which the CSR build drops.
__global__ void rmat_bounded_kernel(uint32_t scale, uint32_t n, uint64_t m, uint64_t ta, uint64_t tab, uint64_t tabc,
                                    uint64_t seed, uint32_t *src, uint32_t *dst) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t base = mix64(seed * 0xD1B54A32D192ED03ull + i);
        uint32_t u = 0, v = 0;
        uint64_t word = 0;
        for (uint32_t b = 0; b < scale; b++) {
            if ((b & 1) == 0) word = mix64(base ^ ((uint64_t)((b >> 1) + 1) * 0xA24BAED4963EE407ull));
            uint32_t r = (uint32_t)(word >> (32 * (b & 1)));
            uint32_t q = r < ta ? 0u : (r < tab ? 1u : (r < tabc ? 2u : 3u));
            u = (u << 1) | (q >> 1);
            v = (v << 1) | (q & 1u);
        }
        if (u >= n || v >= n) u = v = 0;
        src[i] = u;
        dst[i] = v;
    }
}

int gen_rmat_bounded(uint32_t n, uint64_t num_edges, double a, double b, double c, uint64_t seed, uint32_t *d_src,
                     uint32_t *d_dst, cudaStream_t s) {
    if (n < 2) return fail(KC_ERR_INVALID, "bounded R-MAT needs n >= 2");
    uint32_t scale = 1;
    while (scale < 32 && (1ull << scale) < n) scale++;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return fail(KC_ERR_INVALID, "R-MAT probabilities invalid");
    if (!num_edges) return KC_OK;
    uint64_t blocks = (num_edges + 255) / 256;
    if (blocks > 65535ull * 16) blocks = 65535ull * 16;
    rmat_bounded_kernel<<<(unsigned)blocks, 256, 0, s>>>(scale, n, num_edges, prob_threshold(a), prob_threshold(a + b),
                                                         prob_threshold(a + b + c), seed, d_src, d_dst);
    KC_CUDA(cudaGetLastError());
    return KC_OK;
}

// ----------------------------------------------------- Barabasi-Albert ----
// Batagelj and Brandes' linear-time formulation ("Efficient generation of
// large random networks", Phys. Rev. E 71, 2005): an array M of 2*n*d slots
// where M[2k] = k / d is the vertex that created edge k and M[2k+1] = M[r]
// for r uniform in [0, 2k+1) -- choosing an endpoint of an earlier edge is
// choosing a vertex with probability proportional to its degree.  Each odd
// slot is resolved independently by following r back until it lands on an
// even slot (expected O(log) steps), with r drawn from a counter hash, so the
// whole array is generated in parallel.  Edge k = (k / d, M[2k+1]).
__global__ void ba_kernel(uint32_t n, uint32_t d, uint64_t seed, uint32_t *src, uint32_t *dst) {
    const uint64_t m = (uint64_t)n * d;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t slot = 2 * k + 1;
        uint32_t target = 0;
        for (int guard = 0; guard < 4096; guard++) {
            uint64_t r = mix64(seed * 0x9FB21C651E98DF25ull + slot) % slot;
            if ((r & 1) == 0) {
                target = (uint32_t)((r >> 1) / d);
                break;
            }
            slot = r;
        }
        src[k] = (uint32_t)(k / d);
        dst[k] = target;
    }
}

int gen_ba(uint32_t n, uint32_t d, uint64_t seed, uint32_t *d_src, uint32_t *d_dst, cudaStream_t s) {
    if (n < 1 || d < 1) return fail(KC_ERR_INVALID, "Barabasi-Albert needs n >= 1 and d >= 1");
    uint64_t m = (uint64_t)n * d;
    uint64_t blocks = (m + 255) / 256;
    if (blocks > 65535ull * 16) blocks = 65535ull * 16;
    ba_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, d, seed, d_src, d_dst);
    KC_CUDA(cudaGetLastError());
    return KC_OK;
}

__global__ void offset_kernel(uint32_t *src, uint32_t *dst, uint64_t m, uint32_t off) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        src[i] += off;
        dst[i] += off;
    }
}

int edges_offset(uint32_t *d_src, uint32_t *d_dst, uint64_t m, uint32_t off, cudaStream_t s) {
    if (!m || !off) return KC_OK;
    uint64_t blocks = (m + 255) / 256;
    if (blocks > 65535ull * 16) blocks = 65535ull * 16;
    offset_kernel<<<(unsigned)blocks, 256, 0, s>>>(d_src, d_dst, m, off);
    KC_CUDA(cudaGetLastError());
    return KC_OK;
}

}  // namespace kc
