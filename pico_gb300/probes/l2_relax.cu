// Throughput probe for the memory pattern of the peel's row walk, used to bound
// what the decomposition kernels can reach on this GPU: a warp reads a run of
// column ids (coalesced), probes one claim bit per id in a 4 MB bitmap that
// stays in L2, and decrements the residual degree of the unclaimed ones with
// atomicSub.  Uniform random ids over 2^25 vertices, 2^30 entries, half the
// bitmap set.  MODE 0: column stream only; 1: + bit probe; 2: + atomicSub.
// Build and run: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o l2_relax l2_relax.cu && ./l2_relax
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>
__device__ __forceinline__ uint64_t mix(uint64_t x) { x += 0x9e3779b97f4a7c15ull; x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull; x = (x ^ (x >> 27)) * 0x94d049bb133111ebull; return x ^ (x >> 31); }
__global__ void fill(uint32_t *col, uint64_t nnz, uint32_t n, uint32_t *bm, uint32_t *deg) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nnz; i += (uint64_t)gridDim.x * blockDim.x) {
        col[i] = (uint32_t)(mix(i) % n);
        if (i < (n + 31) / 32) bm[i] = (uint32_t)mix(i * 7 + 1);  // ~half claimed
        if (i < n) deg[i] = 1u << 30;
    }
}
template <int U, int MODE>  // MODE 0: col only, 1: col+bitmap, 2: col+bitmap+atomicSub
__global__ void __launch_bounds__(512, 2) relax(const uint32_t *__restrict__ col, uint64_t nnz, const uint32_t *bm, uint32_t *deg, unsigned long long *sink) {
    const unsigned lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * 16, w0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    unsigned acc = 0;
    for (uint64_t base = w0 * 32 * U; base < nnz; base += warps * 32 * U) {
        uint32_t u[U]; bool live[U];
#pragma unroll
        for (int k = 0; k < U; k++) { uint64_t e = base + k * 32 + lane; live[k] = e < nnz; u[k] = live[k] ? __ldcs(&col[e]) : 0u; }
        if (MODE >= 1) {
#pragma unroll
            for (int k = 0; k < U; k++) if (live[k]) { unsigned w = __ldcg(&bm[u[k] >> 5]); live[k] = !(w & (1u << (u[k] & 31))); }
        }
        if (MODE >= 2) {
            unsigned a[U];
#pragma unroll
            for (int k = 0; k < U; k++) a[k] = live[k] ? atomicSub(&deg[u[k]], 1u) : 0u;
#pragma unroll
            for (int k = 0; k < U; k++) acc += a[k] & 1;
        } else {
#pragma unroll
            for (int k = 0; k < U; k++) acc += live[k] ? u[k] : 0;
        }
    }
    if (acc == 0x12345678) atomicAdd(sink, 1ull);
}
template <int U, int MODE> float run(const uint32_t *col, uint64_t nnz, const uint32_t *bm, uint32_t *deg, unsigned long long *sink, int sms) {
    cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
    relax<U, MODE><<<sms * 2, 512>>>(col, nnz, bm, deg, sink);
    cudaEventRecord(a);
    for (int r = 0; r < 3; r++) relax<U, MODE><<<sms * 2, 512>>>(col, nnz, bm, deg, sink);
    cudaEventRecord(b); cudaEventSynchronize(b);
    float ms; cudaEventElapsedTime(&ms, a, b); return ms / 3;
}
int main() {
    const uint32_t n = 1u << 25; const uint64_t nnz = 1ull << 30;
    uint32_t *col, *bm, *deg; unsigned long long *sink;
    if (cudaMalloc(&col, nnz * 4) || cudaMalloc(&bm, (n / 32 + 1) * 4) || cudaMalloc(&deg, n * 4ull) || cudaMalloc(&sink, 8)) { printf("alloc failed\n"); return 1; }
    int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    fill<<<sms * 8, 256>>>(col, nnz, n, bm, deg);
    cudaDeviceSynchronize();
    printf("n=%u nnz=%llu sms=%d\n", n, (unsigned long long)nnz, sms);
#define R(U, M) { float ms = run<U, M>(col, nnz, bm, deg, sink, sms); printf("U=%d mode=%d  %.3f ms  %.1f G entries/s  col %.0f GB/s\n", U, M, ms, nnz / ms / 1e6, nnz * 4 / ms / 1e6); }
    R(4, 0) R(8, 0) R(4, 1) R(8, 1) R(16, 1) R(4, 2) R(8, 2) R(16, 2)
    cudaError_t e = cudaDeviceSynchronize();
    printf("status %s\n", cudaGetErrorString(e));
    return 0;
}
