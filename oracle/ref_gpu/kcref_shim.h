// TEST INFRASTRUCTURE ONLY.  Pre-included (nvcc --pre-include) into every
// translation unit of the reference's GPU drivers when they are compiled as
// a second oracle; the reference's sources are compiled unmodified.
//
// Three CUDA runtime calls of the drivers are routed through wrappers:
//   * cudaMalloc allocates KCREF_PAD more bytes and zeroes them.  Several
//     reference kernels read a flag or counter array at the thread index
//     before testing it against the vertex count (count_kernel of
//     index2core/HistoCore.cu:98, NbrCore.cu:89, CntCore.cu:103,
//     scan_nodes of peel/gppeel.cu:31), with grids of n/512+1 blocks, so
//     up to 511 entries past the end are read; the zeroed pad keeps those
//     reads inside the allocation, and a zero there makes each kernel return.
//   * cudaMemcpy, device to host: a copy of exactly KCREF_DUMP_BYTES bytes
//     (4 x the vertex count, set by the harness) is written to the file
//     KCREF_DUMP; the last such copy of each driver is its core array
//     (HistoCore.cu:350, CntCore.cu:425, NbrCore.cu:306, peelone.cu:195,
//     gppeel.cu:239).  Host to device: a copy from the host array registered
//     with kcref_track_host() marks its device destination.
//   * cudaFree of the marked device array first copies its contents back
//     (the peel/src drivers keep the core numbers in the device degrees array
//     and free it without reading it back, peel/src/gpu_memory_allocation.cu:18-21).
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define KCREF_PAD ((size_t)65536)

struct KcrefState {
    const void *track_host = nullptr;  // host array whose device copy is watched
    size_t track_bytes = 0;
    void *tracked_dev = nullptr;
    std::vector<unsigned char> captured;  // contents of the watched array at its cudaFree
    bool have_capture = false;
};

inline KcrefState &kcref_state() {
    static KcrefState s;
    return s;
}

inline void kcref_track_host(const void *host, size_t bytes) {
    KcrefState &s = kcref_state();
    s.track_host = host;
    s.track_bytes = bytes;
    s.tracked_dev = nullptr;
    s.have_capture = false;
}

inline cudaError_t kcref_malloc(void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes + KCREF_PAD);
    if (e == cudaSuccess) e = cudaMemset(static_cast<unsigned char *>(*p) + bytes, 0, KCREF_PAD);
    return e;
}

inline cudaError_t kcref_memcpy(void *dst, const void *src, size_t n, cudaMemcpyKind kind) {
    cudaError_t e = cudaMemcpy(dst, src, n, kind);
    if (e != cudaSuccess) return e;
    KcrefState &s = kcref_state();
    if (kind == cudaMemcpyHostToDevice && s.track_host && src == s.track_host && n == s.track_bytes)
        s.tracked_dev = dst;
    if (kind == cudaMemcpyDeviceToHost) {
        const char *want = std::getenv("KCREF_DUMP_BYTES");
        const char *path = std::getenv("KCREF_DUMP");
        if (want && path && n == (size_t)std::strtoull(want, nullptr, 10)) {
            FILE *f = std::fopen(path, "wb");
            if (f) {
                std::fwrite(dst, 1, n, f);
                std::fclose(f);
            }
        }
    }
    return e;
}

inline cudaError_t kcref_free(void *p) {
    KcrefState &s = kcref_state();
    if (p && p == s.tracked_dev) {
        s.captured.resize(s.track_bytes);
        if (cudaMemcpy(s.captured.data(), p, s.track_bytes, cudaMemcpyDeviceToHost) == cudaSuccess)
            s.have_capture = true;
        s.tracked_dev = nullptr;
    }
    return cudaFree(p);
}

#define cudaMalloc(p, bytes) kcref_malloc((void **)(p), (size_t)(bytes))
#define cudaMemcpy(dst, src, n, kind) kcref_memcpy((void *)(dst), (const void *)(src), (size_t)(n), (kind))
#define cudaFree(p) kcref_free((void *)(p))
