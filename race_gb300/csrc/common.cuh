// Shared definitions for the engine's CUDA translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/race_gb300.h"

namespace race {

// Thrown inside the engine and turned into a RACE_error at the C boundary.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void cudaCheck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(RACE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define RACE_CUDA(call) ::race::cudaCheck((call), #call)

// Device-side status word codes (written by kernels, read by the host).
enum DevStatus : int {
    DEV_OK = 0,
    DEV_WAIT_TIMEOUT = 1,   // a bounded spin gave up
    DEV_BAD_SCHEDULE = 2,   // a schedule table was inconsistent
};

// Upper bound on the iterations of any device spin-wait. Each iteration
// sleeps at least 32-64 ns plus an L2 round trip, so this is a fraction of a
// second to a few seconds: far above any legitimate wait (a whole kernel
// runs in milliseconds), small enough that a broken schedule ends the kernel
// with an error status instead of hanging.
constexpr long long kSpinLimit = 1LL << 22;

// Matrix-power rows longer than this are summed by a whole warp: lane l
// takes entries l, l+32, ... as one fma chain, then an xor butterfly over
// offsets 16, 8, 4, 2, 1 combines the 32 partial sums.
constexpr int kMpkHubRowLen = 256;
// Largest column window of the MPK's 16-bit column layout (14-bit offsets).
constexpr int kMpkColWindow = 1 << 14;

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) {
            free();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { free(); }
    void alloc(size_t count) {
        free();
        if (count) RACE_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
        n = count;
    }
    void ensure(size_t count) {
        if (count > n) alloc(count);
    }
    void free() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // Copies count elements from h; h may be null (an empty host vector's
    // data()) when the caller only needs a placeholder of at least one
    // element, which is then allocated but left unset.
    void upload(const T *h, size_t count, cudaStream_t s = 0) {
        ensure(count);
        if (count && h) RACE_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
};

inline int ceilDiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace race
