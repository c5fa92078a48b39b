// L2 die map of the current GPU.
//
// GB300 is two dies with an L2 each, and a line an SM reads is cached in
// the L2 of the SM's own die: data that SMs of both dies read is held twice,
// so for it the L2 holds about half as much as for data each die reads
// alone (measured: repeated reads of a working set stay in L2 up to about
// 100 MB when every SM keeps reading its own part, but only up to about
// 64 MB when each part is read by SMs of both dies). Kernels that reuse
// data between work items (the matrix-power wavefront) keep an item's data
// on one die once they know which SMs share a die. The map is measured,
// not assumed (floor-swept chips number their SMs differently): one block
// writes a pointer chain into one region per timing block, so those lines
// sit in the writer's die's L2; then every block walks its own region once
// and times it. SMs of the writer's die hit their L2 (about 300 cycles per
// load on GB300), SMs of the other die fetch across the die boundary (about
// 480). A device whose latencies do not split into two clear groups is
// treated as one die.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "dies.h"

namespace race {

namespace {

constexpr int kChaseLines = 256;  // lines of 128 bytes per region
constexpr int kLineWords = 16;    // 8-byte words per line
constexpr int kChaseStep = 97;    // odd step: one cycle through all lines

__device__ __forceinline__ unsigned smIndex() {
    unsigned r;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
    return r;
}

__device__ __forceinline__ long long ldL2(const long long *p) {
    long long v;
    asm volatile("ld.global.cg.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ long long clockNow() {
    long long c;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(c)::"memory");
    return c;
}

// One block: writes every region's chain, reads it back, records its SM.
__global__ void kDieWrite(long long *buf, int regions, int *writerSm, long long *sink) {
    const long long words = (long long)regions * kChaseLines * kLineWords;
    for (long long w = threadIdx.x; w < words; w += blockDim.x) {
        const int i = (int)((w / kLineWords) % kChaseLines);
        buf[w] = (w % kLineWords) == 0 ? (i + kChaseStep) % kChaseLines : 0;
    }
    __syncthreads();
    long long s = 0;
    for (long long w = (long long)threadIdx.x * kLineWords; w < words; w += (long long)blockDim.x * kLineWords)
        s += ldL2(buf + w);
    if (threadIdx.x == 0) *writerSm = (int)smIndex();
    if (s == -1) *sink = s;
}

// One lane per block walks region blockIdx (no other block reads it, so
// only the writer has brought its lines into an L2) and records (SM, cycles).
__global__ void kDieChase(const long long *buf, long long *out) {
    if (threadIdx.x != 0) return;
    const long long *base = buf + (long long)blockIdx.x * kChaseLines * kLineWords;
    long long idx = 0;
    const long long t0 = clockNow();
    for (int i = 0; i < kChaseLines; ++i) idx = ldL2(base + idx * kLineWords);
    const long long t1 = clockNow() + (idx == -1);
    out[2 * blockIdx.x] = smIndex();
    out[2 * blockIdx.x + 1] = (t1 - t0) / kChaseLines;
}

DieMap measure() {
    DieMap m;
    int dev = 0, sms = 0;
    RACE_CUDA(cudaGetDevice(&dev));
    RACE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    m.smDie.assign(sms, 0);
    m.smsPerDie = {sms, 0};
    if (const char *v = getenv("RACE_GPU_DIE_AFFINITY"))
        if (atoi(v) == 0) return m;
    const int blocks = 4 * sms, regions = blocks;
    DevBuf<long long> buf((size_t)regions * kChaseLines * kLineWords), out(2 * (size_t)blocks), sink(1);
    DevBuf<int> writer(1);
    kDieWrite<<<1, 256>>>(buf.p, regions, writer.p, sink.p);
    kDieChase<<<blocks, 32>>>(buf.p, out.p);
    RACE_CUDA(cudaGetLastError());
    std::vector<long long> h(2 * (size_t)blocks);
    int w = -1;
    RACE_CUDA(cudaMemcpy(h.data(), out.p, sizeof(long long) * h.size(), cudaMemcpyDeviceToHost));
    RACE_CUDA(cudaMemcpy(&w, writer.p, sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<long long> lat(sms, -1);
    for (int b = 0; b < blocks; ++b) {
        const long long s = h[2 * (size_t)b], c = h[2 * (size_t)b + 1];
        if (s < 0 || s >= sms) continue;
        lat[s] = lat[s] < 0 ? c : std::min(lat[s], c);
    }
    if (getenv("RACE_GPU_DIE_DEBUG")) {
        fprintf(stderr, "die map: writer SM %d; cycles per load:", w);
        for (int s = 0; s < sms; ++s) fprintf(stderr, " %d:%lld", s, lat[s]);
        fprintf(stderr, "\n");
    }
    if (w < 0 || w >= sms || std::count(lat.begin(), lat.end(), -1LL) > 0) return m;
    // two groups split at the widest gap of the sorted latencies, accepted
    // when the gap is at least a quarter of the fastest latency and the
    // writer's SM is in the faster group
    std::vector<long long> sorted(lat);
    std::sort(sorted.begin(), sorted.end());
    size_t cut = 0;
    long long gap = 0;
    for (size_t i = 0; i + 1 < sorted.size(); ++i)
        if (sorted[i + 1] - sorted[i] > gap) {
            gap = sorted[i + 1] - sorted[i];
            cut = i;
        }
    if (gap * 4 < sorted[0] || sorted[0] <= 0) return m;
    const long long threshold = sorted[cut];
    if (lat[w] > threshold) return m;
    DieMap two;
    two.numDies = 2;
    two.smDie.assign(sms, 0);
    two.smsPerDie = {0, 0};
    for (int s = 0; s < sms; ++s) {
        two.smDie[s] = lat[s] <= threshold ? 0 : 1;
        ++two.smsPerDie[two.smDie[s]];
    }
    if (two.smsPerDie[0] == 0 || two.smsPerDie[1] == 0) return m;
    return two;
}

}  // namespace

const DieMap &dieMap() {
    static std::mutex mu;
    static std::vector<std::unique_ptr<DieMap>> maps;
    std::lock_guard<std::mutex> lock(mu);
    int dev = 0;
    RACE_CUDA(cudaGetDevice(&dev));
    if (maps.size() <= (size_t)dev) maps.resize(dev + 1);
    if (!maps[dev]) {
        auto m = std::make_unique<DieMap>(measure());
        m->smDieDev.upload(m->smDie.data(), m->smDie.size());
        RACE_CUDA(cudaDeviceSynchronize());
        maps[dev] = std::move(m);
    }
    return *maps[dev];
}

}  // namespace race
