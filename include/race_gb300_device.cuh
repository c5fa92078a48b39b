// race_gb300_device.cuh -- header-only CUDA counterpart of RACE's callback
// registration. The reference calls a host function on row ranges of its
// schedule: f(start, end, args) for colored kernels and
// f(start, end, pow, numa, args) for the matrix power (registerFunction,
// include/interface.h:143-157; FuncManager::Run, src/functionManager.cpp).
// Here the function is a __device__ functor (its members play the role of
// `args`, holding device pointers) and the engine's schedule calls it on the
// GPU:
//
//   struct MyGs {
//       const int *rowPtr, *col; const double *val, *b; double *x;
//       __device__ void operator()(int start, int end) const {...}
//   };
//   RACE::gb300::DeviceFunction<MyGs> gs(ce.handle(), MyGs{...});
//   gs.execute(/*rev=*/false, stream);
//
// Colored functions: every phase of the engine's flattened zone tree is one
// launch; each leaf of the phase is one call f(start, end) on one thread,
// start > end meaning rows start, start-1, ..., end+1 (the reference's
// reverse sweep convention). Leaves of one phase never conflict, so the
// calls of a launch may run in any order, exactly as the reference's threads
// do.
//
// Matrix power: DevicePowerFunction calls f(start, end, pow), pow = 1..p
// (or f(start, end, pow, subPow) with sub-powers), on the engine's MPK level
// groups in a wavefront of stride 2 (step s holds power k of group s-2k, so
// every call of a step depends only on earlier steps: rows of a group
// reference rows of the neighbouring groups only); one launch per step, each
// group cut into ranges of at most rowsPerCall rows. The matrix the functor
// reads must be permuted with the engine's permutation (getPerm/getInvPerm),
// as for the built-in MPK.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "race_gb300.h"

namespace RACE {
namespace gb300 {

namespace detail {

template <class F>
__global__ void kColorPhase(F f, const int *leafLo, const int *leafHi, int first, int last) {
    for (int l = first + blockIdx.x * blockDim.x + threadIdx.x; l < last; l += gridDim.x * blockDim.x)
        f(leafLo[l], leafHi[l]);
}

// A power call: f(start, end, pow, subPow) when the functor takes four
// arguments (main and sub power, both 1-based), else f(start, end, step)
// with the 1-based step of power * subPower steps.
template <class F>
__host__ __device__ auto invokePower(const F &f, int start, int end, int step, int subPower, int)
    -> decltype(f(start, end, step, step), void()) {
    f(start, end, (step - 1) / subPower + 1, (step - 1) % subPower + 1);
}
template <class F>
__host__ __device__ void invokePower(const F &f, int start, int end, int step, int subPower, long) {
    (void)subPower;
    f(start, end, step);
}

template <class F>
__global__ void kPowerStep(F f, const int4 *calls, int count, int subPower) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int4 c = calls[i];
        invokePower(f, c.x, c.y, c.z, subPower, 0);
    }
}

// The calls of a wavefront of `steps` powers over level groups (groupPtr:
// groups+1 row offsets) with stride 2: wavefront step s holds power k+1 of
// group s-2k (k = 0, 1, ...), each group cut into ranges of at most
// rowsPerCall rows; calls[stepPtr[s] .. stepPtr[s+1]) are (start, end, k+1).
inline void powerCalls(const std::vector<int> &groupPtr, int steps, int rowsPerCall, std::vector<int4> &calls,
                       std::vector<int> &stepPtr) {
    const int G = (int)groupPtr.size() - 1;
    calls.clear();
    stepPtr.assign(1, 0);
    for (int st = 0; G > 0 && st < G + 2 * (steps - 1); ++st) {
        for (int k = 0; k < steps; ++k) {
            const int g = st - 2 * k;
            if (g < 0 || g >= G) continue;
            for (int r = groupPtr[g]; r < groupPtr[g + 1]; r += rowsPerCall)
                calls.push_back(make_int4(r, std::min(r + rowsPerCall, groupPtr[g + 1]), k + 1, 0));
        }
        stepPtr.push_back((int)calls.size());
    }
}

constexpr int kThreads = 128;
constexpr int kMaxBlocks = 152 * 8;

inline int blocksFor(int count) { return std::max(1, std::min((count + kThreads - 1) / kThreads, kMaxBlocks)); }

}  // namespace detail

// A colored function over the engine's schedule (both directions). The
// engine must be colored (race_color) and outlive this object, and must not
// be colored again while it is used (the schedule is read at construction).
template <class F>
class DeviceFunction {
  public:
    DeviceFunction(race_engine *e, const F &f) : f_(f) {
        for (int dir = 0; dir < 2; ++dir) {
            Schedule &d = sched_[dir];
            int np = 0, nl = 0;
            rc_ = race_get_phases(e, dir, nullptr, nullptr, nullptr, 0, &np, &nl);
            if (rc_ != RACE_SUCCESS) return;
            const int cap = std::max(np + 1, nl);
            std::vector<int> lo(cap), hi(cap);
            d.phasePtr.resize(cap);
            rc_ = race_get_phases(e, dir, d.phasePtr.data(), lo.data(), hi.data(), cap, &np, &nl);
            if (rc_ != RACE_SUCCESS) return;
            d.phasePtr.resize(np + 1);
            rc_ = race_get_device_phases(e, dir, &d.leafLo, &d.leafHi, &nl);
            if (rc_ != RACE_SUCCESS) return;
        }
    }
    // RACE_SUCCESS, or the error of the constructor's schedule queries.
    int status() const { return rc_; }
    // Enqueues the sweep on `stream` (no synchronisation); RACE_ERR_CUDA if a
    // launch failed.
    int execute(bool rev = false, cudaStream_t stream = 0) const {
        if (rc_ != RACE_SUCCESS) return rc_;
        const Schedule &d = sched_[rev ? 1 : 0];
        for (size_t p = 0; p + 1 < d.phasePtr.size(); ++p) {
            const int first = d.phasePtr[p], last = d.phasePtr[p + 1];
            detail::kColorPhase<F><<<detail::blocksFor(last - first), detail::kThreads, 0, stream>>>(
                f_, d.leafLo, d.leafHi, first, last);
        }
        return cudaGetLastError() == cudaSuccess ? RACE_SUCCESS : RACE_ERR_CUDA;
    }

  private:
    struct Schedule {
        std::vector<int> phasePtr;
        const int *leafLo = nullptr, *leafHi = nullptr;
    };
    F f_;
    Schedule sched_[2];
    int rc_ = RACE_SUCCESS;
};

// A matrix-power function of `power` powers, each of `subPower` sub-steps
// (registerFunction(f, args, power, subPower), interface.h:149-153: the
// wavefront runs power * subPower steps), over the engine's level groups
// (after RACEColor(highestPower, cacheSize, safety, mtxType,
// highestSubPower)). The functor takes (start, end, pow, subPow) or, for
// subPower 1, (start, end, pow). Owns one device table of calls.
template <class F>
class DevicePowerFunction {
  public:
    DevicePowerFunction(race_engine *e, const F &f, int power, int rowsPerCall = 32, int subPower = 1)
        : e_(e), f_(f), power_(power), subPower_(subPower), rowsPerCall_(rowsPerCall) {
        rc_ = build();
    }
    ~DevicePowerFunction() {
        if (calls_) cudaFree(calls_);
    }
    DevicePowerFunction(const DevicePowerFunction &) = delete;
    DevicePowerFunction &operator=(const DevicePowerFunction &) = delete;
    int status() const { return rc_; }
    int getPower() const { return power_; }
    int getSubPower() const { return subPower_; }
    // Interface::setPower / setSubPower (interface.cpp:574-582): the next
    // execute runs power * subPower steps; the call table is rebuilt.
    // Returns the new status.
    int setPower(int power) {
        power_ = power;
        return rc_ = build();
    }
    int setSubPower(int subPower) {
        subPower_ = subPower;
        return rc_ = build();
    }
    int execute(cudaStream_t stream = 0) const {
        if (rc_ != RACE_SUCCESS) return rc_;
        for (size_t st = 0; st + 1 < stepPtr_.size(); ++st) {
            const int count = stepPtr_[st + 1] - stepPtr_[st];
            if (count == 0) continue;
            detail::kPowerStep<F><<<detail::blocksFor(count), detail::kThreads, 0, stream>>>(
                f_, calls_ + stepPtr_[st], count, subPower_);
        }
        return cudaGetLastError() == cudaSuccess ? RACE_SUCCESS : RACE_ERR_CUDA;
    }

  private:
    // The call table of power_ * subPower_ steps over the engine's groups.
    int build() {
        if (calls_) cudaFree(calls_);
        calls_ = nullptr;
        stepPtr_.clear();
        if (power_ < 1 || subPower_ < 1 || rowsPerCall_ < 1) return RACE_ERR_INVALID_ARG;
        int len = 0;
        int rc = race_get_power_groups(e_, nullptr, 0, &len);
        if (rc != RACE_SUCCESS) return rc;
        std::vector<int> gp(len);
        rc = race_get_power_groups(e_, gp.data(), len, &len);
        if (rc != RACE_SUCCESS) return rc;
        std::vector<int4> calls;
        detail::powerCalls(gp, power_ * subPower_, rowsPerCall_, calls, stepPtr_);
        if (!calls.empty() && (cudaMalloc(&calls_, sizeof(int4) * calls.size()) != cudaSuccess ||
                               cudaMemcpy(calls_, calls.data(), sizeof(int4) * calls.size(),
                                          cudaMemcpyHostToDevice) != cudaSuccess))
            return RACE_ERR_CUDA;
        return RACE_SUCCESS;
    }

    race_engine *e_;
    F f_;
    int power_, subPower_, rowsPerCall_;
    std::vector<int> stepPtr_;
    int4 *calls_ = nullptr;
    int rc_ = RACE_SUCCESS;
};

namespace detail {

// MAT_NUM_VEC_ACCESSES (interface.cpp:1060-1080): each row counts its
// visits; a visit that leaves the count other than pow is an error.
struct CoverageCount {
    double *x;
    int *errors;
    __device__ void operator()(int start, int end, int pow) const {
        for (int row = start; row < end; ++row) {
            x[row] += 1;
            if (x[row] != (double)pow) atomicAdd(errors, 1);
        }
    }
};

}  // namespace detail

// Interface::checkPowerCoverage (interface.cpp:1082-1095): a counting
// function of the engine's highest power runs over its level groups
// (after race_power_prepare); *errors gets the number of row visits out of
// turn (missing or repeated computations), 0 for a sound schedule. The
// reference prints each such visit instead. Synchronises the device.
inline int checkPowerCoverage(race_engine *e, int *errors) {
    if (!errors) return RACE_ERR_INVALID_ARG;
    *errors = -1;
    int hp = 0, len = 0;
    int rc = race_get_highest_power(e, &hp);
    if (rc == RACE_SUCCESS) rc = race_get_power_groups(e, nullptr, 0, &len);
    if (rc != RACE_SUCCESS) return rc;
    std::vector<int> gp(len);
    rc = race_get_power_groups(e, gp.data(), len, &len);
    if (rc != RACE_SUCCESS) return rc;
    const int n = gp.empty() ? 0 : gp.back();
    double *x = nullptr;
    int *err = nullptr;
    if (cudaMalloc(&x, sizeof(double) * (size_t)std::max(n, 1)) != cudaSuccess ||
        cudaMalloc(&err, sizeof(int)) != cudaSuccess || cudaMemset(x, 0, sizeof(double) * (size_t)n) != cudaSuccess ||
        cudaMemset(err, 0, sizeof(int)) != cudaSuccess) {
        rc = RACE_ERR_CUDA;
    } else {
        DevicePowerFunction<detail::CoverageCount> f(e, detail::CoverageCount{x, err}, hp);
        rc = f.status();
        if (rc == RACE_SUCCESS) rc = f.execute(0);
        if (rc == RACE_SUCCESS && (cudaDeviceSynchronize() != cudaSuccess ||
                                   cudaMemcpy(errors, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
            rc = RACE_ERR_CUDA;
    }
    if (x) cudaFree(x);
    if (err) cudaFree(err);
    return rc;
}

}  // namespace gb300
}  // namespace RACE
