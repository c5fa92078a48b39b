// race_gb300.hpp -- header-only C++ view of the GB300 engine with the shape of
// RACE::Interface (include/interface.h:54-205 of the reference), forwarding
// to the C ABI in race_gb300.h. Method names, argument meaning and return
// codes follow the reference; the callback is a built-in device kernel with
// device operands instead of a host function pointer.
#pragma once
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "race_gb300.h"

namespace RACE {
namespace gb300 {

enum dist { ONE = RACE_DIST_ONE, TWO = RACE_DIST_TWO, POWER = RACE_DIST_POWER };
enum d2Method { TWO_BLOCK = RACE_TWO_BLOCK, THREE_BLOCK = RACE_THREE_BLOCK };
enum LBTarget { ROW = RACE_LB_ROW, NNZ = RACE_LB_NNZ };
enum PinMethod { FILL = 0, SCATTER = 1 };
enum Kernel {
    SPMV = RACE_K_SPMV,
    SPMTV = RACE_K_SPMTV,
    SYMMSPMV = RACE_K_SYMMSPMV,
    GS = RACE_K_GS,
    KACZ = RACE_K_KACZ,
    MPK = RACE_K_MPK
};

// Prints a zone tree in race_get_zone_tree's flat form ([numNodes], then per
// node [nthreadsZ, idealNthreadsZ, totalSubBlocks, parentZ, effRowZ, stage,
// reachedLimit, nValueZ, valueZ..., nChildren, children...]).
inline void printZoneTreeFlat(const std::vector<int> &t) {
    size_t k = 1;
    for (int i = 0; i < t[0]; ++i) {
        const int nth = t[k], ideal = t[k + 1], sub = t[k + 2], parent = t[k + 3], eff = t[k + 4], stage = t[k + 5],
                  reached = t[k + 6];
        k += 7;
        printf("%d. Range:[", i);
        for (int j = 0, nv = t[k++]; j < nv; ++j) printf("%d, ", t[k++]);
        printf("] Children:[");
        for (int j = 0, nc = t[k++]; j < nc; ++j) printf("%d, ", t[k++]);
        printf("], Parent: %d, nthreads: %d, idealNThreads:%d, stage:%d, subBLocks:%d, effRow: %d, reachedLimit: %s\n",
               parent, nth, ideal, stage, sub, eff, reached ? "true" : "false");
    }
}

class Interface {
  public:
    // Interface(nrow, nthreads, dist, rowPtr, col, symm_hint, SMT, pinMethod,
    //           initPerm, initInvPerm, d2Type, lbTarget) (interface.h:124).
    // rowPtr/col are host arrays; SMT and pinMethod have no GPU meaning.
    Interface(int nrow, int nthreads, dist d, int *rowPtr, int *col, bool symm_hint = false, int SMT = 1,
              PinMethod pin = SCATTER, int *initPerm = nullptr, int *initInvPerm = nullptr,
              d2Method d2Type = TWO_BLOCK, LBTarget lbTarget = NNZ)
        : nrow_(nrow) {
        (void)SMT;
        (void)pin;
        int rc = race_create(&e_, nrow, nthreads, (int)d, rowPtr, col, symm_hint ? 1 : 0, initPerm, initInvPerm,
                             (int)d2Type, (int)lbTarget, nullptr);
        if (rc != RACE_SUCCESS) throw std::runtime_error("race_create failed: " + std::to_string(rc));
    }
    ~Interface() {
        if (e_) race_destroy(e_);
    }
    Interface(const Interface &) = delete;
    Interface &operator=(const Interface &) = delete;

    // RACEColor() and RACEColor(highestPower, cacheSize, ...) (interface.h:127-128)
    int RACEColor() { return race_color(e_); }
    int RACEColor(int highestPower, double cacheSize, double safetyFactor = 2, std::string mtxType = "N",
                  int highestSubPower = 1) {
        return race_power_prepare(e_, highestPower, cacheSize, safetyFactor, mtxType.c_str(), highestSubPower);
    }
    // RACEing(): the same two entry points under the name the RACE papers
    // use for the coloring / partitioning step
    int RACEing() { return RACEColor(); }
    int RACEing(int highestPower, double cacheSize, double safetyFactor = 2, std::string mtxType = "N",
                int highestSubPower = 1) {
        return RACEColor(highestPower, cacheSize, safetyFactor, mtxType, highestSubPower);
    }

    // getPerm / getInvPerm hand over new[]-allocated arrays, as the reference
    // does (the caller delete[]s them; interface.cpp:333-383).
    void getPerm(int **perm, int *len) {
        *perm = new int[nrow_];
        race_get_perm(e_, *perm, nullptr);
        *len = nrow_;
    }
    void getInvPerm(int **invPerm, int *len) {
        *invPerm = new int[nrow_];
        race_get_perm(e_, nullptr, *invPerm);
        *len = nrow_;
    }
    int getNumThreads() {
        int v = 0;
        race_get_num_threads(e_, &v);
        return v;
    }
    double getEfficiency() {
        double v = 0;
        race_get_efficiency(e_, &v);
        return v;
    }
    int getMaxStageDepth() {
        int v = 0;
        race_get_max_stage_depth(e_, &v);
        return v;
    }
    // printZoneTree (interface.cpp:328-331, zone_tree.cpp:307-339): one line
    // per zone-tree node with its row ranges, children, parent, thread counts,
    // stage, sub-blocks, effective rows and limit flag (no pinning or timing
    // fields: they have no GPU meaning).
    void printZoneTree() {
        int len = 0;
        if (race_get_zone_tree(e_, nullptr, 0, &len) != RACE_SUCCESS) return;
        std::vector<int> t(len);
        race_get_zone_tree(e_, t.data(), len, &len);
        printZoneTreeFlat(t);
    }

    // registerFunction with a device kernel (interface.h:149-157); returns the
    // function id, or the error code as the reference does.
    int registerFunction(Kernel k, const race_operands &args, int power = 1) {
        int id = -1;
        int rc = race_register_function(e_, (int)k, &args, power, &id);
        return rc == RACE_SUCCESS ? id : rc;
    }
    int executeFunction(int funcId, bool rev = false) { return race_execute_function(e_, funcId, rev ? 1 : 0); }
    // No counterpart in the reference: enqueue without waiting, and the
    // status word of the last launch (waits for the stream).
    int executeFunctionAsync(int funcId, bool rev = false) {
        return race_execute_function_async(e_, funcId, rev ? 1 : 0);
    }
    int getStatus() { return race_get_status(e_); }
    // Matrix power over nrhs right-hand sides (race_register_mpk_block);
    // returns the function id, or the error code like registerFunction.
    int registerMpkBlock(const race_operands &args, int power, int nrhs) {
        int id = -1;
        int rc = race_register_mpk_block(e_, &args, power, nrhs, &id);
        return rc == RACE_SUCCESS ? id : rc;
    }
    void setPower(int funcId, int pow) { race_set_power(e_, funcId, pow); }
    int getPower(int funcId) {
        int v = 0;
        race_get_power(e_, funcId, &v);
        return v;
    }
    // built-in functions have sub-power 1 (race_set_sub_power); device
    // power functors carry their own (DevicePowerFunction::setSubPower)
    void setSubPower(int funcId, int subPow) { race_set_sub_power(e_, funcId, subPow); }
    int getSubPower(int funcId) {
        int v = 0;
        race_get_sub_power(e_, funcId, &v);
        return v;
    }
    int getHighestPower() {
        int v = 0;
        race_get_highest_power(e_, &v);
        return v;
    }
    // SELL-C-sigma preparation (interface.h:179-185): true on success, false
    // when a row cannot be placed, as in the reference.
    bool simdify(int simdWidth, int C, int nrows, int *col, int *chunkStart, int *rl, int *clp, double *val,
                 bool diagFirst = false) {
        return race_simdify(e_, simdWidth, C, nrows, col, chunkStart, rl, clp, val, RACE_VAL_F64, diagFirst ? 1 : 0,
                            nullptr) == RACE_SUCCESS;
    }
    bool simdify(int simdWidth, int C, int nrows, int *col, int *chunkStart, int *rl, int *clp, float *val,
                 bool diagFirst = false) {
        return race_simdify(e_, simdWidth, C, nrows, col, chunkStart, rl, clp, val, RACE_VAL_F32, diagFirst ? 1 : 0,
                            nullptr) == RACE_SUCCESS;
    }
    bool simdifyD1(int simdWidth, int C, int nrows, int *col, int *chunkStart, int *rl, int *clp, double *val,
                   bool dist2Compatible = false) {
        return race_simdify_d1(simdWidth, C, nrows, col, chunkStart, rl, clp, val, RACE_VAL_F64,
                               dist2Compatible ? 1 : 0) == RACE_SUCCESS;
    }
    bool simdifyD1(int simdWidth, int C, int nrows, int *col, int *chunkStart, int *rl, int *clp, float *val,
                   bool dist2Compatible = false) {
        return race_simdify_d1(simdWidth, C, nrows, col, chunkStart, rl, clp, val, RACE_VAL_F32,
                               dist2Compatible ? 1 : 0) == RACE_SUCCESS;
    }
    // getNumaSplitting (interface.cpp:1042-1053): the row split of the
    // level groups over shared-cache domains, malloc()ed as in the
    // reference. The reference always uses one domain (interface.cpp:207),
    // so the split is {0, nrow}.
    void getNumaSplitting(int **split, int *splitLen) {
        *split = (int *)malloc(2 * sizeof(int));
        (*split)[0] = 0;
        (*split)[1] = nrow_;
        *splitLen = 2;
    }

    // CPU thread and memory placement (interface.h:139, 172-177, 188-198):
    // the GPU engine has no host threads to pin, put to sleep or run
    // serially and no NUMA first touch, and its results do not depend on a
    // thread count. Kept so that callers of the reference compile; they do
    // nothing.
    void sleep() {}
    // MPI placeholders whose bodies are empty in the reference too (all code
    // commented out, interface.cpp:62-67 and compressColIdx after it): kept
    // so that callers compile.
    void passGlobalRows(int globalStartRow, int globalEndRow) { (void)globalStartRow, (void)globalEndRow; }
    void compressColIdx() {}
    void pinThread(int threadId) { (void)threadId; }
    void setSerial(int funcId) { (void)funcId; }
    void unsetSerial(int funcId) { (void)funcId; }
    void resetTime() {}
    void numaInitRowPtr(int *rowPtr) { (void)rowPtr; }
    void numaInitRowPtr(int **rowPtr) { (void)rowPtr; }
    void numaInitMtxVec(int *rowPtr, int *col, double *val, double *x, int power = 1) {
        (void)rowPtr, (void)col, (void)val, (void)x, (void)power;
    }
    void numaInitMtxVec(int **rowPtr, int **col, double **val, int power = 1) {
        (void)rowPtr, (void)col, (void)val, (void)power;
    }

    // tuneFunction (interface.cpp:605-647): runs the function with powers
    // 1..p for at least 0.2 s each, keeps the power with the lowest time per
    // power step and sets it. p is the power the function was registered
    // with (the reference takes highestPower), so that its x, sized for p,
    // is never overrun. The choice is kept per function.
    int tuneFunction(int funcId, bool rev = false) {
        auto known = tuned_.find(funcId);
        if (known != tuned_.end()) {
            setPower(funcId, known->second);
            return known->second;
        }
        const int hp = std::max(1, getPower(funcId));
        std::vector<double> perStep(hp, 0.0);
        for (int p = 1; p <= hp; ++p) {
            setPower(funcId, p);
            const auto start = std::chrono::steady_clock::now();
            double elapsed = 0;
            int iter = 0;
            do {
                executeFunction(funcId, rev);
                ++iter;
                elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
            } while (elapsed < 0.2);
            perStep[p - 1] = elapsed / (iter * (double)p);
        }
        const int best = (int)(std::min_element(perStep.begin(), perStep.end()) - perStep.begin()) + 1;
        tuned_[funcId] = best;
        setPower(funcId, best);
        return best;
    }
    void setStream(void *cudaStream) { race_set_stream(e_, cudaStream); }
    race_engine *handle() { return e_; }

  private:
    race_engine *e_ = nullptr;
    int nrow_;
    std::map<int, int> tuned_;
};

// Block-MPK functions of several Interfaces in one persistent launch
// (race_batch_*; no counterpart in the reference). The Interfaces and their
// operands must outlive the batch.
class Batch {
  public:
    Batch() {
        if (race_batch_create(&b_) != RACE_SUCCESS) throw std::runtime_error("race_batch_create failed");
    }
    ~Batch() { race_batch_destroy(b_); }
    Batch(const Batch &) = delete;
    Batch &operator=(const Batch &) = delete;
    int add(Interface &ce, int funcId) { return race_batch_add(b_, ce.handle(), funcId); }
    int prepare(void *cudaStream = nullptr) { return race_batch_prepare(b_, cudaStream); }
    int execute(void *cudaStream = nullptr) { return race_batch_execute(b_, cudaStream); }
    // first call captures the launch into a CUDA graph, later calls replay it
    int graphLaunch(void *cudaStream = nullptr) { return race_batch_graph_launch(b_, cudaStream); }
    int getStatus(void *cudaStream = nullptr) { return race_batch_get_status(b_, cudaStream); }
    const char *lastError() { return race_batch_last_error(b_); }

  private:
    race_batch *b_ = nullptr;
};

}  // namespace gb300
}  // namespace RACE
