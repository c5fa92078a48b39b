// race_gb300.hpp -- header-only C++ view of the GB300 engine with the shape of
// RACE::Interface (include/interface.h:54-205 of the reference), forwarding
// to the C ABI in race_gb300.h. Method names, argument meaning and return
// codes follow the reference; the callback is a built-in device kernel with
// device operands instead of a host function pointer.
#pragma once
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

    // registerFunction with a device kernel (interface.h:149-157); returns the
    // function id, or the error code as the reference does.
    int registerFunction(Kernel k, const race_operands &args, int power = 1) {
        int id = -1;
        int rc = race_register_function(e_, (int)k, &args, power, &id);
        return rc == RACE_SUCCESS ? id : rc;
    }
    int executeFunction(int funcId, bool rev = false) { return race_execute_function(e_, funcId, rev ? 1 : 0); }
    void setPower(int funcId, int pow) { race_set_power(e_, funcId, pow); }
    int getPower(int funcId) {
        int v = 0;
        race_get_power(e_, funcId, &v);
        return v;
    }
    void setStream(void *cudaStream) { race_set_stream(e_, cudaStream); }
    race_engine *handle() { return e_; }

  private:
    race_engine *e_ = nullptr;
    int nrow_;
};

}  // namespace gb300
}  // namespace RACE
