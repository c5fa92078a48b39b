// Custom device functions run through the engine's schedule
// (include/race_gb300_device.cuh): the example kernels' bodies
// (examples/src/helpers/kernels.cpp: GS :174-186, MAT_SPMV_KERNEL
// :749-777) written as functors, with every multiply-add an explicit fma
// (built with --fmad=false) so that results compare bit for bit with the
// oracle. Built and loaded by tests/test_device_functors.py; test
// infrastructure only.
#include "race_gb300_device.cuh"

namespace {

struct GsFn {
    const int *rowPtr, *col;
    const double *val, *b;
    double *x;
    __device__ void operator()(int start, int end) const {
        const int inc = start > end ? -1 : 1;
        for (int row = start; row != end; row += inc) {
            const int d = rowPtr[row];
            double tmp = b[row];
            for (int idx = d + 1; idx < rowPtr[row + 1]; ++idx) tmp = fma(-val[idx], x[col[idx]], tmp);
            x[row] = tmp / val[d];
        }
    }
};

struct MpkFn {
    const int *rowPtr, *col;
    const double *val;
    double *x;
    int n;
    __device__ void operator()(int start, int end, int pow) const {
        const double *in = x + (size_t)(pow - 1) * n;
        double *out = x + (size_t)pow * n;
        for (int row = start; row < end; ++row) {
            double tmp = 0;
            for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx) tmp = fma(val[idx], in[col[idx]], tmp);
            out[row] = tmp;
        }
    }
};

// MAT_NUM_VEC_ACCESSES_w_subPower (examples/src/helpers/sparsemat.cpp:1399-1412)
// with the sub-power count as a member: every row is visited once per
// (pow, subPow), in order; a visit out of order counts an error.
struct CountFn {
    double *x;
    int subPower;
    int *errors;
    __device__ void operator()(int start, int end, int pow, int subPow) const {
        for (int row = start; row < end; ++row) {
            x[row] += 1;
            if (x[row] != (double)((pow - 1) * subPower + subPow)) atomicAdd(errors, 1);
        }
    }
};

int finish(int rc) {
    if (rc == RACE_SUCCESS && cudaDeviceSynchronize() != cudaSuccess) rc = RACE_ERR_CUDA;
    return rc;
}

}  // namespace

extern "C" int fn_gs(race_engine *e, const int *rowPtr, const int *col, const double *val, const double *b, double *x,
                     int rev) {
    RACE::gb300::DeviceFunction<GsFn> f(e, GsFn{rowPtr, col, val, b, x});
    if (f.status() != RACE_SUCCESS) return f.status();
    return finish(f.execute(rev != 0, 0));
}

extern "C" int fn_mpk(race_engine *e, const int *rowPtr, const int *col, const double *val, double *x, int n, int power,
                      int rowsPerCall) {
    RACE::gb300::DevicePowerFunction<MpkFn> f(e, MpkFn{rowPtr, col, val, x, n}, power, rowsPerCall);
    if (f.status() != RACE_SUCCESS) return f.status();
    return finish(f.execute(0));
}

extern "C" int fn_count_subpower(race_engine *e, double *x, int power, int subPower, int *errors) {
    RACE::gb300::DevicePowerFunction<CountFn> f(e, CountFn{x, subPower, errors}, power, 32, subPower);
    if (f.status() != RACE_SUCCESS) return f.status();
    return finish(f.execute(0));
}

// The same count after setPower / setSubPower on a function registered
// with power 1 and sub-power 1 (Interface::setPower / setSubPower).
extern "C" int fn_count_after_set(race_engine *e, double *x, int power, int subPower, int *errors) {
    RACE::gb300::DevicePowerFunction<CountFn> f(e, CountFn{x, subPower, errors}, 1, 32, 1);
    if (f.status() != RACE_SUCCESS) return f.status();
    if (f.setPower(power) != RACE_SUCCESS || f.getPower() != power) return RACE_ERR_INVALID_ARG;
    if (f.setSubPower(subPower) != RACE_SUCCESS || f.getSubPower() != subPower) return RACE_ERR_INVALID_ARG;
    return finish(f.execute(0));
}

extern "C" int fn_check_coverage(race_engine *e, int *errors) { return RACE::gb300::checkPowerCoverage(e, errors); }
