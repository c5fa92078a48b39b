// The caller's own kernel body as a device functor (compiled by the test
// suite for sm_103a; INTEGRATION.md quotes it).
#include "race_gb300.hpp"
#include "race_gb300_device.cuh"

struct MyGs {  // the reference's GS callback body, args as members
    const int *rowPtr, *col;
    const double *val, *b;
    double *x;
    __device__ void operator()(int start, int end) const {
        const int inc = start > end ? -1 : 1;  // start > end: reverse sweep
        for (int row = start; row != end; row += inc) {
            double tmp = b[row];
            for (int idx = rowPtr[row] + 1; idx < rowPtr[row + 1]; ++idx) tmp -= val[idx] * x[col[idx]];
            x[row] = tmp / val[rowPtr[row]];
        }
    }
};

void example(RACE::gb300::Interface &ce, int *d_rowPtr, int *d_col, double *d_val, double *d_b, double *d_x,
             cudaStream_t stream) {
    // after ce.RACEColor() and permuting A:
    RACE::gb300::DeviceFunction<MyGs> gs(ce.handle(), MyGs{d_rowPtr, d_col, d_val, d_b, d_x});
    gs.execute(false, stream);  // forward sweep
    gs.execute(true, stream);   // backward sweep
}
