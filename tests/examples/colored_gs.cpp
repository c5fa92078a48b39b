// Colored symmetric Gauss-Seidel through the C++ Interface (compiled by the
// test suite; INTEGRATION.md quotes it).
#include "race_gb300.hpp"

void example(int n, int *rowPtr, int *col, int *d_rowPtr, int *d_col, double *d_val, double *d_x, double *d_b) {
    // host CRS of A (rowPtr, col), diagonal first
    RACE::gb300::Interface ce(n, 4096, RACE::gb300::TWO, rowPtr, col, /*symm_hint=*/true);
    ce.RACEing();  // the same as ce.RACEColor()
    int *perm, *invPerm, len;
    ce.getPerm(&perm, &len);
    ce.getInvPerm(&invPerm, &len);
    // permute A as sparsemat::permute does, copy it and x, b to the device ...
    race_operands ops{n, d_rowPtr, d_col, d_val, RACE_VAL_F64, d_x, d_b, RACE_VAL_F64};
    int gs = ce.registerFunction(RACE::gb300::GS, ops);
    ce.executeFunction(gs);        // forward sweep
    ce.executeFunction(gs, true);  // backward sweep
    delete[] perm;
    delete[] invPerm;
}
