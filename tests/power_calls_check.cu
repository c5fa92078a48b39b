// Host-only check of the device header's matrix-power schedule
// (include/race_gb300_device.cuh): prints the call table that
// DevicePowerFunction would run for level groups read from stdin, and how a
// three- and a four-argument functor see each call. Built and run by
// tests/test_device_functors.py without a GPU; test infrastructure only.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "race_gb300_device.cuh"

namespace {
struct Three {
    int *out;
    void operator()(int start, int end, int pow) const { out[0] = start, out[1] = end, out[2] = pow, out[3] = 0; }
};
struct Four {
    int *out;
    void operator()(int start, int end, int pow, int subPow) const {
        out[0] = start, out[1] = end, out[2] = pow, out[3] = subPow;
    }
};
}  // namespace

int main(int argc, char **argv) {
    if (argc != 4) return 2;
    const int power = atoi(argv[1]), subPower = atoi(argv[2]), rowsPerCall = atoi(argv[3]);
    std::vector<int> groupPtr;
    int v;
    while (scanf("%d", &v) == 1) groupPtr.push_back(v);
    std::vector<int4> calls;
    std::vector<int> stepPtr;
    RACE::gb300::detail::powerCalls(groupPtr, power * subPower, rowsPerCall, calls, stepPtr);
    printf("%zu\n", stepPtr.size() - 1);
    for (size_t s = 0; s + 1 < stepPtr.size(); ++s)
        for (int i = stepPtr[s]; i < stepPtr[s + 1]; ++i) {
            int a[4], b[4];
            RACE::gb300::detail::invokePower(Three{a}, calls[i].x, calls[i].y, calls[i].z, subPower, 0);
            RACE::gb300::detail::invokePower(Four{b}, calls[i].x, calls[i].y, calls[i].z, subPower, 0);
            printf("%zu %d %d %d %d %d\n", s, a[0], a[1], a[2], b[2], b[3]);
        }
    return 0;
}
