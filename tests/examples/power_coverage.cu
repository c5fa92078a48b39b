// The reference's checkPowerCoverage as a device-header call (compiled by
// the test suite for sm_103a; INTEGRATION.md quotes it).
#include "race_gb300.hpp"
#include "race_gb300_device.cuh"

int example(RACE::gb300::Interface &ce) {
    // after ce.RACEColor(p, cacheSize):
    int errors = -1;
    RACE::gb300::checkPowerCoverage(ce.handle(), &errors);  // 0 for a sound schedule
    return errors;
}
