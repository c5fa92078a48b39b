/* Minimal atomics used by RACE's BFS (traverse_GAP_graphSoA.cpp:178-204):
 * compare_and_swap(x, old, new) returns true when x held `old` and now holds `new`.
 * Written for the oracle build from RACE's call sites. Test infrastructure only. */
#ifndef ORACLE_PLATFORM_ATOMICS_H
#define ORACLE_PLATFORM_ATOMICS_H
#include <cstddef>
template <typename T>
inline bool compare_and_swap(T &x, const T &old_val, const T &new_val) {
    return __sync_bool_compare_and_swap(&x, old_val, new_val);
}
template <typename T>
inline T fetch_and_add(T &x, T inc) { return __sync_fetch_and_add(&x, inc); }
#endif
