/* No-op topology stand-in with the hwloc calls RACE's pinning layer makes
 * (machine.cpp:34-150). It reports one package holding ORACLE_HWLOC_PUS cores
 * (default 4096) with one PU each, so RACE never runs out of places to "pin"
 * (RACE may return more threads than requested; pin.cpp:143). Binding is a
 * no-op that succeeds: CPU affinity plays no part in the schedule RACE
 * computes. Written for the oracle build from RACE's call sites.
 * Test infrastructure only. */
#ifndef ORACLE_HWLOC_STUB_H
#define ORACLE_HWLOC_STUB_H
#include <cstdlib>

typedef int hwloc_obj_type_t;
enum { HWLOC_OBJ_PACKAGE = 1, HWLOC_OBJ_CORE = 2, HWLOC_OBJ_PU = 3 };
enum { HWLOC_CPUBIND_THREAD = 2 };

struct oracle_hwloc_bitmap { int id; };
typedef oracle_hwloc_bitmap *hwloc_cpuset_t;
typedef oracle_hwloc_bitmap *hwloc_bitmap_t;

struct oracle_hwloc_obj { hwloc_cpuset_t cpuset; };
typedef oracle_hwloc_obj *hwloc_obj_t;

struct oracle_hwloc_topology { int npus; oracle_hwloc_bitmap set; oracle_hwloc_obj obj; };
typedef oracle_hwloc_topology *hwloc_topology_t;

static inline int oracle_hwloc_npus() {
    const char *e = getenv("ORACLE_HWLOC_PUS");
    int n = e ? atoi(e) : 4096;
    return n > 0 ? n : 4096;
}
static inline int hwloc_topology_init(hwloc_topology_t *t) {
    *t = new oracle_hwloc_topology;
    (*t)->npus = oracle_hwloc_npus();
    (*t)->set.id = 0;
    (*t)->obj.cpuset = &(*t)->set;
    return 0;
}
static inline int hwloc_topology_load(hwloc_topology_t) { return 0; }
static inline void hwloc_topology_destroy(hwloc_topology_t t) { delete t; }
static inline int hwloc_get_nbobjs_by_type(hwloc_topology_t, hwloc_obj_type_t type) {
    return type == HWLOC_OBJ_PACKAGE ? 1 : 0;
}
static inline hwloc_obj_t hwloc_get_obj_by_type(hwloc_topology_t t, hwloc_obj_type_t, unsigned) { return &t->obj; }
static inline int hwloc_get_nbobjs_inside_cpuset_by_type(hwloc_topology_t t, hwloc_cpuset_t, hwloc_obj_type_t type) {
    return type == HWLOC_OBJ_CORE ? t->npus : 1;
}
static inline hwloc_obj_t hwloc_get_obj_inside_cpuset_by_type(hwloc_topology_t t, hwloc_cpuset_t, hwloc_obj_type_t, unsigned) {
    return &t->obj;
}
static inline int hwloc_set_cpubind(hwloc_topology_t, hwloc_cpuset_t, int) { return 0; }
static inline int hwloc_get_cpubind(hwloc_topology_t, hwloc_cpuset_t, int) { return 0; }
static inline hwloc_bitmap_t hwloc_bitmap_dup(hwloc_cpuset_t s) { return s; }
static inline void hwloc_bitmap_singlify(hwloc_bitmap_t) {}
static inline void hwloc_bitmap_free(hwloc_bitmap_t) {}
static inline hwloc_bitmap_t hwloc_bitmap_alloc() { return nullptr; }
#endif
