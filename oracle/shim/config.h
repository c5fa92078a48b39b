/* Oracle build configuration for compiling the RACE reference sources in place.
 * Mirrors the reference's CMake defaults (CMakeLists.txt:14-16, 80-83, 232-236):
 * OpenMP kernel threads, GAP BFS containers, SoA graph, permute-on-fly, C++17.
 * MPI MPK is off (the reference default). Test infrastructure only. */
#ifndef RACE_CONFIG_H
#define RACE_CONFIG_H
#define RACE_VERBOSITY 1
#define RACE_KERNEL_THREAD_OMP
#define RACE_USE_GAP
#define RACE_PERMUTE_ON_FLY
#define RACE_USE_SOA_GRAPH
#define RACE_HAVE_CPP_17
#endif
