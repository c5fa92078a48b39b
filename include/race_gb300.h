/* race_gb300.h -- C ABI of the GB300-native RACE execution engine.
 *
 * The entry points mirror RACE::Interface (include/interface.h in the
 * reference) one to one; every function returns a RACE_error code and no
 * C++ exception crosses the boundary. Matrices are CRS with int32 indices.
 * Arrays passed as `host` are read during the call and not retained;
 * arrays passed as `dev` are device pointers owned by the caller that must
 * stay valid while a registered function that uses them can run.
 *
 * Threading: one host thread drives a handle at a time. Work is enqueued on
 * the handle's CUDA stream (race_set_stream); calls that return results to
 * the host synchronise that stream.
 */
#ifndef RACE_GB300_H
#define RACE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* RACE_error, include/error.h:29-41 of the reference, plus engine codes. */
enum {
    RACE_SUCCESS = 0,
    RACE_ERR_INVALID_ARG = 1,
    RACE_ERR_MATRIX_SYMM = 2,
    RACE_ERR_D2_COLOR = 3,
    RACE_ERR_D1_COLOR = 4,
    RACE_ERR_GRAPH_TRAVERSAL = 5,
    RACE_ERR_INCOMPATIBILITY = 6,
    RACE_ERR_HWLOC = 7,
    RACE_ERR_PIN = 8,
    RACE_ERR_INTERNAL = 9,
    RACE_ERR_NOT_IMPLEMENTED = 10,
    RACE_ERR_CUDA = 100,    /* a CUDA runtime call failed */
    RACE_ERR_TIMEOUT = 101  /* a device wait hit its iteration limit */
};

/* RACE::dist, include/type.h:31-35 */
enum { RACE_DIST_ONE = 1, RACE_DIST_TWO = 2, RACE_DIST_POWER = 3 };
/* RACE::d2Method, RACE::LBTarget, include/type.h:37-46 */
enum { RACE_TWO_BLOCK = 0, RACE_THREE_BLOCK = 1 };
enum { RACE_LB_ROW = 0, RACE_LB_NNZ = 1 };

/* Built-in device kernels (the example kernels of the reference,
 * examples/src/helpers/kernels.cpp). */
enum {
    RACE_K_SPMV = 0,      /* b = A x                                          */
    RACE_K_SPMTV = 1,     /* b += A^T x (scatter; needs distance-2)           */
    RACE_K_SYMMSPMV = 2,  /* b += A x from the upper triangle, diag first     */
    RACE_K_GS = 3,        /* x <- Gauss-Seidel step for A x = b, diag first   */
    RACE_K_KACZ = 4,      /* x <- Kaczmarz projection step (needs distance-2) */
    RACE_K_MPK = 5        /* x_k = A x_{k-1}, k = 1..power, power-major x     */
};

/* Value storage of a registered operand set. */
enum { RACE_VAL_F64 = 0, RACE_VAL_F32 = 1, RACE_VAL_BF16 = 2 };

/* Execution of colored sweeps. WAVE: RACE's order compiled into
 * conflict-free waves, one thread per row, results identical bit for bit to
 * RACE's sequential walk (rows above 512 entries use a warp reduction).
 * LEAF: one warp per RACE leaf, rows in order, warp-shuffle row reductions.
 * GATHER (SpMV, SpMTV, SymmSpMV only): one launch, one thread per entry of b
 * replaying RACE's updates to it in RACE's order (bit-identical to WAVE).
 * AUTO (default): GATHER for SpMV, SpMTV and SymmSpMV; for GS and KACZ, per
 * function and direction, whichever of WAVE and LEAF is estimated cheaper. */
enum { RACE_SWEEP_AUTO = 0, RACE_SWEEP_WAVE = 1, RACE_SWEEP_LEAF = 2, RACE_SWEEP_GATHER = 3 };

typedef struct race_engine race_engine;

/* Device operands of a built-in kernel (the `args` of registerFunction). */
typedef struct {
    int n;                  /* rows of the (permuted) matrix */
    const int *rowPtr;      /* dev, n+1 */
    const int *col;         /* dev, nnz */
    const void *val;        /* dev, nnz, type val_type */
    int val_type;           /* RACE_VAL_* */
    void *x;                /* dev, type vec_type; MPK: (power+1)*n doubles, power-major */
    void *b;                /* dev, type vec_type, n (unused by MPK) */
    int vec_type;           /* RACE_VAL_F64 or RACE_VAL_F32 (sweeps, block MPK); RACE_K_MPK vectors are FP64 */
} race_operands;

/* Pre-processing knobs; the reference reads them from the environment
 * (RACE_EFFICIENCY, RACE_THREADS, RACE_CACHE_VIOLATION_CUTOFF[_DEFAULT],
 * RACE_MAX_RECURSION_STAGES). race_params_from_env fills them the same way. */
typedef struct {
    int n_eff;
    double eff[16];          /* eff[0] default threshold (40), eff[k] stage k */
    int n_lvl_threads;
    int lvl_threads[16];
    int cache_violation_cutoff;
    int max_recursion_stages; /* -1: the reference's default; 0: MPK partition without recursion */
    int n_cutoffs;            /* RACE_CACHE_VIOLATION_CUTOFF: cut-off of MPK recursion stage k is cutoffs[k] */
    int cutoffs[16];          /* for k < n_cutoffs, else cache_violation_cutoff */
} race_params;

int race_params_from_env(race_params *p);

/* Interface::Interface (interface.h:124, interface.cpp:33-36). rowPtr/col are
 * host arrays; symm_hint=0 symmetrises the pattern first (graph.cpp:47-142).
 * initPerm/initInvPerm may be NULL. params may be NULL (read the environment). */
int race_create(race_engine **out, int nrow, int nthreads, int dist, const int *rowPtr_host, const int *col_host,
                int symm_hint, const int *initPerm_host, const int *initInvPerm_host, int d2type, int lbtarget,
                const race_params *params);
/* Interface::~Interface (interface.cpp:38-60) */
int race_destroy(race_engine *e);

/* Work is enqueued on this stream (default: the legacy default stream). */
int race_set_stream(race_engine *e, void *cuda_stream);

/* Interface::RACEColor() (interface.h:128, interface.cpp:260-301) */
int race_color(race_engine *e);
/* Interface::RACEColor(highestPower, cacheSize, safetyFactor, mtxType,
 * highestSubPower) (interface.h:127, interface.cpp:205-257); cacheSize in bytes.
 * A repeated call on the same engine (another power or cache budget, e.g. a
 * parameter search) regroups the BFS levels of the first call: the
 * permutation stays that of the first call. */
int race_power_prepare(race_engine *e, int highestPower, double cacheSize, double safetyFactor, const char *mtxType,
                       int highestSubPower);

/* Interface::getPerm / getInvPerm (interface.cpp:333-383): copy into
 * caller-provided host arrays of nrow ints. */
int race_get_perm(race_engine *e, int *perm_host, int *invPerm_host);
/* Interface::getNumThreads / getEfficiency / getMaxStageDepth (interface.cpp:304-331, 385) */
int race_get_num_threads(race_engine *e, int *out);
int race_get_efficiency(race_engine *e, double *out);
int race_get_max_stage_depth(race_engine *e, int *out);
/* Zone tree in the flat layout documented in race_gb300/csrc/coloring.h
 * (no counterpart in the reference API; printZoneTree prints the same data,
 * interface.cpp:328-331). *len receives the length; data is written when
 * cap is large enough. */
int race_get_zone_tree(race_engine *e, int *buf, int cap, int *len);
/* Flattened execution phases: phasePtr (numPhases+1) and leaf ranges. */
int race_get_phases(race_engine *e, int rev, int *phasePtr, int *leafLo, int *leafHi, int cap, int *numPhases,
                    int *numLeaves);
/* The same leaf ranges in device memory owned by the engine (valid until
 * race_color runs again or race_destroy), for custom device functions
 * (race_gb300_device.cuh). */
int race_get_device_phases(race_engine *e, int rev, const int **leafLo, const int **leafHi, int *numLeaves);
/* MPK level groups (consolidated levelPtr of the reference's MPLeaf::lp,
 * matrixPowerRecursive.h:27-62), *len = groups+1. */
int race_get_power_groups(race_engine *e, int *buf, int cap, int *len);
/* The MPK partition's leaf tree (mtxPowerRecursive's MPLeaf tree,
 * matrixPowerRecursive.h:27-62; the reference prints it with printTree):
 * count, then per leaf lo, hi, stage, parent, numGroups,
 * groupPtr[numGroups+1], numHopeless, hopeless[numHopeless]; the root alone
 * without hopeless regions. *len receives the length; data is written when
 * cap is large enough. */
int race_get_power_tree(race_engine *e, int *buf, int cap, int *len);

/* Interface::registerFunction (interface.h:149-157, interface.cpp:391-485)
 * with a built-in device kernel in place of a host callback; `power`
 * (1..255) is used by RACE_K_MPK. */
int race_register_function(race_engine *e, int kernel, const race_operands *ops, int power, int *func_id);
/* Interface::executeFunction (interface.h:167, interface.cpp:541-572):
 * enqueues the kernel on the engine's stream, waits for it and returns
 * RACE_ERR_TIMEOUT if a device wait gave up. */
int race_execute_function(race_engine *e, int func_id, int rev);
/* Same work without waiting (stream-ordered, like a CUDA library call);
 * race_get_status later synchronises and reports the device status word of
 * the last launch. No counterpart in the reference, whose executor is
 * synchronous. */
int race_execute_function_async(race_engine *e, int func_id, int rev);
int race_get_status(race_engine *e);
/* RACE_SWEEP_GATHER runs SpMV, SpMTV and SymmSpMV without the coloring's
 * phases: every entry of b is produced by one thread in one launch, from the
 * updates RACE's sequential walk makes to it, replayed in that walk's order
 * (identical results, bit for bit; the gather plan is built at the first
 * such call per direction). GS and KACZ, which depend on earlier rows, run
 * as in RACE_SWEEP_AUTO. */
/* Sweep execution mode of this engine (RACE_SWEEP_*), and the schedule
 * sizes of a registered sweep function in one direction: waves and the
 * largest wave, phases and the longest leaf, and the mode that runs
 * (*waveModeChosen: 0 leaf, 1 wave, 2 gather). No
 * counterpart in the reference (its executor has one mode). */
int race_set_sweep_mode(race_engine *e, int mode);
int race_get_sweep_info(race_engine *e, int func_id, int rev, int *numWaves, int *maxWaveRows, int *numPhases,
                        int *maxLeafRows, int *waveModeChosen);

/* Interface::setPower / getPower (interface.cpp:574-590) */
int race_set_power(race_engine *e, int func_id, int power);
int race_get_power(race_engine *e, int func_id, int *out);
/* Interface::setSubPower / getSubPower (interface.cpp:579-592) for a
 * built-in function. The built-in kernels have no sub-steps, so only 1 is
 * accepted (RACE_ERR_INCOMPATIBILITY otherwise) and getSubPower gives 1.
 * The caller's own power functions with sub-powers are device functors
 * (DevicePowerFunction::setSubPower in race_gb300_device.cuh). */
int race_set_sub_power(race_engine *e, int func_id, int subPower);
int race_get_sub_power(race_engine *e, int func_id, int *out);

/* Plain FP64 CRS SpMV b = A x (no schedule; the traditional baseline the
 * reference compares MPK against, kernels.cpp:90-105). */
int race_spmv_plain(race_engine *e, int n, const int *rowPtr_dev, const int *col_dev, const double *val_dev,
                    const double *x_dev, double *b_dev);

/* Symmetric Gauss-Seidel solve of A x = b with FP64 iterative refinement
 * (the reference's GS driver loop, examples/src/colorSymmGS.cpp:147-267,
 * with a mixed-precision inner solve). inner_func_id is a registered
 * RACE_K_GS function whose operands hold the inner matrix (FP32/BF16 values
 * with FP32 vectors, or FP64) and whose x/b buffers receive the correction d
 * and the residual r. Each refinement computes r = b - A x in FP64 from the
 * FP64 matrix (rowPtr/col/val, dev, same permuted matrix), runs `sweeps`
 * forward+backward sweeps on A d = r from d = 0, and updates x += d in FP64;
 * it stops when ||r||_2 <= tol ||b||_2 or after maxIter refinements.
 * *iters and *relres receive the refinement count and the final relative
 * residual. No counterpart in the reference API. */
int race_symmgs_ir(race_engine *e, int inner_func_id, int n, const int *rowPtr_dev, const int *col_dev,
                   const double *val_dev, const double *b_dev, double *x_dev, double tol, int maxIter, int sweeps,
                   int *iters, double *relres);

/* One plain SpMV x_{k+1} = A x_k (0 <= k < power) of a registered RACE_K_MPK
 * function, on its internal layout and operands, without the level-blocked
 * schedule: the traditional p-SpMV path on the same data (no counterpart in
 * the reference, whose examples time it separately as tradPower). */
int race_spmv_power_layout(race_engine *e, int func_id, int k);

/* The device layout of a registered RACE_K_MPK function (no counterpart in
 * the reference, which keeps the caller's CRS): SELL-32 chunks, the bits of
 * a stored column index (16: a 2-bit window and a 14-bit offset from one of
 * the chunk's four window bases; 32: plain indices), the chunks that keep
 * 32-bit columns in the 16-bit layout, the SELL slots with padding, and the
 * bytes of the matrix arrays one power reads (values, columns, row lengths,
 * chunk tables, hub copies), and the schedule that runs (see
 * race_set_mpk_schedule). */
int race_get_mpk_layout(race_engine *e, int func_id, int *numChunks, int *colBits, int *wideChunks,
                        long long *sellSlots, long long *matrixBytes, int *schedule);

/* Schedule of a registered RACE_K_MPK function (no counterpart in the
 * reference, whose executor always runs the level-group wavefront):
 * RACE_MPK_WAVEFRONT runs all powers in one persistent kernel in the
 * chunk-level wavefront order; RACE_MPK_SWEEPS runs p plain SpMV launches on
 * the same layout (no level blocking); RACE_MPK_AUTO (the default) times
 * both once, at the function's first call on a stream that is not being
 * captured (that call synchronises), and keeps the faster; while capturing
 * it runs the wavefront for FP64 values and the sweeps otherwise. All give
 * bit-identical powers. Triangular partitions (mtxType L/U) always run
 * their own step-by-step schedule. race_get_mpk_layout's *schedule reports
 * the schedule that runs (RACE_MPK_AUTO before the first timed call). */
enum { RACE_MPK_AUTO = 0, RACE_MPK_WAVEFRONT = 1, RACE_MPK_SWEEPS = 2 };
int race_set_mpk_schedule(race_engine *e, int func_id, int schedule);

/* Matrix power without any device allocation. No counterpart in the
 * reference (its executor runs on the host and allocates freely).
 * For callers that cannot allocate device memory when they run the kernel:
 * code whose device memory is owned by its own pool, real-time loops with a
 * fixed memory budget, library code that must not trigger a cudaMalloc (and
 * the device synchronisation it may cause). All scratch lives in one
 * built-in device array of 16 MiB (2^22 ints) held by every GPU that loads
 * the library; a problem needing more than about power * ceil(n/32) +
 * 2 * numGroups + 2 * power ints is rejected with RACE_ERR_INVALID_ARG.
 * Inputs: the FP64 CRS matrix permuted with the engine's MPK permutation
 * (device), the level groups from race_get_power_groups (numGroups+1 row
 * offsets, both a device and a host copy holding the same offsets: the host
 * copy sizes the scratch, the kernel reads the device copy; both must run
 * from 0 to n without decreasing and the device copy must give the same
 * number of 32-row chunks, otherwise RACE_ERR_INVALID_ARG before any work
 * item runs), and x with (power+1)*n doubles, power-major, x[0:n] the input
 * vector (device). A matrix not in the engine's level order is refused with
 * RACE_ERR_INVALID_ARG too. Results equal the registered RACE_K_MPK path bit
 * for bit, rows above 256 entries included. The first call on a device looks
 * up the array's device address, so make that first call before any CUDA
 * stream capture. Calls share the array: calls that overlap on the GPU
 * (other streams, other host threads) race and must be serialised by the
 * caller. Synchronises `stream` before returning. */
int race_mpk_noalloc(int n, const int *rowPtr_dev, const int *col_dev, const double *val_dev,
                     const int *groupPtr_dev, const int *groupPtr_host, int numGroups, int power, double *x_dev,
                     void *stream);

/* Matrix power over a block of nrhs right-hand sides (nrhs in 1, 2, 4, 8,
 * 16, 32): x_k = A x_{k-1} for every right-hand side, k = 1..power, on the
 * engine's level groups. Extends the power callback of registerFunction
 * (interface.h:151-153, one vector) to a vector block. x (device) holds
 * (power+1) * n * nrhs elements: power-major, then row, then right-hand side
 * (x[(k*n + r)*nrhs + j]); x[0 : n*nrhs] is the input block. Types: FP64
 * values with FP64 x (results equal p sequential fma SpMVs per right-hand
 * side bit for bit), or FP32/BF16 values with FP32 x (FP32 accumulation).
 * The matrix must be permuted with the engine's MPK permutation. Executed
 * with race_execute_function[_async]; race_spmv_power_layout runs one plain
 * SpMV of it; race_set_power rebuilds its schedule. */
int race_register_mpk_block(race_engine *e, const race_operands *ops, int power, int nrhs, int *func_id);

/* Batches: block-MPK functions of one or more engines (matrices of any size,
 * each with its own level groups and power) executed by ONE persistent
 * kernel launch; members must share value type, vector type and nrhs. No
 * counterpart in the reference (one matrix per RACE::Interface).
 * race_batch_add records (engine, function); the batch reads the members'
 * schedules and operand pointers at race_batch_prepare (called implicitly
 * by the first execute), so engines and operands must outlive the batch and
 * a member changed afterwards (race_set_power) needs a new prepare.
 * race_batch_execute enqueues the launch on `stream` (a cudaStream_t).
 * race_batch_graph_launch captures that launch sequence once into a CUDA
 * graph and replays the graph on every call (inputs are read through the
 * recorded pointers, so new data in the same buffers is picked up).
 * race_batch_get_status synchronises `stream` and returns RACE_ERR_TIMEOUT
 * if a device wait of the last launch gave up. race_batch_info reports
 * members, chunks and work items (0 before prepare). */
typedef struct race_batch race_batch;
int race_batch_create(race_batch **out);
int race_batch_destroy(race_batch *b);
int race_batch_add(race_batch *b, race_engine *e, int func_id);
int race_batch_prepare(race_batch *b, void *stream);
int race_batch_execute(race_batch *b, void *stream);
int race_batch_graph_launch(race_batch *b, void *stream);
int race_batch_get_status(race_batch *b, void *stream);
int race_batch_info(race_batch *b, int *members, int *chunks, int *items);
const char *race_batch_last_error(race_batch *b);

/* Multilayer perceptron of the parameter tuner (FP32; no counterpart in the
 * reference, whose only tuning is the wall-clock power sweep of
 * Interface::tuneFunction, interface.cpp:605-647). Shape: `in` inputs,
 * `hidden_layers` ReLU layers of `hidden` units, `out` linear outputs; every
 * layer y = x W^T + b with W row-major [out_l][in_l], parameters flattened
 * layer by layer as W then b (race_mlp_num_params values, all zero after
 * create). X, T and Y are device arrays, row-major [batch][in|out].
 * race_mlp_loss_grad evaluates the mean squared error sum (y-t)^2/(batch*out)
 * and its gradient with respect to every parameter (kept on the device;
 * copied to grad_host when non-NULL; *loss_host likewise), synchronising
 * `stream` when it copies. race_mlp_adam_step applies one Adam update with
 * the last gradient. */
typedef struct race_mlp race_mlp;
int race_mlp_create(race_mlp **out, int in, int hidden, int hidden_layers, int out_dim);
int race_mlp_destroy(race_mlp *m);
int race_mlp_num_params(race_mlp *m, long long *count);
int race_mlp_set_params(race_mlp *m, const float *params_host, long long count);
int race_mlp_get_params(race_mlp *m, float *params_host, long long count);
int race_mlp_forward(race_mlp *m, const float *X_dev, int batch, float *Y_dev, void *stream);
int race_mlp_loss_grad(race_mlp *m, const float *X_dev, const float *T_dev, int batch, float *loss_host,
                       float *grad_host, void *stream);
int race_mlp_adam_step(race_mlp *m, float lr, float beta1, float beta2, float eps, void *stream);
const char *race_mlp_last_error(race_mlp *m);

/* Host-only helpers (no GPU needed), exposed for inspection and tests:
 * the level load balancer (LB::balance, lb.cpp:188-771) on given level data,
 * out = [nScale, scale..., totalBlocks, zonePtr(totalBlocks+1)...,
 *        totalSubBlocks, subZonePtr(totalSubBlocks+1)..., numBlocks(totalBlocks)...];
 * and the phase flattening of a zone tree given in the flat layout of
 * race_get_zone_tree. Both return the written length (or the needed length
 * when cap is too small) through *len. */
int race_lb_balance(const int *levelRow, const int *levelNnz, int totalLevel, int nthreads, double eff, int dist,
                    int d2type, int lbtarget, int base, int *out, int cap, int *len);
int race_flatten_zone_tree(const int *tree, int treeLen, int dist, int d2type, int rev, int serialLo, int serialHi,
                           int *phasePtr, int *leafLo, int *leafHi, int cap, int *numPhases, int *numLeaves);

/* Host-only: RACE's single-stage MPK partition (mtxPower::findPartition,
 * matrixPower.cpp:505-605) of BFS levels levelRow/levelNnz (totalLevel
 * levels from row 0): cache-violating levels, hopeless regions
 * (identifyHopelessRegions, :147-503) and the consolidated level groups
 * (consolidatePartition, :685-940). power = highestPower * highestSubPower;
 * graphRows/graphNnz give the bytes per non-zero; cutoff is the cache
 * violation cut-off (INT_MAX: no hopeless regions). Writes groupPtr
 * (numGroups+1 row offsets, the reference's MPLeaf::lp) and hopeless
 * (numHopeless group indices, MPLeaf::hid) when cap is large enough for both. */
int race_mpk_stage_partition(const int *levelRow, const int *levelNnz, int totalLevel, int graphRows,
                             long long graphNnz, int power, double cacheSize, double safety, int cutoff, int *groupPtr,
                             int *hopeless, int cap, int *numGroups, int *numHopeless);

/* Host-only: the permutation of the MPK partition's recursion into its
 * hopeless groups (one stage, the reference's default;
 * matrixPowerRecursive.cpp:156-298): for each hopeless group, a BFS of its
 * rows through the boundary groups ceil(power/2)-1 on either side, then the
 * group and those boundary groups sorted by level. rowPtr/col: the
 * traversal pattern (original rows); totalPerm/totalInvPerm (n each, new
 * index -> original row and back) are updated in place; groupPtr and
 * hopeless as from race_mpk_stage_partition. */
int race_mpk_recursion_permute(int n, const int *rowPtr, const int *col, int *totalPerm, int *totalInvPerm,
                               const int *groupPtr, int numGroups, const int *hopeless, int numHopeless, int power);

/* Host-only: the MPK partition's recursion at any depth
 * (mtxPowerRecursive::recursivePartition, matrixPowerRecursive.cpp:156-338):
 * below the stage-0 groups and hopeless groups of race_mpk_stage_partition,
 * every hopeless group is traversed with its boundaries, partitioned again
 * (a level's size includes its boundary rows' non-zeros) with the cut-off
 * of its stage, stageCutoff[s] (INT_MAX for s >= numStages; stageCutoff[0]
 * is not read), and recursed into depth first. totalPerm/totalInvPerm are
 * updated in place. treeBuf (when cap >= *treeLen) gets the leaves in the
 * reference's order: count, then per leaf lo, hi, stage, parent, numGroups,
 * groupPtr[numGroups+1], numHopeless, hopeless[numHopeless]. */
int race_mpk_recursive_partition(int n, const int *rowPtr, const int *col, int *totalPerm, int *totalInvPerm,
                                 const int *groupPtr, int numGroups, const int *hopeless, int numHopeless, int power,
                                 long long graphNnz, double cacheSize, double safety, const int *stageCutoff,
                                 int numStages, int *treeBuf, int cap, int *treeLen);

/* Host-only: one traversal of rows [lo,hi) of the current permuted space
 * with RACE's distance-1 or distance-2 rules (dist 1 or 2;
 * traverse_GAP_graphSoA.cpp:135-641): the engine's own traversal, which it
 * runs on the host for ranges shorter than RACE_GPU_HOST_TRAVERSE_BELOW.
 * rowPtr/col: the traversal graph (original rows); totalPerm/totalInvPerm
 * (n each) are updated in place and levelRow/levelNnz written when
 * cap >= *totalLevel (otherwise nothing changes and *totalLevel says how
 * much room is needed). */
int race_traverse_host(int n, const int *rowPtr, const int *col, int *totalPerm, int *totalInvPerm, int lo, int hi,
                       int dist, int *levelRow, int *levelNnz, int cap, int *totalLevel);

/* Host-only: RACE's level recursion (level_recursion.cpp:149-376, the
 * zone tree of race_color) with the traversal supplied by the caller instead
 * of the engine's GPU BFS. `trav` runs one traversal of rows [lo,hi) of the
 * current permuted index space (BFS levels, stable level sort composed into
 * the caller's running permutation) and writes the per-level row and
 * non-zero counts (at most cap levels; returns 0, or nonzero to abort);
 * `rangeNnz` returns the non-zeros of rows [lo,hi) in the current
 * permutation. Writes the serialised zone tree (format of
 * race_get_zone_tree) when cap >= *treeLen. For tests and for callers with
 * their own traversal. */
typedef int (*race_traverse_fn)(void *user, int lo, int hi, int *levelRow, int *levelNnz, int cap, int *totalLevel);
typedef long long (*race_range_nnz_fn)(void *user, int lo, int hi);
int race_zone_tree_host(int nrow, int nthreads, int dist, int d2type, int lbTarget, const race_params *params,
                        race_traverse_fn trav, race_range_nnz_fn rangeNnz, void *user, int *treeBuf, int cap,
                        int *treeLen, int *availableThreads);

/* Host-only: the gather plan of RACE_SWEEP_GATHER for SpMTV or SymmSpMV on
 * a CRS pattern and a phase table: for every entry y of b, the updates
 * ptr[y] .. ptr[y+1] in RACE's execution order, each a matrix entry (-1:
 * row y's own SymmSpMV update) and the row whose x it reads. Written when
 * cap >= *numUpdates and cap >= n + 1. */
int race_gather_plan(int kernel, int n, const int *rowPtr, const int *col, const int *phasePtr, const int *leafLo,
                     const int *leafHi, int numPhases, int *ptr, int *entry, int *row, int cap, int *numUpdates);

/* Host-only: the wave plan of built-in kernel `kernel` on a CRS pattern
 * (host arrays) for a phase table (as from race_get_phases): rows grouped
 * into conflict-free waves that keep RACE's order between every pair of
 * conflicting accesses. wavePtr (numWaves+1) and rows (numRows) are written
 * when cap is large enough for both (call once with cap 0 for the sizes).
 * No counterpart in the reference; exposed for inspection and tests. */
int race_wave_plan(int kernel, int n, const int *rowPtr, const int *col, const int *phasePtr, const int *leafLo,
                   const int *leafHi, int numPhases, int *wavePtr, int *rows, int cap, int *numWaves, int *numRows);

/* Host-only: the issue order of the persistent matrix-power kernel for
 * numChunks chunks whose dependency intervals are depRange (6 ints per
 * chunk: the chunk intervals [lo,hi] its columns fall in within the
 * previous, own and next level group; hi < lo when empty). order 0: the
 * chunk-level wavefront in runs of up to runLen chunks (1..32) per ticket,
 * powers in segments of segLen (0: one segment), each item at least `lag`
 * chunks of issue time after its inputs; chunkDie (NULL: one die) gives the
 * L2 die (0 or 1) whose SMs run each chunk, and the runs are grouped into one
 * queue per die. order 1: RACE's level-group order
 * (functionManager.cpp:618-823) with stride `stride`, one chunk per run,
 * chunkGroup giving each chunk's level group. Writes, when
 * cap >= *numRuns, per run head[4] (first chunk, end chunk, power, flags),
 * dep[8] (four chunk intervals that must be complete at the previous
 * power) and rank (its position in the global order; may be NULL), and
 * dieStart[3] (die d's queue is runs dieStart[d] .. dieStart[d+1]-1). The
 * dependency ranges are first widened to the kernel's completion blocks
 * (at most 16 consecutive chunks inside one level group of chunkGroup, or
 * by index alone when chunkGroup is NULL), as the engine does. No
 * counterpart in the reference; exposed for tests. */
int race_mpk_issue_order(const int *depRange, const int *chunkGroup, const int *chunkDie, int numChunks, int power,
                         int order, int stride, int segLen, int runLen, int lag, int *head, int *dep, int *rank,
                         int *dieStart, int cap, int *numRuns);

/* The L2 die map of the current device as the engine measured it (once per
 * process and device, at the first matrix-power registration or at this
 * call): *numDies (1 or 2), *numSms and, when cap >= *numSms, smDie[sm] for
 * every SM index. GB300's two dies each cache what their own SMs read; the
 * matrix-power kernel keeps each chunk's work on one die. Synchronises the
 * device on the first call. No counterpart in the reference. */
int race_device_dies(int *numDies, int *smDie, int cap, int *numSms);

/* RACE::Interface::getHighestPower (interface.cpp:1055-1058): the highest
 * power given to race_power_prepare (1 before it). */
int race_get_highest_power(race_engine *e, int *power);

/* SELL-C-sigma preparation for SIMD kernels, RACE::Interface::simdify and
 * simdifyD1 (include/interface.h:179-185; include/simdify.h,
 * src/sell_c_sigmize.cpp). Host arrays in the reference's layout: entry j of
 * row r at chunkStart[r/C] + r%C + j*C, rl[r] row r's length, clp[c] chunk
 * c's padded length; C a multiple of simdWidth; the matrix in the engine's
 * permuted order. col and val (val_type RACE_VAL_F64/F32/BF16; val may be
 * NULL) are rewritten in place.
 *
 * race_simdify (distance-2 scatter kernels): pads each row of each leaf
 * [start, end) of the forward schedule with columns start + (row-start) %
 * simdWidth, then reorders the rows so that the simdWidth rows of a SIMD
 * group hold pairwise different columns in every slot (diagonal kept in slot
 * 0 with diagFirst). The engine must be colored and nrows its row count.
 * RACE_ERR_INCOMPATIBILITY when a row cannot be placed (the reference's
 * `false`; the arrays are then partly rearranged, as there). collisions
 * (nullable): rows that needed a move. */
int race_simdify(race_engine *e, int simdWidth, int C, int nrows, int *col, const int *chunkStart, const int *rl,
                 const int *clp, void *val, int val_type, int diagFirst, int *collisions);

/* Host-only: race_simdify on an explicit forward schedule (leaves as from
 * race_get_phases or race_flatten_zone_tree). No engine needed. */
int race_simdify_schedule(int simdWidth, int C, int nrows, int *col, const int *chunkStart, const int *rl,
                          const int *clp, void *val, int val_type, int diagFirst, const int *leafLo,
                          const int *leafHi, int numLeaves, int *collisions);

/* Host-only, simdifyD1 (distance-1 kernels such as Gauss-Seidel): moves each
 * row's entries on the earlier rows of its SIMD group to the row's last
 * slots, nearest row last (dist2Compatible = 0) or first (1). rl is unused,
 * as in the reference. */
int race_simdify_d1(int simdWidth, int C, int nrows, int *col, const int *chunkStart, const int *rl, const int *clp,
                    void *val, int val_type, int dist2Compatible);

/* Last error message of this engine (NUL-terminated, owned by the engine). */
const char *race_last_error(race_engine *e);

#ifdef __cplusplus
}
#endif
#endif
