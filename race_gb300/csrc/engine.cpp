// Engine driver: pre-processing (coloring, matrix-power partition),
// function registration and execution, and the C ABI of include/race_gb300.h.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>

#include "dies.h"
#include "engine.h"
#include "mpk_order.h"
#include "partition.h"
#include "simdify.h"

namespace race {

std::unique_ptr<MpkPlan> buildMpkPlan(Engine &e, const race_operands &ops, int power);
void runMpk(Engine &e, MpkPlan &plan, const race_operands &ops, int power);
void runSpmvSell(Engine &e, MpkPlan &plan, double *x, int n, int k);
void uploadPhases(Engine &e, int dir);
void buildSweepWaves(Engine &e, FuncEntry &f);
void runSweep(Engine &e, FuncEntry &f, bool rev);
bool useWaveMode(const Engine &e, const FuncEntry &f, int dir);
bool usesGather(const Engine &e, const FuncEntry &f);
void symmGsIr(Engine &e, int inner, int n, const int *rowPtr, const int *col, const double *val, const double *b,
              double *x, double tol, int maxIter, int sweeps, int *itersOut, double *relresOut);
std::unique_ptr<BlockPlan> buildBlockPlan(Engine &e, const race_operands &ops, int power, int nrhs);
void buildBatchTables(BatchTables &t, const std::vector<const BlockPlan *> &plans, cudaStream_t s);
void runBatch(BatchTables &t, cudaStream_t s);
void runBlockSpmv(const BlockPlan &p, int k, cudaStream_t s);

// Interface::RACEColor() (interface.cpp:260-301): level recursion over the
// whole matrix, then the execution phases of both sweep directions.
void Engine::color() {
    if (dist == DIST_POWER) throw Error(RACE_ERR_INVALID_ARG, "coloring needs dist ONE or TWO");
    LevelRecursion lr(
        n, requested, dist, d2, lbTarget, params, [this](int lo, int hi) { return traverse(lo, hi, dist); },
        [this](int lo, int hi) { return rangeNnz(lo, hi); });
    lr.levelBalancing();
    syncDevicePerm();
    availableThreads = lr.availableThreads;
    tree = std::make_unique<ZoneTree>(lr.tree);
    for (int dir = 0; dir < 2; ++dir) {
        phases[dir] = flattenZoneTree(*tree, dir == 1, n, n);
        uploadPhases(*this, dir);
    }
    RACE_CUDA(cudaStreamSynchronize(stream));
    colored = true;
}

// Interface::RACEColor(p, cacheSize, ...) (interface.cpp:205-257) for the
// first stage of mtxPowerRecursive (matrixPowerRecursive.cpp:340-436):
// BFS levels of the whole matrix, cache-violation check, level groups.
void Engine::powerPrepare(int hp, double cacheSize, double safety, const std::string &mtxType, int subPow) {
    if (subPow < 1) throw Error(RACE_ERR_INVALID_ARG, "highest sub power must be >= 1");
    if (dist != DIST_POWER) throw Error(RACE_ERR_INVALID_ARG, "matrix power needs dist POWER");
    if (mtxType != "N" && mtxType != "L" && mtxType != "U") throw Error(RACE_ERR_INVALID_ARG, "mtxType must be N, L or U");
    highestPower = hp;
    highestSubPower = subPow;
    const int P = hp * subPow;
    // The BFS levels depend on neither the power nor the cache budget: a
    // repeated call (a parameter search) regroups the cached levels instead
    // of traversing the already permuted matrix again, so the permutation
    // stays the one of the first call.
    if (!powerLevelsCached || powerLevelsType != mtxType) {
        powerLevels = traverse(0, n, DIST_POWER, mtxType);
        powerLevelsType = mtxType;
        powerLevelsCached = true;
    }
    const LevelData &ld = powerLevels;
    const int L = ld.totalLevel;
    levelPtr.assign(L + 1, 0);
    for (int l = 0; l < L; ++l) levelPtr[l + 1] = levelPtr[l] + ld.levelRow[l];
    // getBytePerNNZ / getElemUpperLimit (matrixPower.cpp:88-99, 134-140)
    double nnzr = nnz / (double)n;
    double bpn = (double)(((1 + P / nnzr) * sizeof(double) + (1 + 1 / nnzr) * sizeof(int)));
    double cacheElem = cacheSize / bpn;
    // stage-0 cut-off (matrixPowerRecursive.cpp:37-95)
    int maxRec = params.maxRecStages >= 0 ? params.maxRecStages
                                          : std::max(0, (int)(params.cacheViolationCutoff.size() - 1 + 1));
    int cutoff = 50;
    if (0 >= maxRec)
        cutoff = INT_MAX;
    else
        cutoff = (0 < (int)params.cacheViolationCutoff.size() - 1) ? params.cacheViolationCutoff[1]
                                                                    : params.cacheViolationCutoff[0];
    // Levels over the cut-off form a hopeless region only where two of them
    // are consecutive (identifyHopelessRegions, matrixPower.cpp:147-210);
    // isolated ones are grouped like any other level.
    bool hopeless = false;
    for (int l = 0, prev = -2; l < L; ++l) {
        double e = safety * (P + 1) * ld.levelNnz[l];
        if (e > cacheElem && static_cast<int>(std::ceil(e / cacheElem)) > cutoff) {
            hopeless = hopeless || l == prev + 1;
            prev = l;
        }
    }
    if (hopeless) {
        // Hopeless regions: the reference's stage-0 groups around them
        // (stagePartition) and, for mtxType N, its recursion, which reorders
        // the rows of each hopeless group and of its boundary groups
        // (recursivePartition: one stage by default, deeper stages reorder
        // rows inside those groups again) and gives the leaf tree.
        // Every stage-0 group keeps its row range, so the MPK's
        // neighbour-group dependencies still hold.
        const StagePartition sp = stagePartition(ld, 0, P, n, nnz, cacheSize, safety, cutoff);
        powerTree.assign(1, MpkLeaf{0, n, 0, -1, sp.groupPtr, sp.hopeless});
        if (mtxType == "N" && !sp.hopeless.empty()) {
            // cut-off of stage s (get_cache_violation_cutoff, matrixPowerRecursive.cpp:81-100);
            // stages from maxRec on have none
            std::vector<int> stageCutoff(std::min(std::max(maxRec, 1), 1 << 16));
            const std::vector<int> &cv = params.cacheViolationCutoff;
            for (int s = 0; s < (int)stageCutoff.size(); ++s)
                stageCutoff[s] = s < (int)cv.size() - 1 ? cv[s + 1] : cv[0];
            const bool ok = recursivePartition(n, hRowPtr.data(), hCol.data(), hPerm, hInvPerm, sp, P, nnz, cacheSize,
                                               safety, stageCutoff, powerTree);
            if (!ok)
                throw Error(RACE_ERR_GRAPH_TRAVERSAL,
                            "MPK recursion: rows of a hopeless group went missing, or its boundary groups do not exist");
            dPerm.upload(hPerm.data(), n, stream);
            dInvPerm.upload(hInvPerm.data(), n, stream);
            RACE_CUDA(cudaStreamSynchronize(stream));
            powerLevelsCached = false;  // the BFS levels no longer follow the row order
        }
        groupPtr = sp.groupPtr;
        unlockRow = sp.unlockRow;
        dangerRow = sp.dangerRow;
        powerReady = true;
        return;
    }
    // consolidatePartition without hopeless regions (matrixPower.cpp:685-883)
    groupPtr.assign(1, levelPtr[0]);
    unlockRow.assign(1, L > 0 ? levelPtr[std::min(1, L)] : 0);
    dangerRow.clear();
    double sumElem = 0;
    for (int l = 0; l < L; ++l) {
        double cur = safety * (P + 1) * ld.levelNnz[l];
        sumElem += cur;
        if (l > 0 && sumElem >= cacheElem) {
            sumElem = cur;
            groupPtr.push_back(levelPtr[l]);
            dangerRow.push_back(levelPtr[l - 1]);
            unlockRow.push_back(levelPtr[l + 1]);
        }
    }
    groupPtr.push_back(levelPtr[L]);
    dangerRow.push_back(levelPtr[L > 0 ? L - 1 : 0]);
    powerTree.assign(1, MpkLeaf{0, n, 0, -1, groupPtr, {}});
    powerReady = true;
}

int Engine::registerFunction(int kernel, const race_operands &ops, int power) {
    if (ops.n != n) throw Error(RACE_ERR_INVALID_ARG, "operand rows differ from the engine's");
    if (!ops.rowPtr || !ops.col || !ops.val) throw Error(RACE_ERR_INVALID_ARG, "missing matrix operand");
    FuncEntry f;
    f.kernel = kernel;
    f.ops = ops;
    f.power = power;
    if (kernel == RACE_K_MPK) {
        // interface.cpp:438-458
        if (dist != DIST_POWER || !powerReady) throw Error(RACE_ERR_INVALID_ARG, "MPK needs RACEColor(power, ...) first");
        if (power < 1 || power > 255) throw Error(RACE_ERR_INVALID_ARG, "power must be in 1..255");
        if (!ops.x) throw Error(RACE_ERR_INVALID_ARG, "missing x");
        f.mpk = buildMpkPlan(*this, ops, power);
    } else {
        // interface.cpp:397-431
        if (dist == DIST_POWER) throw Error(RACE_ERR_INVALID_ARG, "coloring kernels need dist ONE or TWO");
        if (!colored) throw Error(RACE_ERR_INVALID_ARG, "RACEColor() first");
        if (kernel < RACE_K_SPMV || kernel > RACE_K_KACZ) throw Error(RACE_ERR_INVALID_ARG, "unknown kernel");
        if (!ops.x || !ops.b) throw Error(RACE_ERR_INVALID_ARG, "missing x or b");
        if ((kernel == RACE_K_SPMTV || kernel == RACE_K_KACZ || kernel == RACE_K_SYMMSPMV) && dist != DIST_TWO)
            throw Error(RACE_ERR_D2_COLOR, "scatter kernels need distance-2 coloring");
        if (ops.vec_type == RACE_VAL_F64 && ops.val_type != RACE_VAL_F64)
            throw Error(RACE_ERR_INVALID_ARG, "FP64 vectors need FP64 values");
        if (ops.vec_type == RACE_VAL_F32 && ops.val_type == RACE_VAL_F64)
            throw Error(RACE_ERR_INVALID_ARG, "FP32 vectors need FP32 or BF16 values");
        buildSweepWaves(*this, f);
    }
    funcs.push_back(std::move(f));
    return (int)funcs.size() - 1;
}

// Matrix power over nrhs right-hand sides (no counterpart in the reference,
// whose power callback takes one vector).
int Engine::registerMpkBlock(const race_operands &ops, int power, int nrhs) {
    if (ops.n != n) throw Error(RACE_ERR_INVALID_ARG, "operand rows differ from the engine's");
    if (!ops.rowPtr || !ops.col || !ops.val || !ops.x) throw Error(RACE_ERR_INVALID_ARG, "missing operand");
    if (dist != DIST_POWER || !powerReady) throw Error(RACE_ERR_INVALID_ARG, "MPK needs RACEColor(power, ...) first");
    if (power < 1 || power > 255) throw Error(RACE_ERR_INVALID_ARG, "power must be in 1..255");
    FuncEntry f;
    f.kernel = RACE_K_MPK;
    f.ops = ops;
    f.power = power;
    f.block = buildBlockPlan(*this, ops, power, nrhs);
    funcs.push_back(std::move(f));
    return (int)funcs.size() - 1;
}

void Engine::launch(int id, bool rev) {
    if (id < 0 || id >= (int)funcs.size()) throw Error(RACE_ERR_INVALID_ARG, "unknown function id");
    FuncEntry &f = funcs[id];
    if (f.block) {
        runBatch(f.block->tables, stream);
        lastStatus = f.block->tables.status.p;
    } else if (f.kernel == RACE_K_MPK) {
        runMpk(*this, *f.mpk, f.ops, f.power);
        lastStatus = f.mpk->status.p;
    } else {
        runSweep(*this, f, rev);
        lastStatus = dStatus.p;
    }
}

void Engine::checkStatus() {
    int st = 0;
    if (lastStatus) RACE_CUDA(cudaMemcpyAsync(&st, lastStatus, sizeof(int), cudaMemcpyDeviceToHost, stream));
    RACE_CUDA(cudaStreamSynchronize(stream));
    if (st != DEV_OK) throw Error(RACE_ERR_TIMEOUT, "a device wait gave up (schedule dependency or grid barrier)");
}

void Engine::execute(int id, bool rev) {
    launch(id, rev);
    checkStatus();
}

}  // namespace race

using race::Engine;
using race::Error;

struct race_engine {
    std::unique_ptr<Engine> eng;
    std::string err;
};

namespace {
template <typename F>
int guard(race_engine *h, F &&f) {
    try {
        f();
        return RACE_SUCCESS;
    } catch (const Error &ex) {
        if (h) h->err = ex.what();
        return ex.code;
    } catch (const std::exception &ex) {
        if (h) h->err = ex.what();
        return RACE_ERR_INTERNAL;
    }
}
race::Params toParams(const race_params *p) {
    if (!p) return race::Params::fromEnv();
    race::Params q;
    q.effVec.assign(p->eff, p->eff + std::max(1, std::min(p->n_eff, 16)));
    q.lvlThreads.assign(p->lvl_threads, p->lvl_threads + std::max(0, std::min(p->n_lvl_threads, 16)));
    // as from the environment: a thread request for a stage drops its
    // efficiency threshold to 0 (level_recursion.cpp:86-90)
    for (size_t lvl = 1; lvl < q.lvlThreads.size() + 1 && lvl < q.effVec.size(); ++lvl) q.effVec[lvl] = 0;
    q.cacheViolationCutoffDefault = p->cache_violation_cutoff > 0 ? p->cache_violation_cutoff : 50;
    q.cacheViolationCutoff.assign(1, q.cacheViolationCutoffDefault);
    q.cacheViolationCutoff.insert(q.cacheViolationCutoff.end(), p->cutoffs,
                                  p->cutoffs + std::max(0, std::min(p->n_cutoffs, 16)));
    q.maxRecStages = p->max_recursion_stages >= 0 ? p->max_recursion_stages : -1;
    return q;
}
}  // namespace

extern "C" {

int race_params_from_env(race_params *p) {
    if (!p) return RACE_ERR_INVALID_ARG;
    race::Params q = race::Params::fromEnv();
    memset(p, 0, sizeof(*p));
    p->n_eff = (int)std::min<size_t>(q.effVec.size(), 16);
    for (int i = 0; i < p->n_eff; ++i) p->eff[i] = q.effVec[i];
    p->n_lvl_threads = (int)std::min<size_t>(q.lvlThreads.size(), 16);
    for (int i = 0; i < p->n_lvl_threads; ++i) p->lvl_threads[i] = q.lvlThreads[i];
    p->cache_violation_cutoff = q.cacheViolationCutoffDefault;
    p->max_recursion_stages = q.maxRecStages;
    p->n_cutoffs = (int)std::min<size_t>(q.cacheViolationCutoff.size() - 1, 16);
    for (int i = 0; i < p->n_cutoffs; ++i) p->cutoffs[i] = q.cacheViolationCutoff[i + 1];
    return RACE_SUCCESS;
}

int race_create(race_engine **out, int nrow, int nthreads, int dist, const int *rowPtr, const int *col, int symm_hint,
                const int *initPerm, const int *initInvPerm, int d2type, int lbtarget, const race_params *params) {
    if (!out) return RACE_ERR_INVALID_ARG;
    *out = nullptr;
    race_engine *h = new race_engine;
    int rc = guard(h, [&] {
        h->eng = std::make_unique<Engine>(nrow, nthreads, dist, rowPtr, col, symm_hint != 0, initPerm, initInvPerm,
                                          d2type, lbtarget, toParams(params));
    });
    if (rc != RACE_SUCCESS) {
        fprintf(stderr, "[RACE-GB300] race_create: %s\n", h->err.c_str());
        delete h;
        return rc;
    }
    *out = h;
    return RACE_SUCCESS;
}

int race_destroy(race_engine *e) {
    delete e;
    return RACE_SUCCESS;
}

int race_set_stream(race_engine *e, void *s) {
    if (!e) return RACE_ERR_INVALID_ARG;
    e->eng->stream = (cudaStream_t)s;
    return RACE_SUCCESS;
}

int race_color(race_engine *e) {
    if (!e) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] { e->eng->color(); });
}

int race_power_prepare(race_engine *e, int hp, double cacheSize, double safety, const char *mtxType, int subPow) {
    if (!e) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] { e->eng->powerPrepare(hp, cacheSize, safety, mtxType ? mtxType : "N", subPow); });
}

int race_get_perm(race_engine *e, int *perm, int *invPerm) {
    if (!e) return RACE_ERR_INVALID_ARG;
    if (perm) memcpy(perm, e->eng->hPerm.data(), sizeof(int) * e->eng->n);
    if (invPerm) memcpy(invPerm, e->eng->hInvPerm.data(), sizeof(int) * e->eng->n);
    return RACE_SUCCESS;
}

int race_get_num_threads(race_engine *e, int *out) {
    if (!e || !out) return RACE_ERR_INVALID_ARG;
    *out = e->eng->availableThreads;
    return RACE_SUCCESS;
}

int race_get_efficiency(race_engine *e, double *out) {
    if (!e || !out) return RACE_ERR_INVALID_ARG;
    Engine &g = *e->eng;
    if (g.dist == race::DIST_POWER || !g.tree) return RACE_ERR_INVALID_ARG;
    // interface.cpp:316-319
    double effThreads = ((double)g.n / (double)g.tree->nodes[0].effRowZ);
    *out = effThreads / g.requested;
    return RACE_SUCCESS;
}

int race_get_max_stage_depth(race_engine *e, int *out) {
    if (!e || !out || !e->eng->tree) return RACE_ERR_INVALID_ARG;
    *out = e->eng->tree->maxStage;
    return RACE_SUCCESS;
}

int race_get_zone_tree(race_engine *e, int *buf, int cap, int *len) {
    if (!e || !len || !e->eng->tree) return RACE_ERR_INVALID_ARG;
    std::vector<int> v = race::serializeZoneTree(*e->eng->tree);
    *len = (int)v.size();
    if (buf && cap >= (int)v.size()) memcpy(buf, v.data(), sizeof(int) * v.size());
    return RACE_SUCCESS;
}

int race_get_phases(race_engine *e, int rev, int *phasePtr, int *leafLo, int *leafHi, int cap, int *numPhases,
                    int *numLeaves) {
    if (!e || !numPhases || !numLeaves || !e->eng->colored) return RACE_ERR_INVALID_ARG;
    const race::PhaseTable &pt = e->eng->phases[rev ? 1 : 0];
    *numPhases = pt.numPhases();
    *numLeaves = (int)pt.leafLo.size();
    if (phasePtr && leafLo && leafHi && cap >= *numLeaves && cap >= *numPhases + 1) {
        memcpy(phasePtr, pt.phasePtr.data(), sizeof(int) * pt.phasePtr.size());
        memcpy(leafLo, pt.leafLo.data(), sizeof(int) * pt.leafLo.size());
        memcpy(leafHi, pt.leafHi.data(), sizeof(int) * pt.leafHi.size());
    }
    return RACE_SUCCESS;
}

int race_get_device_phases(race_engine *e, int rev, const int **leafLo, const int **leafHi, int *numLeaves) {
    if (!e || !leafLo || !leafHi || !numLeaves || !e->eng->colored) return RACE_ERR_INVALID_ARG;
    const race::DevPhases &d = e->eng->dPhases[rev ? 1 : 0];
    *leafLo = d.leafLo.p;
    *leafHi = d.leafHi.p;
    *numLeaves = d.numLeaves;
    return RACE_SUCCESS;
}

int race_get_power_tree(race_engine *e, int *buf, int cap, int *len) {
    if (!e || !len || !e->eng->powerReady) return RACE_ERR_INVALID_ARG;
    std::vector<int> flat{(int)e->eng->powerTree.size()};
    for (const race::MpkLeaf &l : e->eng->powerTree) {
        flat.insert(flat.end(), {l.lo, l.hi, l.stage, l.parent, (int)l.groupPtr.size() - 1});
        flat.insert(flat.end(), l.groupPtr.begin(), l.groupPtr.end());
        flat.push_back((int)l.hopeless.size());
        flat.insert(flat.end(), l.hopeless.begin(), l.hopeless.end());
    }
    *len = (int)flat.size();
    if (buf && cap >= *len) memcpy(buf, flat.data(), sizeof(int) * flat.size());
    return RACE_SUCCESS;
}

int race_get_power_groups(race_engine *e, int *buf, int cap, int *len) {
    if (!e || !len || !e->eng->powerReady) return RACE_ERR_INVALID_ARG;
    const std::vector<int> &g = e->eng->groupPtr;
    *len = (int)g.size();
    if (buf && cap >= (int)g.size()) memcpy(buf, g.data(), sizeof(int) * g.size());
    return RACE_SUCCESS;
}

int race_register_function(race_engine *e, int kernel, const race_operands *ops, int power, int *func_id) {
    if (!e || !ops || !func_id) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] { *func_id = e->eng->registerFunction(kernel, *ops, power); });
}

int race_execute_function(race_engine *e, int func_id, int rev) {
    if (!e) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] { e->eng->execute(func_id, rev != 0); });
}

int race_execute_function_async(race_engine *e, int func_id, int rev) {
    if (!e) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] { e->eng->launch(func_id, rev != 0); });
}

int race_get_status(race_engine *e) {
    if (!e) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] { e->eng->checkStatus(); });
}

int race_set_sweep_mode(race_engine *e, int mode) {
    if (!e || mode < RACE_SWEEP_AUTO || mode > RACE_SWEEP_GATHER) return RACE_ERR_INVALID_ARG;
    e->eng->sweepMode = mode;
    return RACE_SUCCESS;
}

int race_get_sweep_info(race_engine *e, int func_id, int rev, int *numWaves, int *maxWaveRows, int *numPhases,
                        int *maxLeafRows, int *waveModeChosen) {
    if (!e || func_id < 0 || func_id >= (int)e->eng->funcs.size() || !numWaves || !maxWaveRows || !numPhases ||
        !maxLeafRows || !waveModeChosen)
        return RACE_ERR_INVALID_ARG;
    const race::FuncEntry &f = e->eng->funcs[func_id];
    if (f.kernel == RACE_K_MPK) return RACE_ERR_INVALID_ARG;
    const int dir = rev ? 1 : 0;
    *numWaves = f.waves[dir].numWaves;
    *maxWaveRows = f.waves[dir].maxRows;
    *numPhases = e->eng->dPhases[dir].numPhases;
    *maxLeafRows = e->eng->dPhases[dir].maxLeafRows;
    *waveModeChosen = race::usesGather(*e->eng, f) ? 2 : race::useWaveMode(*e->eng, f, dir) ? 1 : 0;
    return RACE_SUCCESS;
}

int race_get_mpk_layout(race_engine *e, int func_id, int *numChunks, int *colBits, int *wideChunks,
                        long long *sellSlots, long long *matrixBytes, int *schedule) {
    if (!e || func_id < 0 || func_id >= (int)e->eng->funcs.size() || !numChunks || !colBits || !wideChunks ||
        !sellSlots || !matrixBytes || !schedule)
        return RACE_ERR_INVALID_ARG;
    const race::FuncEntry &f = e->eng->funcs[func_id];
    if (f.kernel != RACE_K_MPK || !f.mpk) return RACE_ERR_INVALID_ARG;
    const race::MpkPlan &p = *f.mpk;
    *numChunks = p.numChunks;
    *colBits = p.col16 ? 16 : 32;
    *wideChunks = p.wideChunks;
    *sellSlots = p.sellSlots;
    const long long vb = p.valType == RACE_VAL_F64 ? 8 : p.valType == RACE_VAL_F32 ? 4 : 2;
    *matrixBytes = p.sellSlots * vb + (p.col16 ? 2 * p.sellSlots + 4 * p.wideSlots + 16LL * p.numChunks
                                                : 4 * p.sellSlots) +
                   4LL * (long long)p.rowLen.n + 12LL * p.numChunks + 4LL * (long long)p.hubRow.n +
                   (vb + 4) * (long long)p.hubCol.n;
    *schedule = p.schedule != RACE_MPK_AUTO ? p.schedule : p.chosen;
    return RACE_SUCCESS;
}

int race_set_mpk_schedule(race_engine *e, int func_id, int schedule) {
    if (!e || func_id < 0 || func_id >= (int)e->eng->funcs.size() || schedule < RACE_MPK_AUTO ||
        schedule > RACE_MPK_SWEEPS)
        return RACE_ERR_INVALID_ARG;
    race::FuncEntry &f = e->eng->funcs[func_id];
    if (f.kernel != RACE_K_MPK || !f.mpk) return RACE_ERR_INVALID_ARG;
    f.mpk->schedule = schedule;
    f.mpk->chosen = 0;
    return RACE_SUCCESS;
}

int race_set_power(race_engine *e, int func_id, int power) {
    if (!e || func_id < 0 || func_id >= (int)e->eng->funcs.size()) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] {
        race::FuncEntry &f = e->eng->funcs[func_id];
        if (f.block && power != f.power) {
            if (power < 1 || power > 255) throw Error(RACE_ERR_INVALID_ARG, "power must be in 1..255");
            f.block = race::buildBlockPlan(*e->eng, f.ops, power, f.block->nrhs);
        } else if (f.kernel == RACE_K_MPK && power != f.power) {
            if (power < 1 || power > 255) throw Error(RACE_ERR_INVALID_ARG, "power must be in 1..255");
            f.mpk = race::buildMpkPlan(*e->eng, f.ops, power);
        }
        f.power = power;
    });
}

int race_get_power(race_engine *e, int func_id, int *out) {
    if (!e || !out || func_id < 0 || func_id >= (int)e->eng->funcs.size()) return RACE_ERR_INVALID_ARG;
    *out = e->eng->funcs[func_id].power;
    return RACE_SUCCESS;
}

int race_set_sub_power(race_engine *e, int func_id, int subPower) {
    if (!e || func_id < 0 || func_id >= (int)e->eng->funcs.size() || subPower < 1) return RACE_ERR_INVALID_ARG;
    return subPower == 1 ? RACE_SUCCESS : RACE_ERR_INCOMPATIBILITY;
}

int race_get_sub_power(race_engine *e, int func_id, int *out) {
    if (!e || !out || func_id < 0 || func_id >= (int)e->eng->funcs.size()) return RACE_ERR_INVALID_ARG;
    *out = 1;
    return RACE_SUCCESS;
}

int race_symmgs_ir(race_engine *e, int inner_func_id, int n, const int *rowPtr, const int *col, const double *val,
                   const double *b, double *x, double tol, int maxIter, int sweeps, int *iters, double *relres) {
    if (!e || !rowPtr || !col || !val || !b || !x || !iters || !relres || sweeps < 1 || maxIter < 0)
        return RACE_ERR_INVALID_ARG;
    return guard(e, [&] {
        race::symmGsIr(*e->eng, inner_func_id, n, rowPtr, col, val, b, x, tol, maxIter, sweeps, iters, relres);
    });
}

int race_spmv_power_layout(race_engine *e, int func_id, int k) {
    if (!e || func_id < 0 || func_id >= (int)e->eng->funcs.size()) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] {
        race::FuncEntry &f = e->eng->funcs[func_id];
        if (f.kernel != RACE_K_MPK || (!f.mpk && !f.block))
            throw Error(RACE_ERR_INVALID_ARG, "not a matrix-power function");
        if (k < 0 || k >= f.power) throw Error(RACE_ERR_INVALID_ARG, "k out of range");
        if (f.block)
            race::runBlockSpmv(*f.block, k, e->eng->stream);
        else
            race::runSpmvSell(*e->eng, *f.mpk, (double *)f.ops.x, f.ops.n, k);
    });
}

int race_spmv_plain(race_engine *e, int n, const int *rowPtr, const int *col, const double *val, const double *x,
                    double *b) {
    if (!e || !rowPtr || !col || !val || !x || !b || n < 0) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] { e->eng->spmvPlain(n, rowPtr, col, val, x, b); });
}

int race_lb_balance(const int *levelRow, const int *levelNnz, int totalLevel, int nthreads, double eff, int dist,
                    int d2type, int lbtarget, int base, int *out, int cap, int *len) {
    if (!levelRow || !levelNnz || totalLevel < 0 || !len) return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        race::LevelData ld;
        ld.totalLevel = totalLevel;
        ld.levelRow.assign(levelRow, levelRow + totalLevel);
        ld.levelNnz.assign(levelNnz, levelNnz + totalLevel);
        for (int i = 0; i < totalLevel; ++i) {
            ld.nrow += levelRow[i];
            ld.nnz += levelNnz[i];
        }
        race::LBResult r = race::lbBalance(ld, nthreads, eff, dist, d2type, lbtarget, base);
        std::vector<int> v;
        v.push_back((int)r.scale.size());
        v.insert(v.end(), r.scale.begin(), r.scale.end());
        v.push_back((int)r.numBlocks.size());
        v.insert(v.end(), r.zonePtr.begin(), r.zonePtr.end());
        v.push_back((int)r.subZonePtr.size() - 1);
        v.insert(v.end(), r.subZonePtr.begin(), r.subZonePtr.end());
        v.insert(v.end(), r.numBlocks.begin(), r.numBlocks.end());
        *len = (int)v.size();
        if (out && cap >= (int)v.size()) memcpy(out, v.data(), sizeof(int) * v.size());
    });
}

int race_flatten_zone_tree(const int *tree, int treeLen, int dist, int d2type, int rev, int serialLo, int serialHi,
                           int *phasePtr, int *leafLo, int *leafHi, int cap, int *numPhases, int *numLeaves) {
    if (!tree || treeLen < 1 || !numPhases || !numLeaves) return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        race::ZoneTree t(dist, d2type, race::LB_NNZ);
        int k = 1;
        auto take = [&]() {
            if (k >= treeLen) throw Error(RACE_ERR_INVALID_ARG, "truncated zone tree");
            return tree[k++];
        };
        for (int i = 0, nn = tree[0]; i < nn; ++i) {
            race::ZoneNode z;
            z.nthreadsZ = take();
            z.idealNthreadsZ = take();
            z.totalSubBlocks = take();
            z.parentZ = take();
            z.effRowZ = take();
            z.stage = take();
            z.reachedLimit = take() != 0;
            z.valueZ.resize(take());
            for (auto &v : z.valueZ) v = take();
            z.children.resize(take());
            for (auto &c : z.children) c = take();
            t.nodes.push_back(z);
        }
        race::PhaseTable pt = race::flattenZoneTree(t, rev != 0, serialLo, serialHi);
        *numPhases = pt.numPhases();
        *numLeaves = (int)pt.leafLo.size();
        if (phasePtr && leafLo && leafHi && cap >= *numLeaves && cap >= *numPhases + 1) {
            memcpy(phasePtr, pt.phasePtr.data(), sizeof(int) * pt.phasePtr.size());
            memcpy(leafLo, pt.leafLo.data(), sizeof(int) * pt.leafLo.size());
            memcpy(leafHi, pt.leafHi.data(), sizeof(int) * pt.leafHi.size());
        }
    });
}

int race_mpk_stage_partition(const int *levelRow, const int *levelNnz, int totalLevel, int graphRows,
                             long long graphNnz, int power, double cacheSize, double safety, int cutoff, int *groupPtr,
                             int *hopeless, int cap, int *numGroups, int *numHopeless) {
    if (totalLevel < 0 || (totalLevel > 0 && (!levelRow || !levelNnz)) || graphRows < 1 || graphNnz < 1 ||
        power < 1 || !(cacheSize > 0) || !numGroups || !numHopeless)
        return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        race::LevelData ld;
        ld.totalLevel = totalLevel;
        ld.levelRow.assign(levelRow, levelRow + totalLevel);
        ld.levelNnz.assign(levelNnz, levelNnz + totalLevel);
        const race::StagePartition sp =
            race::stagePartition(ld, 0, power, graphRows, graphNnz, cacheSize, safety, cutoff);
        *numGroups = (int)sp.groupPtr.size() - 1;
        *numHopeless = (int)sp.hopeless.size();
        if (groupPtr && hopeless && cap >= (int)sp.groupPtr.size() && cap >= (int)sp.hopeless.size()) {
            memcpy(groupPtr, sp.groupPtr.data(), sizeof(int) * sp.groupPtr.size());
            if (!sp.hopeless.empty()) memcpy(hopeless, sp.hopeless.data(), sizeof(int) * sp.hopeless.size());
        }
    });
}

int race_mpk_recursion_permute(int n, const int *rowPtr, const int *col, int *totalPerm, int *totalInvPerm,
                               const int *groupPtr, int numGroups, const int *hopeless, int numHopeless, int power) {
    if (n < 0 || !rowPtr || !col || !totalPerm || !totalInvPerm || !groupPtr || numGroups < 0 || numHopeless < 0 ||
        (numHopeless > 0 && !hopeless) || power < 1 || groupPtr[0] < 0 || groupPtr[numGroups] > n)
        return RACE_ERR_INVALID_ARG;
    for (int g = 0; g < numGroups; ++g)
        if (groupPtr[g + 1] < groupPtr[g]) return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        std::vector<int> tp(totalPerm, totalPerm + n), ti(totalInvPerm, totalInvPerm + n);
        std::vector<int> gp(groupPtr, groupPtr + numGroups + 1), hid(hopeless, hopeless + numHopeless);
        if (!race::recursePermutation(n, rowPtr, col, tp, ti, gp, hid, power))
            throw Error(RACE_ERR_GRAPH_TRAVERSAL, "rows of a hopeless group went missing in its traversal");
        memcpy(totalPerm, tp.data(), sizeof(int) * n);
        memcpy(totalInvPerm, ti.data(), sizeof(int) * n);
    });
}

int race_mpk_recursive_partition(int n, const int *rowPtr, const int *col, int *totalPerm, int *totalInvPerm,
                                 const int *groupPtr, int numGroups, const int *hopeless, int numHopeless, int power,
                                 long long graphNnz, double cacheSize, double safety, const int *stageCutoff,
                                 int numStages, int *treeBuf, int cap, int *treeLen) {
    if (n < 1 || !rowPtr || !col || !totalPerm || !totalInvPerm || !groupPtr || numGroups < 1 || numHopeless < 0 ||
        (numHopeless > 0 && !hopeless) || power < 1 || graphNnz < 1 || !(cacheSize > 0) || numStages < 0 ||
        (numStages > 0 && !stageCutoff) || !treeLen || groupPtr[0] != 0 || groupPtr[numGroups] != n)
        return RACE_ERR_INVALID_ARG;
    for (int g = 0; g < numGroups; ++g)
        if (groupPtr[g + 1] < groupPtr[g]) return RACE_ERR_INVALID_ARG;
    for (int h = 0; h < numHopeless; ++h)
        if (hopeless[h] < 0 || hopeless[h] >= numGroups) return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        std::vector<int> tp(totalPerm, totalPerm + n), ti(totalInvPerm, totalInvPerm + n);
        race::StagePartition root;
        root.groupPtr.assign(groupPtr, groupPtr + numGroups + 1);
        root.hopeless.assign(hopeless, hopeless + numHopeless);
        std::vector<int> cut(stageCutoff, stageCutoff + numStages);
        std::vector<race::MpkLeaf> tree;
        if (!race::recursivePartition(n, rowPtr, col, tp, ti, root, power, graphNnz, cacheSize, safety, cut, tree))
            throw Error(RACE_ERR_GRAPH_TRAVERSAL,
                        "MPK recursion: rows of a hopeless group went missing, or its boundary groups do not exist");
        std::vector<int> buf{(int)tree.size()};
        for (const race::MpkLeaf &l : tree) {
            buf.insert(buf.end(), {l.lo, l.hi, l.stage, l.parent, (int)l.groupPtr.size() - 1});
            buf.insert(buf.end(), l.groupPtr.begin(), l.groupPtr.end());
            buf.push_back((int)l.hopeless.size());
            buf.insert(buf.end(), l.hopeless.begin(), l.hopeless.end());
        }
        *treeLen = (int)buf.size();
        if (treeBuf && cap >= *treeLen) memcpy(treeBuf, buf.data(), sizeof(int) * buf.size());
        memcpy(totalPerm, tp.data(), sizeof(int) * n);
        memcpy(totalInvPerm, ti.data(), sizeof(int) * n);
    });
}

int race_traverse_host(int n, const int *rowPtr, const int *col, int *totalPerm, int *totalInvPerm, int lo, int hi,
                       int dist, int *levelRow, int *levelNnz, int cap, int *totalLevel) {
    if (n < 1 || !rowPtr || !col || !totalPerm || !totalInvPerm || lo < 0 || hi > n || lo > hi ||
        (dist != race::DIST_ONE && dist != race::DIST_TWO) || !totalLevel || (cap > 0 && (!levelRow || !levelNnz)))
        return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        std::vector<int> tp(totalPerm, totalPerm + n), ti(totalInvPerm, totalInvPerm + n);
        race::HostTraverseScratch sc;
        race::LevelData ld;
        if (!race::traverseRangeHost(n, rowPtr, col, tp, ti, lo, hi, dist, sc, ld))
            throw Error(RACE_ERR_GRAPH_TRAVERSAL, "some rows went missing in BFS");
        *totalLevel = ld.totalLevel;
        if (cap < ld.totalLevel) return;
        std::copy(ld.levelRow.begin(), ld.levelRow.end(), levelRow);
        std::copy(ld.levelNnz.begin(), ld.levelNnz.end(), levelNnz);
        memcpy(totalPerm, tp.data(), sizeof(int) * n);
        memcpy(totalInvPerm, ti.data(), sizeof(int) * n);
    });
}

int race_zone_tree_host(int nrow, int nthreads, int dist, int d2type, int lbTarget, const race_params *params,
                        race_traverse_fn trav, race_range_nnz_fn rangeNnz, void *user, int *treeBuf, int cap,
                        int *treeLen, int *availableThreads) {
    if (nrow < 0 || nthreads < 1 || (dist != race::DIST_ONE && dist != race::DIST_TWO) || !trav || !rangeNnz ||
        !treeLen || !availableThreads)
        return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        auto traverse = [&](int lo, int hi) {
            race::LevelData ld;
            if (hi <= lo) return ld;
            // a distance-2 BFS may pass through rows outside [lo,hi) and an
            // island restart adds an empty level, so allow twice the graph
            const int levelCap = 2 * nrow + 2;
            ld.levelRow.assign(levelCap, 0);
            ld.levelNnz.assign(levelCap, 0);
            int total = 0;
            if (trav(user, lo, hi, ld.levelRow.data(), ld.levelNnz.data(), levelCap, &total) != 0 || total < 0 ||
                total > levelCap)
                throw Error(RACE_ERR_GRAPH_TRAVERSAL, "the caller's traversal failed");
            ld.levelRow.resize(total);
            ld.levelNnz.resize(total);
            ld.totalLevel = total;
            for (int l = 0; l < total; ++l) {
                ld.nrow += ld.levelRow[l];
                ld.nnz += ld.levelNnz[l];
            }
            return ld;
        };
        race::LevelRecursion lr(nrow, nthreads, dist, d2type, lbTarget, toParams(params), traverse,
                                [&](int lo, int hi) { return rangeNnz(user, lo, hi); });
        lr.levelBalancing();
        std::vector<int> v = race::serializeZoneTree(lr.tree);
        *treeLen = (int)v.size();
        *availableThreads = lr.availableThreads;
        if (treeBuf && cap >= (int)v.size()) memcpy(treeBuf, v.data(), sizeof(int) * v.size());
    });
}

int race_gather_plan(int kernel, int n, const int *rowPtr, const int *col, const int *phasePtr, const int *leafLo,
                     const int *leafHi, int numPhases, int *ptr, int *entry, int *row, int cap, int *numUpdates) {
    if (!rowPtr || !col || !phasePtr || !leafLo || !leafHi || n < 0 || numPhases < 0 || !numUpdates ||
        (kernel != RACE_K_SPMTV && kernel != RACE_K_SYMMSPMV) || phasePtr[0] != 0)
        return RACE_ERR_INVALID_ARG;
    for (int p = 0; p < numPhases; ++p)
        if (phasePtr[p + 1] < phasePtr[p]) return RACE_ERR_INVALID_ARG;
    for (int l = 0; l < phasePtr[numPhases]; ++l) {
        const int lo = leafLo[l], hi = leafHi[l];
        if (!(lo <= hi ? (lo >= 0 && hi <= n) : (hi >= -1 && lo < n))) return RACE_ERR_INVALID_ARG;
    }
    return guard(nullptr, [&] {
        race::PhaseTable pt;
        pt.phasePtr.assign(phasePtr, phasePtr + numPhases + 1);
        pt.leafLo.assign(leafLo, leafLo + pt.phasePtr.back());
        pt.leafHi.assign(leafHi, leafHi + pt.phasePtr.back());
        race::GatherPlan gp = race::buildGatherPlan(kernel, n, rowPtr, col, pt);
        *numUpdates = (int)gp.entry.size();
        if (ptr && entry && row && cap >= (int)gp.entry.size() && cap >= n + 1) {
            memcpy(ptr, gp.ptr.data(), sizeof(int) * gp.ptr.size());
            if (!gp.entry.empty()) {
                memcpy(entry, gp.entry.data(), sizeof(int) * gp.entry.size());
                memcpy(row, gp.row.data(), sizeof(int) * gp.row.size());
            }
        }
    });
}

int race_mpk_issue_order(const int *depRange, const int *chunkGroup, const int *chunkDie, int numChunks, int power,
                         int order, int stride, int segLen, int runLen, int lag, int *head, int *dep, int *rank,
                         int *dieStart, int cap, int *numRuns) {
    if (numChunks < 0 || (numChunks > 0 && !depRange) || power < 1 || power > 255 || !numRuns || lag < 0 ||
        (order == 1 && numChunks > 0 && !chunkGroup) || (order != 0 && order != 1) || runLen < 1 ||
        runLen > race::kMpkMaxRunLen)
        return RACE_ERR_INVALID_ARG;
    int numGroups = 0;
    for (int c = 0; c < numChunks; ++c) {
        for (int d = 0; d < 3; ++d) {
            const int lo = depRange[6 * c + 2 * d], hi = depRange[6 * c + 2 * d + 1];
            if (hi >= lo && (lo < 0 || hi >= numChunks)) return RACE_ERR_INVALID_ARG;
        }
        if (order == 1) {
            if (chunkGroup[c] < 0 || (c > 0 && chunkGroup[c] < chunkGroup[c - 1])) return RACE_ERR_INVALID_ARG;
            numGroups = chunkGroup[c] + 1;
        }
        if (chunkDie && chunkDie[c] != 0 && chunkDie[c] != 1) return RACE_ERR_INVALID_ARG;
    }
    return guard(nullptr, [&] {
        const std::vector<int> cg =
            chunkGroup ? std::vector<int>(chunkGroup, chunkGroup + numChunks) : std::vector<int>();
        const std::vector<int> dr = race::widenDepsToBlocks(
            std::vector<int>(depRange, depRange + 6 * (size_t)numChunks), race::mpkFlagBlocks(numChunks, cg));
        const std::vector<int> cd = chunkDie ? std::vector<int>(chunkDie, chunkDie + numChunks) : std::vector<int>();
        const race::MpkOrder o =
            order == 1 ? race::mpkGroupOrder(dr, cg, numGroups, power, stride == 1 ? 1 : 2, segLen)
                       : race::mpkRunOrder(dr, numChunks, power, segLen, runLen, lag, cd);
        *numRuns = o.numRuns();
        if (head && dep && cap >= o.numRuns()) {
            memcpy(head, o.head.data(), sizeof(int) * o.head.size());
            memcpy(dep, o.dep.data(), sizeof(int) * o.dep.size());
            if (rank) memcpy(rank, o.rank.data(), sizeof(int) * o.rank.size());
        }
        if (dieStart) memcpy(dieStart, o.dieStart.data(), sizeof(int) * 3);
    });
}

int race_device_dies(int *numDies, int *smDie, int cap, int *numSms) {
    if (!numDies || !numSms) return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        const race::DieMap &m = race::dieMap();
        *numDies = m.numDies;
        *numSms = (int)m.smDie.size();
        if (smDie && cap >= (int)m.smDie.size()) memcpy(smDie, m.smDie.data(), sizeof(int) * m.smDie.size());
    });
}

int race_wave_plan(int kernel, int n, const int *rowPtr, const int *col, const int *phasePtr, const int *leafLo,
                   const int *leafHi, int numPhases, int *wavePtr, int *rows, int cap, int *numWaves, int *numRows) {
    if (!rowPtr || !col || !phasePtr || !leafLo || !leafHi || n < 0 || numPhases < 0 || !numWaves || !numRows)
        return RACE_ERR_INVALID_ARG;
    if (kernel < RACE_K_SPMV || kernel > RACE_K_KACZ || phasePtr[0] != 0) return RACE_ERR_INVALID_ARG;
    for (int p = 0; p < numPhases; ++p)
        if (phasePtr[p + 1] < phasePtr[p]) return RACE_ERR_INVALID_ARG;
    for (int l = 0; l < phasePtr[numPhases]; ++l) {
        // forward leaf [lo, hi) or backward leaf (hi, lo], inside 0..n-1
        const int lo = leafLo[l], hi = leafHi[l];
        const bool ok = lo <= hi ? (lo >= 0 && hi <= n) : (hi >= -1 && lo < n);
        if (!ok) return RACE_ERR_INVALID_ARG;
    }
    return guard(nullptr, [&] {
        race::PhaseTable pt;
        pt.phasePtr.assign(phasePtr, phasePtr + numPhases + 1);
        pt.leafLo.assign(leafLo, leafLo + pt.phasePtr.back());
        pt.leafHi.assign(leafHi, leafHi + pt.phasePtr.back());
        race::WavePlan wp = race::buildWavePlan(kernel, n, rowPtr, col, pt);
        *numWaves = wp.numWaves();
        *numRows = (int)wp.rows.size();
        if (wavePtr && rows && cap >= (int)wp.rows.size() && cap >= wp.numWaves() + 1) {
            memcpy(wavePtr, wp.wavePtr.data(), sizeof(int) * wp.wavePtr.size());
            memcpy(rows, wp.rows.data(), sizeof(int) * wp.rows.size());
        }
    });
}

namespace {
race::SellArrays sellArrays(int simdWidth, int C, int nrows, int *col, const int *chunkStart, const int *rl,
                            const int *clp, void *val, int valType) {
    if (valType < RACE_VAL_F64 || valType > RACE_VAL_BF16) throw Error(RACE_ERR_INVALID_ARG, "simdify: bad val_type");
    race::SellArrays m;
    m.simdWidth = simdWidth;
    m.C = C;
    m.nrows = nrows;
    m.col = col;
    m.chunkStart = chunkStart;
    m.rl = rl;
    m.clp = clp;
    m.val = static_cast<unsigned char *>(val);
    m.valBytes = valType == RACE_VAL_F64 ? 8 : valType == RACE_VAL_F32 ? 4 : 2;
    return m;
}

void throwSimdify(int st, const std::string &msg) {
    if (st == race::SIMDIFY_BAD_ARG) throw Error(RACE_ERR_INVALID_ARG, msg);
    if (st == race::SIMDIFY_UNPLACEABLE) throw Error(RACE_ERR_INCOMPATIBILITY, msg);
}
}  // namespace

int race_get_highest_power(race_engine *e, int *power) {
    if (!e || !power) return RACE_ERR_INVALID_ARG;
    *power = e->eng->highestPower;
    return RACE_SUCCESS;
}

int race_simdify(race_engine *e, int simdWidth, int C, int nrows, int *col, const int *chunkStart, const int *rl,
                 const int *clp, void *val, int val_type, int diagFirst, int *collisions) {
    if (!e) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] {
        race::Engine &E = *e->eng;
        if (!E.colored) throw Error(RACE_ERR_INVALID_ARG, "simdify needs a colored engine (race_color)");
        if (nrows != E.n) throw Error(RACE_ERR_INVALID_ARG, "simdify: nrows must be the engine's row count");
        race::SellArrays m = sellArrays(simdWidth, C, nrows, col, chunkStart, rl, clp, val, val_type);
        std::string msg;
        int coll = 0;
        const int st = race::simdifyD2(m, E.phases[0].leafLo, E.phases[0].leafHi, diagFirst != 0, &coll, msg);
        if (collisions) *collisions = coll;
        throwSimdify(st, msg);
    });
}

int race_simdify_schedule(int simdWidth, int C, int nrows, int *col, const int *chunkStart, const int *rl,
                          const int *clp, void *val, int val_type, int diagFirst, const int *leafLo,
                          const int *leafHi, int numLeaves, int *collisions) {
    if (numLeaves < 0 || (numLeaves > 0 && (!leafLo || !leafHi))) return RACE_ERR_INVALID_ARG;
    return guard(nullptr, [&] {
        race::SellArrays m = sellArrays(simdWidth, C, nrows, col, chunkStart, rl, clp, val, val_type);
        std::vector<int> lo(leafLo, leafLo + numLeaves), hi(leafHi, leafHi + numLeaves);
        std::string msg;
        int coll = 0;
        const int st = race::simdifyD2(m, lo, hi, diagFirst != 0, &coll, msg);
        if (collisions) *collisions = coll;
        throwSimdify(st, msg);
    });
}

int race_simdify_d1(int simdWidth, int C, int nrows, int *col, const int *chunkStart, const int *rl, const int *clp,
                    void *val, int val_type, int dist2Compatible) {
    (void)rl;
    return guard(nullptr, [&] {
        race::SellArrays m = sellArrays(simdWidth, C, nrows, col, chunkStart, rl, clp, val, val_type);
        std::string msg;
        throwSimdify(race::simdifyD1(m, dist2Compatible != 0, msg), msg);
    });
}

const char *race_last_error(race_engine *e) { return e ? e->err.c_str() : "null engine"; }

int race_register_mpk_block(race_engine *e, const race_operands *ops, int power, int nrhs, int *func_id) {
    if (!e || !ops || !func_id) return RACE_ERR_INVALID_ARG;
    return guard(e, [&] { *func_id = e->eng->registerMpkBlock(*ops, power, nrhs); });
}

}  // extern "C"

// A batch: block-MPK functions of several engines run by one persistent
// launch; the launch sequence is captured once in a CUDA graph on request.
struct race_batch {
    std::vector<std::pair<race_engine *, int>> members;
    race::BatchTables tables;
    bool prepared = false;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::string err;
    void dropGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
    ~race_batch() {
        dropGraph();
        if (capture) cudaStreamDestroy(capture);
    }
    void prepare(cudaStream_t s) {
        std::vector<const race::BlockPlan *> plans;
        for (auto &m : members) {
            const auto &funcs = m.first->eng->funcs;
            if (m.second < 0 || m.second >= (int)funcs.size() || !funcs[m.second].block)
                throw Error(RACE_ERR_INVALID_ARG, "batch member is not a block-MPK function");
            plans.push_back(funcs[m.second].block.get());
        }
        dropGraph();
        race::buildBatchTables(tables, plans, s);
        prepared = true;
    }
};

namespace {
template <typename F>
int guardBatch(race_batch *b, F &&f) {
    try {
        f();
        return RACE_SUCCESS;
    } catch (const Error &ex) {
        b->err = ex.what();
        return ex.code;
    } catch (const std::exception &ex) {
        b->err = ex.what();
        return RACE_ERR_INTERNAL;
    }
}
}  // namespace

extern "C" {

int race_batch_create(race_batch **out) {
    if (!out) return RACE_ERR_INVALID_ARG;
    *out = new race_batch;
    return RACE_SUCCESS;
}

int race_batch_destroy(race_batch *b) {
    delete b;
    return RACE_SUCCESS;
}

int race_batch_add(race_batch *b, race_engine *e, int func_id) {
    if (!b || !e) return RACE_ERR_INVALID_ARG;
    return guardBatch(b, [&] {
        const auto &funcs = e->eng->funcs;
        if (func_id < 0 || func_id >= (int)funcs.size() || !funcs[func_id].block)
            throw Error(RACE_ERR_INVALID_ARG, "not a block-MPK function (race_register_mpk_block)");
        b->members.emplace_back(e, func_id);
        b->prepared = false;
        b->dropGraph();
    });
}

int race_batch_prepare(race_batch *b, void *stream) {
    if (!b) return RACE_ERR_INVALID_ARG;
    return guardBatch(b, [&] { b->prepare((cudaStream_t)stream); });
}

int race_batch_execute(race_batch *b, void *stream) {
    if (!b) return RACE_ERR_INVALID_ARG;
    return guardBatch(b, [&] {
        if (!b->prepared) b->prepare((cudaStream_t)stream);
        race::runBatch(b->tables, (cudaStream_t)stream);
    });
}

int race_batch_graph_launch(race_batch *b, void *stream) {
    if (!b) return RACE_ERR_INVALID_ARG;
    return guardBatch(b, [&] {
        if (!b->prepared) b->prepare((cudaStream_t)stream);
        if (!b->exec) {
            if (!b->capture) RACE_CUDA(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking));
            RACE_CUDA(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeRelaxed));
            try {
                race::runBatch(b->tables, b->capture);
            } catch (...) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(b->capture, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            RACE_CUDA(cudaStreamEndCapture(b->capture, &b->graph));
            RACE_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
        }
        RACE_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    });
}

int race_batch_get_status(race_batch *b, void *stream) {
    if (!b) return RACE_ERR_INVALID_ARG;
    return guardBatch(b, [&] {
        if (!b->prepared) return;
        int st = 0;
        RACE_CUDA(cudaMemcpyAsync(&st, b->tables.status.p, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
        RACE_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
        if (st != race::DEV_OK) throw Error(RACE_ERR_TIMEOUT, "a device wait gave up (schedule dependency)");
    });
}

int race_batch_info(race_batch *b, int *members, int *chunks, int *items) {
    if (!b || !members || !chunks || !items) return RACE_ERR_INVALID_ARG;
    *members = (int)b->members.size();
    *chunks = b->prepared ? b->tables.numChunks : 0;
    *items = b->prepared ? b->tables.numItems : 0;
    return RACE_SUCCESS;
}

const char *race_batch_last_error(race_batch *b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"
