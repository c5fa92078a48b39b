/* C-ABI harness around the RACE reference classes, compiled together with the
 * reference sources where they lie (see oracle/build_ref.sh). It exists only
 * to produce golden data (levels, permutations, zone trees, MPK schedules,
 * sweep outputs, simdify outputs) and to pin the C restatement in
 * oracle/race_oracle.c.
 * TEST INFRASTRUCTURE ONLY: nothing in the product links or loads this.
 *
 * Pre-processing follows RACE::Interface exactly, minus CPU pinning:
 *   coloring: Graph ctor (interface.cpp:33-36) then LevelRecursion +
 *             levelBalancing + getPerm/getInvPerm/getZoneTree
 *             (interface.cpp:273-281). The LevelPool/Pin step
 *             (interface.cpp:284-289) only binds OpenMP threads to cores and
 *             does not change the schedule, so it is skipped.
 *   power:    Graph ctor then mtxPowerRecursive + findPartition + getPerm
 *             (interface.cpp:205-257).
 * Execution goes through the reference FuncManager (functionManager.cpp).
 * The kernel bodies handed to FuncManager restate the example kernels
 * (examples/src/helpers/kernels.cpp: SpMV :5-15, SpMTV :107-115, GS :174-186,
 * KACZ :285-302, SymmSpMV :403-417, MPK :749-777) with each multiply-add
 * written as a fused fma(), the same arithmetic as the GPU path.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>
#include <unistd.h>
#include <fcntl.h>

#include "graph.h"
#include "level_recursion.h"
#include "zone_tree.h"
#include "lb.h"
#include "functionManager.h"
#include "matrixPowerRecursive.h"
#include "traverse.h"
#include "interface.h"

namespace {

struct Quiet {
    /* The reference prints progress to stdout unconditionally; route it to
     * /dev/null while a harness call runs when ORACLE_QUIET is set. */
    int saved = -1;
    Quiet() {
        if (getenv("ORACLE_QUIET")) {
            fflush(stdout);
            saved = dup(1);
            int dn = open("/dev/null", O_WRONLY);
            dup2(dn, 1);
            close(dn);
        }
    }
    ~Quiet() {
        if (saved >= 0) {
            fflush(stdout);
            dup2(saved, 1);
            close(saved);
        }
    }
};

struct ColorHandle {
    int n = 0;
    int requested = 0;
    RACE::dist dist = RACE::ONE;
    RACE::Graph *graph = nullptr;
    ZoneTree *tree = nullptr;
    int *perm = nullptr;
    int *invPerm = nullptr;
    int available = 0;
};

struct PowerHandle {
    int n = 0;
    int highestPower = 1;
    RACE::Graph *graph = nullptr;
    mtxPowerRecursive *mp = nullptr;
    int *perm = nullptr;
    int *invPerm = nullptr;
};

struct CsrArgs {
    int n;
    const int *rowPtr;
    const int *col;
    const double *val;
    double *x;
    double *b;
};

/* Kernel bodies (restated; see file header for the reference lines). */
void k_spmv(int start, int end, void *a) {
    CsrArgs *p = (CsrArgs *)a;
    for (int row = start; row < end; ++row) {
        double tmp = 0;
        for (int idx = p->rowPtr[row]; idx < p->rowPtr[row + 1]; ++idx)
            tmp = fma(p->val[idx], p->x[p->col[idx]], tmp);
        p->b[row] = tmp;
    }
}
void k_spmtv(int start, int end, void *a) {
    CsrArgs *p = (CsrArgs *)a;
    for (int row = start; row < end; ++row) {
        double xr = p->x[row];
        for (int idx = p->rowPtr[row]; idx < p->rowPtr[row + 1]; ++idx)
            p->b[p->col[idx]] = fma(p->val[idx], xr, p->b[p->col[idx]]);
    }
}
void k_symmspmv(int start, int end, void *a) {
    CsrArgs *p = (CsrArgs *)a;
    for (int row = start; row < end; ++row) {
        double xr = p->x[row];
        p->b[row] = fma(p->val[p->rowPtr[row]], xr, p->b[row]);
        double temp = 0;
        for (int idx = p->rowPtr[row] + 1; idx < p->rowPtr[row + 1]; ++idx) {
            double m = p->val[idx];
            int c = p->col[idx];
            temp = fma(m, p->x[c], temp);
            p->b[c] = fma(m, xr, p->b[c]);
        }
        p->b[row] += temp;
    }
}
void k_gs(int start, int end, void *a) {
    CsrArgs *p = (CsrArgs *)a;
    int inc = (start > end) ? -1 : 1;
    for (int row = start; row != end; row += inc) {
        int d = p->rowPtr[row];
        double tmp = p->b[row];
        for (int idx = d + 1; idx < p->rowPtr[row + 1]; ++idx)
            tmp = fma(-p->val[idx], p->x[p->col[idx]], tmp);
        p->x[row] = tmp / p->val[d];
    }
}
void k_kacz(int start, int end, void *a) {
    CsrArgs *p = (CsrArgs *)a;
    int inc = (start > end) ? -1 : 1;
    for (int row = start; row != end; row += inc) {
        double rowNorm = 0.0, scale = -p->b[row];
        for (int idx = p->rowPtr[row]; idx < p->rowPtr[row + 1]; ++idx) {
            double m = p->val[idx];
            scale = fma(m, p->x[p->col[idx]], scale);
            rowNorm = fma(m, m, rowNorm);
        }
        scale /= rowNorm;
        for (int idx = p->rowPtr[row]; idx < p->rowPtr[row + 1]; ++idx) {
            int c = p->col[idx];
            p->x[c] = fma(-scale, p->val[idx], p->x[c]);
        }
    }
}

struct PowArgs {
    int n;
    const int *rowPtr;
    const int *col;
    const double *val;
    double *x; /* (p+1)*n, power-major */
    int *coverage; /* optional: per (pow,row) visit counters, p*n */
};

void k_mpk(int start, int end, int pow, int numa, void *a) {
    (void)numa;
    PowArgs *p = (PowArgs *)a;
    if (p->coverage) {
        for (int row = start; row < end; ++row)
            __sync_fetch_and_add(&p->coverage[(size_t)(pow - 1) * p->n + row], 1);
        return;
    }
    const size_t in = (size_t)(pow - 1) * p->n, out = (size_t)pow * p->n;
    for (int row = start; row < end; ++row) {
        double tmp = 0;
        for (int idx = p->rowPtr[row]; idx < p->rowPtr[row + 1]; ++idx)
            tmp = fma(p->val[idx], p->x[in + p->col[idx]], tmp);
        p->x[out + row] = tmp;
    }
}

void k_mpk_wrapped(std::function<void(int, int, int, int, void *)> f, int s, int e, int pw, int sp, int nl, void *a) {
    (void)sp;
    f(s, e, pw, nl, a);
}

void push_vec(std::vector<int> &out, const std::vector<int> &v) {
    out.push_back((int)v.size());
    out.insert(out.end(), v.begin(), v.end());
}

int copy_out(const std::vector<int> &buf, int *out, int cap) {
    if (out && cap >= (int)buf.size()) memcpy(out, buf.data(), buf.size() * sizeof(int));
    return (int)buf.size();
}

} // namespace

extern "C" {

/* ---------------- coloring ---------------- */

/* Coloring of a graph whose running permutation starts at initPerm (the
 * Interface ctor's initPerm/initInvPerm, graph_SoA.cpp:63-79); NULL for the
 * identity. */
void *refc_color_init(int n, int *rowPtr, int *col, int dist, int nthreads, int symm_hint, int d2type, int lbtarget,
                      int *initPerm, int *initInvPerm) {
    Quiet q;
    ColorHandle *h = new ColorHandle;
    h->n = n;
    h->requested = nthreads;
    h->dist = (RACE::dist)dist;
    h->graph = new RACE::Graph(n, n, rowPtr, col, h->dist, symm_hint != 0, initPerm, initInvPerm);
    LevelRecursion lr(h->graph, nthreads, h->dist, (RACE::d2Method)d2type, (RACE::LBTarget)lbtarget);
    lr.levelBalancing();
    h->available = lr.getAvailableThreads();
    int len;
    lr.getPerm(&h->perm, &len);
    lr.getInvPerm(&h->invPerm, &len);
    h->tree = lr.getZoneTree();
    return h;
}

void *refc_color(int n, int *rowPtr, int *col, int dist, int nthreads, int symm_hint, int d2type, int lbtarget) {
    Quiet q;
    ColorHandle *h = new ColorHandle;
    h->n = n;
    h->requested = nthreads;
    h->dist = (RACE::dist)dist;
    h->graph = new RACE::Graph(n, n, rowPtr, col, h->dist, symm_hint != 0, NULL, NULL);
    LevelRecursion lr(h->graph, nthreads, h->dist, (RACE::d2Method)d2type, (RACE::LBTarget)lbtarget);
    lr.levelBalancing();
    h->available = lr.getAvailableThreads();
    int len;
    lr.getPerm(&h->perm, &len);
    lr.getInvPerm(&h->invPerm, &len);
    h->tree = lr.getZoneTree();
    return h;
}

void refc_color_free(void *vh) {
    ColorHandle *h = (ColorHandle *)vh;
    /* getPerm/getInvPerm hand the arrays over (graph_SoA.cpp:616-628). */
    delete[] h->perm;
    delete[] h->invPerm;
    delete h->tree;
    delete h->graph;
    delete h;
}

void refc_color_perm(void *vh, int *perm, int *invPerm) {
    ColorHandle *h = (ColorHandle *)vh;
    memcpy(perm, h->perm, sizeof(int) * h->n);
    memcpy(invPerm, h->invPerm, sizeof(int) * h->n);
}

int refc_color_threads(void *vh) { return ((ColorHandle *)vh)->available; }

double refc_color_efficiency(void *vh) {
    ColorHandle *h = (ColorHandle *)vh;
    double effThreads = ((double)h->n / (double)h->tree->at(0).effRowZ);
    return effThreads / h->requested; /* interface.cpp:316-319 */
}

int refc_color_max_stage(void *vh) { return ((ColorHandle *)vh)->tree->maxStages(); }

void refc_color_serial_part(void *vh, int *out2) {
    ColorHandle *h = (ColorHandle *)vh;
    out2[0] = h->graph->serialPart[0];
    out2[1] = h->graph->serialPart[1];
}

/* Zone tree, flattened: [numNodes] then per node
 * [nthreadsZ, idealNthreadsZ, totalSubBlocks, parentZ, effRowZ, stage,
 *  reachedLimit, nValueZ, valueZ..., nChildren, children...].
 * Returns the length; writes only when cap is large enough. */
int refc_color_tree(void *vh, int *out, int cap) {
    ColorHandle *h = (ColorHandle *)vh;
    std::vector<int> buf;
    int nn = h->tree->size();
    buf.push_back(nn);
    for (int i = 0; i < nn; ++i) {
        ZoneLeaf &z = h->tree->at(i);
        buf.push_back(z.nthreadsZ);
        buf.push_back(z.idealNthreadsZ);
        buf.push_back(z.totalSubBlocks);
        buf.push_back(z.parentZ);
        buf.push_back(z.effRowZ);
        buf.push_back(z.stage);
        buf.push_back(z.reachedLimit ? 1 : 0);
        push_vec(buf, z.valueZ);
        push_vec(buf, z.children);
    }
    return copy_out(buf, out, cap);
}

/* Run one built-in kernel through the reference executor (FuncManager::Run,
 * functionManager.cpp:1453-1501) on a matrix the caller has already permuted.
 * kernel: 0 SpMV, 1 SpMTV, 2 SymmSpMV, 3 GS, 4 KACZ. */
int refc_color_exec(void *vh, int kernel, int rev, int n, const int *rowPtr, const int *col, const double *val,
                    double *x, double *b) {
    ColorHandle *h = (ColorHandle *)vh;
    Quiet q;
    CsrArgs args{n, rowPtr, col, val, x, b};
    void (*f)(int, int, void *) = nullptr;
    switch (kernel) {
    case 0: f = k_spmv; break;
    case 1: f = k_spmtv; break;
    case 2: f = k_symmspmv; break;
    case 3: f = k_gs; break;
    case 4: f = k_kacz; break;
    default: return 1;
    }
    std::function<void(int, int, void *)> fn = f;
    FuncManager fm(fn, &args, h->tree, NULL, h->graph->serialPart);
    fm.Run(rev != 0);
    return 0;
}

/* ---------------- traversal (one BFS over a range) ---------------- */

/* BFS of rows [lo,hi) of a fresh graph, as Traverse::calculateDistance does
 * (traverse_GAP_graphSoA.cpp:236-383). Outputs the composed permutation
 * (graph->totalPerm after the step), and the per-level row/nnz counts.
 * Returns totalLevel, or -1 if levelCap is too small. */
int refc_traverse(int n, int *rowPtr, int *col, int dist, int lo, int hi, int symm_hint, int *perm, int *invPerm,
                  int *levelRow, int *levelNnz, int levelCap) {
    Quiet q;
    RACE::Graph g(n, n, rowPtr, col, (RACE::dist)dist, symm_hint != 0, NULL, NULL);
    int total;
    {
        RACE::Traverse t(&g, (RACE::dist)dist, lo, hi);
        t.calculateDistance();
        LevelData *ld = t.getLevelData();
        total = ld->totalLevel;
        if (total > levelCap) {
            delete ld;
            return -1;
        }
        for (int i = 0; i < total; ++i) {
            levelRow[i] = ld->levelRow[i];
            levelNnz[i] = ld->levelNnz[i];
        }
        delete ld;
    }
    memcpy(perm, g.totalPerm, sizeof(int) * n);
    memcpy(invPerm, g.totalInvPerm, sizeof(int) * n);
    return total;
}

/* ---------------- load balancer ---------------- */

/* LB::balance on given level data (lb.cpp:188-667, 767-771). Outputs:
 * out = [currLvlThreads, scale..., totalBlocks, zonePtr(totalBlocks+1)...,
 *        totalSubBlocks, subZonePtr(totalSubBlocks+1)..., numBlocks(totalBlocks)...]. */
int refc_lb(const int *levelRow, const int *levelNnz, int totalLevel, int nthreads, double eff, int dist, int d2type,
            int lbtarget, int base, int *out, int cap) {
    Quiet q;
    LevelData *ld = new LevelData;
    ld->totalLevel = totalLevel;
    ld->levelRow = new int[totalLevel > 0 ? totalLevel : 1];
    ld->levelNnz = new int[totalLevel > 0 ? totalLevel : 1];
    ld->nrow = 0;
    ld->nnz = 0;
    for (int i = 0; i < totalLevel; ++i) {
        ld->levelRow[i] = levelRow[i];
        ld->levelNnz[i] = levelNnz[i];
        ld->nrow += levelRow[i];
        ld->nnz += levelNnz[i];
    }
    std::vector<int> buf;
    {
        LB lb(nthreads, eff, ld, (RACE::dist)dist, (RACE::d2Method)d2type, (RACE::LBTarget)lbtarget);
        lb.balance();
        int *scale = nullptr, slen = 0;
        lb.getNxtLvlThreads(&scale, &slen);
        buf.push_back(slen);
        for (int i = 0; i < slen; ++i) buf.push_back(scale[i]);
        delete[] scale;
        int *zp = nullptr, zlen = 0, *szp = nullptr, szlen = 0, *nb = nullptr, nblen = 0;
        lb.getZonePtr(&zp, &zlen, base);
        lb.getSubZonePtr(&szp, &szlen, base);
        lb.getNumBlocks(&nb, &nblen);
        buf.push_back(nblen);
        for (int i = 0; i < zlen; ++i) buf.push_back(zp[i]);
        buf.push_back(szlen - 1);
        for (int i = 0; i < szlen; ++i) buf.push_back(szp[i]);
        for (int i = 0; i < nblen; ++i) buf.push_back(nb[i]);
        delete[] zp;
        delete[] szp;
        delete[] nb;
    }
    delete ld;
    return copy_out(buf, out, cap);
}

/* ---------------- matrix power ---------------- */

void *refc_power(int n, int *rowPtr, int *col, int highestPower, double cacheSize, double safety, const char *mtxType,
                 int symm_hint) {
    Quiet q;
    PowerHandle *h = new PowerHandle;
    h->n = n;
    h->highestPower = highestPower;
    h->graph = new RACE::Graph(n, n, rowPtr, col, RACE::POWER, symm_hint != 0, NULL, NULL);
    h->mp = new mtxPowerRecursive(h->graph, highestPower, 1, cacheSize, safety, std::string(mtxType));
    h->mp->findPartition();
    int len;
    h->mp->getPerm(&h->perm, &len);
    h->mp->getInvPerm(&h->invPerm, &len);
    return h;
}

void refc_power_free(void *vh) {
    PowerHandle *h = (PowerHandle *)vh;
    /* getPerm/getInvPerm hand the arrays over (matrixPowerRecursive.cpp:537-549). */
    delete[] h->perm;
    delete[] h->invPerm;
    delete h->mp;
    delete h->graph;
    delete h;
}

void refc_power_perm(void *vh, int *perm, int *invPerm) {
    PowerHandle *h = (PowerHandle *)vh;
    memcpy(perm, h->perm, sizeof(int) * h->n);
    memcpy(invPerm, h->invPerm, sizeof(int) * h->n);
}

/* MPK tree, flattened: [numLeaves] then per leaf
 * [rangeLo, rangeHi, stage, parent, nodeId, lp, hid, unlockRow, dangerRow,
 *  unlockCtr, nodePtr, unitPtr, unitNodePtr, children] (vectors length-prefixed). */
int refc_power_tree(void *vh, int *out, int cap) {
    PowerHandle *h = (PowerHandle *)vh;
    std::vector<int> buf;
    buf.push_back((int)h->mp->tree.size());
    for (auto &L : h->mp->tree) {
        buf.push_back(L.range.lo);
        buf.push_back(L.range.hi);
        buf.push_back(L.stage);
        buf.push_back(L.parent);
        buf.push_back(L.nodeId);
        push_vec(buf, L.lp);
        push_vec(buf, L.hid);
        push_vec(buf, L.unlockRow);
        push_vec(buf, L.dangerRow);
        push_vec(buf, L.unlockCtr);
        push_vec(buf, L.nodePtr);
        push_vec(buf, L.unitPtr);
        push_vec(buf, L.unitNodePtr);
        push_vec(buf, L.children);
    }
    return copy_out(buf, out, cap);
}

/* y_k = A^k x through the reference MPK executor (functionManager.cpp:618-823,
 * 1139-1331). x holds (power+1)*n doubles, power-major; x[0:n] is the input. */
int refc_power_exec(void *vh, int power, int n, const int *rowPtr, const int *col, const double *val, double *x) {
    PowerHandle *h = (PowerHandle *)vh;
    Quiet q;
    PowArgs args{n, rowPtr, col, val, x, nullptr};
    using namespace std::placeholders;
    std::function<void(int, int, int, int, void *)> f4 = k_mpk;
    std::function<void(int, int, int, int, int, void *)> f6 = std::bind(k_mpk_wrapped, f4, _1, _2, _3, _4, _5, _6);
    FuncManager fm(f6, &args, power, 1, h->mp, false);
    fm.Run();
    return 0;
}

/* Per-row visit counts of every power (the checkPowerCoverage invariant,
 * interface.cpp:1060-1095): cover[(k-1)*n + row] = number of times row was
 * computed at power k; a correct schedule gives all ones. */
int refc_power_coverage(void *vh, int power, int *cover) {
    PowerHandle *h = (PowerHandle *)vh;
    Quiet q;
    memset(cover, 0, sizeof(int) * (size_t)power * h->n);
    PowArgs args{h->n, nullptr, nullptr, nullptr, nullptr, cover};
    using namespace std::placeholders;
    std::function<void(int, int, int, int, void *)> f4 = k_mpk;
    std::function<void(int, int, int, int, int, void *)> f6 = std::bind(k_mpk_wrapped, f4, _1, _2, _3, _4, _5, _6);
    FuncManager fm(f6, &args, power, 1, h->mp, false);
    fm.Run();
    return 0;
}

/* ---------------- simdify (interface.cpp:824-842) ---------------- */

/* A RACE::Interface colored by RACEColor() (interface.cpp:260-301; its
 * pinning step binds nothing with the hwloc stand-in), for simdify, whose
 * padding pass runs a callback through the interface's own executor
 * (sell_c_sigmize.cpp:48-62). The CRS arrays are copied and outlive the
 * interface, which borrows them. */
struct IfaceHandle {
    RACE::Interface *ce = nullptr;
    int n = 0;
    std::vector<int> rowPtr, col;
};

void *refc_iface(int n, const int *rowPtr, const int *col, int dist, int nthreads, int symm_hint, int d2type,
                 int lbtarget) {
    Quiet q;
    IfaceHandle *h = new IfaceHandle;
    h->n = n;
    h->rowPtr.assign(rowPtr, rowPtr + n + 1);
    h->col.assign(col, col + rowPtr[n]);
    h->ce = new RACE::Interface(n, nthreads, (RACE::dist)dist, h->rowPtr.data(), h->col.data(), symm_hint != 0, 1,
                                RACE::SCATTER, NULL, NULL, (RACE::d2Method)d2type, (RACE::LBTarget)lbtarget);
    if (h->ce->RACEColor() != RACE_SUCCESS) {
        delete h->ce;
        delete h;
        return nullptr;
    }
    return h;
}

void refc_iface_free(void *vh) {
    IfaceHandle *h = (IfaceHandle *)vh;
    delete h->ce;
    delete h;
}

void refc_iface_perm(void *vh, int *perm, int *invPerm) {
    IfaceHandle *h = (IfaceHandle *)vh;
    int *p = nullptr, *ip = nullptr, len = 0;
    h->ce->getPerm(&p, &len);
    h->ce->getInvPerm(&ip, &len);
    memcpy(perm, p, sizeof(int) * h->n);
    memcpy(invPerm, ip, sizeof(int) * h->n);
    delete[] p;
    delete[] ip;
}

/* Interface::simdify (double values); returns its bool. */
int refc_simdify(void *vh, int simdWidth, int C, int nrows, int *col, int *chunkStart, int *rl, int *clp,
                 double *val, int diagFirst) {
    IfaceHandle *h = (IfaceHandle *)vh;
    Quiet q;
    return h->ce->simdify(simdWidth, C, nrows, col, chunkStart, rl, clp, val, diagFirst != 0) ? 1 : 0;
}

/* Interface::simdifyD1 (double values); returns its bool. */
int refc_simdify_d1(void *vh, int simdWidth, int C, int nrows, int *col, int *chunkStart, int *rl, int *clp,
                    double *val, int dist2Compatible) {
    IfaceHandle *h = (IfaceHandle *)vh;
    Quiet q;
    return h->ce->simdifyD1(simdWidth, C, nrows, col, chunkStart, rl, clp, val, dist2Compatible != 0) ? 1 : 0;
}

} // extern "C"
