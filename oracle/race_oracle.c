/* race_oracle.c -- CPU restatement of RACE's hot path, used as the checker.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load this library. The product (race_gb300)
 * never links, loads or calls it.
 *
 * Contents (each function cites the reference lines it restates):
 *   - BFS level construction over a row range with RACE's distance-1,
 *     distance-2 and matrix-power rules, its island restarts, the per-level
 *     row/nnz histogram and the stable level sort that yields the permutation
 *     (src/traverse_GAP_graphSoA.cpp, include/utility.h).
 *   - The kernel bodies of the example kernels (SpMV, SpMTV, SymmSpMV,
 *     Gauss-Seidel, Kaczmarz, matrix-power SpMV;
 *     examples/src/helpers/kernels.cpp), every multiply-add written as
 *     C99 fma(): the GPU path issues the same fused operations in the same
 *     order, so outputs of sequential row sums match bit for bit.
 *   - A sequential walk of a RACE zone tree in the executor's order
 *     (src/functionManager.cpp:201-265, 1453-1501).
 *   - The matrix-power partition of a single stage (levels grouped to fit a
 *     cache budget, hopeless regions, unlock/danger rows, per-level unlock
 *     counters; src/matrixPower.cpp:88-140, 147-605, 685-940, 958-1044) and the level
 *     wavefront executor that runs it on OpenMP threads
 *     (src/functionManager.cpp:560-823). This is the CPU baseline for the
 *     matrix-power kernel.
 *
 * Parity of this file is pinned against the reference compiled in place
 * (oracle/build_ref.sh) through the golden fixtures in tests/golden/.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_ONE 1
#define ORC_TWO 2
#define ORC_POWER 3

/* ------------------------------------------------------------------------ */
/* BFS levels over [lo,hi)                                                   */
/* ------------------------------------------------------------------------ */

/* Distances of the rows of [lo,hi) (in the current permuted index space)
 * from root `lo`, following Traverse::calculateDistance and TDStep
 * (traverse_GAP_graphSoA.cpp:135-221, 236-330) for mtxType "N" without
 * boundary regions:
 *   - node u of the current space is original row totalPerm[u]; its
 *     neighbours are totalInvPerm[col] (RACE_PERMUTE_ON_FLY, :156-170);
 *   - an in-range unvisited neighbour gets distance = current level;
 *   - distance-2 mode also pushes out-of-range neighbours of an in-range
 *     parent; they carry no distance and expand once (:199-209);
 *   - when the frontier empties before every in-range row is reached, the
 *     lowest unvisited row after the previous island start restarts the BFS,
 *     one empty level apart for coloring and with no gap for power (:282-306).
 * Level-synchronous BFS distances do not depend on the order inside a
 * frontier, so a sequential FIFO reproduces the parallel result.
 * dist_out has n entries (-1 outside the range). Returns totalLevel, or -1
 * if some row could not be reached (the reference exits there). */
int orc_bfs(int n, const int *rowPtr, const int *col, const int *totalPerm, const int *totalInvPerm, int dist,
            int lo, int hi, int *dist_out) {
    int *parent = (int *)malloc(sizeof(int) * (size_t)n);
    int *queue = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    for (int i = 0; i < n; ++i) {
        dist_out[i] = -1;
        parent[i] = -1;
    }
    int qlo = 0, qhi = 0, qin = 0;
    int counter = 0;
    int currLvl = 0;
    if (lo < hi) {
        queue[qin++] = lo;
        dist_out[lo] = 0;
        parent[lo] = 0;
        counter = 1;
    }
    qlo = qhi;
    qhi = qin;
    int prevIslandStop = lo;
    while (qlo != qhi) {
        currLvl += 1;
        for (int q = qlo; q < qhi; ++q) {
            int u = queue[q];
            int pu = totalPerm[u];
            for (int idx = rowPtr[pu]; idx < rowPtr[pu + 1]; ++idx) {
                int child = col[idx];
                if (child >= n) continue; /* remote column guard, :172 */
                child = totalInvPerm[child];
                if (parent[child] != -1) continue;
                if (child >= lo && child < hi) {
                    parent[child] = u;
                    queue[qin++] = child;
                    dist_out[child] = currLvl;
                    counter++;
                } else if (dist == ORC_TWO) {
                    if (u >= lo && u < hi) {
                        parent[child] = u;
                        queue[qin++] = child;
                    }
                }
            }
        }
        qlo = qhi;
        qhi = qin;
        if (qlo == qhi && counter != (hi - lo)) {
            for (int i = prevIslandStop; i < hi; ++i) {
                if (dist_out[i] == -1) {
                    if (dist != ORC_POWER) currLvl += 1;
                    queue[qin++] = i;
                    counter++;
                    qlo = qhi;
                    qhi = qin;
                    dist_out[i] = currLvl;
                    parent[i] = i;
                    prevIslandStop = i;
                    break;
                }
            }
            if (qlo == qhi) {
                free(parent);
                free(queue);
                return -1;
            }
        }
    }
    free(parent);
    free(queue);
    return currLvl;
}

/* BFS of the rows [lo,hi) of a recursion stage of the MPK partition
 * together with its boundary regions [bLo[k], bHi[k]) (Traverse with a
 * boundaryRange and dist POWER, traverse_GAP_graphSoA.cpp:31-90, 135-221,
 * 236-330): from row lo, a child inside [lo,hi) takes the next level and
 * counts toward the range; a child in a boundary region also takes the next
 * level and carries the search on but does not count; other rows are not
 * visited. When the search dies out before the range is covered, the first
 * unvisited row of the range restarts it on the same level (no extra level
 * for POWER). Boundary rows left unvisited get the level after the last one
 * (createLevelData, :452-472). Returns the number of levels (at least 1),
 * or -1 if rows of the range went missing. */
int orc_bfs_boundary(int n, const int *rowPtr, const int *col, const int *totalPerm, const int *totalInvPerm, int lo,
                     int hi, int nb, const int *bLo, const int *bHi, int *dist_out) {
    char *inB = (char *)calloc((size_t)n + 1, 1);
    for (int k = 0; k < nb; ++k)
        for (int i = bLo[k]; i < bHi[k]; ++i) inB[i] = 1;
    int *parent = (int *)malloc(sizeof(int) * (size_t)n);
    int *queue = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    for (int i = 0; i < n; ++i) {
        dist_out[i] = -1;
        parent[i] = -1;
    }
    int qlo = 0, qhi = 0, qin = 0, counter = 0, currLvl = 0;
    if (lo < hi) {
        queue[qin++] = lo;
        dist_out[lo] = 0;
        parent[lo] = 0;
        counter = 1;
    }
    qhi = qin;
    int prevIslandStop = lo;
    while (qlo != qhi) {
        currLvl += 1;
        for (int q = qlo; q < qhi; ++q) {
            int u = queue[q];
            int pu = totalPerm[u];
            for (int idx = rowPtr[pu]; idx < rowPtr[pu + 1]; ++idx) {
                int child = col[idx];
                if (child >= n) continue;
                child = totalInvPerm[child];
                if (parent[child] != -1) continue;
                if (child >= lo && child < hi) {
                    parent[child] = u;
                    queue[qin++] = child;
                    dist_out[child] = currLvl;
                    counter++;
                } else if (inB[child]) {
                    parent[child] = u;
                    queue[qin++] = child;
                    dist_out[child] = currLvl;
                }
            }
        }
        qlo = qhi;
        qhi = qin;
        if (qlo == qhi && counter != (hi - lo)) {
            for (int i = prevIslandStop; i < hi; ++i) {
                if (dist_out[i] == -1) {
                    queue[qin++] = i;
                    counter++;
                    qlo = qhi;
                    qhi = qin;
                    dist_out[i] = currLvl;
                    parent[i] = i;
                    prevIslandStop = i;
                    break;
                }
            }
            if (qlo == qhi) {
                currLvl = -1;
                break;
            }
        }
    }
    if (currLvl >= 0) {
        int untouched = 0;
        for (int k = 0; k < nb; ++k)
            for (int i = bLo[k]; i < bHi[k]; ++i)
                if (dist_out[i] == -1) {
                    dist_out[i] = currLvl;
                    untouched = 1;
                }
        currLvl += untouched;
        if (currLvl < 1) currLvl = 1;
    }
    free(inB);
    free(parent);
    free(queue);
    return currLvl;
}

/* Per-level row and nnz counts over [lo,hi) (findLevelData,
 * traverse_GAP_graphSoA.cpp:385-447). Row lengths are taken from the original
 * row totalPerm[i]. */
void orc_level_data(const int *rowPtr, const int *totalPerm, const int *dist, int lo, int hi, int totalLevel,
                    int *levelRow, int *levelNnz) {
    for (int l = 0; l < totalLevel; ++l) levelRow[l] = levelNnz[l] = 0;
    for (int i = lo; i < hi; ++i) {
        int d = dist[i];
        int pr = totalPerm[i];
        levelRow[d] += 1;
        levelNnz[d] += rowPtr[pr + 1] - rowPtr[pr];
    }
}

/* Stable sort of the rows of [lo,hi) by distance, composed into the running
 * permutation (permuteGraph + sortPerm + updatePerm,
 * traverse_GAP_graphSoA.cpp:506-575; utility.h:50-58, 114-151):
 *   local[i] = i outside the range, rows of the range ordered by level with
 *   ties kept in index order; totalPerm'[i] = totalPerm[local[i]];
 *   totalInvPerm'[totalPerm'[i]] = i.
 * A stable counting sort gives the same order as std::stable_sort. */
void orc_level_permute(int n, const int *dist, int lo, int hi, int totalLevel, int *totalPerm, int *totalInvPerm) {
    int *start = (int *)calloc((size_t)totalLevel + 1, sizeof(int));
    for (int i = lo; i < hi; ++i) start[dist[i] + 1]++;
    for (int l = 0; l < totalLevel; ++l) start[l + 1] += start[l];
    int *local = (int *)malloc(sizeof(int) * (size_t)(hi - lo > 0 ? hi - lo : 1));
    for (int i = lo; i < hi; ++i) local[start[dist[i]]++] = i;
    int *old = (int *)malloc(sizeof(int) * (size_t)(hi - lo > 0 ? hi - lo : 1));
    for (int i = lo; i < hi; ++i) old[i - lo] = totalPerm[i];
    for (int i = lo; i < hi; ++i) totalPerm[i] = old[local[i - lo] - lo];
    for (int i = 0; i < n; ++i) totalInvPerm[totalPerm[i]] = i;
    free(old);
    free(local);
    free(start);
}

/* ------------------------------------------------------------------------ */
/* Kernel bodies (examples/src/helpers/kernels.cpp)                          */
/* ------------------------------------------------------------------------ */

/* SPMV_KERNEL, kernels.cpp:5-25 */
void orc_spmv_range(int start, int end, const int *rowPtr, const int *col, const double *val, const double *x,
                    double *b) {
    for (int row = start; row < end; ++row) {
        double tmp = 0;
        for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx) tmp = fma(val[idx], x[col[idx]], tmp);
        b[row] = tmp;
    }
}

/* SPMTV_KERNEL, kernels.cpp:107-125 */
void orc_spmtv_range(int start, int end, const int *rowPtr, const int *col, const double *val, const double *x,
                     double *b) {
    for (int row = start; row < end; ++row) {
        double xr = x[row];
        for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx) b[col[idx]] = fma(val[idx], xr, b[col[idx]]);
    }
}

/* SYMM_SPMV_KERNEL on the upper triangle with the diagonal first,
 * kernels.cpp:403-428 */
void orc_symmspmv_range(int start, int end, const int *rowPtr, const int *col, const double *val, const double *x,
                        double *b) {
    for (int row = start; row < end; ++row) {
        double xr = x[row];
        b[row] = fma(val[rowPtr[row]], xr, b[row]);
        double temp = 0;
        for (int idx = rowPtr[row] + 1; idx < rowPtr[row + 1]; ++idx) {
            int c = col[idx];
            temp = fma(val[idx], x[c], temp);
            b[c] = fma(val[idx], xr, b[c]);
        }
        b[row] += temp;
    }
}

/* GS_KERNEL, diagonal first; descending rows when start > end,
 * kernels.cpp:174-200 */
void orc_gs_range(int start, int end, const int *rowPtr, const int *col, const double *val, double *x,
                  const double *b) {
    int inc = (start > end) ? -1 : 1;
    for (int row = start; row != end; row += inc) {
        int d = rowPtr[row];
        double tmp = b[row];
        for (int idx = d + 1; idx < rowPtr[row + 1]; ++idx) tmp = fma(-val[idx], x[col[idx]], tmp);
        x[row] = tmp / val[d];
    }
}

/* KACZ_KERNEL with omega = 1, kernels.cpp:285-317 */
void orc_kacz_range(int start, int end, const int *rowPtr, const int *col, const double *val, double *x,
                    const double *b) {
    int inc = (start > end) ? -1 : 1;
    for (int row = start; row != end; row += inc) {
        double rowNorm = 0.0, scale = -b[row];
        for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx) {
            double m = val[idx];
            scale = fma(m, x[col[idx]], scale);
            rowNorm = fma(m, m, rowNorm);
        }
        scale /= rowNorm;
        for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx) x[col[idx]] = fma(-scale, val[idx], x[col[idx]]);
    }
}

/* Kernel ids shared with the Python side. */
enum { ORC_K_SPMV = 0, ORC_K_SPMTV = 1, ORC_K_SYMMSPMV = 2, ORC_K_GS = 3, ORC_K_KACZ = 4 };

static void orc_call(int kernel, int start, int end, const int *rowPtr, const int *col, const double *val, double *x,
                     double *b) {
    switch (kernel) {
    case ORC_K_SPMV: orc_spmv_range(start, end, rowPtr, col, val, x, b); break;
    case ORC_K_SPMTV: orc_spmtv_range(start, end, rowPtr, col, val, x, b); break;
    case ORC_K_SYMMSPMV: orc_symmspmv_range(start, end, rowPtr, col, val, x, b); break;
    case ORC_K_GS: orc_gs_range(start, end, rowPtr, col, val, x, b); break;
    case ORC_K_KACZ: orc_kacz_range(start, end, rowPtr, col, val, x, b); break;
    default: break;
    }
}

/* ------------------------------------------------------------------------ */
/* Sequential zone-tree walk (functionManager.cpp:201-265, 1453-1501)        */
/* ------------------------------------------------------------------------ */

typedef struct {
    int nnodes;
    const int *valueStart; /* nnodes+1 offsets into value */
    const int *value;      /* valueZ of every node */
    const int *childStart; /* nnodes+1 offsets into child */
    const int *child;      /* children pairs of every node */
    const int *subBlocks;  /* totalSubBlocks of every node */
} orc_tree;

static void orc_walk(const orc_tree *t, int node, int blockPerThread, int rev, int kernel, const int *rowPtr,
                     const int *col, const double *val, double *x, double *b) {
    const int *ch = t->child + t->childStart[node];
    int nch = t->childStart[node + 1] - t->childStart[node];
    const int *v = t->value + t->valueStart[node];
    for (int sb = 0; sb < t->subBlocks[node]; ++sb) {
        int currNthreads = nch ? (ch[2 * sb + 1] - ch[2 * sb]) / blockPerThread : 0;
        if (currNthreads <= 1) {
            /* a node with at most one thread in this sub-block runs its own
             * first range as a leaf (functionManager.cpp:218-230) */
            int s = v[0], e = v[1];
            if (rev) {
                s = v[1] - 1;
                e = v[0] - 1;
            }
            orc_call(kernel, s, e, rowPtr, col, val, x, b);
        } else {
            int b0 = rev ? blockPerThread - 1 : 0, b1 = rev ? -1 : blockPerThread, inc = rev ? -1 : 1;
            for (int blk = b0; blk != b1; blk += inc)
                for (int tid = 0; tid < currNthreads; ++tid)
                    orc_walk(t, ch[2 * sb] + blockPerThread * tid + blk, blockPerThread, rev, kernel, rowPtr, col,
                             val, x, b);
        }
    }
}

/* Execute `kernel` over a zone tree sequentially in the executor's order,
 * then the dense-row serial tail (functionManager.cpp:1493-1500). */
void orc_exec_tree(int nnodes, const int *valueStart, const int *value, const int *childStart, const int *child,
                   const int *subBlocks, int blockPerThread, int serialLo, int serialHi, int kernel, int rev,
                   const int *rowPtr, const int *col, const double *val, double *x, double *b) {
    orc_tree t = {nnodes, valueStart, value, childStart, child, subBlocks};
    orc_walk(&t, 0, blockPerThread, rev, kernel, rowPtr, col, val, x, b);
    if (!rev)
        orc_call(kernel, serialLo, serialHi, rowPtr, col, val, x, b);
    else
        orc_call(kernel, serialHi, serialLo, rowPtr, col, val, x, b);
}

/* The colored executor on OpenMP threads over a zone tree flattened into
 * phases (the engine's race_get_phases; leaves of one phase are
 * conflict-free for the coloring's distance): the leaves of a phase run in
 * parallel, one static share per thread, and the phases run in order with a
 * barrier between them, as RACE's executor runs block 0 of all threads, a
 * barrier, then block 1 (functionManager.cpp:201-265, 1453-1501). A leaf
 * with lo > hi runs backwards (a reverse sweep). reps calls are made in one
 * parallel region, as the reference's thread pool stays up between calls. */
void orc_exec_phases_omp(int kernel, int numPhases, const int *phasePtr, const int *leafLo, const int *leafHi,
                         int nthreads, int reps, const int *rowPtr, const int *col, const double *val, double *x,
                         double *b) {
#pragma omp parallel num_threads(nthreads)
    for (int r = 0; r < reps; ++r)
        for (int ph = 0; ph < numPhases; ++ph) {
#pragma omp for schedule(static)
            for (int l = phasePtr[ph]; l < phasePtr[ph + 1]; ++l)
                orc_call(kernel, leafLo[l], leafHi[l], rowPtr, col, val, x, b);
        }
}

/* ------------------------------------------------------------------------ */
/* Matrix power                                                              */
/* ------------------------------------------------------------------------ */

/* y_k = A y_{k-1}, k = 1..p, each row a sequential fma chain: the output of
 * the reference's MPK executor for MAT_SPMV_KERNEL (kernels.cpp:749-777),
 * which depends only on the per-row arithmetic. x holds (p+1)*n values,
 * power-major. Rows are split over OpenMP threads when available. */
void orc_mpk_plain(int n, int p, const int *rowPtr, const int *col, const double *val, double *x) {
    for (int k = 1; k <= p; ++k) {
        const double *in = x + (size_t)(k - 1) * n;
        double *out = x + (size_t)k * n;
#pragma omp parallel for schedule(static)
        for (int row = 0; row < n; ++row) {
            double tmp = 0;
            for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx) tmp = fma(val[idx], in[col[idx]], tmp);
            out[row] = tmp;
        }
    }
}

/* The same power chain applied to a block of nrhs vectors stored row-major
 * (x[(k*n + r)*nrhs + j]): each right-hand side is MAT_SPMV_KERNEL's
 * sequential fma chain (kernels.cpp:749-777), in FP64 and, for the
 * reduced-precision block path, in FP32 with fmaf. */
void orc_mpk_block(int n, int p, int nrhs, const int *rowPtr, const int *col, const double *val, double *x) {
    for (int k = 1; k <= p; ++k) {
        const double *in = x + (size_t)(k - 1) * n * nrhs;
        double *out = x + (size_t)k * n * nrhs;
#pragma omp parallel for schedule(static)
        for (int row = 0; row < n; ++row)
            for (int j = 0; j < nrhs; ++j) {
                double tmp = 0;
                for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx)
                    tmp = fma(val[idx], in[(size_t)col[idx] * nrhs + j], tmp);
                out[(size_t)row * nrhs + j] = tmp;
            }
    }
}

void orc_mpk_block_f32(int n, int p, int nrhs, const int *rowPtr, const int *col, const float *val, float *x) {
    for (int k = 1; k <= p; ++k) {
        const float *in = x + (size_t)(k - 1) * n * nrhs;
        float *out = x + (size_t)k * n * nrhs;
#pragma omp parallel for schedule(static)
        for (int row = 0; row < n; ++row)
            for (int j = 0; j < nrhs; ++j) {
                float tmp = 0;
                for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx)
                    tmp = fmaf(val[idx], in[(size_t)col[idx] * nrhs + j], tmp);
                out[(size_t)row * nrhs + j] = tmp;
            }
    }
}

/* Cache-violation bookkeeping of one MPK stage (matrixPower.cpp:88-99,
 * 134-140): nnz budget of a level = safety * (p+1) * levelNnz; bytes per nnz
 * = (1 + p/nnzr) * 8 + (1 + 1/nnzr) * 4 with nnzr = NNZ/NROW. */
static double orc_byte_per_nnz(int p, int nrow, long long nnz) {
    double nnzr = (double)nnz / (double)nrow;
    return (double)(((1 + p / nnzr) * sizeof(double) + (1 + 1 / nnzr) * sizeof(int)));
}

/* Level groups of a single-stage MPK partition (consolidatePartition without
 * hopeless regions, matrixPower.cpp:685-883): consecutive levels are merged
 * while the running sum of level budgets stays below cacheSize/bytePerNnz;
 * the level that reaches it opens the next group. Also returns unlockRow and
 * dangerRow per group (rows before unlockRow are what the previous group's
 * next power needs; rows from dangerRow on need the next group).
 * levelPtr has totalLevel+1 row offsets starting at lo. Outputs have room
 * for totalLevel+1 entries. Returns the number of groups, or -1 when the
 * stage has a hopeless region: two consecutive levels whose budgets exceed
 * the cache by more than cutoff (identifyHopelessRegions,
 * matrixPower.cpp:147-210; an isolated such level is grouped normally). */
int orc_mpk_groups(int p, int nrow, long long nnz, double cacheSize, double safety, int cutoff, int totalLevel,
                   const int *levelPtr, const int *levelNnz, int *groupPtr, int *unlockRow, int *dangerRow) {
    double bpn = orc_byte_per_nnz(p, nrow, nnz);
    double cacheElem = cacheSize / bpn;
    int prevViolated = -2;
    for (int l = 0; l < totalLevel; ++l) {
        double e = safety * (p + 1) * levelNnz[l];
        if (e > cacheElem && (int)ceil(e / cacheElem) > cutoff) {
            if (l == prevViolated + 1) return -1;
            prevViolated = l;
        }
    }
    int ng = 0;
    groupPtr[0] = levelPtr[0];
    unlockRow[0] = totalLevel > 1 ? levelPtr[1] : levelPtr[totalLevel];
    double sumElem = 0;
    for (int l = 0; l < totalLevel; ++l) {
        double cur = safety * (p + 1) * levelNnz[l];
        sumElem += cur;
        if (l > 0 && sumElem >= cacheElem) {
            sumElem = cur;
            groupPtr[ng + 1] = levelPtr[l];
            dangerRow[ng] = levelPtr[l - 1];
            if (l + 1 <= totalLevel) unlockRow[ng + 1] = levelPtr[l + 1];
            ng += 1;
        }
    }
    groupPtr[ng + 1] = levelPtr[totalLevel];
    dangerRow[ng] = levelPtr[totalLevel - 1];
    ng += 1;
    return ng;
}

/* Level groups of one stage of the MPK partition with hopeless regions
 * (mtxPower::findPartition for one shared-cache domain, matrixPower.cpp:
 * 505-605: identifyHopelessRegions :147-503 and consolidatePartition
 * :685-940), stated from what they compute:
 *   - a level is violated when its budget b(l) = safety*(p+1)*levelNnz[l]
 *     exceeds the cache by more than `cutoff` (ceil(b/cacheElem) > cutoff);
 *   - every run of two or more consecutive violated levels is a hopeless
 *     region; regions with fewer than p-1 levels between them merge;
 *   - the first region starts no earlier than level p-1 and the last ends
 *     no later than level L-p (a region left empty is dropped);
 *   - grouping walks the levels once, opening a group at a level (not the
 *     first) when the running budget reaches the cache or the level is
 *     forced: the p-1 levels before a region and its first level, the p-1
 *     levels after it and the one after those; the levels inside a region
 *     after its first never open a group, so a region is one group, whose
 *     index is reported (MPLeaf::hid). Opening a group restarts the
 *     running budget at the level's own.
 * levelNnz includes the non-zeros of boundary rows of each level
 * (getElemUpperLimit, :88-99). levelPtr holds L+1 row offsets; bndPtr holds
 * nb regions' L+1 offsets each. Writes groupPtr (ng+1), hid (*numHid) and
 * each region's offsets at the group starts into bndGroupPtr (nb*(ng+1),
 * region-major with stride L+1). Returns ng, or -1 when L < 1 or a region
 * lacks p-1 levels on either side. */
int orc_mpk_partition(int p, int nrow, long long nnz, double cacheSize, double safety, int cutoff, int L,
                      const int *levelPtr, const int *levelNnz, int nb, const int *bndPtr, int *groupPtr, int *hid,
                      int *numHid, int *bndGroupPtr) {
    if (L < 1) return -1;
    double cacheElem = cacheSize / orc_byte_per_nnz(p, nrow, nnz);
    int *viol = (int *)calloc((size_t)L, sizeof(int));
    int *rs = (int *)malloc(sizeof(int) * (size_t)L), *re = (int *)malloc(sizeof(int) * (size_t)L);
    int nr = 0;
    for (int l = 0; l < L; ++l) {
        double b = safety * (p + 1) * levelNnz[l];
        viol[l] = b > cacheElem && (int)ceil(b / cacheElem) > cutoff;
    }
    for (int l = 0; l + 1 < L; ++l) /* runs of length >= 2 */
        if (viol[l] && viol[l + 1] && (l == 0 || !viol[l - 1])) {
            int e = l + 1;
            while (e + 1 < L && viol[e + 1]) ++e;
            if (nr > 0 && l - re[nr - 1] - 1 < p - 1) {
                re[nr - 1] = e; /* merge with the previous region */
            } else {
                rs[nr] = l;
                re[nr] = e;
                ++nr;
            }
        }
    int first = 0, last = nr - 1;
    if (nr > 0 && rs[0] < p) { /* keep p-1 levels before the first region */
        if (re[0] < p - 1) first = 1;
        else rs[0] = p - 1;
    }
    if (nr > 0 && re[nr - 1] > L - 1 - p) { /* and after the last */
        if (rs[nr - 1] > L - p) last = nr - 2;
        else re[nr - 1] = L - p;
    }
    /* classify the levels: 1 forced, 2 inside a region after its first level, 3 first level of a region */
    int *kind = (int *)calloc((size_t)L + 1, sizeof(int));
    int ok = 1;
    for (int r = first; r <= last; ++r) {
        int a = rs[r], z = re[r], b = p - 1;
        if (a - b < 0 || z + b > L - 1) ok = 0;
        for (int l = a - b; l <= z + b + 1 && ok; ++l) {
            if (l < 0 || l >= L) continue;
            if (l == a) kind[l] = 3;
            else if (l > a && l <= z) kind[l] = 2;
            else if (kind[l] == 0) kind[l] = 1;
        }
    }
    int ng = 0, nh = 0;
    if (ok) {
        groupPtr[0] = levelPtr[0];
        for (int k = 0; k < nb; ++k) bndGroupPtr[(size_t)k * (L + 1)] = bndPtr[(size_t)k * (L + 1)];
        double sum = 0;
        for (int l = 0; l < L; ++l) {
            double b = safety * (p + 1) * levelNnz[l];
            sum += b;
            if (kind[l] == 3) hid[nh++] = ng + 1;
            if (l > 0 && kind[l] != 2 && (sum >= cacheElem || kind[l] != 0)) {
                sum = b;
                ++ng;
                groupPtr[ng] = levelPtr[l];
                for (int k = 0; k < nb; ++k) bndGroupPtr[(size_t)k * (L + 1) + ng] = bndPtr[(size_t)k * (L + 1) + l];
            }
        }
        ++ng;
        groupPtr[ng] = levelPtr[L];
        for (int k = 0; k < nb; ++k) bndGroupPtr[(size_t)k * (L + 1) + ng] = bndPtr[(size_t)k * (L + 1) + L];
    }
    *numHid = nh;
    free(viol);
    free(rs);
    free(re);
    free(kind);
    return ok ? ng : -1;
}

/* Per-group unlock counters for `nthreads` threads (findUnlockCtr,
 * matrixPower.cpp:958-1001 with one node): the number of threads whose
 * slice of group l starts before unlockRow[l]. Slices follow
 * SPLIT_LEVEL_PER_THREAD_P2P (macros.h:51-61). */
void orc_mpk_unlock_ctr(int ngroups, const int *groupPtr, const int *unlockRow, int nthreads, int *unlockCtr) {
    for (int l = 0; l < ngroups; ++l) {
        int s = groupPtr[l], e = groupPtr[l + 1];
        int per = (e - s) / nthreads;
        unlockCtr[l] = 0;
        for (int t = 0; t < nthreads; ++t)
            if (unlockRow[l] > s + t * per) unlockCtr[l]++;
    }
}

/* Level-group wavefront on OpenMP threads (powerCallGeneral for one node
 * without boundary regions, functionManager.cpp:560-823): for every step
 * `level` and power `pow`, thread t computes its slice of group level-pow
 * after the group has been released by all threads at pow-1, and (for the
 * rows from dangerRow on) after the next group's first rows at pow-1 are
 * done. Spins use a plain busy wait, as the reference does. */
void orc_mpk_wavefront(int n, int p, int ngroups, const int *groupPtr, const int *unlockRow, const int *dangerRow,
                       int nthreads, const int *rowPtr, const int *col, const double *val, double *x) {
    volatile int *lockCtr = (volatile int *)calloc((size_t)ngroups, sizeof(int));
    volatile int *lockTable = (volatile int *)calloc((size_t)ngroups * (size_t)p + 1, sizeof(int));
    int *unlockCtr = (int *)malloc(sizeof(int) * (size_t)(ngroups > 0 ? ngroups : 1));
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
    {
        int nthr = 1, tid = 0;
#ifdef _OPENMP
        nthr = omp_get_num_threads();
        tid = omp_get_thread_num();
#endif
        /* the unlock counters count the threads of the team that actually
         * runs (findUnlockCtr uses the live team size, matrixPower.cpp:970) */
#pragma omp single
        orc_mpk_unlock_ctr(ngroups, groupPtr, unlockRow, nthr, unlockCtr);
        for (int level = 0; level < ngroups + p - 1; ++level) {
            for (int pow = 0; pow < p; ++pow) {
                int L = level - pow;
                if (L < 0 || L >= ngroups) continue;
                while (__atomic_load_n(&lockCtr[L], __ATOMIC_ACQUIRE) < nthr * pow) {
                }
                int s = groupPtr[L], e = groupPtr[L + 1];
                int per = (e - s) / nthr;
                int st = s + tid * per;
                int en = (tid == nthr - 1) ? e : s + (tid + 1) * per;
                int cu = unlockRow[L], dr = dangerRow[L];
                const double *in = x + (size_t)pow * n;
                double *out = x + (size_t)(pow + 1) * n;
#define ORC_ROWS(a, z)                                                                                    \
    for (int row = (a); row < (z); ++row) {                                                               \
        double tmp = 0;                                                                                   \
        for (int idx = rowPtr[row]; idx < rowPtr[row + 1]; ++idx) tmp = fma(val[idx], in[col[idx]], tmp); \
        out[row] = tmp;                                                                                   \
    }
#define ORC_WAIT()                                                                                        \
    if (nthr > 1 && pow != 0 && L != ngroups - 1)                                                         \
        while (__atomic_load_n(&lockTable[(size_t)L * p + pow], __ATOMIC_ACQUIRE) != unlockCtr[L + 1]) {  \
        }
#define ORC_UNLOCK()                                                                                      \
    if (L - 1 >= 0 && pow + 1 <= p - 1 && tid < unlockCtr[L])                                             \
        __atomic_fetch_add(&lockTable[(size_t)(L - 1) * p + pow + 1], 1, __ATOMIC_ACQ_REL);
                if (dr <= st || dr < cu) {
                    ORC_WAIT();
                    ORC_ROWS(st, en);
                    ORC_UNLOCK();
                } else {
                    int till = st;
                    if (st < cu) till = cu < en ? cu : en;
                    ORC_ROWS(st, till);
                    ORC_UNLOCK();
                    int nxt = till;
                    if (dr > en) nxt = en;
                    ORC_ROWS(till, nxt);
                    ORC_WAIT();
                    ORC_ROWS(nxt, en);
                }
                __atomic_fetch_add(&lockCtr[L], 1, __ATOMIC_ACQ_REL);
#undef ORC_ROWS
#undef ORC_WAIT
#undef ORC_UNLOCK
            }
        }
    }
    free((void *)lockCtr);
    free((void *)lockTable);
    free(unlockCtr);
}
