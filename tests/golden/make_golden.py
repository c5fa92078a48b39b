"""Generates tests/golden/golden.npz from the RACE reference compiled in
place (oracle/build_ref.sh -> oracle/_ref/librace_ref.so).

Run on the build host (where the reference sources are):
    ./oracle/build_ref.sh && python tests/golden/make_golden.py

Stored per case: matrix digest, permutation and inverse, zone tree (flat),
threads/efficiency/stage depth, MPK level groups and the reference's sweep
and MPK outputs for a few small cases; coloring variants (THREE_BLOCK, an
initial permutation, row balancing, environment knobs, unsymmetric
patterns); MPK partitions with hopeless regions (level groups, hopeless
groups, the permutation after the recursion), without recursion, with
recursion deeper than one stage (the whole leaf tree), and of triangular
matrices; the load balancer on level histograms; simdify /
simdifyD1 outputs. The reference's executor runs on
OpenMP threads; its outputs are deterministic for valid colorings.
Full-size configurations are stored as digests only.
"""
from __future__ import annotations

import os
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

os.environ.setdefault("ORACLE_QUIET", "1")
os.environ.setdefault("OMP_NUM_THREADS", "8")

from cases import (COLOR3_CASES, COLOR_CASES, COLOR_ENV_CASES, COLOR_INIT_CASES, COLOR_ROW_CASES,  # noqa: E402
                   COLOR_UNSYM_CASES, EXEC_CASES, POWER_SAFETY_CASES, key_power_safety, HOPELESS_CASES, MATRICES, POWER_CASES, POWER_FLAT_CASES, POWER_TRI_CASES,  # noqa: E402
                   SIMDIFY_CASES, TRAVERSE_CASES, arr_digest, digest, key_color, key_power, key_power_flat,
                   init_perm, key_color3, key_color_env, key_color_init, key_color_row, key_color_unsym,
                   key_hopeless, key_power_tri, key_simdify, key_trav, sell_layout, triangle,
                   DEEP_CASES, DEEP_EXEC_CASES, key_deep, COLOR_EDGE_CASES, COLOR_EDGE_EXEC, key_color_edge,
                   POWER_EDGE_CASES, key_power_edge, f64_digest)
from oracle import refpy  # noqa: E402
from oracle.refpy import RefInterface  # noqa: E402
from race_gb300 import matgen  # noqa: E402

OUT = pathlib.Path(__file__).resolve().parent / "golden.npz"

# full-size MPK configuration: 128^3 27-point stencil, p=8, 100 MB cache budget
FULL_POWER = ("st27_128", 8, 100e6)


def flat_power_tree(tr):
    """An MPK leaf tree flattened: count, then per leaf lo, hi, stage,
    parent, groups, lp, hopeless count, hid."""
    flat = [len(tr)]
    for leaf in tr:
        flat += [leaf["lo"], leaf["hi"], leaf["stage"], leaf["parent"], len(leaf["lp"]) - 1] + leaf["lp"]
        flat += [len(leaf["hid"])] + leaf["hid"]
    return np.array(flat, np.int32)


def exec_outputs(rc, A, d, p, ip):
    """The reference executor's outputs of the example kernels on its own
    coloring (SymmSpMV and KACZ need distance 2)."""
    P = A.permuted(p, ip)
    U = P.upper()
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    out = {}
    for kern, name, mat, rev in [(2, "symmspmv", U, False), (3, "gs", P, False), (3, "gsrev", P, True),
                                 (4, "kacz", P, False), (0, "spmv", P, False)]:
        if kern in (2, 4) and d != 2:
            continue
        x = x0.copy()
        b = np.zeros(A.n) if kern in (0, 2) else b0.copy()
        rc.execute(kern, rev, mat, x, b)
        out[name] = b if kern in (0, 2) else x
    return out


def main():
    g = {}
    mats = {}

    def M(name):
        if name not in mats:
            mats[name] = MATRICES[name]()
        return mats[name]

    for m, d in TRAVERSE_CASES:
        A = M(m)
        p, ip, lr, ln = refpy.traverse(A, d, 0, A.n)
        k = key_trav(m, d)
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = p
        g[k + "__levelRow"] = lr
        g[k + "__levelNnz"] = ln
        print(k, len(lr), "levels")

    # load balancer on the level data of each traversal case
    lb_rows = []
    for m, d in TRAVERSE_CASES:
        if d == 3:
            continue
        lr = g[key_trav(m, d) + "__levelRow"]
        ln = g[key_trav(m, d) + "__levelNnz"]
        for nt in (2, 5, 8, 33, 128):
            for eff in (40.0, 10.0, 80.0):
                for tgt in (0, 1):
                    r = refpy.lb(lr, ln, nt, eff, d, 0, tgt, 7)
                    flat = [len(r["scale"])] + r["scale"] + [len(r["numBlocks"])] + r["zonePtr"] + \
                           [len(r["subZonePtr"]) - 1] + r["subZonePtr"] + r["numBlocks"]
                    lb_rows.append((m, d, nt, eff, tgt, flat))
    g["lb__index"] = np.array([f"{m}|{d}|{nt}|{eff}|{tgt}" for m, d, nt, eff, tgt, _ in lb_rows])
    lens = np.array([len(f) for *_, f in lb_rows], np.int32)
    g["lb__offsets"] = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    g["lb__data"] = np.concatenate([np.array(f, np.int32) for *_, f in lb_rows])
    print("lb cases", len(lb_rows))

    for m, d, t in COLOR_CASES:
        A = M(m)
        rc = refpy.RefColor(A, d, t)
        k = key_color(m, d, t)
        p, ip = rc.perm()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = p
        g[k + "__tree"] = rc.tree_flat()
        g[k + "__threads"] = np.array(rc.threads())
        g[k + "__eff"] = np.array(rc.efficiency())
        g[k + "__stage"] = np.array(rc.max_stage())
        g[k + "__serial"] = rc.serial_part()
        if (m, d, t) in EXEC_CASES:
            for name, out in exec_outputs(rc, A, d, p, ip).items():
                g[k + f"__out_{name}"] = out
        rc.close()
        print(k, "threads", int(g[k + "__threads"]), "eff %.3f" % float(g[k + "__eff"]))

    # simdify / simdifyD1 through a colored RACE::Interface, on the matrix
    # in the interface's own permutation (checked equal to the coloring's,
    # whose zone tree gives the test its schedule)
    for m, d, t, w, cl, extra, flag, kind in SIMDIFY_CASES:
        A = M(m)
        rc = refpy.RefColor(A, d, t)
        p, ip = rc.perm()
        tree = rc.tree_flat()
        rc.close()
        ri = RefInterface(A, d, t)
        assert np.array_equal(ri.perm()[0], p), "interface and coloring permutations differ"
        sell = sell_layout(A.permuted(p, ip), cl, extra, diag_first=(kind == "d2" and flag))
        ok = ri.simdify(w, cl, sell, flag) if kind == "d2" else ri.simdify_d1(w, cl, sell, flag)
        ri.close()
        k = key_simdify(m, d, t, w, cl, extra, flag, kind)
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = p
        g[k + "__tree"] = tree
        g[k + "__ok"] = np.array(int(ok))
        g[k + "__col"] = sell[0]
        g[k + "__src"] = sell[1].astype(np.int32)
        print(k, "ok" if ok else "cannot simdify")

    # colorings of unsymmetric patterns (symm_hint false)
    for m, tri, d, t in COLOR_UNSYM_CASES:
        T = triangle(M(m), tri)
        rc = refpy.RefColor(T, d, t, symm_hint=False)
        k = key_color_unsym(m, tri, d, t)
        p, ip = rc.perm()
        g[k + "__digest"] = np.array(digest(T))
        g[k + "__perm"] = p
        g[k + "__tree"] = rc.tree_flat()
        g[k + "__threads"] = np.array(rc.threads())
        rc.close()
        print(k, "threads", int(g[k + "__threads"]))

    # colorings that balance rows (LBTarget ROW)
    for m, d, t in COLOR_ROW_CASES:
        A = M(m)
        rc = refpy.RefColor(A, d, t, lbtarget=0)
        k = key_color_row(m, d, t)
        p, ip = rc.perm()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = p
        g[k + "__tree"] = rc.tree_flat()
        g[k + "__threads"] = np.array(rc.threads())
        rc.close()
        print(k, "threads", int(g[k + "__threads"]))

    # colorings at the edges of the thread count
    for m, d, t in COLOR_EDGE_CASES:
        A = M(m)
        rc = refpy.RefColor(A, d, t)
        k = key_color_edge(m, d, t)
        p, ip = rc.perm()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = p
        g[k + "__tree"] = rc.tree_flat()
        g[k + "__threads"] = np.array(rc.threads())
        g[k + "__eff"] = np.array(rc.efficiency())
        if (m, d, t) in COLOR_EDGE_EXEC:
            g[k + "__serial"] = rc.serial_part()
            for name, out in exec_outputs(rc, A, d, p, ip).items():
                g[k + f"__out_{name}"] = out
        rc.close()
        print(k, "threads", int(g[k + "__threads"]))

    # colorings under RACE's environment knobs
    for m, d, t, env in COLOR_ENV_CASES:
        A = M(m)
        os.environ.update(env)
        try:
            rc = refpy.RefColor(A, d, t)
        finally:
            for var in env:
                del os.environ[var]
        k = key_color_env(m, d, t, env)
        p, ip = rc.perm()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = p
        g[k + "__tree"] = rc.tree_flat()
        g[k + "__threads"] = np.array(rc.threads())
        rc.close()
        print(k, "threads", int(g[k + "__threads"]))

    # colorings that start from an initial permutation
    for m, d, t in COLOR_INIT_CASES:
        A = M(m)
        ip0 = init_perm(A.n)
        rc = refpy.RefColor(A, d, t, init_perm=ip0)
        k = key_color_init(m, d, t)
        p, ip = rc.perm()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__init"] = ip0
        g[k + "__perm"] = p
        g[k + "__tree"] = rc.tree_flat()
        g[k + "__threads"] = np.array(rc.threads())
        g[k + "__eff"] = np.array(rc.efficiency())
        rc.close()
        print(k, "threads", int(g[k + "__threads"]))

    # load balancer with THREE_BLOCK (distance 2 only)
    lb3_rows = []
    for m, d in TRAVERSE_CASES:
        if d != 2:
            continue
        lr = g[key_trav(m, d) + "__levelRow"]
        ln = g[key_trav(m, d) + "__levelNnz"]
        for nt in (2, 5, 8, 33, 128):
            for eff in (40.0, 10.0):
                for tgt in (0, 1):
                    r = refpy.lb(lr, ln, nt, eff, d, 1, tgt, 7)
                    flat = [len(r["scale"])] + r["scale"] + [len(r["numBlocks"])] + r["zonePtr"] + \
                           [len(r["subZonePtr"]) - 1] + r["subZonePtr"] + r["numBlocks"]
                    lb3_rows.append((m, nt, eff, tgt, flat))
    g["lb3__index"] = np.array([f"{m}|{nt}|{eff}|{tgt}" for m, nt, eff, tgt, _ in lb3_rows])
    lens = np.array([len(f) for *_, f in lb3_rows], np.int32)
    g["lb3__offsets"] = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    g["lb3__data"] = np.concatenate([np.array(f, np.int32) for *_, f in lb3_rows])
    print("lb three-block cases", len(lb3_rows))

    # distance-2 colorings with THREE_BLOCK, and the reference executor's
    # sweeps on them
    for m, t in COLOR3_CASES:
        A = M(m)
        rc = refpy.RefColor(A, 2, t, d2type=1)
        k = key_color3(m, t)
        p, ip = rc.perm()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = p
        g[k + "__tree"] = rc.tree_flat()
        g[k + "__threads"] = np.array(rc.threads())
        g[k + "__eff"] = np.array(rc.efficiency())
        g[k + "__stage"] = np.array(rc.max_stage())
        g[k + "__serial"] = rc.serial_part()
        P = A.permuted(p, ip)
        U = P.upper()
        x0 = matgen.uniform_vector(A.n, 0)
        b0 = matgen.uniform_vector(A.n, 1)
        for kern, name, mat, rev in [(2, "symmspmv", U, False), (3, "gs", P, False), (3, "gsrev", P, True),
                                     (4, "kacz", P, False), (1, "spmtv", P, False)]:
            x = x0.copy()
            b = np.zeros(A.n) if kern in (1, 2) else b0.copy()
            rc.execute(kern, rev, mat, x, b)
            g[k + f"__out_{name}"] = b if kern in (1, 2) else x
        rc.close()
        print(k, "threads", int(g[k + "__threads"]))

    for m, p, c in POWER_CASES:
        A = M(m)
        rp = refpy.RefPower(A, p, c)
        k = key_power(m, p, c)
        perm, ip = rp.perm()
        tr = rp.tree()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = perm
        g[k + "__lp"] = np.array(tr[0]["lp"], np.int32)
        g[k + "__leaves"] = np.array(len(tr))
        g[k + "__hid"] = np.array(tr[0]["hid"] + [-1], np.int32)
        cov = rp.coverage()
        assert (cov == 1).all()
        if m in ("st27_24", "aniso5_120x90"):
            P = A.permuted(perm, ip)
            x0 = matgen.uniform_vector(A.n, 0)
            g[k + "__out"] = rp.execute(P, x0)[1:]
        rp.close()
        print(k, "groups", len(tr[0]["lp"]) - 1, "leaves", len(tr))

    # hopeless regions: the reference's default recursion (leaf count only)
    # and its partition with RACE_MAX_RECURSION_STAGES=0
    for m, p, c in POWER_FLAT_CASES:
        A = M(m)
        k = key_power_flat(m, p, c)
        rp = refpy.RefPower(A, p, c)
        g[k + "__default_leaves"] = np.array(len(rp.tree()))
        rp.close()
        os.environ["RACE_MAX_RECURSION_STAGES"] = "0"
        try:
            rp = refpy.RefPower(A, p, c)
            perm, ip = rp.perm()
            tr = rp.tree()
            assert (rp.coverage() == 1).all()
            rp.close()
        finally:
            del os.environ["RACE_MAX_RECURSION_STAGES"]
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = perm
        g[k + "__lp"] = np.array(tr[0]["lp"], np.int32)
        g[k + "__leaves"] = np.array(len(tr))
        print(k, "default leaves", int(g[k + "__default_leaves"]), "flat groups", len(tr[0]["lp"]) - 1)

    # default partitions with hopeless regions: stage-0 level groups and the
    # consolidated hopeless groups
    for m, p, c in HOPELESS_CASES:
        A = M(m)
        k = key_hopeless(m, p, c)
        rp = refpy.RefPower(A, p, c)
        tr = rp.tree()
        perm, ip = rp.perm()
        cov = rp.coverage()
        assert (cov == 1).all()
        if (m, p, c) in (("band_5k", 8, 3000), ("plaw_3k", 4, 2e3)):  # the reference executor, recursive partition
            g[key_hopeless(m, p, c) + "__out"] = rp.execute(A.permuted(perm, ip), matgen.uniform_vector(A.n, 0))[1:]
        rp.close()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__lp"] = np.array(tr[0]["lp"], np.int32)
        g[k + "__hid"] = np.array(tr[0]["hid"], np.int32)
        g[k + "__leaves"] = np.array(len(tr))
        g[k + "__perm"] = perm  # after the recursion into the hopeless groups
        print(k, "groups", len(tr[0]["lp"]) - 1, "hopeless", tr[0]["hid"], "leaves", len(tr))

    # other safety factors
    for m, p, c, sf in POWER_SAFETY_CASES:
        A = M(m)
        k = key_power_safety(m, p, c, sf)
        rp = refpy.RefPower(A, p, c, safety=sf)
        perm, _ = rp.perm()
        tr = rp.tree()
        rp.close()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__perm"] = perm
        g[k + "__lp"] = np.array(tr[0]["lp"], np.int32)
        g[k + "__hid"] = np.array(tr[0]["hid"], np.int32)
        print(k, "groups", len(tr[0]["lp"]) - 1, "hopeless", tr[0]["hid"])

    # triangular matrix power: mtxType L / U on the lower / upper triangle
    for m, tri, p, c in POWER_TRI_CASES:
        T = triangle(M(m), tri)
        k = key_power_tri(m, tri, p, c)
        rp = refpy.RefPower(T, p, c, mtx_type=tri)
        perm, ip = rp.perm()
        tr = rp.tree()
        assert (rp.coverage() == 1).all()
        rp.close()
        g[k + "__digest"] = np.array(digest(T))
        g[k + "__perm"] = perm
        g[k + "__lp"] = np.array(tr[0]["lp"], np.int32)
        g[k + "__leaves"] = np.array(len(tr))
        print(k, "groups", len(tr[0]["lp"]) - 1)

    # recursion deeper than one stage: the whole leaf tree (count, then per
    # leaf lo, hi, stage, parent, groups, lp, hopeless count, hid) and the
    # permutation
    for m, p, c, stages, cuts in DEEP_CASES:
        A = M(m)
        k = key_deep(m, p, c, stages, cuts)
        env = {"RACE_MAX_RECURSION_STAGES": str(stages) if stages >= 0 else None,
               "RACE_CACHE_VIOLATION_CUTOFF": ",".join(str(v) for v in cuts) or None}
        for var, val in env.items():
            if val is not None:
                os.environ[var] = val
        try:
            rp = refpy.RefPower(A, p, c)
            perm, ip = rp.perm()
            tr = rp.tree()
            assert (rp.coverage() == 1).all()
            if (m, p, c, stages, cuts) in DEEP_EXEC_CASES:
                g[k + "__out"] = rp.execute(A.permuted(perm, ip), matgen.uniform_vector(A.n, 0))[1:]
            rp.close()
        finally:
            for var in env:
                os.environ.pop(var, None)
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__tree"] = flat_power_tree(tr)
        g[k + "__perm"] = perm
        print(k, "leaves", len(tr), "deepest stage", max(leaf["stage"] for leaf in tr))

    # MPK partitions at edge parameters, default recursion
    for m, p, c in POWER_EDGE_CASES:
        A = M(m)
        k = key_power_edge(m, p, c)
        rp = refpy.RefPower(A, p, c)
        perm, ip = rp.perm()
        tr = rp.tree()
        assert (rp.coverage() == 1).all()
        out = rp.execute(A.permuted(perm, ip), matgen.uniform_vector(A.n, 0))[1:]
        rp.close()
        g[k + "__digest"] = np.array(digest(A))
        g[k + "__tree"] = flat_power_tree(tr)
        g[k + "__perm"] = perm
        g[k + "__out_digest"] = np.array(f64_digest(out))  # the reference MPK executor's outputs
        print(k, "leaves", len(tr), "groups", len(tr[0]["lp"]) - 1, "hopeless", tr[0]["hid"])

    # full-size MPK configuration: digests only
    A = matgen.stencil3d_27pt(128)
    m, p, c = FULL_POWER
    rp = refpy.RefPower(A, p, c)
    perm, ip = rp.perm()
    tr = rp.tree()
    k = key_power(m, p, c)
    g[k + "__digest"] = np.array(digest(A))
    g[k + "__perm_digest"] = np.array(arr_digest(perm))
    g[k + "__lp"] = np.array(tr[0]["lp"], np.int32)
    g[k + "__leaves"] = np.array(len(tr))
    rp.close()
    print(k, "groups", len(tr[0]["lp"]) - 1)

    np.savez_compressed(OUT, **g)
    print("wrote", OUT, OUT.stat().st_size // 1024, "KB")


if __name__ == "__main__":
    main()
