"""Host logic of the parameter tuner (no GPU): features, config spaces,
dataset files and regret arithmetic."""
import numpy as np
import pytest

from race_gb300 import matgen, tuner


def test_features_deterministic_and_finite():
    fam, A = tuner.dataset_matrix(3, seed=1, nmin=5000, nmax=20000)
    f1, f2 = tuner.matrix_features(A), tuner.matrix_features(A)
    assert f1.shape == (tuner.N_MATRIX_FEATURES,) and np.array_equal(f1, f2)
    for task in (tuner.MPK_TASK, tuner.SWEEP_TASK):
        rows = tuner.feature_rows(f1, task)
        assert rows.shape == (len(task.configs), tuner.N_FEATURES)
        assert np.isfinite(rows).all()
        # configs are distinguishable by their features
        assert len({r.tobytes() for r in rows[:, tuner.N_MATRIX_FEATURES:]}) == len(task.configs)


def test_bfs_levels_of_a_chain():
    A = matgen.chain_with_empty_rows(10, ())
    lev = tuner.bfs_levels(A)
    np.testing.assert_array_equal(lev, np.arange(10))


def test_dataset_roundtrip_and_merge(tmp_path):
    rng = np.random.Generator(np.random.PCG64(0))
    mk = lambda k: tuner.Dataset(rng.random((k, tuner.N_MATRIX_FEATURES)).astype(np.float32),  # noqa: E731
                                 rng.random((k, len(tuner.SWEEP_CONFIGS))) + 0.1, np.array(["lap7"] * k),
                                 np.ones((k, 2), np.int64), "symmgs")
    a, b = mk(3), mk(4)
    pa, pb, pm = tmp_path / "a.npz", tmp_path / "b.npz", tmp_path / "m.npz"
    a.save(pa)
    b.save(pb)
    la = tuner.Dataset.load(pa)
    assert la.task == "symmgs" and np.array_equal(la.times, a.times)
    tuner.main(["merge", "--out", str(pm), str(pa), str(pb)])
    m = tuner.Dataset.load(pm)
    assert m.task == "symmgs" and m.times.shape == (7, len(tuner.SWEEP_CONFIGS))
    np.testing.assert_array_equal(m.times[3:], b.times)


def test_committed_search_files_match_config_spaces():
    import pathlib
    g = pathlib.Path(__file__).resolve().parent / "golden"
    for name, task in (("tuner_search.npz", "mpk"), ("tuner_search_symmgs.npz", "symmgs")):
        if not (g / name).exists():
            pytest.skip("no committed search timings")
        d = tuner.Dataset.load(g / name)
        assert d.task == task and d.times.shape[1] == len(tuner.TASKS[task].configs)
        assert (d.times[np.isfinite(d.times)] > 0).all()


def test_regret_and_best_fixed_config():
    times = np.array([[1.0, 2.0, 1.5], [3.0, 1.0, 1.2], [2.0, 2.2, 1.0]])
    assert tuner.regret(times[0], 0) == 0.0
    assert tuner.regret(times[1], 0) == pytest.approx(2.0)
    ds = tuner.Dataset(np.zeros((3, tuner.N_MATRIX_FEATURES), np.float32),
                       np.pad(times, ((0, 0), (0, len(tuner.SWEEP_CONFIGS) - 3)), constant_values=np.inf),
                       np.array(["x"] * 3), np.ones((3, 2), np.int64), "symmgs")
    # config 2 has the lowest mean regret (0.5+0.2+0)/3
    assert tuner.best_fixed_config(ds) == 2


def test_tuning_matrices_have_no_hopeless_regions():
    """The recursion depth (RACE_MAX_RECURSION_STAGES) changes a partition
    only where two consecutive levels exceed the budget by more than the
    cut-off (50). On the seeded tuning matrices none does at any searched
    power and budget, so the depth is not a tuning knob there (the first
    matrices up to at least 8 and all four families; the oracle's BFS
    levels)."""
    from oracle import oracle as orc
    families = set()
    idx = 0
    while idx < 8 or len(families) < 4:
        fam, A = tuner.dataset_matrix(idx)
        idx += 1
        families.add(fam)
        _, _, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
        lp = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
        for p, c in tuner.CONFIGS:
            part = orc.mpk_partition(p, A.n, A.nnz, c * 1e6, 2.0, 50, lp, ln)
            assert part is not None and part[1].size == 0, (idx - 1, fam, p, c)
    assert families == {"lap7", "st27", "band", "plaw"}
