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
        assert rows.shape[0] == len(task.configs) and rows.shape[1] > tuner.N_MATRIX_FEATURES
        if task is tuner.MPK_TASK:
            assert rows.shape[1] == tuner.N_FEATURES
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
    # each row keeps the index of its matrix in the seeded set
    c = tuner.Dataset(a.features, a.times, a.families, a.sizes, "symmgs", np.array([4, 9, 11]))
    c.save(pa)
    np.testing.assert_array_equal(tuner.Dataset.load(pa).index, [4, 9, 11])
    np.testing.assert_array_equal(tuner.Dataset.load(pa).subset(np.array([False, True, True])).index, [9, 11])
    np.testing.assert_array_equal(m.index, [0, 1, 2, 0, 1, 2, 3])


def test_committed_search_files_match_config_spaces():
    import pathlib
    g = pathlib.Path(__file__).resolve().parent / "golden"
    for name, task in (("tuner_search.npz", "mpk"), ("tuner_search_symmgs.npz", "symmgs")):
        if not (g / name).exists():
            pytest.skip("no committed search timings")
        d = tuner.Dataset.load(g / name)
        assert d.task == task and d.times.shape[1] == len(tuner.TASKS[task].configs)
        assert (d.times[np.isfinite(d.times)] > 0).all()
        assert len(np.unique(d.index)) == len(d.index) and (np.diff(d.index) > 0).all()


def test_regret_and_best_fixed_config():
    times = np.array([[1.0, 2.0, 1.5], [3.0, 1.0, 1.2], [2.0, 2.2, 1.0]])
    assert tuner.regret(times[0], 0) == 0.0
    assert tuner.regret(times[1], 0) == pytest.approx(2.0)
    ds = tuner.Dataset(np.zeros((3, tuner.N_MATRIX_FEATURES), np.float32),
                       np.pad(times, ((0, 0), (0, len(tuner.SWEEP_CONFIGS) - 3)), constant_values=np.inf),
                       np.array(["x"] * 3), np.ones((3, 2), np.int64), "symmgs")
    # config 2 has the lowest mean regret (0.5+0.2+0)/3
    assert tuner.best_fixed_config(ds) == 2


def test_recursion_depth_configs_and_hopeless_trees():
    """Every blocked (power, budget) pair is searched at recursion depths 0,
    1 and 2 (RACE_MAX_RECURSION_STAGES), distinguishable by their features;
    the search times the other depths only where the default depth's leaf
    tree shows hopeless regions (more than the root, or hopeless groups in
    it)."""
    assert (1, 512, 1) in tuner.CONFIGS
    for p in (2, 4, 8):
        for c in tuner.CACHE_MB:
            assert all((p, c, r) in tuner.CONFIGS for r in tuner.RECURSION_STAGES)
    # trees: count, then lo, hi, stage, parent, numGroups, groupPtr..., numHopeless, hopeless...
    root_only = np.array([1, 0, 100, 0, -1, 2, 0, 40, 100, 0])
    root_hopeless = np.array([1, 0, 100, 0, -1, 3, 0, 30, 70, 100, 1, 1])
    two_leaves = np.array([2, 0, 100, 0, -1, 3, 0, 30, 70, 100, 1, 1, 30, 70, 1, 0, 1, 0, 40, 0])
    assert not tuner.has_hopeless(root_only)
    assert tuner.has_hopeless(root_hopeless)
    assert tuner.has_hopeless(two_leaves)
    assert not tuner.has_hopeless(np.zeros(0, np.int64))


def test_seeded_set_covers_the_configured_sizes_and_families():
    """The default tuning set: n log-uniform in [50k, 2M] rows, the four
    families (stencils 7/27-point, scrambled banded, power-law); checked on
    the seeds alone (no matrix is built)."""
    import math
    fams, sizes = set(), []
    for i in range(400):
        rng = np.random.Generator(np.random.PCG64([0, i]))
        fams.add(int(rng.integers(0, 4)))
        sizes.append(int(math.exp(rng.uniform(math.log(50_000), math.log(2_000_000)))))
    assert fams == {0, 1, 2, 3}
    assert 50_000 <= min(sizes) < 60_000 and 1_700_000 < max(sizes) <= 2_000_000


def test_build_dataset_keeps_every_matrix_in_order(monkeypatch):
    """The search over spawned matrix-making processes (workers > 0) sees
    matrices start .. start+count-1, each once and in order, and records
    their indices; the GPU search is replaced by a stand-in here."""
    calls = []

    def fake_search(A):
        calls.append(A.n)
        return np.full(len(tuner.SWEEP_CONFIGS), 1e-3)

    monkeypatch.setitem(tuner.TASKS, "fake", tuner.Task("fake", tuner.SWEEP_CONFIGS, tuner.sweep_config_features,
                                                        fake_search))
    monkeypatch.setitem(tuner.TASKS, "symmgs", tuner.TASKS["fake"])
    for workers in (0, 2):
        calls.clear()
        ds = tuner.build_dataset(7, seed=3, nmin=2000, nmax=4000, task="symmgs", start=5, workers=workers)
        np.testing.assert_array_equal(ds.index, np.arange(5, 12))
        want = [tuner.dataset_matrix(i, 3, 2000, 4000)[1].n for i in range(5, 12)]
        assert calls == want and list(ds.sizes[:, 0]) == want
