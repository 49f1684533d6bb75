"""The launch-shape autotuner on the GPU: its trials leave no trace in the results, and its
decisions land in the process-wide table under the kernel's key."""
import numpy as np
import pytest

from tdep_gb300 import Options, Problem, QLists, ScatteringRates, device_count
from tdep_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _fresh_table(built):
    assert device_count() > 0, "GPU tests need a CUDA device; the GB300 path has no CPU fallback"
    N.check(N.lib().tdg_autotune_clear(), "tdg_autotune_clear")
    yield
    N.check(N.lib().tdg_autotune_clear(), "tdg_autotune_clear")


def _run(sr, opts, lists):
    lw = sr.generate(opts, lists).copy()
    _, ki = sr.kappa(opts)
    return lw, ki


def test_fused_kernel_grid_is_tuned_without_changing_results(configs, monkeypatch):
    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=9, precision="fp64")
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    monkeypatch.setenv("TDG_AUTOTUNE", "0")
    a, ka = _run(sr, opts, lists)
    assert N.autotune_table() == {}  # no trials, nothing recorded
    monkeypatch.setenv("TDG_AUTOTUNE", "1")
    b, kb = _run(sr, opts, lists)
    table = N.autotune_table()
    keys = [k for k in table if k.startswith("threephonon/n6/p0/")]
    assert len(keys) == 1 and 1 <= table[keys[0]] <= 32, table
    c, kc = _run(sr, opts, lists)  # the recorded decision, no new trials
    sr.close()
    assert N.autotune_table() == table
    # only the order of the atomic FP64 sums may differ
    np.testing.assert_allclose(b, a, rtol=1e-12, atol=0)
    np.testing.assert_allclose(c, a, rtol=1e-12, atol=0)
    np.testing.assert_allclose(kb, ka, rtol=1e-11, atol=0)
    np.testing.assert_allclose(kc, ka, rtol=1e-11, atol=0)


def test_large_cell_shapes_are_tuned_without_changing_results(configs, monkeypatch, tmp_path):
    prob = Problem.load(configs["supercell"], (3, 3, 3), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=6, precision="mixed",
                   qg3ph=(2, 2, 2))
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    monkeypatch.setenv("TDG_AUTOTUNE", "0")
    a, ka = _run(sr, opts, lists)
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("TDG_AUTOTUNE", "1")
    monkeypatch.setenv("TDG_TUNE_CACHE", str(cache))
    N.check(N.lib().tdg_autotune_clear(), "tdg_autotune_clear")
    b, kb = _run(sr, opts, lists)
    sr.close()
    table = N.autotune_table()
    keys = [k for k in table if k.startswith("largecell/n30/p1/")]
    assert len(keys) == 1 and table[keys[0]] in (324, 164, 323, 163), table
    # the decision was written to the cache file named by the environment
    saved = dict(line.split() for line in cache.read_text().splitlines() if line and not line.startswith("#"))
    assert int(saved[keys[0]]) == table[keys[0]]
    # the GEMM depth does not change results; the delta row block changes only the order of
    # the FP64 column sums
    np.testing.assert_allclose(b, a, rtol=1e-10, atol=1e-14 * np.abs(a).max())
    np.testing.assert_allclose(kb, ka, rtol=1e-9, atol=0)


def _graph_counts(sr):
    import ctypes as C

    counts = np.zeros(3, dtype=np.int64)
    N.check(N.lib().tdg_graph_counts(sr._ctx, N.ptr(counts, C.c_int64)), "tdg_graph_counts")
    return counts.tolist()


@pytest.mark.parametrize("path", ["fused", "large_cell"])
def test_three_phonon_part_is_recorded_once_and_replayed(configs, monkeypatch, path):
    """First call direct, second recorded as a CUDA graph, later calls replay it; the
    results of every call agree."""
    monkeypatch.delenv("TDG_GRAPHS", raising=False)
    if path == "fused":
        prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
        opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=9, precision="fp64")
        rtol = 1e-12
    else:
        prob = Problem.load(configs["supercell"], (3, 3, 3), readiso=True)
        opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=6, precision="mixed",
                       qg3ph=(2, 2, 2))
        rtol = 1e-10
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    runs = [_run(sr, opts, lists) for _ in range(4)]
    counts = _graph_counts(sr)
    assert counts == [1, 1, 2], counts
    # another temperature changes only device data: the same graph replays
    hot = Options(**{**opts.__dict__, "temperature": 700.0})
    lw_hot, _ = _run(sr, hot, lists)
    assert _graph_counts(sr) == [1, 1, 3]
    monkeypatch.setenv("TDG_GRAPHS", "0")
    lw_hot_direct, _ = _run(sr, hot, lists)
    sr.close()
    for lw, ki in runs[1:]:
        np.testing.assert_allclose(lw, runs[0][0], rtol=rtol, atol=0)
        np.testing.assert_allclose(ki, runs[0][1], rtol=10 * rtol, atol=0)
    np.testing.assert_allclose(lw_hot, lw_hot_direct, rtol=rtol, atol=0)
    assert np.max(lw_hot) > 1.5 * np.max(runs[0][0])  # the replay saw the new occupations
