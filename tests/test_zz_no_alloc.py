"""tdg_triplets_static (device scratch in one fixed array, no allocation) against
tdg_triplets, the allocating entry point it mirrors. Integer output: the bar is
bit-exact. Collected last on purpose, and written to pass alone in a fresh process too."""
import ctypes as C

import numpy as np
import pytest

from tdep_gb300 import Problem, ScatteringRates, device_count
from tdep_gb300 import _native as N

pytestmark = pytest.mark.gpu

MAX_SAMPLE = 32768


@pytest.fixture(scope="module", autouse=True)
def _require_gpu(built):
    assert device_count() > 0, "GPU tests need a CUDA device; the GB300 path has no CPU fallback"


def _call(sr, name, q1, sample, cap=None):
    sample = np.ascontiguousarray(sample, dtype=np.int32)
    if cap is None:
        cap = max(64, sample.size * (3 + 2 * 2 * sr.prob.n_op))
    out = np.full(cap, -7, np.int32)
    w = C.c_int64(-1)
    rc = getattr(N.lib(), name)(sr._ctx, int(q1), N.ptr(sample, C.c_int32), sample.size, N.ptr(out, C.c_int32),
                                cap, C.byref(w))
    return rc, out[: max(w.value, 0)].copy()


def _both(sr, q1, sample):
    rc_d, ref = _call(sr, "tdg_triplets", q1, sample)
    rc_s, got = _call(sr, "tdg_triplets_static", q1, sample)
    assert rc_d == 0 and rc_s == 0, N.lib().tdg_last_error()
    return ref, got


@pytest.mark.parametrize("name,grid", [("fcc", (8, 8, 8)), ("rocksalt", (6, 6, 6)), ("perovskite", (4, 4, 4))])
def test_static_matches_allocating_two_calls_in_a_row(configs, name, grid):
    prob = Problem.load(configs[name], grid)
    sr = ScatteringRates(prob)
    rng = np.random.default_rng(5)
    full = np.arange(1, prob.n_full + 1, dtype=np.int32)
    total = 0
    for q1 in range(1, prob.n_irr + 1):
        small = rng.permutation(full)[: max(1, prob.n_full // 5)]
        big = rng.permutation(full)
        # large then small, then large again: a stale tail of the scratch cannot hide
        for sample in (big, small, big):
            ref, got = _both(sr, q1, sample)
            np.testing.assert_array_equal(got, ref)
            total += ref.size
    assert total > 0
    sr.close()


def test_static_at_the_sample_limit(configs):
    """A 32x32x32 mesh sampled in full is exactly the stated maximum."""
    prob = Problem.load(configs["fcc"], (32, 32, 32))
    assert prob.n_full == MAX_SAMPLE
    sr = ScatteringRates(prob)
    full = np.arange(1, prob.n_full + 1, dtype=np.int32)
    for q1 in (1, 2, prob.n_irr // 2, prob.n_irr):
        for _ in range(2):
            ref, got = _both(sr, q1, full)
            np.testing.assert_array_equal(got, ref)
    sr.close()


def test_static_rejects_and_edges(configs):
    prob = Problem.load(configs["rocksalt"], (6, 6, 6))
    sr = ScatteringRates(prob)
    # beyond the limit: a clear parameter error naming the limit, nothing written
    rc, got = _call(sr, "tdg_triplets_static", 1, np.ones(MAX_SAMPLE + 1, np.int32), cap=16)
    assert rc == 5 and got.size == 0
    assert b"32768" in N.lib().tdg_last_error()
    # empty sample
    rc, got = _call(sr, "tdg_triplets_static", 1, np.zeros(0, np.int32))
    assert rc == 0 and got.size == 0
    # capacity too small, bad q1, bad q' index
    full = np.arange(1, prob.n_full + 1, dtype=np.int32)
    assert _call(sr, "tdg_triplets_static", 1, full, cap=4)[0] == 5
    assert _call(sr, "tdg_triplets_static", prob.n_irr + 1, full)[0] == 5
    assert _call(sr, "tdg_triplets_static", 1, np.array([0, 3], np.int32))[0] == 5
    # still correct after the rejected calls
    ref, got = _both(sr, 2, full)
    np.testing.assert_array_equal(got, ref)
    sr.close()


def test_static_repeated_sample_over_the_pair_limit(configs):
    """A q-point sampled k times adds its equivalent triplets k times: a sample of one
    q-point with at least 5 images, repeated 32768 times, goes over the 131072-pair limit
    and gets the limit error; the next call is still correct."""
    prob = Problem.load(configs["rocksalt"], (6, 6, 6))
    sr = ScatteringRates(prob)
    full = np.arange(1, prob.n_full + 1, dtype=np.int32)
    trip = sr.triplets(1, full)
    q2, _, k = max(((t[0], t[1], len(t[2])) for t in trip), key=lambda x: x[2])
    assert k >= 5, "the Gamma row of the rocksalt mesh has q-triplets with many images"
    rc, got = _call(sr, "tdg_triplets_static", 1, np.full(MAX_SAMPLE, q2, np.int32), cap=16)
    assert rc == 5 and got.size == 0
    assert b"131072" in N.lib().tdg_last_error()
    ref, got = _both(sr, 1, full)
    np.testing.assert_array_equal(got, ref)
    sr.close()


def test_static_allocates_nothing(configs):
    """The property the entry point exists for: around a call on a warmed-up context, the
    device's free memory and the library pool's used and reserved bytes stay the same."""
    import torch

    prob = Problem.load(configs["perovskite"], (4, 4, 4))
    sr = ScatteringRates(prob)
    full = np.arange(1, prob.n_full + 1, dtype=np.int32)
    rc, first = _call(sr, "tdg_triplets_static", 2, full)  # warm-up: module and symbol lookup
    assert rc == 0

    def usage():
        torch.cuda.synchronize()
        used, res = C.c_uint64(), C.c_uint64()
        N.check(N.lib().tdg_pool_usage(0, C.byref(used), C.byref(res)), "tdg_pool_usage")
        return torch.cuda.mem_get_info(0)[0], used.value, res.value

    before = usage()
    for _ in range(3):
        rc, got = _call(sr, "tdg_triplets_static", 2, full)
        assert rc == 0
        np.testing.assert_array_equal(got, first)
    assert usage() == before
    sr.close()
