"""Parity of the GB300 path (through the C-ABI) with the oracle's CPU restatement.

Bars: integer triplet enumeration bit-exact; FP64 linewidths rtol 1e-10, Xi within
1e-9 of its largest entry, kappa rtol 1e-9; mixed precision kappa rtol 1e-4 against the
FP64 GPU path, as the benchmark spec states.
"""
import numpy as np
import pytest

from oracle import binding as orc
from tdep_gb300 import Options, Problem, QLists, ScatteringRates, device_count

pytestmark = pytest.mark.gpu

LW_RTOL = 1e-10
KAPPA_RTOL = 1e-9
XI_REL = 1e-9
MIXED_KAPPA_RTOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _require_gpu(built):
    assert device_count() > 0, "GPU tests need a CUDA device; the GB300 path has no CPU fallback"


def distinct_triplets(prob, lists):
    """Accepted irreducible q-triplets counted once per q1 over the union of its rows' samples
    (the oracle, like the reference, revisits each of them once per row). A q2 that a row
    samples k times counts k times, as it does in the reference's row loop."""
    total = 0
    for q1 in np.unique(lists.row_q1):
        mult = {}
        for r in np.nonzero(lists.row_q1 == q1)[0]:
            vals, counts = np.unique(lists.list3[lists.ptr3[r]:lists.ptr3[r + 1]], return_counts=True)
            for v, c in zip(vals.tolist(), counts.tolist()):
                mult[v] = max(mult.get(v, 0), c)
        union = np.array(sorted(mult), dtype=np.int32)
        total += sum(mult[q2] for q2, _, _ in orc.triplets(prob, int(q1), union))
    return total


def distinct_quartets(prob, lists):
    """Accepted irreducible q-quartets counted once per q1 over all its rows' pair samples; a
    pair that a row forms k times counts k times."""
    total = 0
    for q1 in np.unique(lists.row_q1):
        mult = {}
        for r in np.nonzero(lists.row_q1 == q1)[0]:
            a, b = lists.ptr4[r], lists.ptr4[r + 1]
            cnt = {}
            for q2, q3, q4, _ in orc.quartets(prob, int(q1), lists.list4a[a:b], lists.list4b[a:b]):
                cnt[(q2, q3, q4)] = cnt.get((q2, q3, q4), 0) + 1
            for k, c in cnt.items():
                mult[k] = max(mult.get(k, 0), c)
        total += sum(mult.values())
    return total


def _xi_flips(xi, ref_xi, ratio_check=True, max_frac=1e-4):
    """Entries of Xi that differ by more than XI_REL of the largest element.

    symmetrize_and_distribute averages only entries with od_terms > 0
    (scattering_threephonon.f90:175, scattering_fourphonon.f90:222): a sum that is
    analytically zero can land on either side of 0 depending on summation order (exactly 0
    here, where the phases are exact roots of unity; +-1e-17 relative in the reference's
    cos/sin), which changes how many images enter the average of that orbit. Such an entry
    then differs by the ratio of the two image counts, a fraction p/q with p, q <= 2 * 96.
    Returns the mask of differing entries after checking that they are rare and, when Xi
    holds a single symmetrised order (ratio_check), that every one of them is such a flip;
    with two orders or isotope terms in the same entry the ratio is not a fraction."""
    from fractions import Fraction

    scale = np.abs(ref_xi).max()
    bad = np.abs(xi - ref_xi) > XI_REL * scale
    nbad = int(bad.sum())
    assert bad.mean() < max_frac, f"{nbad} of {bad.size} Xi entries differ"
    for a, b in zip(xi[bad], ref_xi[bad]) if ratio_check else ():
        assert a != 0.0 and b != 0.0, "a differing Xi entry is zero on one side only"
        r = a / b
        f = Fraction(r).limit_denominator(192)
        assert f.numerator <= 192 and abs(r - float(f)) <= 1e-6 * abs(r), f"Xi entry ratio {r} is not an image-count flip"
    return bad


def _compare(prob, opts, lists, lw_rtol=LW_RTOL, kappa_rtol=KAPPA_RTOL, check_xi=True, xi_max_frac=1e-4):
    """GPU path against the oracle. Linewidths and kappa_sma do not depend on Xi and keep
    the tight bars. kappa_iter keeps KAPPA_RTOL when Xi agrees entry by entry; when
    _xi_flips found image-count flips, kappa_iter moves with them and the bar is 1e-3.
    Returns the linewidths, kappa_iter, the oracle's results and the mask of differing Xi
    entries (None without the Xi check)."""
    sr = ScatteringRates(prob)
    lw = sr.generate(opts, lists)
    xi = sr.Xi if check_xi else None
    ks, ki = sr.kappa(opts)
    ref = orc.full_run(prob, opts, lists)
    if opts.thirdorder:
        assert sr.stats["triplets"] == distinct_triplets(prob, lists)
    if opts.fourthorder:
        assert sr.stats["quartets"] == distinct_quartets(prob, lists)
    np.testing.assert_allclose(lw, ref["linewidth"], rtol=lw_rtol, atol=1e-14 * np.abs(ref["linewidth"]).max())
    np.testing.assert_allclose(ks, ref["kappa_sma"], rtol=kappa_rtol, atol=kappa_rtol * np.abs(ref["kappa_sma"]).max())
    single = int(bool(opts.thirdorder)) + int(bool(opts.fourthorder)) == 1 and not opts.isotopescattering
    bad = _xi_flips(xi, ref["xi"], ratio_check=single, max_frac=xi_max_frac) if check_xi else None
    flips = int(bad.sum()) if bad is not None else 0
    krt = kappa_rtol if flips == 0 else max(kappa_rtol, 1e-3)
    np.testing.assert_allclose(ki, ref["kappa_iter"], rtol=krt, atol=krt * np.abs(ref["kappa_iter"]).max())
    if flips == 0:
        assert sr.n_iter == ref["n_iter"]
    sr.close()
    return lw, ki, ref, bad


@pytest.mark.parametrize("name,grid", [("fcc", (8, 8, 8)), ("rocksalt", (6, 6, 6)), ("perovskite", (4, 4, 4))])
def test_triplet_enumeration_bit_exact(configs, name, grid):
    prob = Problem.load(configs[name], grid, readiso=True)
    sr = ScatteringRates(prob)
    rng = np.random.default_rng(3)
    full = np.arange(1, prob.n_full + 1, dtype=np.int32)
    for q1 in range(1, prob.n_irr + 1):
        for sample in (full, rng.permutation(full)[: max(1, prob.n_full // 3)]):
            assert sr.triplets(q1, sample) == orc.triplets(prob, q1, sample)
    sr.close()


def test_fp64_fcc_gaussian(configs):
    """fcc with a broad fixed Gaussian: symmetry-forbidden channels feed od_terms with
    values that are exactly zero on the device (exact root-of-unity phases) and +-1e-17
    relative in the oracle (cos/sin of the Cartesian phase, as in the reference); the
    reference's od_terms > 0 filter turns that into factor-2 changes of a few Xi entries,
    which moves the iterative kappa by ~2e-4. Linewidths and the single-mode kappa do not
    depend on Xi and keep the tight bars."""
    prob = Problem.load(configs["fcc"], (8, 8, 8), readiso=True)
    opts = Options(temperature=300.0, integrationtype=1, sigma=1.0, isotopescattering=False, seed=42, itertol=1e-6)
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    lw = sr.generate(opts, lists)
    ks, ki = sr.kappa(opts)
    sr.close()
    ref = orc.full_run(prob, opts, lists)
    np.testing.assert_allclose(lw, ref["linewidth"], rtol=LW_RTOL, atol=1e-14 * np.abs(ref["linewidth"]).max())
    np.testing.assert_allclose(ks, ref["kappa_sma"], rtol=KAPPA_RTOL, atol=KAPPA_RTOL * np.abs(ks).max())
    np.testing.assert_allclose(ki, ref["kappa_iter"], rtol=1e-3, atol=1e-3 * np.abs(ki).max())


@pytest.mark.parametrize("temperature", [100.0, 300.0, 700.0])
def test_fp64_rocksalt_adaptive(configs, temperature):
    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=temperature, integrationtype=2, isotopescattering=False, seed=7)
    _compare(prob, opts, QLists.monte_carlo(prob, opts))


def test_fp64_perovskite_15_modes(configs):
    prob = Problem.load(configs["perovskite"], (4, 4, 4), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=11)
    _compare(prob, opts, QLists.monte_carlo(prob, opts))


def test_fp64_isotope_boundary_velocity_smearing(configs, tmp_path):
    import shutil

    d = tmp_path / "rs_iso"
    shutil.copytree(configs["rocksalt"], d)
    # two isotopes per site: a non-zero mass-disorder parameter
    (d / "infile.isotopes").write_text("2\n0.75 22.0\n0.25 24.0\n2\n0.7577 34.969\n0.2423 36.966\n")
    prob = Problem.load(d, (6, 6, 6), readiso=True)
    assert prob.mass_disorder.min() > 0
    opts = Options(temperature=300.0, integrationtype=6, isotopescattering=True, mfp_max=1e-7, seed=5)
    _compare(prob, opts, QLists.monte_carlo(prob, opts))


def test_fp64_monte_carlo_rows_differ(configs):
    prob = Problem.load(configs["fcc"], (8, 8, 8), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=42, qg3ph=(4, 4, 4))
    lists = QLists.monte_carlo(prob, opts)
    # every row draws its own stratified sample
    assert not np.array_equal(lists.list3[lists.ptr3[0]:lists.ptr3[1]], lists.list3[lists.ptr3[1]:lists.ptr3[2]])
    _compare(prob, opts, lists)


def test_fp64_monte_carlo_grid_not_dividing_the_mesh(configs):
    """-qg3ph 5 5 5 on a 6x6x6 mesh: the reference's sampler only avoids repeating the
    previous point, so rows sample some q-points twice and count them twice."""
    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=8, qg3ph=(5, 5, 5))
    lists = QLists.monte_carlo(prob, opts)
    r = 0
    assert any(np.unique(lists.list3[lists.ptr3[r]:lists.ptr3[r + 1]]).size < lists.ptr3[r + 1] - lists.ptr3[r]
               for r in range(lists.n_row))
    _compare(prob, opts, lists)


def test_fp64_classical_uneven_per_q1_samples(configs):
    prob = Problem.load(configs["perovskite"], (4, 4, 4), readiso=True)
    rng = np.random.default_rng(17)
    samples = {q: np.sort(rng.choice(np.arange(1, prob.n_full + 1), size=int(rng.integers(8, prob.n_full)),
                                     replace=False)).astype(np.int32) for q in range(1, prob.n_irr + 1)}
    lists = QLists.per_irreducible(prob, samples3=samples)
    opts = Options(temperature=500.0, integrationtype=2, classical=True, isotopescattering=False)
    _compare(prob, opts, lists)


def test_mixed_precision_kappa(configs):
    """Mixed precision against FP64 on rocksalt 8^3 with the BTE converged to 1e-12: at the
    default tolerance (1e-6) the iteration stops 1.7e-4 short of its fixed point on this
    cell, so two runs that stop one iteration apart differ by that much whatever their
    precision. The FP64 run at the default tolerance matches the oracle's, iteration count
    included."""
    prob = Problem.load(configs["rocksalt"], (8, 8, 8), readiso=True)
    o64 = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=3)
    o32 = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=3, precision="mixed")
    lists = QLists.monte_carlo(prob, o64)
    sr = ScatteringRates(prob)
    lw64 = sr.generate(o64, lists).copy()
    _, k64d = sr.kappa(o64)
    nit64 = sr.n_iter
    _, k64 = sr.kappa(o64, maxiter=400, tol=1e-12)
    lw32 = sr.generate(o32, lists).copy()
    _, k32 = sr.kappa(o32, maxiter=400, tol=1e-12)
    sr.close()
    big = lw64 > 1e-3 * lw64.max()
    assert np.max(np.abs(lw32[big] / lw64[big] - 1)) < 1e-4
    np.testing.assert_allclose(k32, k64, rtol=MIXED_KAPPA_RTOL, atol=MIXED_KAPPA_RTOL * np.abs(k64).max())
    ref = orc.full_run(prob, o64, lists)
    np.testing.assert_allclose(k64d, ref["kappa_iter"], rtol=1e-3, atol=1e-3 * np.abs(ref["kappa_iter"]).max())
    assert abs(nit64 - ref["n_iter"]) <= 1


@pytest.mark.parametrize("name,grid,qg4,it", [("fcc", (8, 8, 8), (4, 4, 4), 2),
                                             ("rocksalt", (6, 6, 6), (3, 3, 3), 6),
                                             ("rocksalt", (6, 6, 6), (3, 3, 3), 1)])
def test_fp64_three_plus_four_phonon_monte_carlo(configs4, name, grid, qg4, it):
    """Four-phonon rows with their own two stratified samples per row (every row differs)."""
    prob = Problem.load(configs4[name], grid, fourthorder=True, readiso=True)
    opts = Options(temperature=300.0, integrationtype=it, sigma=1.0, isotopescattering=False, seed=3,
                   fourthorder=True, qg4ph=qg4)
    lists = QLists.monte_carlo(prob, opts)
    _compare(prob, opts, lists)


def test_fp64_four_phonon_only_fcc_monte_carlo(configs4):
    """The fcc case alone, so that every differing Xi entry must be an image-count flip."""
    prob = Problem.load(configs4["fcc"], (8, 8, 8), fourthorder=True, readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, thirdorder=False, isotopescattering=False, seed=3,
                   fourthorder=True, qg4ph=(4, 4, 4))
    _compare(prob, opts, QLists.monte_carlo(prob, opts))


def test_fp64_four_phonon_grid_not_dividing_the_mesh(configs4):
    """-qg4ph 4 4 4 on a 6x6x6 mesh: repeated points in the pair lists count once per pair."""
    prob = Problem.load(configs4["rocksalt"], (6, 6, 6), fourthorder=True, readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=9, fourthorder=True,
                   qg4ph=(4, 4, 4), qg3ph=(4, 4, 4))
    _compare(prob, opts, QLists.monte_carlo(prob, opts))


def test_fp64_four_phonon_perovskite_15_modes(configs4):
    prob = Problem.load(configs4["perovskite"], (4, 4, 4), fourthorder=True, readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=11, fourthorder=True,
                   qg4ph=(2, 2, 2))
    _compare(prob, opts, QLists.monte_carlo(prob, opts))


def test_fp64_four_phonon_only_uneven_per_q1_samples(configs4):
    """--nothirdorder with explicit pair samples of uneven size per q1 (shared by its rows)."""
    prob = Problem.load(configs4["rocksalt"], (6, 6, 6), fourthorder=True, readiso=True)
    rng = np.random.default_rng(23)
    samples4 = {}
    for q in range(1, prob.n_irr + 1):
        k = int(rng.integers(4, 40))
        samples4[q] = tuple(np.sort(rng.choice(np.arange(1, prob.n_full + 1), size=k, replace=False)).astype(np.int32)
                            for _ in range(2))
    lists = QLists.per_irreducible(prob, samples4=samples4)
    opts = Options(temperature=500.0, integrationtype=2, thirdorder=False, fourthorder=True, isotopescattering=False)
    _compare(prob, opts, lists)


def test_mixed_precision_four_phonon_kappa(configs4):
    prob = Problem.load(configs4["rocksalt"], (6, 6, 6), fourthorder=True, readiso=True)
    kw = dict(temperature=300.0, integrationtype=2, isotopescattering=False, seed=3, fourthorder=True, qg4ph=(3, 3, 3))
    o64, o32 = Options(**kw), Options(precision="mixed", **kw)
    lists = QLists.monte_carlo(prob, o64)
    sr = ScatteringRates(prob)
    lw64 = sr.generate(o64, lists).copy()
    _, k64 = sr.kappa(o64, maxiter=400, tol=1e-12)
    lw32 = sr.generate(o32, lists).copy()
    _, k32 = sr.kappa(o32, maxiter=400, tol=1e-12)  # converged: the stopping iteration is not compared
    sr.close()
    big = lw64 > 1e-3 * lw64.max()
    assert np.max(np.abs(lw32[big] / lw64[big] - 1)) < 1e-4
    np.testing.assert_allclose(k32, k64, rtol=MIXED_KAPPA_RTOL, atol=MIXED_KAPPA_RTOL * np.abs(k64).max())


def test_repeat_calls_are_stable(configs):
    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=9)
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    a = sr.generate(opts, lists).copy()
    _, ka = sr.kappa(opts)
    b = sr.generate(opts, lists).copy()
    _, kb = sr.kappa(opts)
    sr.close()
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)
    np.testing.assert_allclose(ka, kb, rtol=1e-12, atol=0)


def test_transfer_counter_counts_the_copies(configs):
    """tdg_transfer_bytes: a Xi download adds exactly its size; once the first kappa call has
    uploaded the symmetry and degeneracy tables, a kappa call uploads qs, F0, Fn and the
    16-byte control word of the device iteration once, and downloads the control word per
    chunk of iterations and Fn once."""
    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=9)
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    h0, d0 = sr.transfer_bytes()
    assert h0 > prob.egv.nbytes and d0 >= 0
    sr.generate(opts, lists)
    h1, d1 = sr.transfer_bytes()
    assert h1 > h0 and d1 >= d0 + lists.n_row * 8
    xi = sr.Xi
    h2, d2 = sr.transfer_bytes()
    assert (h2, d2) == (h1, d1 + xi.nbytes)
    n = prob.n_mode
    sr.kappa(opts, maxiter=1, tol=0.0)
    h2, d2 = sr.transfer_bytes()
    sr.kappa(opts, maxiter=1, tol=0.0)
    h3, d3 = sr.transfer_bytes()
    m = prob.n_irr * n
    assert h3 - h2 == m * 8 + 2 * m * 3 * 8 + 16
    assert d3 - d2 == 16 + m * 3 * 8
    sr.close()


def test_fp64_reference_mgo_fixture(built):
    """The reference's own MgO inputs (tests/infiles of the reference: polar force
    constants with the long-range Ewald term, natural-isotope masses and disorder)
    through both paths, 5x5x5 mesh as in the reference's test."""
    from pathlib import Path

    prob = Problem.load(Path(__file__).parent / "golden" / "mgo", (5, 5, 5))
    # The polar eigenvectors have irrational components, so more od_terms sums that are
    # analytically zero round to either sign than in the non-polar cells (about 1e-3 of
    # the Xi entries). Without isotope terms every differing entry must be shown to be
    # such an image-count flip (ratio p/q). With them the ratio is not a fraction, so the
    # isotope-on run (same seed, hence the same samples) must differ only at positions where
    # the isotope-off run was shown to flip: the isotope terms are added outside the
    # od_terms > 0 filter and cannot create a flip of their own.
    opts0 = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=42)
    bad0 = _compare(prob, opts0, QLists.monte_carlo(prob, opts0), xi_max_frac=2e-3)[3]
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=True, seed=42)
    bad1 = _compare(prob, opts, QLists.monte_carlo(prob, opts), xi_max_frac=2e-3)[3]
    extra = bad1 & ~bad0
    assert not extra.any(), f"{int(extra.sum())} Xi entries differ with isotope terms that were not flips without them"


def test_driver_matches_api(configs, tmp_path):
    """The C++ thermal_conductivity driver writes the kappa the Python API computes."""
    import shutil
    import subprocess
    from pathlib import Path

    from tdep_gb300 import KAPPA_AU_TO_SI

    d = tmp_path / "drv"
    shutil.copytree(configs["rocksalt"], d)
    exe = Path(__file__).resolve().parent.parent / "tdep_gb300" / "bin" / "thermal_conductivity"
    r = subprocess.run([str(exe), "-qg", "6", "6", "6", "--readiso", "--noisotope", "--seed", "4",
                        "--temperature", "300", "--dir", str(d)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = np.loadtxt(d / "outfile.thermal_conductivity")
    prob = Problem.load(d, (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=4)
    sr = ScatteringRates(prob)
    sr.generate(opts)
    ks, ki = sr.kappa(opts)
    ko = sr.kappa_offdiag(opts)
    sr.close()
    np.testing.assert_allclose(vals[0][:3], np.diag(ks) * KAPPA_AU_TO_SI, rtol=1e-9)
    np.testing.assert_allclose(vals[2][:3], np.diag(ko) * KAPPA_AU_TO_SI, rtol=1e-9)
    np.testing.assert_allclose(vals[3][:3], np.diag(ki + ko) * KAPPA_AU_TO_SI, rtol=1e-9)


def test_device_exponential_accuracy(built):
    """The FP64 exp(-t) of the delta weights (Cody-Waite reduction, 2^(-j/64) table,
    Taylor series) stays within 2 ulp of the host libm over the lo_gauss window."""
    import ctypes as C
    import math

    from tdep_gb300 import _native as N

    rng = np.random.default_rng(0)
    t = np.concatenate([np.linspace(0.0, 40.0, 20001), rng.uniform(0.0, 40.0, 50000), [0.0, 1e-300, 1e-12, 32.0]])
    out = np.zeros_like(t)
    N.check(N.lib().tdg_check_exp(N.ptr(t, C.c_double), t.size, N.ptr(out, C.c_double)), "tdg_check_exp")
    ref = np.array([math.exp(-x) for x in t])
    ulp = np.spacing(ref)
    assert np.max(np.abs(out - ref) / ulp) <= 2.0


@pytest.mark.parametrize("name,grid,it", [("rocksalt", (6, 6, 6), 2), ("perovskite", (4, 4, 4), 2),
                                          ("fcc", (8, 8, 8), 6)])
def test_tensor_core_contraction_matches_fp64(configs, name, grid, it):
    """The large-cell path (tcgen05 BF16x3 contraction of n^3 tensors in HBM, batched
    q-triplets), forced at small n, against the FP64 shared-memory path: the spec bar
    for mixed precision (kappa within 1e-4)."""
    prob = Problem.load(configs[name], grid, readiso=True)
    kw = dict(temperature=300.0, integrationtype=it, isotopescattering=False, seed=21)
    o64 = Options(**kw)
    otc = Options(precision="mixed", tensor_cores=True, **kw)
    lists = QLists.monte_carlo(prob, o64)
    sr = ScatteringRates(prob)
    lw64 = sr.generate(o64, lists).copy()
    n64 = sr.stats["triplets"]
    _, k64 = sr.kappa(o64, maxiter=400, tol=1e-12)
    lwtc = sr.generate(otc, lists).copy()
    assert sr.stats["triplets"] == n64
    _, ktc = sr.kappa(otc, maxiter=400, tol=1e-12)  # converged: the stopping iteration is not compared
    sr.close()
    # BF16x3 drops the lo*lo product (2^-16 of a term) and keeps 16 of the 24 mantissa bits of
    # each operand; through three stages and the square a single linewidth can be off by a few
    # 1e-4 where its Psi sums cancel. The kappa bar below is the benchmark spec's 1e-4.
    np.testing.assert_allclose(lwtc, lw64, rtol=3e-4, atol=1e-6 * lw64.max())
    np.testing.assert_allclose(ktc, k64, rtol=MIXED_KAPPA_RTOL, atol=MIXED_KAPPA_RTOL * np.abs(k64).max())


def test_large_cell_tensor_core_path_matches_oracle(configs):
    """A displaced 2x1x1 perovskite supercell (30 modes, identity only): beyond 18 modes the
    contraction runs on the tensor cores in mixed precision; against the oracle's FP64
    restatement at the mixed-precision bar."""
    prob = Problem.load(configs["supercell"], (3, 3, 3), readiso=True)
    assert prob.n_mode == 30 and prob.n_op == 1
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=6, precision="mixed",
                   qg3ph=(2, 2, 2))
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    lw = sr.generate(opts, lists)
    ks, ki = sr.kappa(opts)
    trip = sr.stats["triplets"]
    sr.close()
    ref = orc.full_run(prob, opts, lists)
    assert trip == distinct_triplets(prob, lists)
    big = ref["linewidth"] > 1e-3 * ref["linewidth"].max()
    assert np.max(np.abs(lw[big] / ref["linewidth"][big] - 1)) < 1e-4
    np.testing.assert_allclose(ks, ref["kappa_sma"], rtol=MIXED_KAPPA_RTOL, atol=MIXED_KAPPA_RTOL * np.abs(ks).max())
    np.testing.assert_allclose(ki, ref["kappa_iter"], rtol=MIXED_KAPPA_RTOL, atol=MIXED_KAPPA_RTOL * np.abs(ki).max())


def test_large_cell_needs_mixed_precision(configs):
    from tdep_gb300._native import TdgError

    prob = Problem.load(configs["supercell"], (3, 3, 3), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=6, precision="fp64")
    sr = ScatteringRates(prob)
    with pytest.raises(TdgError) as e:
        sr.generate(opts, QLists.monte_carlo(prob, opts))
    assert e.value.code == 5
    sr.close()


@pytest.mark.parametrize("name,grid,classical", [("rocksalt", (6, 6, 6), False), ("perovskite", (4, 4, 4), False),
                                                 ("fcc", (8, 8, 8), True)])
def test_offdiag_kappa_matches_oracle(configs, name, grid, classical):
    """get_kappa_offdiag on the device (little-group sandwich per point, shared-memory work
    arrays) against the oracle's literal Kronecker form, from the same linewidths."""
    prob = Problem.load(configs[name], grid, readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=5, classical=classical)
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    lw = sr.generate(opts, lists)
    kod = sr.kappa_offdiag(opts)
    sr.close()
    ref = orc.kappa_offdiag(prob, opts, lw)
    assert np.abs(ref).max() > 0
    np.testing.assert_allclose(kod, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())


def test_offdiag_kappa_large_cell_matches_oracle(configs):
    """30 modes: the work arrays live in global memory."""
    prob = Problem.load(configs["supercell"], (3, 3, 3), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=6, precision="mixed",
                   qg3ph=(2, 2, 2))
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    lw = sr.generate(opts, lists)
    kod = sr.kappa_offdiag(opts)
    sr.close()
    ref = orc.kappa_offdiag(prob, opts, lw)
    assert np.abs(ref).max() > 0
    np.testing.assert_allclose(kod, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())


def test_contexts_reuse_pooled_memory_and_release_it(configs):
    """A context created after another one reuses the pooled device memory and gives the
    same results (up to the order of atomic additions); the cache can be released once no
    context is alive."""
    from tdep_gb300 import release_cached_memory

    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=9)
    lists = QLists.monte_carlo(prob, opts)
    out = []
    for _ in range(3):
        sr = ScatteringRates(prob)
        lw = sr.generate(opts, lists).copy()
        _, ki = sr.kappa(opts)
        out.append((lw, ki))
        sr.close()
    release_cached_memory(0)
    for lw, ki in out[1:]:  # equal up to the order of FP64 atomic additions
        np.testing.assert_allclose(lw, out[0][0], rtol=1e-12, atol=0)
        np.testing.assert_allclose(ki, out[0][1], rtol=1e-12, atol=0)


def test_rocksalt16_rows_against_the_oracle(configs):
    """Parity at a benchmarked mesh size (rocksalt 16^3, the adjoint configuration's mesh,
    full q' grid): the oracle runs a few whole q1 groups, the GPU the whole mesh; their
    linewidths (after degeneracy averaging) and symmetrised Xi rows must agree with the FP64
    bars, and the mixed-precision linewidths within 1e-4."""
    import bench

    prob = Problem.load(configs["rocksalt"], (16, 16, 16), readiso=True)
    o64 = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=1, precision="fp64")
    o32 = Options(**{**o64.__dict__, "precision": "mixed"})
    lists = QLists.monte_carlo(prob, o64)
    sr = ScatteringRates(prob)
    lw64 = sr.generate(o64, lists).copy()
    xi64 = sr.Xi
    lw32 = sr.generate(o32, lists).copy()
    sr.close()
    q1s = np.unique(lists.row_q1)
    kept = []
    for q1 in q1s[[1, len(q1s) // 2, -1]]:
        rows = np.nonzero(lists.row_q1 == q1)[0]
        r0, r1 = int(rows[0]), int(rows[-1]) + 1
        g, x, _ = orc.scattering(prob, o64, lists, rows=(r0, r1))
        kept.append((r0, r1, g, x))
    idx, lw_ref, xi_ref = bench.oracle_rows_finish(prob, o64, lists, kept)
    sel = np.unique(lists.row_q1[idx]) - 1
    np.testing.assert_allclose(lw64[sel], lw_ref[sel], rtol=LW_RTOL, atol=1e-14 * np.abs(lw_ref).max())
    np.testing.assert_allclose(lw32[sel], lw_ref[sel], rtol=1e-4, atol=1e-12 * np.abs(lw_ref).max())
    _xi_flips(xi64[idx], xi_ref)


@pytest.mark.parametrize("name,grid", [("fluorite", (6, 6, 6)), ("l12", (6, 6, 6)), ("perovskite", (5, 5, 5))])
def test_tensor_core_fused_kernel(configs, name, grid):
    """The tcgen05 fused kernel (9, 12 and 15 modes, mixed precision, automatic): the path is
    taken; its linewidths agree with the oracle within 1e-4 (relative, with an absolute floor
    of 1e-6 of the largest), Xi with the FP64 GPU path within 1e-4 of its largest entry, and
    kappa with the FP64 path within 1e-4 (the benchmark spec's bar); it agrees with the FP32 SIMT
    kernel (tensor_cores = 2) to the same bars."""
    prob = Problem.load(configs[name], grid, readiso=True)
    o64 = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=3, precision="fp64")
    otc = Options(**{**o64.__dict__, "precision": "mixed"})
    osimt = Options(**{**otc.__dict__, "tensor_cores": 2})
    lists = QLists.monte_carlo(prob, o64)
    sr = ScatteringRates(prob)
    lw64 = sr.generate(o64, lists).copy()
    assert sr.last_path() == 0
    xi64 = sr.Xi
    _, ki64 = sr.kappa(o64)
    lwtc = sr.generate(otc, lists).copy()
    assert sr.last_path() == 1
    xitc = sr.Xi
    _, kitc = sr.kappa(otc)
    lwsimt = sr.generate(osimt, lists).copy()
    assert sr.last_path() == 0
    sr.close()
    ref = orc.full_run(prob, o64, lists)
    scale = np.abs(ref["linewidth"]).max()
    np.testing.assert_allclose(lw64, ref["linewidth"], rtol=LW_RTOL, atol=1e-14 * scale)
    np.testing.assert_allclose(lwtc, ref["linewidth"], rtol=1e-4, atol=1e-6 * scale)
    np.testing.assert_allclose(lwtc, lwsimt, rtol=1e-4, atol=1e-6 * scale)
    assert np.abs(xitc - xi64).max() <= 1e-4 * np.abs(xi64).max()
    np.testing.assert_allclose(kitc, ki64, rtol=MIXED_KAPPA_RTOL, atol=MIXED_KAPPA_RTOL * np.abs(ki64).max())


def test_grid_hdf5_kappa_identity(configs, tmp_path):
    """The reference's own consistency check of its two outputs
    (tests/thermal_conductivity/test_thermal_conductivity.py:24-40): the diagonal of kappa_SMA
    plus the collective part (= kappa_iter) equals the diagonal of the per-mode
    thermal_conductivity of outfile.thermal_conductivity_grid.hdf5 summed over points and
    modes and divided by number_of_qpoints (rtol 1e-7, numpy's default there); also through
    the C++ driver, which writes both files."""
    import subprocess
    import shutil
    from pathlib import Path

    from h5read import H5File
    from tdep_gb300 import KAPPA_AU_TO_SI, write_grid_hdf5

    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=4)
    sr = ScatteringRates(prob)
    lw = sr.generate(opts).copy()
    ks, ki = sr.kappa(opts)
    fn = sr.Fn.copy()
    sr.close()
    f = H5File(write_grid_hdf5(tmp_path / "grid.hdf5", prob, 300.0, lw, fn))
    k2 = f.datasets["thermal_conductivity"].sum(axis=(0, 1)) / f.attrs["number_of_qpoints"][0]
    np.testing.assert_allclose(np.diag(k2), np.diag(ki) * KAPPA_AU_TO_SI, rtol=1e-7)
    d = tmp_path / "drv"
    shutil.copytree(configs["rocksalt"], d)
    exe = Path(__file__).resolve().parent.parent / "tdep_gb300" / "bin" / "thermal_conductivity"
    r = subprocess.run([str(exe), "-qg", "6", "6", "6", "--readiso", "--noisotope", "--seed", "4",
                        "--temperature", "300", "--dir", str(d)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    data1 = np.loadtxt(d / "outfile.thermal_conductivity")
    g = H5File(d / "outfile.thermal_conductivity_grid.hdf5")
    k3 = np.diag(g.datasets["thermal_conductivity"].sum(axis=(0, 1)) / g.attrs["number_of_qpoints"][0])
    np.testing.assert_allclose(data1[0][:3] + data1[1][:3], k3, rtol=1e-7)
