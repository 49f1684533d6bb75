"""The oracle's restatement against properties the reference's algorithm guarantees (CPU).

Per-linewidth parity with the Fortran binary is unpinned (it cannot be built here); these
tests pin the restatement through invariances of the method instead.
"""
import numpy as np
import pytest

from oracle import binding as orc
from tdep_gb300 import Options, Problem, QLists


@pytest.fixture(scope="module")
def rs6(configs):
    return Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)


def _third(p, f1, q2):
    g = p.grid
    a = np.array([(f1 - 1) // (g[1] * g[2]), ((f1 - 1) // g[2]) % g[1], (f1 - 1) % g[2]])
    b = np.array([(q2 - 1) // (g[1] * g[2]), ((q2 - 1) // g[2]) % g[1], (q2 - 1) % g[2]])
    c = (-a - b) % g
    return int(c[0] * g[1] * g[2] + c[1] * g[2] + c[2] + 1)


@pytest.mark.parametrize("name,grid", [("fcc", (6, 6, 6)), ("rocksalt", (4, 4, 4)), ("perovskite", (3, 3, 3))])
def test_irreducible_triplets_partition_the_mesh(configs, name, grid):
    """For every q1, the equivalent triplets of the accepted representatives cover every
    momentum-conserving pair {q2, q3} exactly once."""
    p = Problem.load(configs[name], grid, readiso=True)
    full = np.arange(1, p.n_full + 1, dtype=np.int32)
    for q1 in range(1, p.n_irr + 1):
        f1 = int(p.irr_full[q1 - 1])
        want = {tuple(sorted((q2, _third(p, f1, q2)))) for q2 in full}
        got = []
        for q2, q3, red in orc.triplets(p, q1, full):
            assert q3 == _third(p, f1, q2) and q3 >= q2
            got.extend(tuple(sorted(x)) for x in red)
        assert len(got) == len(set(got)) and set(got) == want


def test_kappa_is_isotropic_for_cubic_cells(rs6):
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=1)
    r = orc.full_run(rs6, opts, QLists.monte_carlo(rs6, opts), nthreads=4)
    for k in (r["kappa_sma"], r["kappa_iter"]):
        assert k[0, 0] > 0
        np.testing.assert_allclose(np.diag(k), k[0, 0], rtol=1e-10)
        assert np.abs(k - np.diag(np.diag(k))).max() <= 1e-10 * k[0, 0]
    # the collective (iterative) solution differs from the single-mode one
    assert abs(r["kappa_iter"][0, 0] / r["kappa_sma"][0, 0] - 1) > 1e-4


def test_linewidths_positive_and_degenerate_modes_equal(rs6):
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=1)
    r = orc.full_run(rs6, opts, QLists.monte_carlo(rs6, opts), nthreads=4)
    lw = r["linewidth"]
    om = rs6.omega[rs6.irr_full - 1]
    # on a coarse mesh a mode can find no partner inside its 8-sigma windows (zero width)
    assert np.all(lw >= 0) and np.all(lw[om < 1e-9] == 0)
    assert np.mean(lw[om >= 1e-9] > 0) > 0.95
    for q in range(rs6.n_irr):
        f = rs6.irr_full[q] - 1
        for b in range(rs6.n_mode):
            if om[q, b] < 1e-9:
                continue
            for b2 in rs6.degen_mode[f, b, : rs6.degen[f, b]] - 1:
                assert lw[q, b2] == pytest.approx(lw[q, b], rel=1e-12)


def test_linewidth_is_affine_in_temperature_classically(rs6):
    """In the classical limit the occupations are kT/omega, so n2-n3 and n2+n3+1 are
    affine in T and so is every three-phonon linewidth."""
    lists = QLists.monte_carlo(rs6, Options(seed=1))
    lw = []
    for T in (200.0, 400.0, 600.0):
        o = Options(temperature=T, integrationtype=2, isotopescattering=False, classical=True, seed=1)
        g, _, _ = orc.scattering(rs6, o, lists, nthreads=4)
        lw.append(g)
    np.testing.assert_allclose(lw[2] - lw[1], lw[1] - lw[0], rtol=1e-9, atol=1e-12 * np.abs(lw[2]).max())


def test_explicit_full_samples_equal_default(rs6):
    opts = Options(temperature=300.0, integrationtype=1, sigma=0.5, isotopescattering=False, seed=1)
    a = QLists.monte_carlo(rs6, opts)
    full = {q: np.arange(1, rs6.n_full + 1, dtype=np.int32) for q in range(1, rs6.n_irr + 1)}
    b = QLists.per_irreducible(rs6, samples3=full)
    ga, _, _ = orc.scattering(rs6, opts, a, nthreads=4)
    gb, _, _ = orc.scattering(rs6, opts, b, nthreads=4)
    np.testing.assert_array_equal(ga, gb)


def test_planted_error_is_detected(rs6):
    """A mistake planted in the checker's output must fail the parity comparison used by
    the GPU tests (the oracle is perturbed on the CPU, never the device)."""
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=1)
    r = orc.full_run(rs6, opts, QLists.monte_carlo(rs6, opts), nthreads=4)
    lw = r["linewidth"].copy()
    lw[np.unravel_index(np.argmax(lw), lw.shape)] *= 1 + 1e-7
    with pytest.raises(AssertionError):
        np.testing.assert_allclose(lw, r["linewidth"], rtol=1e-10, atol=1e-14 * np.abs(r["linewidth"]).max())


def test_oracle_adjoint_matches_finite_differences(configs):
    """The oracle's reverse-mode restatement of the three-phonon linewidth with respect to
    fc3_mwm against central differences of the oracle's own forward pass."""
    prob = Problem.load(configs["rocksalt"], (4, 4, 4), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=5)
    lists = QLists.monte_carlo(prob, opts)
    rng = np.random.default_rng(0)
    lw_bar = rng.normal(size=(prob.n_irr, prob.n_mode))
    grad = orc.adjoint_fc3(prob, opts, lists, lw_bar)
    m0 = prob.fc3_mwm.copy()
    h = 1e-6 * np.abs(m0).max()

    def loss():
        return float(np.sum(orc.full_run(prob, opts, lists)["linewidth"] * lw_bar))

    for _ in range(6):
        t, e = int(rng.integers(prob.n_fc3)), int(rng.integers(27))
        prob.fc3_mwm[t, e] = m0[t, e] + h
        lp = loss()
        prob.fc3_mwm[t, e] = m0[t, e] - h
        lm = loss()
        prob.fc3_mwm[t, e] = m0[t, e]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grad[t, e]) <= 1e-6 * abs(grad).max() + 1e-6 * abs(fd)


def _offdiag_sandwich(prob, opts, lw):
    """get_kappa_offdiag written as per-operation sandwiches egw^H (dD/dq) egw in numpy,
    an independent form of the oracle's n^2 x n^2 Kronecker product (kappa.f90:171-200)."""
    n, na = prob.n_mode, prob.n_atom
    kb = 8.6173303e-5 / 27.21138602
    hbar = 6.582119514e-16 / 27.21138602
    chop = 1e-10 / ((0.52917721067e-10 / hbar) / 1000.0)

    def cv(T, om):
        x = om / T / kb
        if x > 200:
            return 0.0
        if x > 21:
            return kb * x * x * np.exp(-x)
        if x < 2e-2:
            return kb * (1 - x * x / 12 + x**4 / 240)
        return kb * x * x * np.exp(x) / (np.exp(x) - 1) ** 2

    K = np.zeros((3, 3))
    for q in range(prob.n_irr):
        f = prob.irr_full[q] - 1
        E = prob.egv[f][..., 0] + 1j * prob.egv[f][..., 1]
        G = prob.irr_dyngrad[q][..., 0] + 1j * prob.irr_dyngrad[q][..., 1]
        om = prob.omega[f]
        V = np.zeros((3, n, n), complex)
        for k in range(prob.irr_nop[q]):
            o = prob.irr_ops[q, k] - 1
            R = prob.op_cart[o].reshape(3, 3, order="F")
            egw = np.zeros((n, n), complex)
            for a2 in range(na):
                a1 = prob.op_fmap[o, a2] - 1
                ph = np.exp(-2j * np.pi * prob.atom_shift[o, a2] @ prob.q_full[f])
                egw[:, 3 * a1:3 * a1 + 3] = (E[:, 3 * a2:3 * a2 + 3] @ R.T) * ph
            egw *= np.where(om > 1e-9, 1 / np.sqrt(2 * np.maximum(om, 1e-300)), 0.0)[:, None]
            for x in range(3):
                V[x] += egw.conj() @ G[x].T @ egw.T
        v = (V.real / prob.irr_nop[q]).transpose(1, 2, 0)
        v[np.abs(v) < chop] = 0
        S = np.zeros((3, 3))
        for j in range(n):
            for kk in range(n):
                if j == kk or min(om[j], om[kk], lw[q, j], lw[q, kk]) < 1e-9:
                    continue
                t = lw[q, j] + lw[q, kk]
                f0 = 0.5 * (cv(opts.temperature, om[j]) + cv(opts.temperature, om[kk]))
                S += t / (t * t + (om[j] - om[kk]) ** 2) * f0 * np.outer(v[j, kk], v[j, kk])
        star = np.nonzero(prob.full_irr == q + 1)[0]
        for fq in star:
            R = prob.op_cart[abs(prob.full_op[fq]) - 1].reshape(3, 3, order="F")
            K += R @ S @ R.T * prob.irr_weight[q] / prob.volume / len(star)
    Ks = sum(prob.op_cart[o].reshape(3, 3, order="F") @ K @ prob.op_cart[o].reshape(3, 3, order="F").T
             for o in range(prob.n_op))
    return Ks / prob.n_op


@pytest.mark.parametrize("name,grid", [("rocksalt", (4, 4, 4)), ("perovskite", (3, 3, 3))])
def test_offdiag_kronecker_form_equals_sandwich_form(configs, name, grid):
    """The oracle's off-diagonal kappa (kappa.f90:77-306, literal Kronecker form) equals the
    per-operation sandwich form the device kernel uses, and is isotropic for cubic cells."""
    p = Problem.load(configs[name], grid, readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=3)
    lw = orc.full_run(p, opts, QLists.monte_carlo(p, opts), nthreads=4)["linewidth"]
    ko = orc.kappa_offdiag(p, opts, lw)
    ks = _offdiag_sandwich(p, opts, lw)
    assert ko[0, 0] > 0
    np.testing.assert_allclose(ko, ks, rtol=1e-12, atol=1e-12 * np.abs(ko).max())
    np.testing.assert_allclose(np.diag(ko), ko[0, 0], rtol=1e-10)
