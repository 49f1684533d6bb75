"""Adjoint of the three-phonon linewidths and kappa_sma with respect to Phi3 on the GB300:
against the oracle's reverse-mode restatement (FP64 reference gradient), against central
finite differences of the device forward pass, and through torch.autograd."""
import numpy as np
import pytest

from oracle import binding as orc
from tdep_gb300 import Options, Problem, QLists, ScatteringRates, device_count

pytestmark = pytest.mark.gpu

ROCKSALT_AMU = (22.99, 35.45)


@pytest.fixture(scope="module", autouse=True)
def _require_gpu(built):
    assert device_count() > 0, "GPU tests need a CUDA device; the GB300 path has no CPU fallback"


@pytest.mark.parametrize("name,grid,it", [("rocksalt", (6, 6, 6), 2), ("perovskite", (4, 4, 4), 6),
                                          ("fcc", (8, 8, 8), 1)])
def test_adjoint_fp64_matches_oracle_gradient(configs, name, grid, it):
    prob = Problem.load(configs[name], grid, readiso=True)
    opts = Options(temperature=300.0, integrationtype=it, sigma=1.0, isotopescattering=False, seed=13)
    lists = QLists.monte_carlo(prob, opts)
    rng = np.random.default_rng(1)
    lw_bar = rng.normal(size=(prob.n_irr, prob.n_mode))
    sr = ScatteringRates(prob)
    sr.generate(opts, lists)
    g = sr.adjoint_fc3(opts, lw_bar)
    again = sr.adjoint_fc3(opts, lw_bar)
    sr.close()
    ref = orc.adjoint_fc3(prob, opts, lists, lw_bar)
    np.testing.assert_allclose(g, ref, rtol=1e-9, atol=1e-10 * np.abs(ref).max())
    np.testing.assert_array_equal(g, again)  # slices are summed in a fixed order


def test_adjoint_mixed_close_to_fp64(configs):
    prob = Problem.load(configs["rocksalt"], (8, 8, 8), readiso=True)
    o64 = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=2)
    o32 = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=2, precision="mixed")
    lists = QLists.monte_carlo(prob, o64)
    sr = ScatteringRates(prob)
    sr.generate(o64, lists)
    sr.kappa(o64, maxiter=0)
    kb = np.zeros((3, 3))
    kb[0, 0] = 1.0
    lw_bar = sr.kappa_sma_vjp(o64, kb)
    g64 = sr.adjoint_fc3(o64, lw_bar)
    g32 = sr.adjoint_fc3(o32, lw_bar)
    sr.close()
    assert np.linalg.norm(g32 - g64) <= 1e-4 * np.linalg.norm(g64)


def test_dkappa_dphi3_against_central_differences(configs):
    """d kappa_xx(300 K) / d Phi3 on rocksalt 16^3 through ThreePhononKappa, against central
    differences with a step of 1e-4 eV/A^3 on 20 seeded random force-constant entries."""
    torch = pytest.importorskip("torch")
    from tdep_gb300.autograd import FC3_EVA3_TO_AU, linewidth_and_kappa, mass_weights

    prob = Problem.load(configs["rocksalt"], (16, 16, 16), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=1)
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    m0 = torch.tensor(prob.fc3_mwm, dtype=torch.float64, requires_grad=True)
    _, ks = linewidth_and_kappa(m0, sr, opts, lists)
    ks[0, 0].backward()
    grad_mwm = m0.grad.numpy()
    w = mass_weights(prob, ROCKSALT_AMU)
    grad_phi = grad_mwm * (w * FC3_EVA3_TO_AU)[:, None]  # d kappa_xx / d Phi3 [a.u. per eV/A^3]
    rng = np.random.default_rng(20)
    h = 1e-4  # eV/A^3
    base = prob.fc3_mwm.copy()
    scale = np.abs(grad_phi).max()
    for _ in range(20):
        t, e = int(rng.integers(prob.n_fc3)), int(rng.integers(27))
        vals = []
        for sgn in (1.0, -1.0):
            m = base.copy()
            m[t, e] += sgn * h * FC3_EVA3_TO_AU * w[t]
            sr.set_fc3(m)
            sr.generate(opts, lists)
            vals.append(sr.kappa(opts, maxiter=0)[0][0, 0])
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - grad_phi[t, e]) <= 2e-6 * scale + 1e-4 * abs(fd), (t, e, fd, grad_phi[t, e])
    sr.close()


def test_autograd_through_a_parameterisation(configs):
    """Phi3 = Phi3_0 + B x for a random basis B: autograd gives B^T (d kappa / d mwm), and a
    central difference along x agrees."""
    torch = pytest.importorskip("torch")
    from tdep_gb300.autograd import linewidth_and_kappa

    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=4)
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    rng = np.random.default_rng(8)
    B = torch.tensor(rng.normal(size=(prob.n_fc3 * 27, 4)) * np.abs(prob.fc3_mwm).max() * 1e-3)
    m0 = torch.tensor(prob.fc3_mwm.reshape(-1))
    x = torch.zeros(4, dtype=torch.float64, requires_grad=True)
    lw, ks = linewidth_and_kappa((m0 + B @ x).reshape(prob.n_fc3, 27), sr, opts, lists)
    loss = ks[0, 0] + 1e3 * lw.sum() * ks[0, 0].detach() / lw.sum().detach()
    loss.backward()
    gx = x.grad.numpy().copy()
    h = 1e-3
    for j in range(4):
        vals = []
        for sgn in (1.0, -1.0):
            xp = torch.zeros(4, dtype=torch.float64)
            xp[j] = sgn * h
            lw2, ks2 = linewidth_and_kappa((m0 + B @ xp).reshape(prob.n_fc3, 27), sr, opts, lists)
            vals.append(float(ks2[0, 0] + 1e3 * lw2.sum() * ks[0, 0].detach() / lw.sum().detach()))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - gx[j]) <= 1e-5 * np.abs(gx).max() + 1e-4 * abs(fd)
    sr.close()


@pytest.mark.parametrize("name,grid,it", [("rocksalt", (6, 6, 6), 2), ("perovskite", (4, 4, 4), 2)])
def test_adjoint_tensor_core_path_matches_fp64(configs, name, grid, it):
    """After a pass on the large-cell path (forced at small n), the adjoint runs per batch on
    the tensor cores (back-contraction with the transposed eigenvector matrices); against the
    FP64 shared-memory adjoint of the same samples, at the mixed-precision bar."""
    prob = Problem.load(configs[name], grid, readiso=True)
    kw = dict(temperature=300.0, integrationtype=it, isotopescattering=False, seed=17)
    o64 = Options(**kw)
    otc = Options(precision="mixed", tensor_cores=True, **kw)
    lists = QLists.monte_carlo(prob, o64)
    rng = np.random.default_rng(4)
    lw_bar = rng.normal(size=(prob.n_irr, prob.n_mode))
    sr = ScatteringRates(prob)
    sr.generate(o64, lists)
    g64 = sr.adjoint_fc3(o64, lw_bar)
    sr.generate(otc, lists)
    gtc = sr.adjoint_fc3(otc, lw_bar)
    assert sr.adjoint_stats["batches_or_ctas"] >= 1
    sr.close()
    assert np.linalg.norm(gtc - g64) <= 1e-3 * np.linalg.norm(g64)


def test_adjoint_large_cell_matches_oracle(configs):
    """30 modes (displaced 2x1x1 supercell, identity only): the large-cell adjoint against the
    oracle's FP64 reverse-mode restatement."""
    prob = Problem.load(configs["supercell"], (3, 3, 3), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=6, precision="mixed",
                   qg3ph=(2, 2, 2))
    lists = QLists.monte_carlo(prob, opts)
    rng = np.random.default_rng(5)
    lw_bar = rng.normal(size=(prob.n_irr, prob.n_mode))
    sr = ScatteringRates(prob)
    sr.generate(opts, lists)
    g = sr.adjoint_fc3(opts, lw_bar)
    sr.close()
    ref = orc.adjoint_fc3(prob, opts, lists, lw_bar)
    assert np.linalg.norm(g - ref) <= 1e-3 * np.linalg.norm(ref)


def test_dkappa_dirreducible_against_central_differences(configs):
    """d kappa_xx / d x for the symmetry-irreducible third-order parameters x (Phi3 = B x,
    Problem.fc3_irreducible) through fc3_from_irreducible and ThreePhononKappa, against
    central differences of the device forward pass in x on 8 seeded parameters; the
    gradient is B^T of the per-entry gradient."""
    torch = pytest.importorskip("torch")
    from tdep_gb300.autograd import fc3_from_irreducible, linewidth_and_kappa

    prob = Problem.load(configs["rocksalt"], (8, 8, 8), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=5)
    lists = QLists.monte_carlo(prob, opts)
    x0, B = prob.fc3_irreducible()
    sr = ScatteringRates(prob)
    x = torch.tensor(x0, dtype=torch.float64, requires_grad=True)
    _, ks = linewidth_and_kappa(fc3_from_irreducible(x, B), sr, opts, lists)
    ks[0, 0].backward()
    g = x.grad.numpy().copy()

    def kxx(xv):
        sr.set_fc3((B @ xv).reshape(-1, 27))
        sr.generate(opts, lists)
        return sr.kappa(opts, maxiter=0)[0][0, 0]

    rng = np.random.default_rng(7)
    for j in rng.choice(x0.size, size=min(8, x0.size), replace=False):
        h = 1e-4 * max(abs(x0[j]), np.abs(x0).max() * 1e-3)
        xp, xm = x0.copy(), x0.copy()
        xp[j] += h
        xm[j] -= h
        fd = (kxx(xp) - kxx(xm)) / (2 * h)
        assert abs(fd - g[j]) <= 1e-5 * np.abs(g).max() + 1e-4 * abs(g[j]), (j, fd, g[j])
    sr.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dkappa_iter_dphi3_against_central_differences(configs, precision):
    """d kappa_iter,xx / d Phi3 (the BTE's adjoint: tdg_kappa_iter_vjp, then tdg_adjoint_fc3
    with the scattering-matrix cotangent) against central differences of the device forward
    pass (generate + iterative kappa converged to 1e-14) on 10 seeded entries, rocksalt 6^3;
    it differs from the kappa_sma gradient, so the Xi term is exercised."""
    prob = Problem.load(configs["rocksalt"], (6, 6, 6), readiso=True)
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=5, precision=precision)
    lists = QLists.monte_carlo(prob, opts)
    sr = ScatteringRates(prob)
    kb = np.zeros((3, 3))
    kb[0, 0] = 1.0
    sr.generate(opts, lists)
    sr.kappa(opts, maxiter=400, tol=1e-14)
    lw_bar = sr.kappa_iter_vjp(opts, kb, maxiter=400, tol=1e-14)
    g = sr.adjoint_fc3(opts, lw_bar)
    sr.kappa(opts, maxiter=0)
    g_sma = sr.adjoint_fc3(opts, sr.kappa_sma_vjp(opts, kb))
    assert np.linalg.norm(g - g_sma) > 1e-3 * np.linalg.norm(g)
    m0 = prob.fc3_mwm.copy()

    def kxx(m):
        sr.set_fc3(m)
        sr.generate(opts, lists)
        return sr.kappa(opts, maxiter=400, tol=1e-14)[1][0, 0]

    rng = np.random.default_rng(11)
    big = np.argsort(-np.abs(g).ravel())[:40]
    picks = rng.choice(big, size=10, replace=False)
    h = 1e-4 * np.abs(m0).max()
    bar = 1e-3 if precision == "fp64" else 2e-2
    for j in picks:
        t, k = divmod(int(j), 27)
        mp, mm = m0.copy(), m0.copy()
        mp[t, k] += h
        mm[t, k] -= h
        fd = (kxx(mp) - kxx(mm)) / (2 * h)
        assert abs(fd - g[t, k]) <= bar * abs(g[t, k]) + 1e-6 * np.abs(g).max(), (t, k, fd, g[t, k])
    sr.close()


@pytest.mark.parametrize("name,grid", [("perovskite", (4, 4, 4)), ("fluorite", (4, 4, 4)), ("l12", (4, 4, 4))])
def test_fused_tensor_core_adjoint_matches_fp64(configs, name, grid):
    """After the tcgen05 fused forward pass (mixed precision, 15, 9 and 12 modes) the adjoint
    runs on the tensor cores too (Psi again, W = G conj(Psi), back-contraction through the E^T
    images, FP32 weights, two-sum float slices): the linewidth adjoint against the FP64 SIMT
    adjoint of the same samples (norm 2e-4), and d kappa_iter,xx / d Phi3 with the
    scattering-matrix term against the FP64 one (norm 1e-3: mixed kappa_iter moves by 1e-6
    and the BTE adjoint amplifies it by the iteration's condition)."""
    prob = Problem.load(configs[name], grid, readiso=True)
    kw = dict(temperature=300.0, integrationtype=2, isotopescattering=False, seed=19)
    o64, o32 = Options(**kw), Options(precision="mixed", **kw)
    lists = QLists.monte_carlo(prob, o64)
    rng = np.random.default_rng(8)
    lw_bar = rng.normal(size=(prob.n_irr, prob.n_mode))
    kb = np.zeros((3, 3))
    kb[0, 0] = 1.0
    sr = ScatteringRates(prob)
    out = {}
    for tag, o in (("fp64", o64), ("mixed", o32)):
        sr.generate(o, lists)
        assert sr.last_path() == (1 if tag == "mixed" else 0)
        g = sr.adjoint_fc3(o, lw_bar)
        sr.kappa(o, maxiter=400, tol=1e-14)
        gi = sr.adjoint_fc3(o, sr.kappa_iter_vjp(o, kb, maxiter=400, tol=1e-14))
        out[tag] = (g, gi)
    sr.close()
    (g64, gi64), (g32, gi32) = out["fp64"], out["mixed"]
    assert np.linalg.norm(g32 - g64) <= 2e-4 * np.linalg.norm(g64)
    assert np.linalg.norm(gi32 - gi64) <= 1e-3 * np.linalg.norm(gi64)
