"""The library's host stage (tdg_problem_load: readers, symmetry search, FFT mesh, wedge,
little groups, phonons, degeneracies) against the oracle's own numpy construction from the
same input files (oracle/problem.py), which shares no code with it. Integer tables exactly
(the operation that maps an irreducible point onto a mesh point is compared as a matrix,
since equivalent operations may be numbered differently), frequencies and velocities to
1e-10. CPU only."""
import numpy as np
import pytest

from oracle.problem import OracleProblem
from tdep_gb300 import Problem


@pytest.mark.parametrize("name,grid", [("fcc", (8, 8, 8)), ("rocksalt", (6, 6, 6)), ("perovskite", (4, 4, 4)),
                                       ("fluorite", (4, 4, 4)), ("l12", (4, 4, 4)),
                                       # unequal dimensions: only the operations that map the
                                       # mesh onto itself connect its points
                                       ("rocksalt", (6, 5, 4)), ("perovskite", (4, 3, 2))])
def test_host_stage_against_the_oracle_problem(configs, name, grid):
    p = Problem.load(configs[name], grid, readiso=True)
    o = OracleProblem(configs[name], grid)
    # readers
    assert p.n_atom == o.na and p.n_op == len(o.ops)
    np.testing.assert_allclose(p.latvec.reshape(3, 3, order="F"), o.lat, rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(p.mass_disorder, o.disorder, atol=1e-15)
    assert p.n_fc3 == len(o.fc3)
    mine = sorted((t[0], t[1], t[2], *np.round(t[3]).astype(int), *np.round(t[4]).astype(int)) for t in o.fc3)
    theirs = sorted(tuple(int(x) for x in (*(p.fc3_atoms[t] - 1), *p.fc3_lv[t])) for t in range(p.n_fc3))
    assert mine == theirs
    # force-constant values, file order (the library parses the numbers itself; the two
    # mass-weighting orders differ by an ulp or two)
    ism = 1.0 / np.sqrt(o.mass)
    ref = np.array([t[5] * ism[t[0]] * ism[t[1]] * ism[t[2]] for t in o.fc3])
    np.testing.assert_array_equal(p.fc3_atoms - 1, [t[:3] for t in o.fc3])
    np.testing.assert_allclose(p.fc3_mwm, ref, rtol=0, atol=1e-15 * np.abs(ref).max())
    # the same point group (as a set of Cartesian rotations)
    R = {tuple(np.round(p.op_cart[k].reshape(3, 3, order="F"), 8).ravel()) for k in range(p.n_op)}
    Ro = {tuple(np.round(o.lat @ W @ np.linalg.inv(o.lat), 8).ravel()) for W, _ in o.ops}
    assert R == Ro
    # mesh and wedge: the same irreducible points (smallest index of each orbit), weights,
    # orbit membership and little-group sizes
    np.testing.assert_array_equal(p.irr_full - 1, o.irr_full)
    np.testing.assert_array_equal(p.full_irr - 1, o.full_irr)
    np.testing.assert_allclose(p.irr_weight, o.irr_weight, rtol=1e-14)
    np.testing.assert_array_equal(p.irr_nop, o.irr_nop)
    # every mesh point is the image of its irreducible point under its stated operation
    inv_rec = p.inv_reclat.reshape(3, 3, order="F")
    for q in range(p.n_full):
        op = p.full_op[q]
        m = p.op_cart[abs(op) - 1].reshape(3, 3, order="F") * np.sign(op)
        v = inv_rec @ (m @ p.q_full[p.irr_full[p.full_irr[q] - 1] - 1] - p.q_full[q])
        assert np.abs(v - np.round(v)).max() < 1e-8
    # q-points equal modulo reciprocal lattice vectors
    d = inv_rec @ (p.q_full - o.q_cart).T
    assert np.abs(d - np.round(d)).max() < 1e-10
    # phonons
    scale = p.omega.max()
    np.testing.assert_allclose(p.omega, o.omega, rtol=0, atol=1e-10 * scale)
    vs = np.abs(o.vel).max()
    np.testing.assert_allclose(p.vel, o.vel, rtol=0, atol=1e-10 * vs)
    np.testing.assert_array_equal(p.degen, o.degen)


@pytest.mark.parametrize("name,grid,it", [("rocksalt", (6, 6, 6), 2), ("perovskite", (4, 4, 4), 1)])
def test_oracle_runs_on_its_own_problem(configs, name, grid, it):
    """The oracle's scattering and kappa computed from its own problem equal those computed
    from the library's problem: linewidths and kappa_SMA do not depend on the eigenvector
    gauge or on which of two equivalent operations numbers a mesh point (rtol 1e-10).
    kappa_iter does, through the reference's own algorithm: symmetrize_and_distribute
    averages only the entries of a mode that are positive (scattering_threephonon.f90:175),
    and how a degenerate subspace splits its entries among its modes depends on the basis
    chosen inside it (here numpy's, in the library a Jacobi rotation, in the reference LAPACK's
    zheev rotated from the irreducible point), so the bar is 2e-2."""
    from oracle import binding as orc
    from tdep_gb300 import Options

    opts = Options(temperature=300.0, integrationtype=it, sigma=1.0, isotopescattering=False, seed=7,
                   precision="fp64")
    p = Problem.load(configs[name], grid, readiso=True)
    q = OracleProblem(configs[name], grid).to_problem()
    lp, lq = orc.mc_qlists(p, opts), orc.mc_qlists(q, opts)
    np.testing.assert_array_equal(lp.list3, lq.list3)
    rp, rq = orc.full_run(p, opts, lp), orc.full_run(q, opts, lq)
    s = np.abs(rp["linewidth"]).max()
    np.testing.assert_allclose(rq["linewidth"], rp["linewidth"], rtol=1e-10, atol=1e-13 * s)
    np.testing.assert_allclose(rq["kappa_sma"], rp["kappa_sma"], rtol=1e-10, atol=1e-12 * np.abs(rp["kappa_sma"]).max())
    np.testing.assert_allclose(rq["kappa_iter"], rp["kappa_iter"], rtol=2e-2, atol=2e-2 * np.abs(rp["kappa_iter"]).max())


@pytest.mark.parametrize("name,grid", [("rocksalt", (6, 6, 6)), ("perovskite", (4, 4, 4)), ("fluorite", (4, 4, 4))])
def test_unfolded_eigenvectors_diagonalise_the_mesh(configs, name, grid):
    """Only the irreducible points are diagonalised; every other mesh point takes its
    eigenvectors rotated from its irreducible point (lo_eigenvector_transformation_matrix,
    conjugated under time reversal), its frequencies copied and its velocities rotated, as
    type_phonon_dispersions_generation.f90:117-170 does. The rotated eigenvectors must be
    orthonormal eigenvectors of the oracle's own D(q) at that point (residual below 1e-10 of
    the largest eigenvalue) and the frequencies exactly those of the irreducible point."""
    p = Problem.load(configs[name], grid, readiso=True)
    o = OracleProblem(configs[name], grid)
    n = p.n_mode
    lam = (p.omega.max()) ** 2
    for q in range(p.n_full):
        D, _ = o._dyn(o.q_cart[q])
        E = (p.egv[q, ..., 0] + 1j * p.egv[q, ..., 1]).T  # columns are modes
        w = np.sign(p.omega[q]) * p.omega[q] ** 2
        assert np.abs(D @ E - E * w[None, :]).max() < 1e-10 * lam
        assert np.abs(E.conj().T @ E - np.eye(n)).max() < 1e-12
        i = p.irr_full[p.full_irr[q] - 1] - 1
        np.testing.assert_array_equal(p.omega[q], p.omega[i])
        np.testing.assert_array_equal(p.degen[q], p.degen[i])
