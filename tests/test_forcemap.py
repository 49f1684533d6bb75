"""Symmetry-irreducible parameterisation of the third-order force constants (tdg_fc3_irreducible,
after the reference's forcemap, type_forcemap_returntensors.f90:250-362). CPU only."""
import numpy as np
import pytest

from tdep_gb300 import Problem


@pytest.mark.parametrize("name", ["fcc", "rocksalt", "perovskite", "fluorite", "l12"])
def test_symmetric_constants_are_spanned(configs, name):
    """The synthetic constants (pair potentials, symmetric by construction) are B x exactly,
    with far fewer parameters than entries."""
    prob = Problem.load(configs[name], (4, 4, 4))
    x, B = prob.fc3_irreducible()
    m = prob.fc3_mwm.ravel()
    np.testing.assert_allclose(B @ x, m, rtol=0, atol=1e-12 * np.abs(m).max())
    assert B.shape == (prob.n_fc3 * 27, x.size) and x.size < prob.n_fc3 * 27 / 10


@pytest.mark.parametrize("name", ["rocksalt", "perovskite"])
def test_every_parameter_vector_is_symmetric(configs, name):
    """Every member's block is an orthogonal image of its representative's orthonormal
    columns, so B^T B is diagonal with the orbit sizes; the projector B (B^T B)^-1 B^T then
    leaves B z unchanged for any z and maps arbitrary constants onto symmetric ones that B
    spans again."""
    prob = Problem.load(configs[name], (4, 4, 4))
    x, B = prob.fc3_irreducible()
    G = (B.T @ B).toarray()
    d = np.diag(G)
    assert np.abs(G - np.diag(d)).max() < 1e-10 * d.max()
    assert np.all(np.abs(d - np.round(d)) < 1e-10) and d.min() >= 1
    rng = np.random.default_rng(1)
    y = B @ rng.normal(size=x.size)
    np.testing.assert_allclose(B @ ((B.T @ y) / d), y, atol=1e-12 * np.abs(y).max())
    u = rng.normal(size=B.shape[0])
    s1 = B @ ((B.T @ u) / d)
    np.testing.assert_allclose(B @ ((B.T @ s1) / d), s1, atol=1e-12 * np.abs(s1).max())


def test_supercell_without_symmetry(configs):
    """With the identity alone only the site permutations tie triplets together."""
    prob = Problem.load(configs["supercell"], (2, 2, 2))
    assert prob.n_op == 1
    x, B = prob.fc3_irreducible()
    np.testing.assert_allclose(B @ x, prob.fc3_mwm.ravel(), atol=1e-12 * np.abs(prob.fc3_mwm).max())
