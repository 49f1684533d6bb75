"""The harmonic stage on the GPU (tdg_problem_load_device: D(q) and dD/dq at the irreducible
points with the polar Ewald sum, batched Jacobi, degenerate-subspace gauge, velocities,
degeneracy tables, unfold onto the mesh) against the host stage (tdg_problem_load), which the
oracle problem and the reference's dispersion fixture pin. The two run the same algorithm,
so they agree to rounding: frequencies, velocities and dD/dq to 1e-10 of their largest
value, the degeneracy tables exactly, and the eigenvectors through the projector onto each
degenerate subspace (the phase of a single eigenvector is the only freedom left). The
scattering pass and kappa then agree to 1e-9."""
from pathlib import Path

import numpy as np
import pytest

from tdep_gb300 import Options, Problem, QLists, ScatteringRates

pytestmark = pytest.mark.gpu

MGO = Path(__file__).parent / "golden" / "mgo"


def _compare(ph, pd):
    np.testing.assert_array_equal(pd.degen, ph.degen)
    np.testing.assert_array_equal(pd.degen_mode, ph.degen_mode)
    np.testing.assert_allclose(pd.omega, ph.omega, rtol=0, atol=1e-10 * np.abs(ph.omega).max())
    np.testing.assert_allclose(pd.vel, ph.vel, rtol=0, atol=1e-10 * np.abs(ph.vel).max())
    np.testing.assert_allclose(pd.irr_dyngrad, ph.irr_dyngrad, rtol=0, atol=1e-10 * np.abs(ph.irr_dyngrad).max())
    n = ph.n_mode
    for q in range(ph.n_full):
        Eh = ph.egv[q, ..., 0] + 1j * ph.egv[q, ..., 1]
        Ed = pd.egv[q, ..., 0] + 1j * pd.egv[q, ..., 1]
        done = np.zeros(n, bool)
        for b in range(n):
            if done[b]:
                continue
            S = ph.degen_mode[q, b, :ph.degen[q, b]] - 1
            done[S] = True
            Ph = Eh[S].T @ Eh[S].conj()
            Pd = Ed[S].T @ Ed[S].conj()
            assert np.abs(Ph - Pd).max() < 1e-9, (q, b)


@pytest.mark.parametrize("name,grid", [("rocksalt", (6, 6, 6)), ("perovskite", (4, 4, 4)), ("fluorite", (4, 4, 4)),
                                       ("fcc", (8, 8, 8)), ("supercell", (3, 3, 3))])
def test_device_harmonic_stage_matches_host(configs, name, grid):
    ph = Problem.load(configs[name], grid, readiso=True)
    pd = Problem.load(configs[name], grid, readiso=True, device=0)
    _compare(ph, pd)


def test_device_harmonic_stage_polar_mgo():
    """The polar MgO force constants (Born charges, dielectric tensor, reciprocal Ewald sum and
    the non-analytic term at Gamma) on a 6^3 mesh."""
    ph = Problem.load(MGO, (6, 6, 6))
    pd = Problem.load(MGO, (6, 6, 6), device=0)
    _compare(ph, pd)


def test_kappa_from_device_harmonic_stage(configs):
    opts = Options(temperature=300.0, integrationtype=2, isotopescattering=False, seed=3, precision="fp64")
    out = []
    for dev in (None, 0):
        p = Problem.load(configs["perovskite"], (4, 4, 4), readiso=True, device=dev)
        lists = QLists.monte_carlo(p, opts)
        sr = ScatteringRates(p)
        lw = sr.generate(opts, lists).copy()
        ks, ki = sr.kappa(opts, maxiter=400, tol=1e-12)
        sr.close()
        out.append((lw, ks, ki))
    (lh, ksh, kih), (ld, ksd, kid) = out
    np.testing.assert_allclose(ld, lh, rtol=1e-9, atol=1e-12 * lh.max())
    np.testing.assert_allclose(ksd, ksh, rtol=1e-9, atol=1e-12 * np.abs(ksh).max())
    # kappa_iter depends on the basis inside degenerate subspaces through
    # symmetrize_and_distribute's od_terms > 0 filter (scattering_threephonon.f90:175); where
    # the velocity operator is degenerate inside the subspace too (zero at Gamma), the gauge
    # rotation is set by rounding and the two stages may pick different bases (the projectors
    # above agree). Measured 2.4e-5 here.
    np.testing.assert_allclose(kid, kih, rtol=1e-3, atol=1e-3 * np.abs(kih).max())
