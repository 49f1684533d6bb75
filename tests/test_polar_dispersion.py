"""Harmonic stage with polar force constants against the reference's own fixture.

The reference's `tests/phonon_dispersion_relations` runs `phonon_dispersion_relations` on
the polar MgO force constants of `tests/infiles/` and compares every column of
`outfile.dispersion_relations` with numpy's default `assert_allclose` tolerance (rtol 1e-7,
test_dispersion_relations.py:8-15). The file holds the default fcc path
Gamma-X-U|K-Gamma-L, 100 points per segment (lo_phonon_bandstructure_on_path.f90:180-217):
the path length in 1/Bohr, then the six frequencies in THz. This test rebuilds the path,
checks its lengths against the first column and the frequencies against the rest,
through the library's long-range (Ewald, reciprocal-space) dynamical matrix, the
non-analytic term at Gamma along each segment and the natural-isotope masses. Host only.
"""
from pathlib import Path

import numpy as np
import pytest

from tdep_gb300 import scattering as S

GOLD = Path(__file__).parent / "golden" / "mgo"
A_TO_BOHR = 1.0 / 0.52917721067


def _path():
    # Conventional cubic constant from the primitive fcc cell of infile.ucposcar.
    lines = (GOLD / "infile.ucposcar").read_text().split("\n")
    a1 = np.array([float(x) for x in lines[2].split()[:3]]) * float(lines[1].split()[0])
    a = 2.0 * np.max(np.abs(a1)) * A_TO_BOHR
    G, X, U = np.zeros(3), np.array([0, 1, 0.0]), np.array([0.25, 1, 0.25])
    K, L = np.array([0.75, 0.75, 0.0]), np.array([0.5, 0.5, 0.5])
    q, qdir, x, off = [], [], [], 0.0
    for r1, r2 in [(G, X), (X, U), (K, G), (G, L)]:
        d = (r2 - r1) / a
        for i in range(100):
            q.append(r1 / a + d * i / 99)
            qdir.append(d / np.linalg.norm(d))
            x.append(off + np.linalg.norm(d) * i / 99)
        off += np.linalg.norm(d)
    return np.array(q), np.array(qdir), np.array(x)


@pytest.fixture(scope="module")
def polar_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("mgo_polar")
    for f in ("infile.ucposcar", "infile.forceconstant"):
        (d / f).write_bytes((GOLD / f).read_bytes())
    return d


def test_dispersion_matches_reference_fixture(polar_dir):
    ref = np.loadtxt(GOLD / "outfile.dispersion_relations.ref")
    q, qdir, x = _path()
    np.testing.assert_allclose(x, ref[:, 0], rtol=1e-7, atol=1e-12)
    om = S.phonon_frequencies(polar_dir, q, qdir) * S.FREQ_HARTREE_TO_THZ
    np.testing.assert_allclose(om, ref[:, 1:], rtol=1e-7, atol=1e-9)


def test_lo_to_splitting_only_with_direction(polar_dir):
    om_na = S.phonon_frequencies(polar_dir, np.zeros((1, 3)), np.array([[1.0, 0, 0]]))[0]
    om_0 = S.phonon_frequencies(polar_dir, np.zeros((1, 3)), np.zeros((1, 3)))[0]
    thz = S.FREQ_HARTREE_TO_THZ
    # Without the non-analytic term the optical triplet stays degenerate (TO = LO).
    assert np.allclose(om_0[3:] * thz, om_0[3] * thz, rtol=1e-12)
    # With it the longitudinal mode splits off; the cubic cell makes every direction equal.
    assert om_na[5] * thz == pytest.approx(22.5329266, rel=1e-7)
    om_d = S.phonon_frequencies(polar_dir, np.zeros((1, 3)), np.array([[1.0, 1.33, 0.4]]))[0]
    np.testing.assert_allclose(om_d, om_na, rtol=1e-10)
    np.testing.assert_allclose(om_na[:3], 0.0, atol=0)


def test_long_range_term_is_periodic(polar_dir):
    # D(q) and D(q + G) agree: the Ewald sum runs over G + q and the short-range phases
    # use lattice vectors; (1,1,1)/a * 2 is a reciprocal vector of the fcc primitive cell.
    q, _, _ = _path()
    pts = q[[37, 150, 260, 350]]
    lines = (GOLD / "infile.ucposcar").read_text().split("\n")
    a1 = np.array([float(x) for x in lines[2].split()[:3]]) * float(lines[1].split()[0])
    a = 2.0 * np.max(np.abs(a1)) * A_TO_BOHR
    gvec = np.array([1.0, 1.0, 1.0]) / a
    om1 = S.phonon_frequencies(polar_dir, pts)
    om2 = S.phonon_frequencies(polar_dir, pts + gvec)
    np.testing.assert_allclose(om2, om1, rtol=1e-9)
