"""Pin of the three-phonon matrix elements against the reference's own output: the
imaginary three-phonon and isotope self-energies of MgO at the zone centre that the
reference's lineshape program wrote for its test (tests/lineshape/reference/
outfile.phonon_self_energy.hdf5, copied to tests/golden/hdf5/), from the checked-in polar
force constants on its default 26x26x26 mesh at 300 K, against the oracle's restatement of
that computation (oracle/lineshape.py) on this library's host stage (readers, symmetry,
mesh, polar dynamical matrix, natural-isotope masses). CPU only.

The per-mode spectra of degenerate zone-centre modes depend on the eigenvector basis chosen
inside each degenerate subspace, so they are compared summed over each degenerate set (the
reference's own Gamma eigenvectors from the file are used for q1).

Bars. The integral of each spectrum over the energy axis and its first moment do not depend
on the Gaussian widths: they pin |Psi|^2, the weights and the occupations, rtol 1e-7 (they
agree to 3e-9). Point by point the spectra agree to 2e-3 of their largest value: the
reference's mesh frequencies at finite q differ from its dispersion program's (to which this
library's harmonic stage is pinned within 5e-10) by up to about 2e-7 relative -- the end of
the file's energy axis, 2 (1.1 omega_max + 3 max(default_smearing)), implies an LA frequency
1.6e-7 higher at q = b3/26 -- which moves the narrowest Gaussians (0.057 THz) enough to
change single energy points at that level. The energy axis is taken from the file."""
from pathlib import Path

import numpy as np
import pytest

from h5read import H5File
from oracle import lineshape as ls
from tdep_gb300 import Problem

GOLDEN = Path(__file__).parent / "golden"


@pytest.fixture(scope="module")
def fixture_and_oracle(built):
    f = H5File(GOLDEN / "hdf5" / "lineshape_self_energy.hdf5")
    prob = Problem.load(GOLDEN / "mgo", (26, 26, 26))
    assert list(f.datasets["qmesh/grid_dimensions"]) == [26, 26, 26]
    e = f.datasets["harmonic/eigenvectors_re"] + 1j * f.datasets["harmonic/eigenvectors_im"]  # [b][r]
    om = f.datasets["harmonic/harmonic_frequencies"] / ls.FREQ_HARTREE_TO_THZ
    im3, imiso, axis = ls.gamma_selfenergy(prob, e, om, temperature=float(f.attrs["temperature"][0]),
                                           axis_thz=f.datasets["anharmonic/frequency"])
    return f, prob, om, im3, imiso, axis


def _groups(om):
    """Sets of degenerate modes at Gamma (frequencies within 1e-9 relative)."""
    out, cur = [], [0]
    for b in range(1, om.size):
        if abs(om[b] - om[cur[-1]]) <= 1e-9 * max(abs(om[b]), 1e-12):
            cur.append(b)
        else:
            out.append(cur)
            cur = [b]
    out.append(cur)
    return out


def test_energy_axis_and_gamma_frequencies(fixture_and_oracle):
    f, prob, om, im3, imiso, axis = fixture_and_oracle
    # the axis computed from this library's mesh frequencies, against the file's (see above)
    maxf = 2 * (prob.omega[prob.irr_full - 1].max() * 1.1 + 3 * ls.default_smearing(prob).max())
    np.testing.assert_allclose(maxf * ls.FREQ_HARTREE_TO_THZ, f.datasets["anharmonic/frequency"][-1], rtol=1e-7)
    # the library's polar dynamical matrix at Gamma along 1 0 0 against the file's frequencies
    from tdep_gb300.scattering import phonon_frequencies

    mine = phonon_frequencies(GOLDEN / "mgo", np.zeros((1, 3)), np.array([[1.0, 0.0, 0.0]]))[0]
    np.testing.assert_allclose(mine[3:], om[3:], rtol=1e-9)


def _compare(mine, ref, om, ax):
    for g in _groups(om):
        a, b = mine[g].sum(0), ref[g].sum(0)
        scale = np.abs(b).max()
        if scale == 0.0:
            assert np.abs(a).max() == 0.0
            continue
        np.testing.assert_allclose(a.sum(), b.sum(), rtol=1e-7, err_msg=f"integral of modes {g}")
        np.testing.assert_allclose((a * ax).sum() / a.sum(), (b * ax).sum() / b.sum(), rtol=1e-7,
                                   err_msg=f"first moment of modes {g}")
        np.testing.assert_allclose(a, b, rtol=0, atol=2e-3 * scale, err_msg=f"spectrum of modes {g}")


def test_threephonon_selfenergy_matches_the_reference(fixture_and_oracle):
    f, prob, om, im3, imiso, axis = fixture_and_oracle
    ref = f.datasets["anharmonic/imaginary_threephonon_selfenergy"]
    assert np.abs(ref).max() > 0
    _compare(im3, ref, om, f.datasets["anharmonic/frequency"])


def test_isotope_selfenergy_matches_the_reference(fixture_and_oracle):
    f, prob, om, im3, imiso, axis = fixture_and_oracle
    ref = f.datasets["anharmonic/imaginary_isotope_selfenergy"]
    assert np.abs(ref).max() > 0
    _compare(imiso, ref, om, f.datasets["anharmonic/frequency"])
