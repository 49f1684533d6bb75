"""outfile.thermal_conductivity_grid.hdf5 (type_phonon_dispersions.f90:316-641) written by the
library's own HDF5 writer, read back with the tests' reader of the file format (which also
reads the reference's libhdf5-written fixtures). CPU only: the linewidths and Fn are
synthetic; the GPU test of the reference's identity is in test_gpu_parity.py."""
import numpy as np

from h5read import H5File
from tdep_gb300 import Problem, write_grid_hdf5
from tdep_gb300.scattering import FREQ_HARTREE_TO_THZ, KAPPA_AU_TO_SI

REF_FIXTURES = ["lineshape_self_energy.hdf5", "cumulative_kappa_2023.hdf5"]


def test_reader_reads_the_reference_fixtures():
    """The reader against two files libhdf5 wrote for the reference's tests (chunked,
    deflate-compressed datasets in nested groups): shapes, units and a physical identity."""
    from pathlib import Path

    g = Path(__file__).parent / "golden" / "hdf5"
    f = H5File(g / "lineshape_self_energy.hdf5")
    assert f.attrs["temperature"][0] == 300.0
    im = f.datasets["anharmonic/imaginary_threephonon_selfenergy"]
    assert im.shape == (6, 1200) and f.dataset_attrs["anharmonic/frequency"]["unit"] == "Thz"
    assert np.all(np.diff(f.datasets["anharmonic/frequency"]) > 0)
    # the MgO dynamical matrix at the incident q is Hermitian and its eigenvalues are the
    # squared harmonic frequencies the file lists
    d = f.datasets["harmonic/dynamical_matrix_re"] + 1j * f.datasets["harmonic/dynamical_matrix_im"]
    assert np.abs(d - d.conj().T).max() <= 1e-12 * np.abs(d).max()
    h = f.datasets["harmonic/harmonic_frequencies"]
    assert h.shape == (6,) and np.all(np.diff(h) >= -1e-12)
    c = H5File(g / "cumulative_kappa_2023.hdf5")
    assert c.attrs["number_of_temperatures"][0] == 5
    assert c.datasets["temperature_3/spectral_kappa_vs_frequency_per_mode"].shape == (6, 400)


def test_grid_file_round_trip(configs, tmp_path):
    prob = Problem.load(configs["rocksalt"], (4, 4, 4), readiso=True)
    rng = np.random.default_rng(0)
    n, T = prob.n_mode, 300.0
    lw = rng.uniform(1e-7, 1e-6, (prob.n_irr, n))
    fn = rng.normal(size=(prob.n_irr, n, 3))
    path = write_grid_hdf5(tmp_path / "outfile.thermal_conductivity_grid.hdf5", prob, T, lw, fn)
    f = H5File(path)
    assert f.attrs["number_of_atoms"][0] == 2 and f.attrs["number_of_bands"][0] == n
    assert f.attrs["number_of_qpoints"][0] == prob.n_full and f.attrs["meshtype"] == "FFT"
    assert f.attrs["temperature"][0] == T
    ds = f.datasets
    np.testing.assert_array_equal(ds["qpoints"], prob.q_full)
    hz = FREQ_HARTREE_TO_THZ * 1e12 * 2 * np.pi
    np.testing.assert_allclose(ds["frequencies"], prob.omega * hz, rtol=1e-15)
    li = prob.full_irr - 1
    np.testing.assert_allclose(ds["linewidths"], lw[li] * hz, rtol=1e-15)
    np.testing.assert_allclose(ds["lifetimes"], 0.5 / (lw[li] * hz), rtol=1e-15)
    np.testing.assert_array_equal(ds["eigenvectors_re"], prob.egv[..., 0])
    assert f.dataset_attrs["thermal_conductivity"] == {"unit": "W/mK", "dimensions": "q-vector,mode,xyz,xyz"}
    # per-mode conductivity: f0 (R Fn omega/T) x (R v) / (V kB T), the Fn prefactor of main.f90:321-327
    kb = 8.6173303e-5 / 27.21138602
    kap = ds["thermal_conductivity"]
    assert kap.shape == (prob.n_full, n, 3, 3)
    omin = prob.omega[prob.irr_full - 1][prob.omega[prob.irr_full - 1] > 1e-9].min()
    for i in (0, 7, prob.n_full - 1):
        l, k = li[i], prob.full_op[i]
        R = prob.op_cart[abs(k) - 1].reshape(3, 3, order="F") * np.sign(k)
        fi = prob.irr_full[l] - 1
        for j in range(n):
            om = prob.omega[fi, j]
            if prob.omega[i, j] < 0.5 * omin:
                assert not kap[i, j].any()
                continue
            nb = 1.0 / np.expm1(om / (kb * T))
            u = R @ fn[l, j] * om / T
            w = R @ prob.vel[fi, j]
            exp = om * (nb + 1) * nb * np.outer(u, w) / (prob.volume * kb * T) * KAPPA_AU_TO_SI
            np.testing.assert_allclose(kap[i, j], exp.T, rtol=1e-12, atol=1e-14 * np.abs(exp).max())
