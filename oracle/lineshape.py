"""ORACLE -- TEST INFRASTRUCTURE ONLY. A numpy restatement of the reference's lineshape
program at the zone centre (single q-point 0 0 0, the defaults of its own test:
tests/lineshape/Makefile `lineshape`), used to pin the three-phonon matrix elements and the
isotope term of the checked-in MgO force constants against the reference's own output
(tests/lineshape/reference/outfile.phonon_self_energy.hdf5). Only tests import it.

Restated (src/lineshape, src/libolle of tdep):
  energy axis     main.f90:117 maxf = 2 (omega_max 1.1 + 3 max(default_smearing)),
                  phonondamping_generation.f90:79 lo_linspace(0, maxf, n_energy = 1200)
  default_smearing type_phonon_dispersions_generation.f90:204-232 (largest gap of the sorted
                  irreducible frequencies per band, at least a fifth of the largest)
  radius          type_qpointmesh_gridgeneration.f90:436-442
  adaptive_sigma  type_qpointmesh_integrationweights.f90:669-688
  smearingparameter type_qpointmesh_integrationweights.f90:639-666
  psi_3ph at Gamma scatteringrates.f90:100-110, 187-270 (scaled eigenvectors), 437-477
                  (zgeru / zgerc / dot_product over the irreducible points, q3 = -q2),
                  pretransform_phi :756-798 (unweighted m; the eigenvectors carry 1/sqrt(m))
  psi_iso         scatteringrates.f90:369-386, isotope_scattering_strength :723-753
  Im Sigma_3ph    phonondamping_gaussian.f90:135-263 (atgamma branch, -it 2)
  Im Sigma_iso    phonondamping_gaussian.f90:1-80 (atgamma branch, -it 2)
  sanity          phonondamping_generation.f90:209-220 (clip at 0, zero ends)
  units           io.f90:73-77 (self-energies and frequencies in THz)
lo_gauss is gottochblandat_calculus.f90:268-288 (zero beyond 8 sigma), lo_planck
gottochblandat_physics.f90:160-186.

Inputs: the problem of the MgO cell on the 26^3 mesh (host stage of this library), the
Gamma-point eigenvectors and frequencies of the fixture's harmonic group (wp = gpoint,
q direction 1 0 0), temperature 300 K, sigma scale 1.
"""
from __future__ import annotations

import math

import numpy as np

HARTREE_TO_EV = 27.21138602
HBAR_EV = 6.582119514e-16
KB_EV = 8.6173303e-5
KB_HARTREE = KB_EV / HARTREE_TO_EV
HBAR_HARTREE = HBAR_EV / HARTREE_TO_EV
FREQ_HARTREE_TO_THZ = 1e-12 / (2 * math.pi) / HBAR_HARTREE
FREQTOL = 1e-5 * 1e-4
SQRT2PI_INV = 0.398942280401433


def lo_gauss(x, mu, sigma):
    x = np.asarray(x, float)
    invsig = 1.0 / sigma
    g = np.exp(-(x - mu) * (x - mu) * 0.5 * invsig * invsig) * SQRT2PI_INV * invsig
    return np.where(np.abs(x - mu) > 8 * sigma, 0.0, g)


def lo_planck(T, om):
    if om < FREQTOL:
        return 0.0
    x = om / (KB_HARTREE * T)
    return 0.0 if x > 1e2 else 1.0 / (math.exp(x) - 1.0)


def linspace(a, b, n):
    x = np.array([a + ((i + 1) * 1.0 - 1.0) / (n * 1.0 - 1.0) * (b - a) for i in range(n)])
    x[0], x[-1] = a, b
    return x


def default_smearing(prob):
    om = prob.omega[prob.irr_full - 1]  # [n_irr, n]
    ds = np.zeros(prob.n_mode)
    for b in range(prob.n_mode):
        x = np.sort(om[:, b])
        ds[b] = np.max(np.abs(np.diff(x))) if x.size > 1 else 0.0
    return np.maximum(ds, ds.max() / 5.0)


def gamma_selfenergy(prob, egv_gamma, om_gamma, temperature=300.0, n_energy=1200, scale=1.0, axis_thz=None):
    """Im Sigma_3ph and Im Sigma_iso [n_mode, n_energy] in THz and the energy axis in THz at
    q = 0, restated from the reference's lineshape (see the module docstring). axis_thz, when
    given, replaces the computed energy axis (its end point, maxf, depends on the smallest
    gaps of the sorted frequencies, which the reference's numerically non-zero acoustic
    frequencies at the mesh's Gamma shift in the seventh digit)."""
    n, na = prob.n_mode, prob.n_atom
    irr = prob.irr_full - 1
    om_irr = prob.omega[irr].copy()
    ds = default_smearing(prob)
    omax = om_irr.max()
    maxf = 2 * (omax * 1.1 + ds.max() * 3)
    axis = linspace(0.0, maxf, n_energy) if axis_thz is None else np.asarray(axis_thz, float) / FREQ_HARTREE_TO_THZ
    n_energy = axis.size
    invf = n_energy / axis[-1]
    radius = (3.0 / prob.volume / prob.n_full / 4.0 / math.pi) ** (1.0 / 3.0)
    reclat = prob.reclat.reshape(3, 3, order="F")
    scaled = reclat * 2 * math.pi / np.asarray(prob.grid)[None, :]

    # Gamma of the mesh is replaced by the consistent Gamma (scatteringrates.f90:255-275)
    gidx = next(i for i in range(prob.n_irr) if np.sum(prob.q_full[irr[i]] ** 2) < 1e-10)
    egv_irr = prob.egv[irr, ..., 0] + 1j * prob.egv[irr, ..., 1]  # [q, b, r]
    egv_sc = egv_irr.copy()
    om_sc = om_irr.copy()
    egv_sc[gidx] = egv_gamma
    om_sc[gidx] = om_gamma
    # (the q-point mesh's own Gamma keeps the grid's eigenvectors for the isotope term)

    def scale_egv(e, om):  # [b, r] -> e / sqrt(omega) as [r, b]; the 1/sqrt(mass) factors of the
        # reference's scaled eigenvectors are carried by the mass-weighted force constants here
        f0 = np.where(om > FREQTOL, 1.0 / np.sqrt(np.where(om > FREQTOL, om, 1.0)), 0.0)
        return (e * f0[:, None]).T

    ugv1 = scale_egv(egv_gamma, om_gamma)
    # pretransform_phi of m / sqrt(m1 m2 m3) (the problem's mass-weighted force constants)
    at = prob.fc3_atoms - 1
    mraw = prob.fc3_mwm
    lv2, lv3 = prob.fc3_lvcart[:, :3], prob.fc3_lvcart[:, 3:]
    idx = np.empty((prob.n_fc3, 27), np.int64)
    for t in range(prob.n_fc3):
        a1, a2, a3 = at[t]
        for k in range(3):
            for j in range(3):
                for i in range(3):
                    ia, ib, ic = 3 * a1 + i, 3 * a2 + j, 3 * a3 + k
                    idx[t, i + 3 * j + 9 * k] = (ia * n + ib) * n + ic

    im3 = np.zeros((n, n_energy))
    imiso = np.zeros((n, n_energy))
    pref3 = math.pi / 16.0
    prefiso = math.pi / 4.0
    vel_irr = prob.vel[irr]
    for q in range(prob.n_irr):
        qv2 = prob.q_full[irr[q]]
        qv3 = -qv2
        iqr = -(lv2 @ qv2 + lv3 @ qv3) * 2 * math.pi
        ph = np.cos(iqr) + 1j * np.sin(iqr)
        ptf = np.zeros(n ** 3, complex)
        np.add.at(ptf, idx.ravel(), (mraw * ph[:, None]).ravel())
        P = ptf.reshape(n, n, n)  # [ia][ib][ic]
        ugv2 = scale_egv(egv_sc[q], om_sc[q])
        # psi(b1,b2,b3) = sum_abc ugv1(a,b1) ugv2(b,b2) conj(ugv2(c,b3)) P[a,b,c]
        psi = np.einsum("abc,ax,by,cz->xyz", P, ugv1, ugv2, ugv2.conj())
        w = prob.irr_weight[q]
        om_q = om_irr[q]
        s = np.array([adaptive_sigma(radius, vel_irr[q, b], ds[b], scale) for b in range(n)])
        for b1 in range(n):
            for b2 in range(n):
                for b3 in range(b2, n):
                    sigma = math.sqrt(s[b2] ** 2 + s[b3] ** 2)
                    om2, om3 = om_q[b2], om_q[b3]
                    plf1 = 1.0 + lo_planck(temperature, om2) + lo_planck(temperature, om3)
                    plf2 = lo_planck(temperature, om3) - lo_planck(temperature, om2)
                    buf = np.zeros(n_energy)
                    ilo, ihi = 10 ** 9, -10 ** 9
                    for c, fac in ((om2 + om3, plf1), (-om2 - om3, -plf1), (om2 - om3, plf2), (-om2 + om3, -plf2)):
                        ii = max(math.floor((c - 4 * sigma) * invf), 1)
                        jj = min(math.ceil((c + 4 * sigma) * invf), n_energy)
                        ilo, ihi = min(ilo, ii), max(ihi, jj)
                        if jj >= ii:
                            buf[ii - 1:jj] += fac * lo_gauss(axis[ii - 1:jj], c, sigma)
                    if ilo < ihi:
                        p23 = abs(psi[b1, b2, b3] * np.conj(psi[b1, b2, b3])) * pref3 * w
                        if b2 == b3:
                            im3[b1, ilo - 1:ihi] += buf[ilo - 1:ihi] * p23
                        else:
                            p32 = abs(psi[b1, b3, b2] * np.conj(psi[b1, b3, b2])) * pref3 * w
                            im3[b1, ilo - 1:ihi] += buf[ilo - 1:ihi] * (p23 + p32)
        # isotope (phonondamping_gaussian.f90:39-66): eigenvectors of the grid at q
        e2 = egv_irr[q]
        for b1 in range(n):
            sig = np.array([smearing_parameter(scaled, vel_irr[q, b], ds[b], scale) for b in range(n)])
            for b2 in range(n):
                lam = isotope_strength(prob, egv_gamma[b1], e2[b2], om_gamma[b1], om_q[b2])
                ii = max(math.floor((om_q[b2] - 4 * sig[b2]) * invf), 1)
                jj = min(math.ceil((om_q[b2] + 4 * sig[b2]) * invf), n_energy)
                if jj >= ii:
                    imiso[b1, ii - 1:jj] += prefiso * w * lo_gauss(axis[ii - 1:jj], om_q[b2], sig[b2]) * lam
    for a in (im3, imiso):
        np.maximum(a, 0.0, out=a)
        a[:, 0] = 0.0
        a[:, -1] = 0.0
    return im3 * FREQ_HARTREE_TO_THZ, imiso * FREQ_HARTREE_TO_THZ, axis * FREQ_HARTREE_TO_THZ


def adaptive_sigma(radius, gradient, default_sigma, scale):
    pre = 2 * math.pi / math.sqrt(2.0)
    sigma = scale * pre * radius * float(np.linalg.norm(gradient))
    sigma = max(default_sigma * 0.25 * scale, sigma)
    return min(default_sigma * 4.0 * scale, sigma)


def smearing_parameter(scaled_recbasis, gradient, sigma, adaptive):
    w = 0.0
    for i in range(3):
        w += float(np.dot(np.abs(gradient), scaled_recbasis[:, i])) ** 2
    w = math.sqrt(w * 0.083333333333) * adaptive
    w = min(w, adaptive * sigma * 4.0)
    return max(w, adaptive * sigma * 0.25)


def isotope_strength(prob, e1, e2, om1, om2):
    f1 = 0.0
    for i in range(prob.n_atom):
        f0 = float(np.sum(np.abs(np.conj(e1[3 * i:3 * i + 3]) * e2[3 * i:3 * i + 3]))) ** 2
        f1 += f0 * prob.mass_disorder[i]
    return f1 * om1 * om2
