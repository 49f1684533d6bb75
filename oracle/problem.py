"""ORACLE -- TEST INFRASTRUCTURE ONLY. The harmonic problem of the scattering path built
from the input files with numpy alone, independently of this library's host stage, so that
the tests can check the library's readers, symmetry search, mesh and phonons
(tdg_problem_load) against it. Non-polar force constants only (the polar long-range term
is pinned by the reference's own dispersion fixture instead). Only tests import it.

Restated (tdep, src/libolle):
  infile.ucposcar            type_crystalstructure_io.f90:9 (VASP5 layout, lattice in A)
  infile.isotopes            type_crystalstructure_io.f90:921-957 (per atom: count, then
                             concentration and mass per isotope; mean mass, disorder)
  infile.forceconstant       type_forceconstant_secondorder_io.f90:136-200 (per atom: pairs
                             with the neighbour index, its fractional lattice vector and the
                             3x3 block in eV/A^2)
  infile.forceconstant_thirdorder  type_forceconstant_thirdorder.f90:243-311
  space group                lattice rotations (integer matrices that keep the metric) with a
                             fractional translation that maps every atom onto one of its species
  FFT mesh                   type_qpointmesh_gridgeneration.f90:117-123 (row-major index),
                             :297-380 (irreducible points = smallest index of an orbit under the
                             rotations and, with time reversal, their negatives)
  little groups              type_qpointmesh.f90:660-700 (rotations that keep q modulo G)
  dynamical matrix           type_forceconstant_secondorder_dynamicalmatrix.f90:484-650
                             (short-range part, mass-weighted, phases exp(i 2 pi q.R), row
                             (a2, j) and column (a1, i) for the block m(i, j) of a pair a1 -> a2)
  velocities                 :167-200 and the degenerate-subspace rule :313-360 (mean over the
                             subspace per direction), derivative with respect to 2 pi q
  degeneracy                 type_phonon_dispersions.f90:1190-1212 (modes within lo_freqtol)
"""
from __future__ import annotations

import itertools
from pathlib import Path

import numpy as np

A_TO_BOHR = 1.0 / 0.52917721067
EV_TO_HA = 1.0 / 27.21138602
AMU_TO_EMU = 1.660539040e-27 / 9.10938356e-31
FREQTOL = 1e-9
SQTOL = 1e-10


def _lines(path):
    return [ln for ln in Path(path).read_text().splitlines()]


def read_poscar(path):
    ln = _lines(path)
    scale = float(ln[1].split()[0])
    lat = np.array([[float(x) for x in ln[2 + i].split()[:3]] for i in range(3)]).T * scale * A_TO_BOHR
    symbols = ln[5].split()
    counts = [int(x) for x in ln[6].split()]
    cart = ln[7].strip().lower().startswith(("c", "k"))
    frac = []
    for i in range(sum(counts)):
        v = np.array([float(x) for x in ln[8 + i].split()[:3]])
        frac.append(np.linalg.solve(lat, v * scale * A_TO_BOHR) if cart else v)
    species = [s for s, c in zip(symbols, counts) for _ in range(c)]
    return lat, np.array(frac), species


def read_isotopes(path, na):
    tok = Path(path).read_text().split()
    p, mass, disorder = 0, np.zeros(na), np.zeros(na)
    for a in range(na):
        k = int(tok[p])
        p += 1
        c = np.array([float(tok[p + 2 * i]) for i in range(k)])
        m = np.array([float(tok[p + 2 * i + 1]) for i in range(k)]) * AMU_TO_EMU
        p += 2 * k
        c = c / c.sum()
        mean = float(np.dot(c, m))
        mass[a] = mean
        disorder[a] = float(np.dot(c, (m - mean) ** 2)) / mean ** 2
    return mass, disorder


def read_fc2(path, na):
    """[(a, b, lv_frac (3,), block 3x3 in Hartree/Bohr^2)]."""
    ln = _lines(path)
    p = 2
    pairs = []
    conv = EV_TO_HA / A_TO_BOHR ** 2
    for a in range(na):
        nn = int(ln[p].split()[0])
        p += 1
        for _ in range(nn):
            b = int(ln[p].split()[0]) - 1
            lv = np.array([float(x) for x in ln[p + 1].split()[:3]])
            m = np.array([[float(x) for x in ln[p + 2 + i].split()[:3]] for i in range(3)]) * conv
            pairs.append((a, b, lv, m))
            p += 5
    return pairs


def read_fc3(path, na):
    """[(a1, a2, a3, lv2_frac, lv3_frac, m (27,) at i + 3j + 9k, Hartree/Bohr^3)]."""
    ln = _lines(path)
    p = 2
    out = []
    conv = EV_TO_HA / A_TO_BOHR ** 3
    for a in range(na):
        nt = int(ln[p].split()[0])
        p += 1
        for _ in range(nt):
            at = [int(ln[p + i].split()[0]) - 1 for i in range(3)]
            lvs = [np.array([float(x) for x in ln[p + 3 + i].split()[:3]]) for i in range(3)]
            m = np.zeros(27)
            for r in range(9):  # row r: (i, j) = (r // 3, r % 3), values over k
                vals = [float(x) for x in ln[p + 6 + r].split()[:3]]
                i, j = r // 3, r % 3
                for k in range(3):
                    m[i + 3 * j + 9 * k] = vals[k] * conv
            out.append((at[0], at[1], at[2], lvs[1] - lvs[0], lvs[2] - lvs[0], m))
            p += 15
    return out


def space_group(lat, frac, species, tol=1e-5):
    """[(W integer 3x3 acting on fractional coordinates, t fractional translation)], the
    identity first."""
    G = lat.T @ lat
    rots = []
    for e in itertools.product((-1, 0, 1), repeat=9):
        W = np.array(e, float).reshape(3, 3)
        if abs(abs(np.linalg.det(W)) - 1) > 1e-8:
            continue
        if np.abs(W.T @ G @ W - G).max() > tol * np.abs(G).max():
            continue
        rots.append(W)
    rots.sort(key=lambda W: (0 if np.array_equal(W, np.eye(3)) else 1))
    ops = []
    for W in rots:
        for b in range(len(species)):
            if species[b] != species[0]:
                continue
            t = frac[b] - W @ frac[0]
            ok = True
            for a in range(len(species)):
                img = W @ frac[a] + t
                hit = False
                for c in range(len(species)):
                    if species[c] != species[a]:
                        continue
                    d = img - frac[c]
                    d -= np.round(d)
                    if np.abs(d).max() < tol:
                        hit = True
                        break
                if not hit:
                    ok = False
                    break
            if ok:
                ops.append((W, t - np.floor(t + tol)))
                break
    return ops


class OracleProblem:
    """Mesh, wedge, little groups, frequencies, velocities and degeneracies of a non-polar
    cell on a Gamma-centred grid."""

    def __init__(self, directory, grid, readiso=True, timereversal=True):
        d = Path(directory)
        self.lat, self.frac, self.species = read_poscar(d / "infile.ucposcar")
        self.na = len(self.species)
        self.n = 3 * self.na
        if not readiso:
            raise ValueError("the oracle problem takes its masses from infile.isotopes")
        self.mass, self.disorder = read_isotopes(d / "infile.isotopes", self.na)
        self.fc2 = read_fc2(d / "infile.forceconstant", self.na)
        self.fc3 = read_fc3(d / "infile.forceconstant_thirdorder", self.na)
        self.reclat = np.linalg.inv(self.lat).T  # columns b_j with a_i . b_j = delta_ij
        self.ops = space_group(self.lat, self.frac, self.species)
        self.grid = tuple(int(g) for g in grid)
        self._mesh(timereversal)
        self._phonons()

    # ---------------------------------------------------------------- mesh
    def _mesh(self, timereversal):
        g = np.array(self.grid)
        N = int(np.prod(g))
        idx = np.arange(N)
        ijk = np.stack([idx // (g[1] * g[2]), (idx // g[2]) % g[1], idx % g[2]], 1)
        self.gfrac = ijk / g
        # rotation of fractional reciprocal coordinates: q' = (W^-T) q
        rrot = [np.round(np.linalg.inv(W).T).astype(int) for W, _ in self.ops]
        self.rrot = rrot

        def index_of(v):
            # mesh index of each fractional point, -1 where it is not on the mesh (an
            # operation that does not map a mesh with unequal dimensions onto itself)
            x = v * g
            w = np.round(x).astype(int)
            on = np.all(np.abs(x - w) < 1e-6, axis=1)
            w = w % g
            return np.where(on, (w[:, 0] * g[1] + w[:, 1]) * g[2] + w[:, 2], -1)

        imgs = np.stack([index_of((ijk / g) @ R.T) for R in rrot], 1)  # [N, nop]
        self.imgs = imgs
        rev = index_of(-(ijk / g)) if timereversal else None
        irr_of = np.full(N, -1)
        irr_list = []
        for i in range(N):
            if irr_of[i] >= 0:
                continue
            k = len(irr_list)
            irr_list.append(i)
            orbit = set(x for x in imgs[i].tolist() if x >= 0)
            if timereversal:
                orbit |= set(rev[list(orbit)].tolist())
            for j in orbit:
                if irr_of[j] < 0:
                    irr_of[j] = k
        self.irr_full = np.array(irr_list)
        self.full_irr = irr_of
        cnt = np.bincount(irr_of, minlength=len(irr_list))
        self.irr_weight = cnt / N
        self.irr_nop = np.array([int(np.sum(imgs[i] == i)) for i in irr_list])
        self.q_cart = self.gfrac @ self.reclat.T

    # ---------------------------------------------------------------- phonons
    def _pairs(self):
        if not hasattr(self, "_pa"):
            a = np.array([t[0] for t in self.fc2])
            b = np.array([t[1] for t in self.fc2])
            r = np.array([self.lat @ t[2] for t in self.fc2])
            inv = 1.0 / np.sqrt(self.mass)
            blk = np.array([t[3] for t in self.fc2]) * (inv[a] * inv[b])[:, None, None]
            rows = (3 * a[:, None, None] + np.arange(3)[None, :, None]) * np.ones((1, 1, 3), int)
            cols = (3 * b[:, None, None] + np.arange(3)[None, None, :]) * np.ones((1, 3, 1), int)
            self._pa = (r, blk, rows.ravel(), cols.ravel())
        return self._pa

    def _dyn(self, q):
        n = self.n
        r, blk, rows, cols = self._pairs()
        ph = np.exp(2j * np.pi * (r @ q))
        vals = (blk * ph[:, None, None]).ravel()
        D = np.zeros((n, n), complex)
        np.add.at(D, (rows, cols), vals)
        G = np.zeros((3, n, n), complex)
        for x in range(3):
            np.add.at(G[x], (rows, cols), (1j * np.repeat(r[:, x], 9)) * vals)
        # the reference's layout: row (a2, j), column (a1, i) for the pair block m(i, j) of
        # atom a1 and its neighbour a2 (type_forceconstant_secondorder_dynamicalmatrix.f90)
        D = D.T
        G = np.transpose(G, (0, 2, 1))
        D = 0.5 * (D + D.conj().T)
        return D, G

    def _phonons(self):
        N, n = len(self.gfrac), self.n
        self.omega = np.zeros((N, n))
        self.egv = np.zeros((N, n, n), complex)
        self.vel = np.zeros((N, n, 3))
        self.degen = np.zeros((N, n), int)
        for q in range(N):
            D, G = self._dyn(self.q_cart[q])
            w, e = np.linalg.eigh(D)
            if np.sum(self.q_cart[q] ** 2) < SQTOL:
                w[np.argsort(np.abs(w))[:3]] = 0.0
            om = np.sign(w) * np.sqrt(np.abs(w))
            o = np.argsort(om, kind="stable")
            om, e = om[o], e[:, o]
            hf = np.array([[np.real(np.vdot(e[:, b], G[x] @ e[:, b])) for x in range(3)] for b in range(n)])
            sub = -np.ones(n, int)
            ns = 0
            for b in range(n):
                for a in range(b):
                    if abs(om[a] - om[b]) < FREQTOL:
                        sub[b] = sub[a]
                        break
                if sub[b] < 0:
                    sub[b] = ns
                    ns += 1
            for b in range(n):
                mean = hf[sub == sub[b]].mean(0)
                self.vel[q, b] = mean / (2 * om[b]) if om[b] > FREQTOL else 0.0
                self.degen[q, b] = int(np.sum(np.abs(om - om[b]) < FREQTOL))
            self.omega[q] = om
            self.egv[q] = e.T  # [mode b][component r]

    # ---------------------------------------------------------------- as a tdg_problem
    def to_problem(self):
        """The oracle's own problem in the layout of tdg_problem (a tdep_gb300 Problem made
        from numpy arrays; nothing of the library's host stage is called). The operation that
        maps an irreducible point onto a mesh point is the first in the oracle's operation
        order, time-reversed ones after the others, as type_qpointmesh_gridgeneration.f90:
        364-381 picks it."""
        from tdep_gb300.scattering import Problem

        g = np.array(self.grid)
        N, n, nop, nirr = len(self.gfrac), self.n, len(self.ops), len(self.irr_full)
        Li = np.linalg.inv(self.lat)
        op_cart = np.array([(self.lat @ W @ Li).ravel(order="F") for W, _ in self.ops])
        op_recfrac = np.array([R.ravel(order="F") for R in self.rrot])
        full_op = np.zeros(N, int)
        gi = np.round(self.gfrac * g).astype(int)

        def index_of(v):
            # mesh index of the fractional point v, -1 off the mesh
            x = v * g
            w = np.round(x).astype(int)
            if np.any(np.abs(x - w) > 1e-6):
                return -1
            w = w % g
            return (w[0] * g[1] + w[1]) * g[2] + w[2]

        for k, i in enumerate(self.irr_full):
            for j, R in enumerate(self.rrot):
                t = index_of(R @ (gi[i] / g))
                if t >= 0 and full_op[t] == 0 and self.full_irr[t] == k:
                    full_op[t] = j + 1
            for j, R in enumerate(self.rrot):
                t = index_of(-(R @ (gi[i] / g)))
                if t >= 0 and full_op[t] == 0 and self.full_irr[t] == k:
                    full_op[t] = -(j + 1)
        irr_ops = np.zeros((nirr, nop), int)
        for k, i in enumerate(self.irr_full):
            ops = [j + 1 for j in range(nop) if self.imgs[i, j] == i]
            irr_ops[k, :len(ops)] = ops
        degen_mode = np.zeros((N, n, n), int)
        for q in range(N):
            close = np.abs(self.omega[q][:, None] - self.omega[q][None, :]) < FREQTOL  # [b, c]
            for b in range(n):
                mates = np.nonzero(close[b])[0] + 1
                degen_mode[q, b, :mates.size] = mates
        nt = len(self.fc3)
        at = np.array([[t[0], t[1], t[2]] for t in self.fc3])
        lv = np.array([np.concatenate([np.round(t[3]), np.round(t[4])]) for t in self.fc3]).astype(int)
        lvcart = np.array([np.concatenate([self.lat @ t[3], self.lat @ t[4]]) for t in self.fc3])
        mw = 1.0 / np.sqrt(self.mass[at[:, 0]] * self.mass[at[:, 1]] * self.mass[at[:, 2]])
        mwm = np.array([t[5] for t in self.fc3]) * mw[:, None]
        egv = np.stack([self.egv.real, self.egv.imag], -1)
        return Problem(n_atom=self.na, n_mode=n, n_op=nop, n_full=N, n_irr=nirr, n_fc3=nt, n_fc4=0,
                       latvec=self.lat.ravel(order="F"), reclat=self.reclat.ravel(order="F"),
                       inv_reclat=np.linalg.inv(self.reclat).ravel(order="F"), volume=abs(np.linalg.det(self.lat)),
                       grid=g, mass_disorder=self.disorder, op_cart=op_cart, q_full=self.q_cart,
                       irr_weight=self.irr_weight, omega=self.omega, egv=egv, vel=self.vel, fc3_lvcart=lvcart,
                       fc3_mwm=mwm, fc4_lvcart=np.zeros(0), fc4_mwm=np.zeros(0),
                       irr_dyngrad=np.zeros(nirr * 3 * n * n * 2), atom_shift=np.zeros(nop * self.na * 3),
                       op_recfrac=op_recfrac, full_irr=self.full_irr + 1, full_op=full_op, irr_full=self.irr_full + 1,
                       irr_nop=self.irr_nop, irr_ops=irr_ops, degen=self.degen, degen_mode=degen_mode,
                       fc3_atoms=at + 1, fc3_lv=lv, fc4_atoms=np.zeros(0), fc4_lv=np.zeros(0),
                       op_fmap=np.ones(nop * self.na))
