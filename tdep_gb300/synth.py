"""Seeded synthetic inputs for the benchmark configurations.

Force constants are the analytic 2nd/3rd/4th derivatives of pair potentials, written in
TDEP's own file formats (infile.ucposcar, infile.forceconstant,
infile.forceconstant_thirdorder, infile.forceconstant_fourthorder, infile.isotopes), so
the same files feed the reference's readers, the oracle and the GPU path.

For a pair potential phi(|r|) the k-th derivative tensor of F(r) = phi(|r|) follows from
g(u) = phi(sqrt(2u)):
  d_ij F   = g'' r_i r_j + g' d_ij
  d_ijk F  = g''' r_i r_j r_k + g'' (d_ij r_k + d_ik r_j + d_jk r_i)
  d_ijkl F = g'''' r_i r_j r_k r_l + g''' (six d r r terms) + g'' (three d d terms)
with g' = phi'/r, g'' = phi''/r^2 - phi'/r^3, g''' = phi'''/r^3 - 3phi''/r^4 + 3phi'/r^5,
g'''' = phi''''/r^4 - 6phi'''/r^5 + 15phi''/r^6 - 15phi'/r^7.
A pair (home atom h, neighbour s) contributes to every force constant whose sites are
all h or s with sign (-1)^(number of h), which also satisfies the acoustic sum rule.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass
from pathlib import Path

import numpy as np

AMU = {"Al": 26.98, "Na": 22.99, "Cl": 35.45, "Ti": 47.9, "O": 16.0, "Ba": 137.3, "Ca": 40.08, "F": 19.0,
       "Cu": 63.55, "Au": 196.97}


# ---------------------------------------------------------------- pair potentials
def morse(D, alpha, r0):
    def f(r):
        e1 = np.exp(-alpha * (r - r0))
        e2 = e1 * e1
        return np.array([D * (e2 - 2 * e1), D * (-2 * alpha * e2 + 2 * alpha * e1),
                         D * (4 * alpha**2 * e2 - 2 * alpha**2 * e1), D * (-8 * alpha**3 * e2 + 2 * alpha**3 * e1),
                         D * (16 * alpha**4 * e2 - 2 * alpha**4 * e1)])
    return f


def born_mayer(A, rho):
    def f(r):
        e = A * np.exp(-r / rho)
        return np.array([e * (-1.0 / rho) ** k for k in range(5)])
    return f


def lennard_jones(eps, sigma):
    def f(r):
        out = np.zeros(5)
        for m, c in ((12, 4 * eps * sigma**12), (6, -4 * eps * sigma**6)):
            coef = 1.0
            for k in range(5):
                out[k] += c * coef * r ** (-m - k)
                coef *= -(m + k)
        return out
    return f


def spring(k, r0):
    def f(r):
        return np.array([0.5 * k * (r - r0) ** 2, k * (r - r0), k, 0.0, 0.0])
    return f


def combine(*fs):
    def f(r):
        return sum(g(r) for g in fs)
    return f


def radial_tensors(dphi, rvec):
    """(D2, D3, D4) derivative tensors of phi(|r|) at rvec (eV/A^k)."""
    r = float(np.linalg.norm(rvec))
    p1, p2, p3, p4 = dphi[1], dphi[2], dphi[3], dphi[4]
    g1 = p1 / r
    g2 = p2 / r**2 - p1 / r**3
    g3 = p3 / r**3 - 3 * p2 / r**4 + 3 * p1 / r**5
    g4 = p4 / r**4 - 6 * p3 / r**5 + 15 * p2 / r**6 - 15 * p1 / r**7
    d = np.eye(3)
    x = np.asarray(rvec, float)
    D2 = g2 * np.einsum("i,j->ij", x, x) + g1 * d
    D3 = g3 * np.einsum("i,j,k->ijk", x, x, x) + g2 * (
        np.einsum("ij,k->ijk", d, x) + np.einsum("ik,j->ijk", d, x) + np.einsum("jk,i->ijk", d, x))
    drr = (np.einsum("il,j,k->ijkl", d, x, x) + np.einsum("jl,i,k->ijkl", d, x, x) +
           np.einsum("kl,i,j->ijkl", d, x, x) + np.einsum("ik,j,l->ijkl", d, x, x) +
           np.einsum("jk,i,l->ijkl", d, x, x) + np.einsum("ij,k,l->ijkl", d, x, x))
    dd = np.einsum("ik,jl->ijkl", d, d) + np.einsum("jk,il->ijkl", d, d) + np.einsum("ij,kl->ijkl", d, d)
    D4 = g4 * np.einsum("i,j,k,l->ijkl", x, x, x, x) + g3 * drr + g2 * dd
    return D2, D3, D4


# ---------------------------------------------------------------- structures
@dataclass
class Cell:
    lattice: np.ndarray        # rows = lattice vectors (A), as in POSCAR
    frac: np.ndarray           # (na, 3)
    species: list              # symbol per atom
    masses: np.ndarray         # amu per atom

    @property
    def na(self):
        return len(self.species)


def fcc_primitive(a, symbol):
    lat = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
    return Cell(lat, np.zeros((1, 3)), [symbol], np.array([AMU[symbol]]))


def rocksalt(a, s1, s2):
    lat = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
    frac = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]])
    return Cell(lat, frac, [s1, s2], np.array([AMU[s1], AMU[s2]]))


def perovskite(a):
    lat = np.eye(3) * a
    frac = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
    sp = ["Ba", "Ti", "O", "O", "O"]
    return Cell(lat, frac, sp, np.array([AMU[s] for s in sp]))


def fluorite(a, s1, s2):
    """AX2 fluorite (3 atoms, fcc lattice): A at 0, X at +-(1/4, 1/4, 1/4)."""
    lat = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
    frac = np.array([[0.0, 0.0, 0.0], [0.25, 0.25, 0.25], [0.75, 0.75, 0.75]])
    sp = [s1, s2, s2]
    return Cell(lat, frac, sp, np.array([AMU[x] for x in sp]))


def l12(a, s1, s2):
    """AB3 L1_2 (4 atoms, simple cubic lattice): A at the corner, B at the face centres."""
    lat = np.eye(3) * a
    frac = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
    sp = [s1, s2, s2, s2]
    return Cell(lat, frac, sp, np.array([AMU[x] for x in sp]))


def neighbours(cell, cutoff):
    """[(home, j, R(int3), rvec)] for every pair within the cutoff (0 < |r| < cutoff)."""
    lat = cell.lattice
    inv_heights = np.linalg.norm(np.linalg.inv(lat), axis=0)  # 1/plane spacing
    nmax = [int(np.ceil(cutoff * h)) + 1 for h in inv_heights]
    out = []
    for h in range(cell.na):
        for j in range(cell.na):
            for R in itertools.product(*[range(-m, m + 1) for m in nmax]):
                rv = (cell.frac[j] + np.array(R) - cell.frac[h]) @ lat
                d = np.linalg.norm(rv)
                if 1e-8 < d < cutoff:
                    out.append((h, j, np.array(R, int), rv))
    return out


# ---------------------------------------------------------------- writers
def _fmt(v):
    return "  " + "  ".join(f"{x: .16f}" for x in v)


def write_poscar(path, cell: Cell, comment="synthetic"):
    syms = []
    for s in cell.species:
        if s not in syms:
            syms.append(s)
    order = sorted(range(cell.na), key=lambda i: syms.index(cell.species[i]))
    assert order == list(range(cell.na)), "atoms must be grouped by species"
    counts = [cell.species.count(s) for s in syms]
    with open(path, "w") as f:
        f.write(f"{comment}\n1.0\n")
        for v in cell.lattice:
            f.write(_fmt(v) + "\n")
        f.write(" " + " ".join(syms) + "\n")
        f.write(" " + " ".join(str(c) for c in counts) + "\n")
        f.write("Direct\n")
        for x in cell.frac:
            f.write(_fmt(x) + "\n")


def write_isotopes(path, cell: Cell):
    with open(path, "w") as f:
        for m in cell.masses:
            f.write("1\n")
            f.write(f"1.0 {m:.10f}\n")


def build_force_constants(cell: Cell, pot, cutoff, order4=False):
    """FC2/FC3/FC4 dictionaries keyed by home atom: list of (sites, tensor)."""
    pairs = neighbours(cell, cutoff)
    fc2 = {h: {} for h in range(cell.na)}
    fc3 = {h: {} for h in range(cell.na)}
    fc4 = {h: {} for h in range(cell.na)}
    zero = (0, (0, 0, 0))
    for (h, j, R, rv) in pairs:
        dphi = pot(cell.species[h], cell.species[j])(np.linalg.norm(rv))
        D2, D3, D4 = radial_tensors(dphi, rv)
        home = (h, (0, 0, 0))
        site = (j, tuple(int(x) for x in R))
        for combo in itertools.product((0, 1), repeat=1):
            sites = (home,) + tuple(home if c == 0 else site for c in combo)
            nh = 1 + sum(1 for c in combo if c == 0)
            fc2[h][sites] = fc2[h].get(sites, 0) + (-1) ** nh * D2
        for combo in itertools.product((0, 1), repeat=2):
            sites = (home,) + tuple(home if c == 0 else site for c in combo)
            nh = 1 + sum(1 for c in combo if c == 0)
            fc3[h][sites] = fc3[h].get(sites, 0) + (-1) ** nh * D3
        if order4:
            for combo in itertools.product((0, 1), repeat=3):
                sites = (home,) + tuple(home if c == 0 else site for c in combo)
                nh = 1 + sum(1 for c in combo if c == 0)
                fc4[h][sites] = fc4[h].get(sites, 0) + (-1) ** nh * D4
    del zero
    return fc2, fc3, fc4


def _sorted_items(d):
    # self terms first, then by lattice vector and atom for a stable file layout
    return sorted(d.items(), key=lambda kv: [(s[1], s[0]) for s in kv[0][1:]])


def write_fc2(path, cell, fc2, cutoff):
    with open(path, "w") as f:
        f.write(f"{cell.na:>11d}               How many atoms per unit cell\n")
        f.write(f"{cutoff:22.15f}     Realspace cutoff (A)\n")
        for h in range(cell.na):
            items = _sorted_items(fc2[h])
            f.write(f"{len(items):>11d}               How many neighbours does atom {h + 1:3d} have\n")
            for k, (sites, m) in enumerate(items, 1):
                (j, R) = sites[1]
                f.write(f"{j + 1:>11d}               In the unit cell, what is the index of neighbour {k} of atom {h + 1}\n")
                f.write(_fmt(R) + "\n")
                for row in m:
                    f.write(_fmt(row) + "\n")
        f.write("          0               Not polar\n")


def write_fc3(path, cell, fc3, cutoff):
    with open(path, "w") as f:
        f.write(f"{cell.na:>11d}               How many atoms per unit cell\n")
        f.write(f"{cutoff:22.15f}     Realspace cutoff (A)\n")
        for h in range(cell.na):
            items = _sorted_items(fc3[h])
            f.write(f"{len(items):>11d}               How many triplets are atom {h + 1:3d} part of\n")
            for k, (sites, m) in enumerate(items, 1):
                for i, (a, _) in enumerate(sites):
                    f.write(f"{a + 1:>11d}                atom {i + 1} in triplet {k:2d}\n")
                for (_, R) in sites:
                    f.write(_fmt(R) + "\n")
                for ii in range(3):
                    for jj in range(3):
                        f.write(_fmt(m[ii, jj, :]) + "\n")


def write_fc4(path, cell, fc4, cutoff):
    with open(path, "w") as f:
        f.write(f"{cell.na:>11d}               How many atoms per unit cell\n")
        f.write(f"{cutoff:22.15f}     Realspace cutoff (A)\n")
        for h in range(cell.na):
            items = _sorted_items(fc4[h])
            f.write(f"{len(items):>11d}               How many quartets are atom {h + 1:3d} part of\n")
            for k, (sites, m) in enumerate(items, 1):
                for i, (a, _) in enumerate(sites):
                    f.write(f"{a + 1:>11d}                atom {i + 1} in quartet {k:2d}\n")
                for (_, R) in sites:
                    f.write(_fmt(R) + "\n")
                for ii in range(3):
                    for jj in range(3):
                        for kk in range(3):
                            f.write(_fmt(m[ii, jj, kk, :]) + "\n")


# ---------------------------------------------------------------- configurations
def _jitter(rng, x):
    return x * (1.0 + 0.05 * rng.uniform(-1.0, 1.0))


def config_fcc_morse(seed=1):
    """fcc Al-like cell, Morse pairs (D=0.3 eV, alpha=1.2/A, r0=2.86 A, +-5%), 2nd shell."""
    rng = np.random.default_rng(seed)
    cell = fcc_primitive(4.05, "Al")
    D, al, r0 = _jitter(rng, 0.3), _jitter(rng, 1.2), _jitter(rng, 2.86)
    pot = lambda s1, s2: morse(D, al, r0)
    cutoff = 0.5 * (4.05 + 4.05 * np.sqrt(1.5))  # between the 2nd and 3rd shells
    return cell, pot, cutoff


def config_rocksalt(seed=1):
    """Rocksalt Na/Cl, seeded Born-Mayer pairs plus a short-range spring, 3rd shell."""
    rng = np.random.default_rng(seed)
    a = 5.64
    cell = rocksalt(a, "Na", "Cl")
    rnn = a / 2
    A = {k: rng.uniform(1000.0, 3000.0) for k in ("NaCl", "NaNa", "ClCl")}
    rho = {k: _jitter(rng, 0.3) for k in A}
    ks, rs = _jitter(rng, 1.5), rnn - 0.6

    def pot(s1, s2):
        key = "NaCl" if s1 != s2 else s1 + s2
        parts = [born_mayer(A[key], rho[key])]
        if key == "NaCl":
            parts.append(spring(ks, rs))
        else:
            parts.append(spring(0.3 * ks, a / np.sqrt(2) - 0.6))
        return combine(*parts)

    cutoff = 0.5 * (a * np.sqrt(3) / 2 + a)  # between the 3rd and 4th shells
    return cell, pot, cutoff


def config_perovskite(seed=1, cutoff=6.0):
    """Cubic ABO3 (Ba, Ti, O3; a=3.9 A), seeded Lennard-Jones + Born-Mayer pairs."""
    rng = np.random.default_rng(seed)
    a = 3.9
    cell = perovskite(a)
    kinds = {}
    nn = {("Ti", "O"): a / 2, ("Ba", "O"): a / np.sqrt(2), ("O", "O"): a / np.sqrt(2), ("Ba", "Ti"): a * np.sqrt(3) / 2,
          ("Ba", "Ba"): a, ("Ti", "Ti"): a}
    for key, r in nn.items():
        sig = 0.85 * r / 2 ** (1 / 6)
        kinds[key] = (lennard_jones(_jitter(rng, 0.05), _jitter(rng, sig)),
                      born_mayer(_jitter(rng, 800.0), _jitter(rng, 0.25)),
                      spring(_jitter(rng, 2.0), 0.8 * r) if key in (("Ti", "O"), ("Ba", "O"), ("O", "O")) else None)

    def pot(s1, s2):
        key = (s1, s2) if (s1, s2) in kinds else (s2, s1)
        lj, bm, sp = kinds[key]
        if sp is not None:
            r_sp = nn[key]
            base = combine(lj, bm)
            return lambda r: base(r) + (sp(r) if r < r_sp * 1.05 else 0.0)
        return combine(lj, bm)

    return cell, pot, cutoff


def config_fluorite(seed=1):
    """Fluorite CaF2 (a = 5.46 A, 9 modes), seeded Born-Mayer pairs plus nearest-neighbour
    springs, cutoff between the third and fourth shells."""
    rng = np.random.default_rng(seed)
    a = 5.46
    cell = fluorite(a, "Ca", "F")
    r_cf, r_ff = a * np.sqrt(3) / 4, a / 2
    bm = {k: born_mayer(rng.uniform(1000.0, 3000.0), _jitter(rng, 0.3)) for k in ("CaF", "FF", "CaCa")}
    sp = {"CaF": spring(_jitter(rng, 1.5), r_cf - 0.5), "FF": spring(_jitter(rng, 0.5), r_ff - 0.5),
          "CaCa": spring(_jitter(rng, 0.3), a / np.sqrt(2) - 0.6)}

    def pot(s1, s2):
        key = "CaF" if s1 != s2 else s1 + s2
        return combine(bm[key], sp[key])

    return cell, pot, 0.5 * (a / np.sqrt(2) + a * np.sqrt(11) / 4)


def config_l12(seed=1):
    """L1_2 Cu3Au (a = 3.75 A, 12 modes), seeded Morse pairs, cutoff between the second and
    third shells."""
    rng = np.random.default_rng(seed)
    a = 3.75
    cell = l12(a, "Au", "Cu")
    r1 = a / np.sqrt(2)
    ms = {k: morse(_jitter(rng, 0.3), _jitter(rng, 1.4), _jitter(rng, r1)) for k in ("AuCu", "CuCu", "AuAu")}

    def pot(s1, s2):
        key = "AuCu" if s1 != s2 else s1 + s2
        return ms[key]

    return cell, pot, 0.5 * (a + a * np.sqrt(1.5))


def supercell(cell: Cell, reps, rng=None, disp=0.0) -> Cell:
    """reps[0] x reps[1] x reps[2] supercell, atoms grouped by species in first-appearance
    order, optional Gaussian displacements of standard deviation disp (A)."""
    reps = np.asarray(reps, int)
    lat = cell.lattice * reps[:, None]
    order = []
    for sp in cell.species:
        if sp not in order:
            order.append(sp)
    frac, species, masses = [], [], []
    for sp in order:
        for ijk in itertools.product(*[range(r) for r in reps]):
            for a in range(cell.na):
                if cell.species[a] == sp:
                    frac.append((cell.frac[a] + np.array(ijk)) / reps)
                    species.append(sp)
                    masses.append(cell.masses[a])
    frac = np.array(frac)
    if disp > 0.0:
        frac = frac + rng.normal(0.0, disp, frac.shape) @ np.linalg.inv(lat)
    return Cell(lat, frac, species, np.array(masses))


def config_perovskite_supercell(seed=1, reps=(2, 2, 2), disp=0.05, cutoff=5.0):
    """Supercell of the cubic perovskite (2x2x2: 40 atoms, 120 modes) with seeded Gaussian
    atomic displacements, so that only the identity survives as a symmetry operation; the
    pair potentials of config_perovskite, evaluated at the displaced positions."""
    rng = np.random.default_rng(seed + 1000)
    base, pot, _ = config_perovskite(seed=seed)
    return supercell(base, reps, rng, disp), pot, cutoff


CONFIGS = {
    "fcc_morse": config_fcc_morse,
    "rocksalt": config_rocksalt,
    "perovskite": config_perovskite,
    "perovskite_supercell": config_perovskite_supercell,
    "fluorite": config_fluorite,
    "l12": config_l12,
}


def write_config(name, directory, seed=1, order4=False, **kw):
    """Write infile.* for a named configuration into `directory`; returns the directory."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    cell, pot, cutoff = CONFIGS[name](seed=seed, **kw)
    fc2, fc3, fc4 = build_force_constants(cell, pot, cutoff, order4=order4)
    write_poscar(d / "infile.ucposcar", cell, comment=f"{name} seed {seed}")
    write_isotopes(d / "infile.isotopes", cell)
    write_fc2(d / "infile.forceconstant", cell, fc2, cutoff)
    write_fc3(d / "infile.forceconstant_thirdorder", cell, fc3, cutoff)
    if order4:
        write_fc4(d / "infile.forceconstant_fourthorder", cell, fc4, cutoff)
    return d
