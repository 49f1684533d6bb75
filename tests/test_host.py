"""Host stage: mesh, symmetry, phonons, force constants, Monte-Carlo samples (CPU only)."""
import numpy as np
import pytest

from oracle import binding as orc
from tdep_gb300 import Options, Problem, QLists

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def fcc8(configs):
    return Problem.load(configs["fcc"], (8, 8, 8), readiso=True)


def test_mesh_counts_and_weights(fcc8):
    # 8x8x8 Gamma-centred fcc mesh with O_h and time reversal: 29 irreducible points
    assert fcc8.n_op == 48 and fcc8.n_irr == 29
    np.testing.assert_allclose(fcc8.irr_weight.sum(), 1.0, rtol=1e-14)
    counts = np.bincount(fcc8.full_irr - 1, minlength=fcc8.n_irr)
    np.testing.assert_allclose(counts / fcc8.n_full, fcc8.irr_weight)
    # irreducible points are the smallest index of their orbit
    assert np.all(fcc8.full_irr[fcc8.irr_full - 1] == np.arange(1, fcc8.n_irr + 1))
    assert np.all(np.diff(fcc8.irr_full) > 0)


def test_operation_from_irreducible_maps_points(fcc8):
    p = fcc8
    g = p.grid
    idx = np.arange(p.n_full)
    frac = np.stack([idx // (g[1] * g[2]), (idx // g[2]) % g[1], idx % g[2]], 1) / g
    for q in range(p.n_full):
        op = p.full_op[q]
        R = p.op_recfrac[abs(op) - 1].reshape(3, 3, order="F")
        v = R @ frac[p.irr_full[p.full_irr[q] - 1] - 1] * np.sign(op)
        d = (v - frac[q]) % 1.0
        d = np.minimum(d, 1 - d)
        assert np.abs(d).max() < 1e-9


def test_little_groups_leave_q_invariant(fcc8):
    p = fcc8
    for k in range(p.n_irr):
        q = p.q_full[p.irr_full[k] - 1]
        for j in range(p.irr_nop[k]):
            m = p.op_cart[p.irr_ops[k, j] - 1].reshape(3, 3, order="F")
            f = p.inv_reclat.reshape(3, 3, order="F") @ (q - m @ q)
            assert np.abs(f - np.round(f)).max() < 1e-8


def test_phonons_physical(fcc8, configs):
    p = fcc8
    n = p.n_mode
    assert p.omega.min() >= 0.0
    gamma = int(np.argmin(np.linalg.norm(p.q_full, axis=1)))
    assert np.count_nonzero(p.omega[gamma] < 1e-9) == 3
    e = p.egv[..., 0] + 1j * p.egv[..., 1]  # (q, b, r)
    for q in range(0, p.n_full, 17):
        np.testing.assert_allclose(e[q] @ e[q].conj().T, np.eye(n), atol=1e-10)
    # time reversal: omega(q) == omega(-q)
    g = p.grid
    for q in range(p.n_full):
        i, j, k = q // (g[1] * g[2]), (q // g[2]) % g[1], q % g[2]
        mq = ((-i) % g[0]) * g[1] * g[2] + ((-j) % g[1]) * g[2] + (-k) % g[2]
        np.testing.assert_allclose(p.omega[q], p.omega[mq], rtol=1e-9, atol=1e-14)
    # degeneracy tables are symmetric and contain the mode itself
    for q in range(0, p.n_full, 7):
        for b in range(n):
            partners = p.degen_mode[q, b, : p.degen[q, b]] - 1
            assert b in partners
            for b2 in partners:
                assert b in p.degen_mode[q, b2, : p.degen[q, b2]] - 1


@pytest.mark.parametrize("name", ["fcc", "rocksalt", "perovskite"])
def test_third_order_acoustic_sum_rule(configs, name):
    p = Problem.load(configs[name], (2, 2, 2), readiso=True)
    # translate mwm back to plain force constants and sum over the third site
    from tdep_gb300 import synth

    cell = synth.CONFIGS["rocksalt" if name == "rocksalt" else
                         ("perovskite" if name == "perovskite" else "fcc_morse")](seed=1)[0]
    m = np.array(cell.masses)
    sums = {}
    for t in range(p.n_fc3):
        a1, a2, a3 = p.fc3_atoms[t]
        w = np.sqrt(m[a1 - 1] * m[a2 - 1] * m[a3 - 1])
        key = (a1, a2, tuple(p.fc3_lv[t, :3]))
        sums[key] = sums.get(key, 0) + p.fc3_mwm[t] * w
    scale = np.abs(p.fc3_mwm).max() * m.max() ** 1.5
    for v in sums.values():
        assert np.abs(v).max() < 1e-10 * scale


def test_reference_fixtures_parse(built):
    """The reference's own MgO inputs go through the same readers."""
    p = Problem.load(GOLDEN / "mgo", (5, 5, 5))
    assert p.n_atom == 2 and p.n_op == 48 and p.n_irr == 10
    # 19 triplets per atom in tests/infiles/infile.forceconstant_thirdorder
    assert p.n_fc3 == 38
    assert p.omega.min() >= 0 and 10 < p.omega.max() * 6579.683920502 < 25


def test_mt19937_64_known_answer(built):
    """The oracle's restatement of lo_randomnumbers.f90 against the published generator:
    the 10000th output of MT19937-64 seeded with 5489 is 9981545732273789042."""
    seq = orc.mt_sequence(10000, seed=0, word=5489)
    assert int(seq[-1]) == 9981545732273789042


def test_tdep_seeding_word(built):
    import random

    # init_genrand64(iseed=0, rseed=1/42): f0 = 1/42 - 0.5; anint(f0 * 2**30)
    seq = orc.mt_sequence(4, seed=42)
    ref = orc.mt_sequence(4, seed=0, word=(-511305630) & (2**64 - 1))
    assert np.array_equal(seq, ref)
    del random


@pytest.mark.parametrize("qg3,qg4", [((8, 8, 8), (2, 2, 2)), ((4, 4, 4), (3, 3, 3)), ((3, 5, 8), (4, 4, 4))])
def test_mc_samples_match_oracle(fcc8, qg3, qg4):
    opts = Options(seed=7, qg3ph=qg3, qg4ph=qg4, fourthorder=True)
    a = QLists.monte_carlo(fcc8, opts)
    b = orc.mc_qlists(fcc8, opts)
    for f in ("row_q1", "row_b1", "ptr3", "list3", "ptr4", "list4a", "list4b"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    # stratified: one point per Monte-Carlo cell, never the same point twice in a row
    n3 = int(np.prod(qg3))
    for r in range(0, a.n_row, 11):
        s = a.list3[a.ptr3[r]:a.ptr3[r + 1]]
        assert s.size == n3 and np.all(s >= 1) and np.all(s <= fcc8.n_full)
        assert np.all(s[1:] != s[:-1])


def test_full_grid_sample_is_the_mesh_in_order(fcc8):
    a = QLists.monte_carlo(fcc8, Options(seed=3))
    for r in range(a.n_row):
        assert np.array_equal(a.list3[a.ptr3[r]:a.ptr3[r + 1]], np.arange(1, fcc8.n_full + 1))


def test_natural_isotope_table_matches_the_reference():
    """Every element of the library's natural-isotope table (abundances and isotope masses)
    against the reference's own table, extracted into tests/golden/isotopes.json by
    tests/golden/make_isotopes.py; the elements of the synthetic cells and the reference's
    MgO fixture must be there."""
    import ctypes as C
    import json

    from tdep_gb300 import _native as N

    ref = json.loads((GOLDEN / "isotopes.json").read_text())
    lib = N.lib()
    lib.tdg_natural_isotopes.restype = C.c_int
    lib.tdg_natural_isotopes.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    have = []
    for sym, iso in ref.items():
        ab = (C.c_double * 16)()
        ms = (C.c_double * 16)()
        n = lib.tdg_natural_isotopes(sym.encode(), 16, ab, ms)
        if n == 0:
            continue
        have.append(sym)
        assert n == len(iso), sym
        np.testing.assert_allclose(list(ab[:n]), [c for c, _ in iso], rtol=0, atol=1e-12, err_msg=sym)
        np.testing.assert_allclose(list(ms[:n]), [m for _, m in iso], rtol=1e-10, err_msg=sym)
    assert {"Al", "Na", "Cl", "Ti", "O", "Ba", "Mg", "Si"} <= set(have)
    assert len(have) >= 45
    assert lib.tdg_natural_isotopes(b"Xx", 16, None, None) == 0


def test_unknown_isotope_disorder_is_nan(configs, tmp_path):
    """An element without a tabulated natural distribution keeps its standard weight and
    an unknown (NaN) disorder, so isotope scattering fails loudly instead of using zero;
    infile.isotopes supplies it."""
    import shutil

    d = tmp_path / "hf"
    shutil.copytree(configs["fcc"], d)
    pos = (d / "infile.ucposcar").read_text().splitlines()
    sym_line = next(i for i, ln in enumerate(pos) if ln.split() and ln.split()[0] == "Al")
    pos[sym_line] = pos[sym_line].replace("Al", "Hf")
    (d / "infile.ucposcar").write_text("\n".join(pos) + "\n")
    prob = Problem.load(d, (4, 4, 4))
    assert np.isnan(prob.mass_disorder).all()
    prob = Problem.load(d, (4, 4, 4), readiso=True)  # the synthetic cells ship infile.isotopes
    assert np.isfinite(prob.mass_disorder).all()
