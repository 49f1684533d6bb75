"""ORACLE BINDING -- TEST INFRASTRUCTURE ONLY.

ctypes access to oracle/lib/liboracle.so, the CPU restatement of the reference's
scattering path (oracle/oracle.cpp). Imported only by tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py, always as the checker; the product never loads it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from tdep_gb300 import _native as N

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "lib" / "liboracle.so"
_L = None


def build() -> Path:
    LIB_PATH.parent.mkdir(exist_ok=True)
    src = HERE / "oracle.cpp"
    hdr = HERE.parent / "include" / "tdep_gb300.h"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        subprocess.run(["g++", "-O2", "-fPIC", "-std=c++17", "-fopenmp", "-shared", str(src), "-o", str(LIB_PATH)],
                       check=True)
    return LIB_PATH


def lib():
    global _L
    if _L is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        P = C.POINTER
        L.orc_mt_sequence.argtypes = [C.c_int, C.c_uint64, C.c_int64, P(C.c_uint64)]
        L.orc_mc_qlists.argtypes = [P(N.TdgProblem), P(N.TdgOpts), P(C.c_int32), P(C.c_int32), P(C.c_int32),
                                    P(C.c_int64), P(C.c_int32), P(C.c_int64), P(C.c_int32), P(C.c_int32)]
        L.orc_triplets.argtypes = [P(N.TdgProblem), C.c_int, P(C.c_int32), C.c_int64, P(C.c_int32), C.c_int64]
        L.orc_triplets.restype = C.c_int64
        L.orc_quartets.argtypes = [P(N.TdgProblem), C.c_int, P(C.c_int32), P(C.c_int32), C.c_int64, P(C.c_int32),
                                   C.c_int64]
        L.orc_quartets.restype = C.c_int64
        L.orc_adjoint_fc3.argtypes = [P(N.TdgProblem), P(N.TdgOpts), P(N.TdgQlists), P(C.c_double), P(C.c_double),
                                      C.c_int]
        L.orc_scattering_rows.argtypes = [P(N.TdgProblem), P(N.TdgOpts), P(N.TdgQlists), C.c_int, C.c_int,
                                          P(C.c_double), P(C.c_double), C.c_int, P(C.c_int64)]
        L.orc_scattering_finish.argtypes = [P(N.TdgProblem), P(N.TdgOpts), P(N.TdgQlists), P(C.c_double),
                                            P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double)]
        L.orc_kappa.argtypes = [P(N.TdgProblem), P(N.TdgOpts), P(N.TdgQlists), P(C.c_double), P(C.c_double),
                                P(C.c_double), C.c_int, C.c_double, P(C.c_double), P(C.c_double), P(C.c_int32)]
        L.orc_kappa_offdiag.argtypes = [P(N.TdgProblem), P(N.TdgOpts), P(C.c_double), P(C.c_double)]
        _L = L
    return _L


def mt_sequence(count: int, seed: int = 0, word: int = 0) -> np.ndarray:
    out = np.zeros(count, np.uint64)
    lib().orc_mt_sequence(int(seed), C.c_uint64(word), int(count), out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return out


def mc_qlists(prob, opts):
    """Rows and samples from the oracle's own MT19937-64 restatement."""
    from tdep_gb300.scattering import QLists

    q3, q4 = opts.resolved(prob.grid)
    cap = prob.n_irr * prob.n_mode
    np3, np4 = int(np.prod(q3)), int(np.prod(q4))
    rq1 = np.zeros(cap, np.int32)
    rb1 = np.zeros(cap, np.int32)
    p3 = np.zeros(cap + 1, np.int64)
    p4 = np.zeros(cap + 1, np.int64)
    l3 = np.zeros(max(1, cap * np3 if opts.thirdorder else 1), np.int32)
    l4a = np.zeros(max(1, cap * np4 if opts.fourthorder else 1), np.int32)
    l4b = np.zeros(max(1, cap * np4 if opts.fourthorder else 1), np.int32)
    nr = C.c_int32(0)
    ps = prob.struct()
    os_ = opts.struct(prob.grid)
    lib().orc_mc_qlists(C.byref(ps), C.byref(os_), C.byref(nr), N.ptr(rq1, C.c_int32), N.ptr(rb1, C.c_int32),
                        N.ptr(p3, C.c_int64), N.ptr(l3, C.c_int32), N.ptr(p4, C.c_int64), N.ptr(l4a, C.c_int32),
                        N.ptr(l4b, C.c_int32))
    n = nr.value
    return QLists(rq1[:n].copy(), rb1[:n].copy(),
                  p3[: n + 1].copy() if opts.thirdorder else None,
                  l3[: n * np3].copy() if opts.thirdorder else None,
                  p4[: n + 1].copy() if opts.fourthorder else None,
                  l4a[: n * np4].copy() if opts.fourthorder else None,
                  l4b[: n * np4].copy() if opts.fourthorder else None)


def triplets(prob, q1: int, sample: np.ndarray):
    """[(q2, q3, [(q2', q3'), ...]), ...] for one irreducible q1 (1-based)."""
    sample = np.ascontiguousarray(sample, np.int32)
    cap = 64
    while True:
        out = np.zeros(cap, np.int32)
        ps = prob.struct()
        w = lib().orc_triplets(C.byref(ps), int(q1), N.ptr(sample, C.c_int32), sample.size, N.ptr(out, C.c_int32), cap)
        if w >= 0:
            break
        cap *= 4
    res, i = [], 0
    while i < w:
        q2, q3, k = out[i], out[i + 1], out[i + 2]
        pairs = [tuple(out[i + 3 + 2 * j: i + 5 + 2 * j]) for j in range(k)]
        res.append((int(q2), int(q3), [(int(a), int(b)) for a, b in pairs]))
        i += 3 + 2 * k
    return res


def quartets(prob, q1: int, la: np.ndarray, lb: np.ndarray):
    """[(q2, q3, q4, [(q2', q3', q4'), ...]), ...] for one irreducible q1 over the pairs la x lb."""
    la = np.ascontiguousarray(la, np.int32)
    lb = np.ascontiguousarray(lb, np.int32)
    assert la.size == lb.size
    cap = 256
    while True:
        out = np.zeros(cap, np.int32)
        ps = prob.struct()
        w = lib().orc_quartets(C.byref(ps), int(q1), N.ptr(la, C.c_int32), N.ptr(lb, C.c_int32), la.size,
                               N.ptr(out, C.c_int32), cap)
        if w >= 0:
            break
        cap *= 4
    res, i = [], 0
    while i < w:
        q2, q3, q4, k = (int(x) for x in out[i:i + 4])
        trip = [tuple(int(v) for v in out[i + 4 + 3 * j: i + 7 + 3 * j]) for j in range(k)]
        res.append((q2, q3, q4, trip))
        i += 4 + 3 * k
    return res


def scattering(prob, opts, lists, nthreads: int = 0, rows=None):
    """Per-row part of sr%generate. Returns (gamma[rows], xi[rows, N*n], counts)."""
    r0, r1 = (0, lists.n_row) if rows is None else rows
    ld = prob.n_full * prob.n_mode
    gamma = np.zeros(r1 - r0)
    xi = np.zeros((r1 - r0, ld))
    counts = np.zeros(2, np.int64)
    ps = prob.struct()
    os_ = opts.struct(prob.grid)
    qs = lists.struct()
    lib().orc_scattering_rows(C.byref(ps), C.byref(os_), C.byref(qs), int(r0), int(r1), N.ptr(gamma, C.c_double),
                              N.ptr(xi, C.c_double), int(nthreads), N.ptr(counts, C.c_int64))
    return gamma, xi, counts


def finish(prob, opts, lists, gamma, xi):
    """Boundary term, degeneracy averaging, symmetrize_scatmat (xi in place)."""
    n = prob.n_irr * prob.n_mode
    lw = np.zeros(n)
    qs = np.zeros(n)
    f0 = np.zeros(3 * n)
    ps = prob.struct()
    os_ = opts.struct(prob.grid)
    ql = lists.struct()
    g = np.ascontiguousarray(gamma, np.float64)
    lib().orc_scattering_finish(C.byref(ps), C.byref(os_), C.byref(ql), N.ptr(g, C.c_double), N.ptr(xi, C.c_double),
                                N.ptr(lw, C.c_double), N.ptr(qs, C.c_double), N.ptr(f0, C.c_double))
    return lw.reshape(prob.n_irr, prob.n_mode), qs, f0


def kappa(prob, opts, lists, xi, qs, f0, maxiter: int, tol: float):
    ks = np.zeros(9)
    ki = np.zeros(9)
    nit = C.c_int32(0)
    ps = prob.struct()
    os_ = opts.struct(prob.grid)
    ql = lists.struct()
    lib().orc_kappa(C.byref(ps), C.byref(os_), C.byref(ql), N.ptr(xi, C.c_double), N.ptr(qs, C.c_double),
                    N.ptr(f0, C.c_double), int(maxiter), float(tol), N.ptr(ks, C.c_double), N.ptr(ki, C.c_double),
                    C.byref(nit))
    return ks.reshape(3, 3, order="F"), ki.reshape(3, 3, order="F"), nit.value


def kappa_offdiag(prob, opts, linewidth):
    """get_kappa_offdiag + symmetrize_kappa (kappa.f90:77-306, main.f90:243) from the given
    irreducible-point linewidths ([n_irr, n_mode]); a.u. 3x3."""
    lw = np.ascontiguousarray(linewidth, np.float64).reshape(-1)
    out = np.zeros(9)
    ps, os_ = prob.struct(), opts.struct(prob.grid)
    lib().orc_kappa_offdiag(C.byref(ps), C.byref(os_), N.ptr(lw, C.c_double), N.ptr(out, C.c_double))
    return out.reshape(3, 3, order="F")


def adjoint_fc3(prob, opts, lists, lw_bar, nthreads: int = 0):
    """(d linewidth / d fc3_mwm)^T lw_bar of the three-phonon part: [n_fc3, 27]."""
    lb = np.ascontiguousarray(lw_bar, np.float64).reshape(-1)
    out = np.zeros(prob.n_fc3 * 27)
    ps, os_, qs = prob.struct(), opts.struct(prob.grid), lists.struct()
    lib().orc_adjoint_fc3(C.byref(ps), C.byref(os_), C.byref(qs), N.ptr(lb, C.c_double), N.ptr(out, C.c_double),
                          int(nthreads))
    return out.reshape(prob.n_fc3, 27)


def full_run(prob, opts, lists, nthreads: int = 0):
    """Oracle linewidths, symmetrised Xi and kappa tensors for a complete run."""
    gamma, xi, counts = scattering(prob, opts, lists, nthreads)
    lw, qs, f0 = finish(prob, opts, lists, gamma, xi)
    ks, ki, nit = kappa(prob, opts, lists, xi, qs, f0, opts.itermaxsteps, opts.itertol)
    return {"linewidth": lw, "xi": xi, "kappa_sma": ks, "kappa_iter": ki, "n_iter": nit, "triplets": int(counts[0]),
            "quartets": int(counts[1])}
