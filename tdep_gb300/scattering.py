"""Host-side mirror of TDEP's scattering interface over the GB300 C-ABI.

Names follow the reference:
  Problem            the flattened (uc, qp, dr, fct, fcf) that sr%generate consumes
  Options            the hot-path subset of lo_opts (src/thermal_conductivity/options.f90)
  QLists             rows (q1, b1) and their Monte-Carlo q' samples
  ScatteringRates    lo_scattering_rates (scattering.f90:34-55): generate(), Xi, and the
                     kappa solves of kappa.f90 (get_kappa / iterative_solution)
Errors raise TdgError with the reference's exit-code meaning (konstanter.f90:160-172).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _native as N

# Unit conversions used at the interface (src/libolle/konstanter.f90).
HARTREE_TO_EV = 27.21138602
BOHR_TO_M = 0.52917721067e-10
EV_TO_JOULE = 1.6021766208e-19
HBAR_EV = 6.582119514e-16
KAPPA_AU_TO_SI = (HARTREE_TO_EV * EV_TO_JOULE) / (HBAR_EV * EV_TO_JOULE / (HARTREE_TO_EV * EV_TO_JOULE)) / BOHR_TO_M
FREQ_HARTREE_TO_THZ = 1e-12 / 6.283185307179586 / (HBAR_EV / HARTREE_TO_EV)
LO_FREQTOL = 1e-9

_FIELDS_F64 = {
    "mass_disorder": ("n_atom",),
    "op_cart": ("n_op", 9),
    "q_full": ("n_full", 3),
    "irr_weight": ("n_irr",),
    "omega": ("n_full", "n_mode"),
    "egv": ("n_full", "n_mode", "n_mode", 2),
    "vel": ("n_full", "n_mode", 3),
    "fc3_lvcart": ("n_fc3", 6),
    "fc3_mwm": ("n_fc3", 27),
    "fc4_lvcart": ("n_fc4", 9),
    "fc4_mwm": ("n_fc4", 81),
    "irr_dyngrad": ("n_irr", 3, "n_mode", "n_mode", 2),
    "atom_shift": ("n_op", "n_atom", 3),
}
_FIELDS_I32 = {
    "op_recfrac": ("n_op", 9),
    "full_irr": ("n_full",),
    "full_op": ("n_full",),
    "irr_full": ("n_irr",),
    "irr_nop": ("n_irr",),
    "irr_ops": ("n_irr", "n_op"),
    "degen": ("n_full", "n_mode"),
    "degen_mode": ("n_full", "n_mode", "n_mode"),
    "fc3_atoms": ("n_fc3", 3),
    "fc3_lv": ("n_fc3", 6),
    "fc4_atoms": ("n_fc4", 4),
    "fc4_lv": ("n_fc4", 9),
    "op_fmap": ("n_op", "n_atom"),
}
_SCALARS = ("n_atom", "n_mode", "n_op", "n_full", "n_irr", "n_fc3", "n_fc4")


class _LoadedProblem:
    """Owner of a tdg_problem the library allocated: freed (tdg_problem_free) when the last
    array viewing its memory is gone."""

    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            N.lib().tdg_problem_free(self.ptr)
        except Exception:
            pass


class Problem:
    """tdg_problem with numpy arrays in the C-ABI layouts (see include/tdep_gb300.h). A loaded
    problem's arrays view the library's memory (no copy); the library's problem lives as long
    as any of them."""

    def __init__(self, **kw):
        for k in _SCALARS:
            setattr(self, k, int(kw[k]))
        for k in ("latvec", "reclat", "inv_reclat"):
            setattr(self, k, np.ascontiguousarray(kw[k], dtype=np.float64).reshape(9))
        self.volume = float(kw["volume"])
        self.grid = np.ascontiguousarray(kw["grid"], dtype=np.int32).reshape(3)
        for k, shp in _FIELDS_F64.items():
            setattr(self, k, np.ascontiguousarray(kw[k], dtype=np.float64).reshape(self._shape(shp)))
        for k, shp in _FIELDS_I32.items():
            setattr(self, k, np.ascontiguousarray(kw[k], dtype=np.int32).reshape(self._shape(shp)))
        self._struct = None

    def _shape(self, shp):
        return tuple(getattr(self, s) if isinstance(s, str) else s for s in shp)

    @classmethod
    def load(cls, directory, qgrid, fourthorder=False, readiso=False, timereversal=True,
             device: int | None = None) -> "Problem":
        """Read infile.* from `directory` and build mesh and phonons (main.f90:42-181); with
        `device` the harmonic stage runs on that GPU (tdg_problem_load_device)."""
        L = N.lib()
        out = C.POINTER(N.TdgProblem)()
        g = np.ascontiguousarray(qgrid, dtype=np.int32)
        args = (str(directory).encode(), N.ptr(g, C.c_int32), int(bool(fourthorder)), int(bool(readiso)),
                int(bool(timereversal)))
        if device is None:
            N.check(L.tdg_problem_load(*args, C.byref(out)), "tdg_problem_load")
        else:
            N.check(L.tdg_problem_load_device(*args, int(device), C.byref(out)), "tdg_problem_load_device")
        owner = _LoadedProblem(out)
        return cls.from_struct(out.contents, owner)

    @classmethod
    def from_struct(cls, s: N.TdgProblem, owner=None) -> "Problem":
        """The arrays of s, copied, or (owner: the object that frees s) viewed in place."""
        kw = {k: getattr(s, k) for k in _SCALARS}
        for k in ("latvec", "reclat", "inv_reclat"):
            kw[k] = np.array(getattr(s, k)[:], dtype=np.float64)
        kw["volume"] = s.volume
        kw["grid"] = np.array(s.grid[:], dtype=np.int32)
        dims = dict(kw)
        for table, ct in ((_FIELDS_F64, np.float64), (_FIELDS_I32, np.int32)):
            cty = C.c_double if ct is np.float64 else C.c_int32
            for k, shp in table.items():
                n = int(np.prod([dims[x] if isinstance(x, str) else x for x in shp]))
                p = getattr(s, k)
                if n == 0 or not p:
                    kw[k] = np.zeros(n, dtype=ct)
                elif owner is None:
                    kw[k] = np.ctypeslib.as_array(p, shape=(n,)).copy()
                else:
                    buf = (cty * n).from_address(C.cast(p, C.c_void_p).value)
                    buf._owner = owner  # the arrays keep the library's problem alive
                    kw[k] = np.ctypeslib.as_array(buf)
        return cls(**kw)

    def fc3_irreducible(self):
        """Symmetry-irreducible parameters of the third-order force constants
        (tdg_fc3_irreducible): returns (x [n_x], B) with B a scipy.sparse CSR matrix of shape
        (n_fc3 * 27, n_x) such that fc3_mwm.ravel() = B @ x for symmetric constants."""
        import scipy.sparse as sp

        ps = self.struct()
        nx, nc = C.c_int32(0), C.c_int64(0)
        L = N.lib()
        N.check(L.tdg_fc3_irreducible(C.byref(ps), C.byref(nx), C.byref(nc), None, None, None, None),
                "tdg_fc3_irreducible")
        col0 = np.zeros(self.n_fc3, np.int32)
        ncol = np.zeros(self.n_fc3, np.int32)
        coef = np.zeros(max(1, nc.value))
        x = np.zeros(max(1, nx.value))
        N.check(L.tdg_fc3_irreducible(C.byref(ps), C.byref(nx), C.byref(nc), N.ptr(col0, C.c_int32),
                                      N.ptr(ncol, C.c_int32), N.ptr(coef, C.c_double), N.ptr(x, C.c_double)),
                "tdg_fc3_irreducible")
        rows, cols, vals = [], [], []
        off = 0
        for t in range(self.n_fc3):
            k = int(ncol[t])
            blk = coef[off:off + 27 * k].reshape(27, k)
            r, c = np.nonzero(np.abs(blk) > 0)
            rows.append(27 * t + r)
            cols.append(col0[t] + c)
            vals.append(blk[r, c])
            off += 27 * k
        B = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(self.n_fc3 * 27, nx.value))
        return x[: nx.value].copy(), B

    def struct(self) -> N.TdgProblem:
        s = N.TdgProblem()
        for k in _SCALARS:
            setattr(s, k, getattr(self, k))
        for k in ("latvec", "reclat", "inv_reclat"):
            getattr(s, k)[:] = list(getattr(self, k))
        s.volume = self.volume
        s.grid[:] = [int(x) for x in self.grid]
        for k in _FIELDS_F64:
            setattr(s, k, N.ptr(getattr(self, k), C.c_double))
        for k in _FIELDS_I32:
            setattr(s, k, N.ptr(getattr(self, k), C.c_int32))
        self._struct = s  # keep alive with the arrays it points into
        return s

    def rows(self):
        """(q1, b1) 1-based rows with omega >= lo_freqtol (scattering.f90:170-209)."""
        om = self.omega[self.irr_full - 1]
        q1, b1 = np.nonzero(om >= LO_FREQTOL)
        return (q1 + 1).astype(np.int32), (b1 + 1).astype(np.int32)


@dataclass
class Options:
    """Hot-path subset of lo_opts, same flag meaning as options.f90."""

    temperature: float = 300.0
    integrationtype: int = 2
    sigma: float = 1.0
    thirdorder: bool = True
    fourthorder: bool = False
    isotopescattering: bool = True
    classical: bool = False
    mfp_max: float = -1.0  # metres, as --max_mfp
    qg3ph: tuple = (-1, -1, -1)
    qg4ph: tuple = (-1, -1, -1)
    seed: int = 1
    precision: str = "fp64"  # "fp64" or "mixed"
    tensor_cores: int = 0  # 0 automatic, 1 (or True) force the tcgen05 large-cell contraction, 2 SIMT fused kernel
    itertol: float = 1e-5
    itermaxsteps: int = 200

    def resolved(self, qgrid):
        """options.f90:205-235: grids default to (and are capped by) the full q-grid.
        A zero dimension, which the reference would divide by, also takes the full grid."""
        q3 = tuple(int(m) if 0 < int(m) <= int(g) else int(g) for m, g in zip(self.qg3ph, qgrid))
        q4 = tuple(int(m) if 0 < int(m) <= int(g) else int(g) for m, g in zip(self.qg4ph, qgrid))
        return q3, q4

    def struct(self, qgrid) -> N.TdgOpts:
        o = N.TdgOpts()
        o.temperature = float(self.temperature)
        o.integrationtype = int(self.integrationtype)
        o.sigma = float(self.sigma)
        o.thirdorder = int(bool(self.thirdorder))
        o.fourthorder = int(bool(self.fourthorder))
        o.isotope = int(bool(self.isotopescattering))
        o.classical = int(bool(self.classical))
        o.mfp_max = float(self.mfp_max) / BOHR_TO_M if self.mfp_max > 0 else -1.0
        q3, q4 = self.resolved(qgrid)
        o.qg3ph[:] = list(q3)
        o.qg4ph[:] = list(q4)
        o.seed = int(self.seed)
        if self.precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        o.precision = N.TDG_PREC_FP64 if self.precision == "fp64" else N.TDG_PREC_MIXED
        o.tensor_cores = int(self.tensor_cores)
        return o


@dataclass
class QLists:
    """Rows and their q' samples (CSR). All indices 1-based as in the reference."""

    row_q1: np.ndarray
    row_b1: np.ndarray
    ptr3: np.ndarray | None = None
    list3: np.ndarray | None = None
    ptr4: np.ndarray | None = None
    list4a: np.ndarray | None = None
    list4b: np.ndarray | None = None
    _keep: list = field(default_factory=list, repr=False)

    @property
    def n_row(self) -> int:
        return int(self.row_q1.size)

    @classmethod
    def monte_carlo(cls, prob: Problem, opts: Options) -> "QLists":
        """Samples drawn exactly as the reference draws them (tdg_mc_qlists)."""
        L = N.lib()
        q3, q4 = opts.resolved(prob.grid)
        cap = prob.n_irr * prob.n_mode
        np3, np4 = int(np.prod(q3)), int(np.prod(q4))
        rq1 = np.zeros(cap, np.int32)
        rb1 = np.zeros(cap, np.int32)
        p3 = np.zeros(cap + 1, np.int64)
        p4 = np.zeros(cap + 1, np.int64)
        l3 = np.zeros(cap * np3 if opts.thirdorder else 1, np.int32)
        l4a = np.zeros(cap * np4 if opts.fourthorder else 1, np.int32)
        l4b = np.zeros(cap * np4 if opts.fourthorder else 1, np.int32)
        nr = C.c_int32(0)
        ps = prob.struct()
        os_ = opts.struct(prob.grid)
        N.check(L.tdg_mc_qlists(C.byref(ps), C.byref(os_), C.byref(nr), N.ptr(rq1, C.c_int32), N.ptr(rb1, C.c_int32),
                                N.ptr(p3, C.c_int64), N.ptr(l3, C.c_int32), N.ptr(p4, C.c_int64),
                                N.ptr(l4a, C.c_int32), N.ptr(l4b, C.c_int32)), "tdg_mc_qlists")
        n = nr.value
        return cls(rq1[:n].copy(), rb1[:n].copy(),
                   p3[: n + 1].copy() if opts.thirdorder else None,
                   l3[: n * np3].copy() if opts.thirdorder else None,
                   p4[: n + 1].copy() if opts.fourthorder else None,
                   l4a[: n * np4].copy() if opts.fourthorder else None,
                   l4b[: n * np4].copy() if opts.fourthorder else None)

    @classmethod
    def per_irreducible(cls, prob: Problem, samples3: dict | None = None, samples4: dict | None = None) -> "QLists":
        """Explicit samples per irreducible q1 (1-based key), shared by all rows of q1."""
        rq1, rb1 = prob.rows()
        p3 = l3 = p4 = l4a = l4b = None
        if samples3 is not None:
            lists = [np.asarray(samples3[int(q)], np.int32) for q in rq1]
            p3 = np.concatenate([[0], np.cumsum([x.size for x in lists])]).astype(np.int64)
            l3 = np.concatenate(lists).astype(np.int32)
        if samples4 is not None:
            la = [np.asarray(samples4[int(q)][0], np.int32) for q in rq1]
            lb = [np.asarray(samples4[int(q)][1], np.int32) for q in rq1]
            p4 = np.concatenate([[0], np.cumsum([x.size for x in la])]).astype(np.int64)
            l4a = np.concatenate(la).astype(np.int32)
            l4b = np.concatenate(lb).astype(np.int32)
        return cls(rq1, rb1, p3, l3, p4, l4a, l4b)

    def struct(self) -> N.TdgQlists:
        s = N.TdgQlists()
        arrs = [np.ascontiguousarray(x) if x is not None else None
                for x in (self.row_q1, self.row_b1, self.ptr3, self.list3, self.ptr4, self.list4a, self.list4b)]
        self._keep = arrs
        s.n_row = self.n_row
        s.row_q1 = N.ptr(arrs[0], C.c_int32)
        s.row_b1 = N.ptr(arrs[1], C.c_int32)
        s.ptr3 = N.ptr(arrs[2], C.c_int64)
        s.list3 = N.ptr(arrs[3], C.c_int32)
        s.ptr4 = N.ptr(arrs[4], C.c_int64)
        s.list4a = N.ptr(arrs[5], C.c_int32)
        s.list4b = N.ptr(arrs[6], C.c_int32)
        return s


class ScatteringRates:
    """lo_scattering_rates on one GB300 (scattering.f90:34-55)."""

    def __init__(self, prob: Problem, device: int = 0):
        self.prob = prob
        self._lib = N.lib()
        self._ctx = C.c_void_p()
        ps = prob.struct()
        N.check(self._lib.tdg_create(C.byref(self._ctx), C.byref(ps), int(device)), "tdg_create")
        self.linewidth = None
        self.qs = None
        self.stats = None
        self.lists = None

    def close(self):
        if self._ctx:
            self._lib.tdg_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def generate(self, opts: Options, lists: QLists | None = None) -> np.ndarray:
        """sr%generate: linewidths (n_irr, n_mode) in Hartree; Xi stays on the device."""
        p = self.prob
        if lists is None:
            lists = QLists.monte_carlo(p, opts)
        self.lists = lists
        lw = np.zeros(p.n_irr * p.n_mode)
        qs = np.zeros(p.n_irr * p.n_mode)
        st = np.zeros(10)
        o = opts.struct(p.grid)
        q = lists.struct()
        N.check(self._lib.tdg_scattering(self._ctx, C.byref(o), C.byref(q), N.ptr(lw, C.c_double),
                                         N.ptr(qs, C.c_double), N.ptr(st, C.c_double)), "tdg_scattering")
        self.linewidth = lw.reshape(p.n_irr, p.n_mode)
        self.qs = qs.reshape(p.n_irr, p.n_mode)
        self.stats = {"triplets": int(st[0]), "quartets": int(st[1]), "device_ms": float(st[2]),
                      "candidates": int(st[3]), "enumerate_ms": float(st[4]), "threephonon_ms": float(st[5]),
                      "symmetrize_ms": float(st[6]), "isotope_ms": float(st[7]), "launches": int(st[8]),
                      "equivalent_triplets": int(st[9])}
        return self.linewidth

    def triplets(self, q1: int, sample) -> list:
        """Device enumeration of the irreducible triplets of one sample (1-based indices):
        [(q2, q3, [(q2', q3'), ...]), ...] in sample order."""
        sample = np.ascontiguousarray(sample, dtype=np.int32)
        cap = max(64, 8 * sample.size * (2 + 2 * self.prob.n_op))
        out = np.zeros(cap, np.int32)
        w = C.c_int64(0)
        N.check(self._lib.tdg_triplets(self._ctx, int(q1), N.ptr(sample, C.c_int32), sample.size,
                                       N.ptr(out, C.c_int32), cap, C.byref(w)), "tdg_triplets")
        res, i = [], 0
        while i < w.value:
            q2, q3, k = int(out[i]), int(out[i + 1]), int(out[i + 2])
            pairs = [(int(out[i + 3 + 2 * j]), int(out[i + 4 + 2 * j])) for j in range(k)]
            res.append((q2, q3, pairs))
            i += 3 + 2 * k
        return res

    @property
    def Xi(self) -> np.ndarray:
        p = self.prob
        xi = np.zeros((self.lists.n_row, p.n_full * p.n_mode))
        N.check(self._lib.tdg_get_xi(self._ctx, N.ptr(xi, C.c_double)), "tdg_get_xi")
        return xi

    def kappa_offdiag(self, opts: Options) -> np.ndarray:
        """get_kappa_offdiag (kappa.f90:77-306) + symmetrize_kappa from the linewidths of the
        last generate(). Returns the a.u. 3x3 off-diagonal (coherence) tensor."""
        o = opts.struct(self.prob.grid)
        k = np.zeros(9)
        N.check(self._lib.tdg_kappa_offdiag(self._ctx, C.byref(o), N.ptr(k, C.c_double)), "tdg_kappa_offdiag")
        return k.reshape(3, 3, order="F")

    def last_path(self) -> int:
        """Three-phonon path of the last generate(): 0 SIMT fused kernel, 1 tcgen05 fused
        kernel, 2 large-cell tcgen05 batches (tdg_last_path)."""
        v = C.c_int32(-1)
        N.check(self._lib.tdg_last_path(self._ctx, C.byref(v)), "tdg_last_path")
        return int(v.value)

    def last_launch(self) -> dict:
        """Launch shape of the fused three-phonon kernel in the last generate()
        (tdg_last_launch): grid, CTAs per SM used, the runtime's occupancy figure and the
        register/shared-memory count; -1 each on the large-cell path."""
        v = np.zeros(4, dtype=np.int32)
        N.check(self._lib.tdg_last_launch(self._ctx, N.ptr(v, C.c_int32)), "tdg_last_launch")
        return {"grid": int(v[0]), "ctas_per_sm": int(v[1]), "occupancy_api": int(v[2]),
                "occupancy_count": int(v[3])}

    def graph_counts(self) -> list[int]:
        """Direct runs, CUDA-graph recordings and replays of the three-phonon kernels on this
        context (tdg_graph_counts)."""
        c = np.zeros(3, dtype=np.int64)
        N.check(self._lib.tdg_graph_counts(self._ctx, N.ptr(c, C.c_int64)), "tdg_graph_counts")
        return [int(x) for x in c]

    def transfer_bytes(self) -> tuple[int, int]:
        """(host-to-device, device-to-host) bytes copied by this object's calls so far."""
        h, d = C.c_int64(0), C.c_int64(0)
        N.check(self._lib.tdg_transfer_bytes(self._ctx, C.byref(h), C.byref(d)), "tdg_transfer_bytes")
        return int(h.value), int(d.value)

    def kappa(self, opts: Options, maxiter: int | None = None, tol: float | None = None):
        """get_kappa (SMA), iterative_solution, symmetrize_kappa. Returns a.u. 3x3 tensors."""
        p = self.prob
        o = opts.struct(p.grid)
        ks = np.zeros(9)
        ki = np.zeros(9)
        fn = np.zeros(p.n_irr * p.n_mode * 3)
        nit = C.c_int32(0)
        mi = opts.itermaxsteps if maxiter is None else maxiter
        tl = opts.itertol if tol is None else tol
        N.check(self._lib.tdg_kappa(self._ctx, C.byref(o), int(mi), float(tl), N.ptr(ks, C.c_double),
                                    N.ptr(ki, C.c_double), N.ptr(fn, C.c_double), C.byref(nit)), "tdg_kappa")
        self.n_iter = nit.value
        self.Fn = fn.reshape(p.n_irr, p.n_mode, 3)
        return ks.reshape(3, 3, order="F"), ki.reshape(3, 3, order="F")

    # ---- differentiation with respect to the third-order force constants ----
    def set_fc3(self, fc3_mwm: np.ndarray) -> None:
        """Replace the mass-weighted third-order force constants ([n_fc3, 27], the layout of
        Problem.fc3_mwm); the next generate() uses them."""
        m = np.ascontiguousarray(fc3_mwm, dtype=np.float64).reshape(self.prob.n_fc3 * 27)
        N.check(self._lib.tdg_set_fc3(self._ctx, N.ptr(m, C.c_double)), "tdg_set_fc3")

    def kappa_sma_vjp(self, opts: Options, kappa_bar: np.ndarray) -> np.ndarray:
        """(d kappa_sma / d linewidth)^T kappa_bar at the last generate(): [n_irr, n_mode]."""
        p = self.prob
        kb = np.ascontiguousarray(np.asarray(kappa_bar, dtype=np.float64).reshape(3, 3).ravel(order="F"))
        out = np.zeros(p.n_irr * p.n_mode)
        o = opts.struct(p.grid)
        N.check(self._lib.tdg_kappa_sma_vjp(self._ctx, C.byref(o), N.ptr(kb, C.c_double), N.ptr(out, C.c_double)),
                "tdg_kappa_sma_vjp")
        return out.reshape(p.n_irr, p.n_mode)

    def kappa_iter_vjp(self, opts: Options, kappa_bar: np.ndarray, maxiter: int | None = None,
                       tol: float | None = None) -> np.ndarray:
        """Cotangent of the linewidths for d(kappa_bar : kappa_iter) (tdg_kappa_iter_vjp);
        the next adjoint_fc3 also adds the scattering-matrix term it leaves on the device."""
        p = self.prob
        o = opts.struct(p.grid)
        kb = np.ascontiguousarray(np.asarray(kappa_bar, np.float64).reshape(3, 3).ravel(order="F"))
        out = np.zeros(p.n_irr * p.n_mode)
        nit = C.c_int32(0)
        mi = opts.itermaxsteps if maxiter is None else maxiter
        tl = opts.itertol if tol is None else tol
        N.check(self._lib.tdg_kappa_iter_vjp(self._ctx, C.byref(o), N.ptr(kb, C.c_double), int(mi), float(tl),
                                             N.ptr(out, C.c_double), C.byref(nit)), "tdg_kappa_iter_vjp")
        self.vjp_iter = nit.value
        return out.reshape(p.n_irr, p.n_mode)

    def adjoint_fc3(self, opts: Options, lw_bar: np.ndarray) -> np.ndarray:
        """(d linewidth / d fc3_mwm)^T lw_bar over the q-triplets of the last generate():
        [n_fc3, 27]. Timing of the pass in self.adjoint_stats."""
        p = self.prob
        lb = np.ascontiguousarray(lw_bar, dtype=np.float64).reshape(p.n_irr * p.n_mode)
        out = np.zeros(p.n_fc3 * 27)
        st = np.zeros(4)
        o = opts.struct(p.grid)
        N.check(self._lib.tdg_adjoint_fc3(self._ctx, C.byref(o), N.ptr(lb, C.c_double), N.ptr(out, C.c_double),
                                          N.ptr(st, C.c_double)), "tdg_adjoint_fc3")
        self.adjoint_stats = {"ms": float(st[0]), "kernel_ms": float(st[1]), "triplets": int(st[2]),
                              "batches_or_ctas": int(st[3])}
        return out.reshape(p.n_fc3, 27)


def write_outfile(directory, temperature, kappa_sma, kappa_iter, kappa_offdiag=None) -> Path:
    """outfile.thermal_conductivity (main.f90:246-294); tensors in atomic units."""
    L = N.lib()
    ks = np.ascontiguousarray(np.asarray(kappa_sma).reshape(3, 3).ravel(order="F"))
    ki = np.ascontiguousarray(np.asarray(kappa_iter).reshape(3, 3).ravel(order="F"))
    ko = np.zeros(9) if kappa_offdiag is None else np.ascontiguousarray(np.asarray(kappa_offdiag).reshape(3, 3).ravel(order="F"))
    N.check(L.tdg_write_outfile(str(directory).encode(), float(temperature), N.ptr(ks, C.c_double),
                                N.ptr(ki, C.c_double), N.ptr(ko, C.c_double)), "tdg_write_outfile")
    return Path(directory) / "outfile.thermal_conductivity"


def write_grid_hdf5(path, prob: "Problem", temperature, linewidth, fn=None) -> Path:
    """outfile.thermal_conductivity_grid.hdf5 (type_phonon_dispersions.f90:316-641): per-mode
    data of the full mesh from the linewidths (n_irr, n_mode) of generate() and the final Fn
    (n_irr, n_mode, 3) of kappa(), or fn=None for the relaxation-time form."""
    lw = np.ascontiguousarray(np.asarray(linewidth, np.float64).reshape(-1))
    f = None if fn is None else np.ascontiguousarray(np.asarray(fn, np.float64).reshape(-1))
    ps = prob.struct()
    N.check(N.lib().tdg_write_grid_hdf5(str(path).encode(), C.byref(ps), float(temperature), N.ptr(lw, C.c_double),
                                        N.ptr(f, C.c_double) if f is not None else None), "tdg_write_grid_hdf5")
    return Path(path)


def phonon_frequencies(directory, q, qdir=None) -> np.ndarray:
    """Harmonic frequencies in Hartree, ascending, at Cartesian points q (1/Bohr, no 2*pi),
    from infile.ucposcar and infile.forceconstant in `directory`, polar force constants
    included (type_phonon_dispersions.f90:1083-1190). At Gamma the non-analytic term is
    taken along qdir (default [1,0,0]; a zero row leaves it out). Host-side computation."""
    L = N.lib()
    qa = np.ascontiguousarray(np.asarray(q, dtype=np.float64).reshape(-1, 3))
    da = None if qdir is None else np.ascontiguousarray(np.asarray(qdir, dtype=np.float64).reshape(-1, 3))
    if da is not None and da.shape != qa.shape:
        raise ValueError("qdir must have the shape of q")
    nq = qa.shape[0]
    # The mode count is known only after reading the cell: 3 * number of atoms.
    first = Path(directory, "infile.ucposcar").read_text().split("\n")
    na = sum(int(x) for x in first[6].split())
    om = np.zeros((nq, 3 * na))
    N.check(L.tdg_phonon_frequencies(str(directory).encode(), nq, N.ptr(qa, C.c_double),
                                     None if da is None else N.ptr(da, C.c_double), N.ptr(om, C.c_double)),
            "tdg_phonon_frequencies")
    return om


def release_cached_memory(device: int = 0) -> None:
    """Return the device memory the library keeps for reuse after contexts close."""
    N.check(N.lib().tdg_release_cached_memory(int(device)), "tdg_release_cached_memory")


def device_count() -> int:
    return int(N.lib().tdg_device_count())
