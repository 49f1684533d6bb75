"""ctypes binding of include/tdep_gb300.h.

The library is loaded from the package's lib/ directory (built in-tree by
tdep_gb300.build). There is no Python fallback for anything the library computes: if the
shared object is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libtdep_gb300.so"

TDG_PREC_FP64 = 0
TDG_PREC_MIXED = 1

ERRORS = {
    1: "bad dimension",
    2: "linear algebra",
    3: "unphysical value",
    4: "symmetry",
    5: "bad parameter",
    6: "IO",
    8: "device",
}

_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)


class TdgProblem(C.Structure):
    _fields_ = [
        ("n_atom", C.c_int32),
        ("n_mode", C.c_int32),
        ("latvec", C.c_double * 9),
        ("reclat", C.c_double * 9),
        ("inv_reclat", C.c_double * 9),
        ("volume", C.c_double),
        ("mass_disorder", _f64p),
        ("n_op", C.c_int32),
        ("op_cart", _f64p),
        ("op_recfrac", _i32p),
        ("grid", C.c_int32 * 3),
        ("n_full", C.c_int32),
        ("n_irr", C.c_int32),
        ("q_full", _f64p),
        ("full_irr", _i32p),
        ("full_op", _i32p),
        ("irr_full", _i32p),
        ("irr_weight", _f64p),
        ("irr_nop", _i32p),
        ("irr_ops", _i32p),
        ("omega", _f64p),
        ("egv", _f64p),
        ("vel", _f64p),
        ("degen", _i32p),
        ("degen_mode", _i32p),
        ("n_fc3", C.c_int32),
        ("fc3_atoms", _i32p),
        ("fc3_lv", _i32p),
        ("fc3_lvcart", _f64p),
        ("fc3_mwm", _f64p),
        ("n_fc4", C.c_int32),
        ("fc4_atoms", _i32p),
        ("fc4_lv", _i32p),
        ("fc4_lvcart", _f64p),
        ("fc4_mwm", _f64p),
        ("irr_dyngrad", _f64p),
        ("op_fmap", _i32p),
        ("atom_shift", _f64p),
    ]


class TdgOpts(C.Structure):
    _fields_ = [
        ("temperature", C.c_double),
        ("integrationtype", C.c_int32),
        ("sigma", C.c_double),
        ("thirdorder", C.c_int32),
        ("fourthorder", C.c_int32),
        ("isotope", C.c_int32),
        ("classical", C.c_int32),
        ("mfp_max", C.c_double),
        ("qg3ph", C.c_int32 * 3),
        ("qg4ph", C.c_int32 * 3),
        ("seed", C.c_int32),
        ("precision", C.c_int32),
        ("tensor_cores", C.c_int32),
    ]


class TdgQlists(C.Structure):
    _fields_ = [
        ("n_row", C.c_int32),
        ("row_q1", _i32p),
        ("row_b1", _i32p),
        ("ptr3", _i64p),
        ("list3", _i32p),
        ("ptr4", _i64p),
        ("list4a", _i32p),
        ("list4b", _i32p),
    ]


# Every symbol include/tdep_gb300.h declares, with its ctypes signature.
SIGNATURES = {
    "tdg_last_error": (C.c_char_p, []),
    "tdg_version": (C.c_char_p, []),
    "tdg_device_count": (C.c_int, []),
    "tdg_check_exp": (C.c_int, [_f64p, C.c_int32, _f64p]),
    "tdg_check_mma": (C.c_int, [C.c_int32, C.c_int32, _f32p, _f32p, _f32p]),
    "tdg_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(TdgProblem), C.c_int]),
    "tdg_destroy": (None, [C.c_void_p]),
    "tdg_mc_qlists": (C.c_int, [C.POINTER(TdgProblem), C.POINTER(TdgOpts), _i32p, _i32p, _i32p, _i64p, _i32p,
                                _i64p, _i32p, _i32p]),
    "tdg_scattering": (C.c_int, [C.c_void_p, C.POINTER(TdgOpts), C.POINTER(TdgQlists), _f64p, _f64p, _f64p]),
    "tdg_get_xi": (C.c_int, [C.c_void_p, _f64p]),
    "tdg_transfer_bytes": (C.c_int, [C.c_void_p, _i64p, _i64p]),
    "tdg_kappa_offdiag": (C.c_int, [C.c_void_p, C.POINTER(TdgOpts), _f64p]),
    "tdg_release_cached_memory": (C.c_int, [C.c_int]),
    "tdg_write_grid_hdf5": (C.c_int, [C.c_char_p, C.POINTER(TdgProblem), C.c_double, _f64p, _f64p]),
    "tdg_fc3_irreducible": (C.c_int, [C.POINTER(TdgProblem), _i32p, C.POINTER(C.c_int64), _i32p, _i32p, _f64p,
                                      _f64p]),
    "tdg_kappa_iter_vjp": (C.c_int, [C.c_void_p, C.POINTER(TdgOpts), _f64p, C.c_int32, C.c_double, _f64p, _i32p]),
    "tdg_last_path": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "tdg_last_launch": (C.c_int, [C.c_void_p, _i32p]),
    "tdg_pool_usage": (C.c_int, [C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "tdg_natural_isotopes": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "tdg_autotune_load": (C.c_int, [C.c_char_p]),
    "tdg_autotune_save": (C.c_int, [C.c_char_p]),
    "tdg_autotune_report": (C.c_int, [C.c_char_p, C.c_int64, _i64p]),
    "tdg_autotune_clear": (C.c_int, []),
    "tdg_graph_counts": (C.c_int, [C.c_void_p, _i64p]),
    "tdg_triplets": (C.c_int, [C.c_void_p, C.c_int32, _i32p, C.c_int64, _i32p, C.c_int64, _i64p]),
    "tdg_triplets_static": (C.c_int, [C.c_void_p, C.c_int32, _i32p, C.c_int64, _i32p, C.c_int64, _i64p]),
    "tdg_set_fc3": (C.c_int, [C.c_void_p, _f64p]),
    "tdg_kappa_sma_vjp": (C.c_int, [C.c_void_p, C.POINTER(TdgOpts), _f64p, _f64p]),
    "tdg_adjoint_fc3": (C.c_int, [C.c_void_p, C.POINTER(TdgOpts), _f64p, _f64p, _f64p]),
    "tdg_kappa": (C.c_int, [C.c_void_p, C.POINTER(TdgOpts), C.c_int32, C.c_double, _f64p, _f64p, _f64p, _i32p]),
    "tdg_problem_load": (C.c_int, [C.c_char_p, _i32p, C.c_int, C.c_int, C.c_int, C.POINTER(C.POINTER(TdgProblem))]),
    "tdg_problem_load_device": (C.c_int, [C.c_char_p, _i32p, C.c_int, C.c_int, C.c_int, C.c_int32,
                                          C.POINTER(C.POINTER(TdgProblem))]),
    "tdg_problem_free": (None, [C.POINTER(TdgProblem)]),
    "tdg_write_outfile": (C.c_int, [C.c_char_p, C.c_double, _f64p, _f64p, _f64p]),
    "tdg_phonon_frequencies": (C.c_int, [C.c_char_p, C.c_int32, _f64p, _f64p, _f64p]),
}

_LIB = None


def lib() -> C.CDLL:
    """Load libtdep_gb300.so (raises OSError when it has not been built)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise OSError(f"{LIB_PATH} is missing: run `python -m tdep_gb300.build` (no CPU fallback exists)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


class TdgError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib().tdg_last_error().decode(errors="replace")
        super().__init__(f"{where}: {ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


def check(code: int, where: str) -> None:
    if code != 0:
        raise TdgError(code, where)


def ptr(a: np.ndarray | None, ctype):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


def autotune_table() -> dict[str, int]:
    """The launch-shape decisions of the autotuner in this process (key -> value)."""
    L = lib()
    need = C.c_int64(0)
    check(L.tdg_autotune_report(None, 0, C.byref(need)), "tdg_autotune_report")
    buf = C.create_string_buffer(int(need.value) + 1)
    check(L.tdg_autotune_report(buf, len(buf), C.byref(need)), "tdg_autotune_report")
    out = {}
    for line in buf.value.decode().splitlines():
        k, v = line.split()
        out[k] = int(v)
    return out
