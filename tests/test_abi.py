"""The C-ABI library: exports, error codes, behaviour without a GPU (CPU only)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from tdep_gb300 import _native as N
from tdep_gb300 import Options, Problem, device_count

HEADER = Path(__file__).resolve().parent.parent / "include" / "tdep_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tdg_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(built):
    lib = C.CDLL(str(N.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 12
    for name in names:
        assert hasattr(lib, name), name
    # and the Python binding covers all of them
    assert set(names) == set(N.SIGNATURES)


def test_version_and_device_count(built):
    assert b"sm_103a" in N.lib().tdg_version()
    assert device_count() >= 0


def test_no_cpu_fallback_without_gpu(built, configs):
    if device_count() > 0:
        pytest.skip("a GPU is present")
    from tdep_gb300 import ScatteringRates

    prob = Problem.load(configs["fcc"], (4, 4, 4), readiso=True)
    with pytest.raises(N.TdgError) as e:
        ScatteringRates(prob)
    assert e.value.code == 8 and "no CPU fallback" in str(e.value)


def test_io_errors(built, tmp_path):
    with pytest.raises(N.TdgError) as e:
        Problem.load(tmp_path / "missing", (4, 4, 4))
    assert e.value.code == 6


def test_bad_grid_is_a_parameter_error(built, configs):
    with pytest.raises(N.TdgError) as e:
        Problem.load(configs["fcc"], (4, 0, 4), readiso=True)
    assert e.value.code == 5


def test_malformed_forceconstant_is_an_io_error(built, configs, tmp_path):
    import shutil

    d = tmp_path / "bad"
    shutil.copytree(configs["fcc"], d)
    txt = (d / "infile.forceconstant_thirdorder").read_text().splitlines()
    (d / "infile.forceconstant_thirdorder").write_text("\n".join(txt[: len(txt) // 2]) + "\n")
    with pytest.raises(N.TdgError) as e:
        Problem.load(d, (4, 4, 4), readiso=True)
    assert e.value.code == 6


def test_non_lattice_vector_is_rejected(built, configs, tmp_path):
    import shutil

    d = tmp_path / "frac"
    shutil.copytree(configs["fcc"], d)
    lines = (d / "infile.forceconstant_thirdorder").read_text().splitlines()
    # the 6th line of the file is lv2 of the first triplet; make it non-integer
    lines[6] = "  0.5000000000000000  0.0000000000000000  0.0000000000000000"
    (d / "infile.forceconstant_thirdorder").write_text("\n".join(lines) + "\n")
    with pytest.raises(N.TdgError) as e:
        Problem.load(d, (4, 4, 4), readiso=True)
    assert e.value.code == 6 and "lattice vector" in str(e.value)


def test_mc_qlists_rejects_bad_seed(built, configs):
    from tdep_gb300 import QLists

    prob = Problem.load(configs["fcc"], (4, 4, 4), readiso=True)
    with pytest.raises(N.TdgError) as e:
        QLists.monte_carlo(prob, Options(seed=0))
    assert e.value.code == 5


def test_outfile_layout_matches_reference(built, tmp_path):
    """The writer reproduces the reference's outfile.thermal_conductivity layout."""
    from tdep_gb300 import KAPPA_AU_TO_SI, write_outfile

    ref = (Path(__file__).parent / "golden" / "mgo" / "outfile.thermal_conductivity.ref").read_text().splitlines()
    vals = np.loadtxt(Path(__file__).parent / "golden" / "mgo" / "outfile.thermal_conductivity.ref")
    ks = np.diag(vals[0][:3]) / KAPPA_AU_TO_SI
    ki = (np.diag(vals[0][:3]) + np.diag(vals[1][:3])) / KAPPA_AU_TO_SI
    ko = np.diag(vals[2][:3]) / KAPPA_AU_TO_SI
    out = write_outfile(tmp_path, 300.0, ks, ki, ko).read_text().splitlines()
    assert len(out) == len(ref)
    for a, b in zip(out, ref):
        if a.startswith("#"):
            assert a.rstrip() == b.rstrip()
        else:
            np.testing.assert_allclose([float(x) for x in a.split()], [float(x) for x in b.split()], rtol=1e-10,
                                       atol=1e-14)
            assert len(a) == len(b)


def test_autotune_table_round_trip(built, tmp_path):
    """The autotuner's decision table loads, reports and saves its text format (no GPU)."""
    L = N.lib()
    N.check(L.tdg_autotune_clear(), "clear")
    f = tmp_path / "tune.txt"
    f.write_text("# comment\nthreephonon/n6/p1/sm152/NVIDIA_GB300 12\n\nlargecell/n120/p1/sm152/NVIDIA_GB300 164\n")
    N.check(L.tdg_autotune_load(str(f).encode()), "load")
    t = N.autotune_table()
    assert t == {"threephonon/n6/p1/sm152/NVIDIA_GB300": 12, "largecell/n120/p1/sm152/NVIDIA_GB300": 164}
    g = tmp_path / "saved.txt"
    N.check(L.tdg_autotune_save(str(g).encode()), "save")
    N.check(L.tdg_autotune_clear(), "clear")
    assert N.autotune_table() == {}
    N.check(L.tdg_autotune_load(str(g).encode()), "reload")
    assert N.autotune_table() == t
    # truncated report stays NUL-terminated and reports the full size
    need = C.c_int64(0)
    buf = C.create_string_buffer(8)
    N.check(L.tdg_autotune_report(buf, 8, C.byref(need)), "report")
    assert len(buf.value) == 7 and need.value > 8
    bad = tmp_path / "bad.txt"
    bad.write_text("key notanumber\n")
    assert L.tdg_autotune_load(str(bad).encode()) == 6
    assert L.tdg_autotune_load(str(tmp_path / "missing.txt").encode()) == 6
    N.check(L.tdg_autotune_clear(), "clear")
