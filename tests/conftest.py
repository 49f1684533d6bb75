"""Shared fixtures: synthetic crystals written by tdep_gb300.synth into a session tmpdir."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (runs the native sm_103a path)")


@pytest.fixture(scope="session")
def built():
    from tdep_gb300 import build

    build.build_all()
    return True


@pytest.fixture(scope="session")
def configs(tmp_path_factory, built):
    from tdep_gb300 import synth

    base = tmp_path_factory.mktemp("configs")
    return {
        "fcc": synth.write_config("fcc_morse", base / "fcc", seed=1),
        "rocksalt": synth.write_config("rocksalt", base / "rocksalt", seed=1),
        "perovskite": synth.write_config("perovskite", base / "perovskite", seed=1),
        # 10 atoms, 30 modes, no symmetry: the tensor-core path is taken automatically
        "supercell": synth.write_config("perovskite_supercell", base / "supercell", seed=1, reps=(2, 1, 1)),
        # 3 and 4 atoms (9 and 12 modes): the tcgen05 fused kernel's other mode counts
        "fluorite": synth.write_config("fluorite", base / "fluorite", seed=1),
        "l12": synth.write_config("l12", base / "l12", seed=1),
    }


@pytest.fixture(scope="session")
def configs4(tmp_path_factory, built):
    """The same crystals with fourth-order force constants."""
    from tdep_gb300 import synth

    base = tmp_path_factory.mktemp("configs4")
    return {
        "fcc": synth.write_config("fcc_morse", base / "fcc", seed=1, order4=True),
        "rocksalt": synth.write_config("rocksalt", base / "rocksalt", seed=1, order4=True),
        "perovskite": synth.write_config("perovskite", base / "perovskite", seed=1, order4=True),
    }
