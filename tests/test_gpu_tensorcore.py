"""tcgen05 tensor-core building block of the large-cell contraction: one 128 x n x 16 tile
through shared-memory descriptors and tensor memory, BF16 hi/lo operand splits and FP32
accumulation, against the FP64 product on the host."""
import ctypes as C

import numpy as np
import pytest

from tdep_gb300 import _native as N
from tdep_gb300 import device_count

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _require_gpu(built):
    assert device_count() > 0, "GPU tests need a CUDA device; the GB300 path has no CPU fallback"


@pytest.mark.parametrize("n", [16, 64, 240, 256])
@pytest.mark.parametrize("variant", [0, 2])  # MN-major and K-major operands
def test_mma_tile_matches_fp64_product(n, variant):
    rng = np.random.default_rng(n + variant)
    a = rng.normal(size=(128, 16)).astype(np.float32)
    b = rng.normal(size=(16, n)).astype(np.float32)
    d = np.zeros((128, n), np.float32)
    N.check(N.lib().tdg_check_mma(variant, n, N.ptr(a, C.c_float), N.ptr(b, C.c_float), N.ptr(d, C.c_float)),
            "tdg_check_mma")
    ref = a.astype(np.float64) @ b.astype(np.float64)
    # three BF16 products keep about 16 bits per operand
    assert np.abs(d - ref).max() <= 2e-5 * np.abs(ref).max()
