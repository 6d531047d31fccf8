"""The C-ABI library loads (no GPU needed) and exports every function
include/swgb300.h declares; host-only entry points behave."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    text = (ROOT / "include" / "swgb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sw_[a-z0-9_]+)\s*\(", text)))


def test_header_exports(sw):
    lib = sw._lib.load()
    names = _declared()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(sw._lib.EXPORTS) == names


def test_version_and_bad_args(sw):
    lib = sw._lib.load()
    assert lib.sw_version() >= 100
    assert lib.sw_ctx_create(0, None, None) == sw._lib.SW_ERR_ARG
    assert lib.sw_wavesim_destroy(None) == sw._lib.SW_ERR_ARG
    assert lib.sw_profile_enable(None, 1) == sw._lib.SW_ERR_ARG
    n = ctypes.c_int64(-1)
    assert lib.sw_profile_read_kernels(None, 0, ctypes.byref(n)) == sw._lib.SW_ERR_ARG and n.value == -1
    assert lib.sw_wavesim_set_tuning(None, 0, 262144) == sw._lib.SW_ERR_ARG


@pytest.mark.parametrize("halo,freetop", [(20, False), (20, True), (7, False), (1, True), (0, False)])
def test_cpml_coefficients_match_oracle(sw, oracle, halo, freetop):
    vmax, dt, rcoef, h, f0 = 3500.0, 7.5e-4, 1e-4, 10.0, 8.0
    a, ah, b, bh = sw._lib.cpml_coefficients(vmax, dt, halo, rcoef, h, f0, freetop)
    blk = oracle.cpml_block(vmax, dt, halo, rcoef, h, f0, freetop)
    na, nh = 2 * (halo + 1), 2 * halo
    np.testing.assert_allclose(a, blk[:na], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(ah, blk[na:na + nh], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(b, blk[na + nh:2 * na + nh], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(bh, blk[2 * na + nh:], rtol=1e-6, atol=1e-12)
    assert np.all(b > 0) and np.all(b <= 1) and np.all(a <= 0)
    if freetop:
        assert np.all(a[: na // 2] == 0) and np.all(b[: na // 2] == 1)
    # the FP64 entry point (compensated forward) gives the oracle's values to FP64 rounding and
    # rounds to the FP32 ones
    a6, ah6, b6, bh6 = sw._lib.cpml_coefficients64(vmax, dt, halo, rcoef, h, f0, freetop)
    np.testing.assert_allclose(np.concatenate([a6, ah6, b6, bh6]), blk, rtol=1e-13, atol=1e-300)
    for x32, x64 in ((a, a6), (ah, ah6), (b, b6), (bh, bh6)):
        assert np.array_equal(x32, x64.astype(np.float32))
