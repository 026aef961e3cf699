"""The coefficients of the kernels' branch-free atan2 (atan2_poly in
zodipy_gb300/csrc/zl_common.cuh) are the output of the fit in tests/atan2_fit.py:
re-run the fit, compare with the literals compiled into the kernels, and check the
float32-emulated error bound the kernel comment states (CPU only)."""

import os
import re

import numpy as np

import atan2_fit

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "zodipy_gb300", "csrc",
                      "zl_common.cuh")


def _header_coefficients():
    src = open(HEADER).read()
    body = src[src.index("float atan2_poly(") :]
    body = body[: body.index("return copysignf")]
    first = float(re.search(r"float q = ([-0-9.e]+)f;", body).group(1))
    rest = [float(v) for v in re.findall(r"q = fmaf\(q, s, ([-0-9.e]+)f\);", body)]
    return np.array([first, *rest][::-1])  # low order first, as the fit returns them


def test_fit_reproduces_the_compiled_coefficients():
    got = _header_coefficients()
    assert got.size == atan2_fit.DEG + 1
    fit = atan2_fit.fit(atan2_fit.DEG).astype(np.float32).astype(np.float64)
    np.testing.assert_allclose(got, fit, rtol=2e-6, atol=1e-8)


def test_compiled_coefficients_error_bound():
    c = _header_coefficients()
    t = atan2_fit.f32(np.linspace(0, 1, 200001))
    ref = np.arctan(t)
    ulp = np.spacing(np.maximum(ref, 1e-30).astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(atan2_fit.atan_poly(c, t) - ref) / ulp) <= 1.5
    rng = np.random.default_rng(3)
    y, x = atan2_fit.f32(rng.standard_normal(1 << 18)), atan2_fit.f32(rng.standard_normal(1 << 18))
    ref2 = np.arctan2(y, x)
    err = np.abs(atan2_fit.atan2_model(c, y, x) - ref2) / np.spacing(np.abs(ref2).astype(np.float32)).astype(np.float64)
    assert err.max() <= 4.0
