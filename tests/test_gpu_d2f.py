"""The kernels convert doubles (unit vectors, observer positions, upstream gradients) to
float-float pairs and floats by bit operations instead of float64 instructions
(ff_split, d2f_bits in zodipy_gb300/csrc/zl_common.cuh).  Checked against the
conversion instruction and against exact arithmetic on constructed cases: values just
above, at and just below the halfway point between two floats (the rounding decision
then rests on the significand bits below the 47 the pair keeps), random values, and
the range limits."""

import ctypes
import struct

import numpy as np
import pytest

from conftest import cuda_ok



def _cases():
    rng = np.random.default_rng(31)
    base = rng.uniform(1.0, 2.0, 4096).astype(np.float32).astype(np.float64)
    base = base * 2.0 ** rng.integers(-60, 60, base.size) * np.where(rng.random(base.size) < 0.5, -1.0, 1.0)
    mid = base + np.sign(base) * np.spacing(np.abs(base).astype(np.float32)).astype(np.float64) / 2  # exact
    away = np.nextafter(mid, 2 * mid)  # one double ulp beyond halfway: a bit among the six the pair drops
    toward = np.nextafter(mid, 0.0)    # one double ulp short of halfway
    rand = (np.where(rng.random(1 << 16) < 0.5, -1.0, 1.0) * rng.uniform(1.0, 10.0, 1 << 16)
            * 10.0 ** rng.uniform(-20, 20, 1 << 16))
    edge = np.array([1.0, -1.0, 2.0**-69, -(2.0**-69), 3.4e38, -3.4e38, 1.5, 0.1, 1 / 3])
    d = np.concatenate([mid, away, toward, rand, edge])
    assert np.all(np.abs(d) >= 2.0**-70) and np.all(np.abs(d) < 2.0**128)
    # the constructed cases do exercise the dropped bits: rounding away differs from rounding toward
    assert np.all(away[:8].astype(np.float32) != toward[:8].astype(np.float32))
    return d


def _split_mirror(x: float, sticky: bool = True) -> np.float32:
    """ff_split's bit operations in Python (float32 arithmetic through numpy): the rounded hi."""
    b = struct.unpack("<Q", struct.pack("<d", x))[0]
    hw, lw = b >> 32, b & 0xFFFFFFFF
    e, sign = (hw >> 20) & 0x7FF, hw & 0x80000000
    f32 = lambda bits: np.float32(struct.unpack("<f", struct.pack("<I", bits))[0])  # noqa: E731
    hi = f32(sign | ((e - 1023 + 127) << 23) | ((hw & 0xFFFFF) << 3) | (lw >> 29))
    base = sign | ((e - 1023 - 23 + 127) << 23)
    low23 = ((lw & 0x1FFFFFFF) >> 6) | (1 if (sticky and lw & 0x3F) else 0)
    lo = f32(base | low23) - f32(base)
    return np.float32(hi + lo)


def test_bit_split_rounds_like_the_conversion_cpu():
    """CPU mirror of the kernel's bit split: equal to numpy's round-to-nearest-even conversion
    on every case; without the sticky bit the halfway cases round the wrong way."""
    d = _cases()
    got = np.array([_split_mirror(x) for x in d])
    np.testing.assert_array_equal(got, d.astype(np.float32))
    assert sum(_split_mirror(x, sticky=False) != np.float32(x) for x in d) > 0


@pytest.mark.gpu
@pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")
def test_split_and_rounding_match_the_conversion(lib):
    import torch

    d = _cases()
    dd = torch.from_numpy(d).cuda()
    out = torch.empty(3 * d.size, dtype=torch.float32, device="cuda")
    rc = lib.zl_diag_d2f(ctypes.c_void_p(dd.data_ptr()), ctypes.c_void_p(out.data_ptr()), d.size,
                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    o = out.cpu().numpy().reshape(-1, 3).astype(np.float64)
    hi, lo, rounded = o[:, 0], o[:, 1], o[:, 2]
    want = d.astype(np.float32).astype(np.float64)  # round to nearest even of the double
    np.testing.assert_array_equal(rounded, want)
    np.testing.assert_array_equal(hi, want)
    # the pair keeps 47 significand bits (the last one sticky): |hi + lo - d| < 2^-45 |d|
    assert np.all(np.abs((hi + lo) - d) < 2.0**-45 * np.abs(d))


def _float_cases():
    """Float bit patterns: random ones over the whole range (normal, subnormal, inf, NaN of
    either sign), every exponent, and the edges."""
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 1 << 32, 1 << 20, dtype=np.uint64).astype(np.uint32)
    expo = (np.arange(256, dtype=np.uint32) << 23) | rng.integers(0, 1 << 23, 256, dtype=np.uint64).astype(np.uint32)
    edge = np.array([0x00000000, 0x80000000, 0x00000001, 0x807FFFFF, 0x00800000, 0x7F7FFFFF, 0xFF7FFFFF,
                     0x7F800000, 0xFF800000, 0x7FC00000, 0x7F800001, 0x3F800000, 0xBF800000], dtype=np.uint32)
    return np.concatenate([bits, expo, expo | 0x80000000, edge]).view(np.float32)


@pytest.mark.gpu
@pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")
def test_float_to_double_bits_match_the_conversion(lib):
    """The kernels store their float results as doubles by bit operations (f2d_bits): the same
    double as the conversion instruction for every float, NaN payloads included (they take
    the instruction)."""
    import torch

    f = _float_cases()
    fd = torch.from_numpy(f).cuda()
    out = torch.empty(f.size, dtype=torch.float64, device="cuda")
    rc = lib.zl_diag_f2d(ctypes.c_void_p(fd.data_ptr()), ctypes.c_void_p(out.data_ptr()), f.size,
                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    got = out.cpu().numpy()
    want = fd.double().cpu().numpy()  # the conversion instruction
    np.testing.assert_array_equal(got.view(np.uint64), want.view(np.uint64))
