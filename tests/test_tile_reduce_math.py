"""The adjoint's warp reduction (bwd_tile_reduce / warp_halve in zl_bwd_f32.cuh), on the CPU.

Each of a warp's 32 lanes holds K partial sums (the gradient entries a launch writes), padded
to 32 W slots, W = ceil(K / 32).  Five levels of recursive halving (lane masks 16, 8, 4, 2, 1)
leave lane L with the warp's sums of slots L W .. L W + W - 1.  At a level with 2H slots per
lane, slot j's partner H + j is padding on every lane when H + j >= K; there the kernel adds
the partner lane's copy of slot j without selecting, so the upper lane's slot j (a padding
slot after the level) holds whatever it adds up to.  This emulates the 32 lanes with numpy,
shuffles as index permutations, and checks every slot that the kernel stores against the
plain sum, for every K from 1 to 100 (the launches write 20 to 78).
"""

import numpy as np


def warp_reduce(v: np.ndarray, k: int) -> np.ndarray:
    """v: (32, 32 W) per-lane slots; returns (32, W), lane L's final slots."""
    lanes = np.arange(32)
    w = v.shape[1] // 32
    v = v.copy()
    for m, h in ((16, 16 * w), (8, 8 * w), (4, 4 * w), (2, 2 * w), (1, w)):
        up = (lanes & m) != 0
        partner = lanes ^ m
        new = np.empty((32, h), dtype=v.dtype)
        for j in range(h):
            if h + j >= k:
                new[:, j] = v[:, j] + v[partner, j]
            else:
                send = np.where(up, v[:, j], v[:, h + j])
                keep = np.where(up, v[:, h + j], v[:, j])
                new[:, j] = keep + send[partner]
        v = new
    return v


def test_every_stored_slot_is_the_warp_sum():
    rng = np.random.default_rng(5)
    for k in range(1, 101):
        w = (k + 31) // 32
        vals = np.zeros((32, 32 * w))
        vals[:, :k] = rng.integers(-1000, 1000, size=(32, k))  # exact in float64: the sums are exact
        # padding slots start at zero in the kernel; garbage must not reach a real slot either way
        out = warp_reduce(vals, k)
        want = vals.sum(axis=0)
        for lane in range(32):
            for t in range(w):
                g = lane * w + t
                if g < k:
                    assert out[lane, t] == want[g], (k, lane, t)


def test_padding_never_reaches_a_stored_slot():
    """Non-zero values in the padding slots (as an earlier level's shortcut leaves them) do not
    change any slot the kernel stores."""
    rng = np.random.default_rng(6)
    for k in (20, 26, 31, 33, 50, 64, 78):
        w = (k + 31) // 32
        vals = np.zeros((32, 32 * w))
        vals[:, :k] = rng.integers(-1000, 1000, size=(32, k))
        noisy = vals.copy()
        noisy[:, k:] = rng.integers(-10**6, 10**6, size=(32, 32 * w - k))
        a, b = warp_reduce(vals, k), warp_reduce(noisy, k)
        for lane in range(32):
            for t in range(w):
                if lane * w + t < k:
                    assert a[lane, t] == b[lane, t], (k, lane, t)
