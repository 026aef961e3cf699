"""GPU parity: libzodigb's kernels against the reference's golden outputs and the oracle.

Tolerances:
  float64 plain kernel vs reference/oracle ........ 1e-10 relative per component,
      or 1e-15 of the pixel's total brightness, whichever is looser.  The floor
      covers values the reference itself evaluates ill-conditioned: a band's
      inner cutoff 1 - exp(-(R/dr)^20) at y ~ 1e-14 keeps ~2 digits, so a
      1-ulp difference between CUDA's and glibc's exp moves that term by ~1 %;
      and quadrature terms near the subnormal range (e^-729) keep few bits.
  float32-bulk kernel vs float64 ................... 1e-5 relative on the total, and
      per component 1e-5 relative to max(|component|, 1e-3 |total|)
"""

import numpy as np
import pytest

from conftest import cuda_ok, golden_cases, load_case, oracle_desc, product_model
from oracle import zodi_oracle as zo

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]

F64_RTOL = 1e-10
F64_ATOL = 1e-200
F32_RTOL = 1e-5


def assert_f64_close(got, ref, what=""):
    floor = np.maximum(F64_ATOL, 1e-15 * np.abs(ref.sum(axis=0)))[None, :]
    err = np.abs(got - ref) - F64_RTOL * np.abs(ref)
    bad = err > floor
    if bad.any():
        c, i = np.unravel_index(np.argmax(np.where(bad, np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300), 0)), got.shape)
        raise AssertionError(
            f"{what}: {bad.sum()} elements off; worst comp {c} pixel {i}: got {got[c, i]!r} ref {ref[c, i]!r}"
        )


def _ref_fixed(case):
    """Reference output, with the b == 0 rows replaced by the documented finite root."""
    ref = case["ref_out"]
    if np.isnan(ref).any():
        ref = zo.evaluate(oracle_desc(case), case["unit_vectors"], case["obs"], case["earth"], fix_b0=True)
    return ref


def _eval(model, case, precision):
    return model.evaluate_xyz(case["unit_vectors"], case["obs"], case["earth"], return_comps=True, precision=precision)


def rel_err_f32(got, ref):
    tot_ref = ref.sum(axis=0)
    tot = got.sum(axis=0)
    e_tot = np.abs(tot - tot_ref) / np.abs(tot_ref)
    floor = np.maximum(np.abs(ref), 1e-3 * np.abs(tot_ref)[None, :])
    e_comp = np.abs(got - ref) / floor
    return e_tot, e_comp


@pytest.mark.parametrize("name", golden_cases())
def test_f64_matches_reference(lib, name):
    case = load_case(name)
    model = product_model(case)
    got = _eval(model, case, "float64")
    ref = _ref_fixed(case)
    assert got.shape == ref.shape
    assert np.isfinite(got).all()
    assert_f64_close(got, ref, name)


@pytest.mark.parametrize("name", golden_cases())
def test_f32_matches_reference(lib, name):
    case = load_case(name)
    model = product_model(case)
    got = _eval(model, case, "float32")
    ref = _ref_fixed(case)
    e_tot, e_comp = rel_err_f32(got, ref)
    c, i = np.unravel_index(np.argmax(e_comp), e_comp.shape)
    assert e_tot.max() <= F32_RTOL, f"total max rel err {e_tot.max():.3e} at pixel {np.argmax(e_tot)}"
    assert e_comp.max() <= F32_RTOL, (
        f"component max rel err {e_comp.max():.3e}: comp {c} pixel {i} got {got[c, i]!r} ref {ref[c, i]!r} "
        f"total {ref[:, i].sum()!r}"
    )


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_total_is_component_sum_bit_exact(lib, precision):
    """return_comps=False equals the component sum exactly (reference tests/test_evaluate.py:198-212)."""
    case = load_case("dirbe25_nside8")
    model = product_model(case, precision)
    comps = model.evaluate_xyz(case["unit_vectors"], case["obs"], case["earth"], return_comps=True)
    total = model.evaluate_xyz(case["unit_vectors"], case["obs"], case["earth"], return_comps=False)
    np.testing.assert_array_equal(comps.sum(axis=0), total)


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_partition_independent(lib, precision):
    """Splitting the pixels changes no bit (reference tests/test_evaluate.py:215-262)."""
    case = load_case("dirbe25_nside8")
    model = product_model(case, precision)
    u = case["unit_vectors"]
    whole = model.evaluate_xyz(u, case["obs"], case["earth"], return_comps=True)
    parts = np.concatenate(
        [model.evaluate_xyz(p, case["obs"], case["earth"], return_comps=True) for p in np.array_split(u, 7, axis=-1)],
        axis=-1,
    )
    np.testing.assert_array_equal(whole, parts)


def test_f64_vs_oracle_random_observers(lib):
    """Fresh seeded inputs (not a fixture): float64 kernel vs oracle at 1e-10."""
    rng = np.random.default_rng(5)
    case = load_case("dirbe1p25_scatter")
    desc = oracle_desc(case)
    model = product_model(case)
    for _ in range(3):
        v = rng.standard_normal((3, 500))
        v /= np.linalg.norm(v, axis=0)
        d = rng.standard_normal(3)
        obs = d / np.linalg.norm(d) * rng.uniform(0.8, 2.0)
        earth = np.array([np.cos(rng.uniform(0, 6.28)), np.sin(rng.uniform(0, 6.28)), 0.0])
        ref = zo.evaluate(desc, v, obs, earth, fix_b0=True)
        got = model.evaluate_xyz(v, obs, earth, return_comps=True, precision="float64")
        assert_f64_close(got, ref, "random observer")
        e_tot, e_comp = rel_err_f32(model.evaluate_xyz(v, obs, earth, return_comps=True, precision="float32"), ref)
        assert e_tot.max() <= F32_RTOL and e_comp.max() <= F32_RTOL


def test_empty_and_single(lib):
    case = load_case("dirbe25_single")
    model = product_model(case)
    out = model.evaluate_xyz(np.zeros((3, 0)), case["obs"], case["earth"], return_comps=True)
    assert out.shape == (6, 0)
    one = model.evaluate_xyz(case["unit_vectors"], case["obs"], case["earth"], return_comps=True)
    assert_f64_close(one, case["ref_out"], "single")


def test_device_tensors_stay_on_device(lib):
    import torch

    case = load_case("planck18_857")
    model = product_model(case, "float32")
    u = torch.from_numpy(case["unit_vectors"]).cuda()
    out = model.evaluate_xyz(u, case["obs"], case["earth"], return_comps=True)
    assert out.is_cuda and out.dtype == torch.float64
    host = model.evaluate_xyz(case["unit_vectors"], case["obs"], case["earth"], return_comps=True)
    np.testing.assert_array_equal(out.cpu().numpy(), host)


def test_host_calls_restage_the_observer_when_it_changes(lib):
    """Host arrays go through the zero-copy path, which keeps the last observer record staged
    per thread: alternating observers, a changed Earth, and alternating models whose cutoff
    spheres (and so the record's cutoff flags) differ must each give the device path's bits."""
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import units as un

    case = load_case("dirbe25_nside8")
    dirbe = product_model(case, "float32")
    planck = zg.Model(857 * un.GHz, name="planck18", precision="float32")
    u = case["unit_vectors"]
    u_dev = torch.from_numpy(u).cuda()
    cases = [(np.array([1.0, 0.0, 0.0]), np.array([1.0, 0.0, 0.0])),
             (np.array([0.0, 1.6, 0.0]), np.array([0.0, 1.0, 0.0])),   # beyond the ring's and feature's spheres
             (np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0])),   # the first observer, another Earth
             (np.array([1.0, 0.0, 0.0]), np.array([1.0, 0.0, 0.0]))]
    for _ in range(2):
        for obs, earth in cases:
            for model in (dirbe, dirbe, planck):  # a repeated call, then another model, same observer
                host = model.evaluate_xyz(u, obs, earth, return_comps=True)
                dev = model.evaluate_xyz(u_dev, obs, earth, return_comps=True).cpu().numpy()
                np.testing.assert_array_equal(host, dev)
