"""Pin the CPU oracle to the reference's own outputs (golden fixtures)."""

import numpy as np
import pytest

from conftest import golden_cases, load_case, oracle_desc
from oracle import zodi_oracle as zo


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference(name):
    case = load_case(name)
    desc = oracle_desc(case)
    out = zo.evaluate(desc, case["unit_vectors"], case["obs"], case["earth"])
    ref = case["ref_out"]
    assert out.shape == ref.shape
    # same nan pattern (the b == 0 quirk), and a few-ulp agreement elsewhere
    np.testing.assert_array_equal(np.isnan(out), np.isnan(ref))
    finite = np.isfinite(ref)
    np.testing.assert_allclose(out[finite], ref[finite], rtol=1e-13, atol=0)


def test_oracle_b0_quirk_documented():
    """Where the reference yields nan (b == 0), fix_b0 gives the finite root."""
    case = load_case("dirbe25_b0")
    desc = oracle_desc(case)
    ref = case["ref_out"]
    assert np.isnan(ref).all()
    fixed = zo.evaluate(desc, case["unit_vectors"], case["obs"], case["earth"], fix_b0=True)
    assert np.isfinite(fixed).all() and (fixed[0] > 0).all()


def test_dirbe_idl_known_answers():
    """The reference's path with the restated blackbody table and approximate
    Earth reproduces the DIRBE IDL prediction software within the reference's
    own 1 % bound (tests/test_evaluate.py:48-66 of the reference)."""
    with np.load("tests/golden/dirbe_idl.npz") as z:
        ref_total, tab = z["ref_total"], z["tabulated"]
    np.testing.assert_allclose(ref_total, tab, rtol=0.01)


def test_planck_table_restatement_matches_fixture():
    import json

    with open("tests/golden/spectral.json") as f:
        spec = json.load(f)
    for key, rec in spec.items():
        x = np.asarray(rec["x"], dtype=np.float64)
        w = rec["weights"]
        w_norm = None if w is None else np.asarray(w) / np.trapezoid(np.asarray(w), x)
        got = zo.planck_table(x, w_norm, unit=rec["unit"])
        np.testing.assert_allclose(got, np.asarray(rec["bb_table"]), rtol=1e-14, err_msg=key)


def test_oracle_chunked_is_partition_independent():
    case = load_case("dirbe25_nside8")
    desc = oracle_desc(case)
    u = case["unit_vectors"]
    whole = zo.evaluate(desc, u, case["obs"], case["earth"])
    parts = np.concatenate(
        [zo.evaluate(desc, part, case["obs"], case["earth"]) for part in np.array_split(u, 5, axis=-1)], axis=-1
    )
    np.testing.assert_array_equal(whole, parts)


GRID_CASES = ["dirbe_wide", "dirbe_near_earth", "planck13_wide", "planck18_ring", "rrm_wide", "rrm_inner"]


def grid_desc(name):
    from conftest import ref_models

    m = ref_models()[name]
    return {"labels": list(m["comps"]), "comps": m["comps"]}


@pytest.mark.parametrize("key", GRID_CASES)
def test_oracle_grid_matches_reference(key):
    """grid_number_density restatement vs the reference's own output, bit for bit (nan where R = 0)."""
    import os

    from conftest import GOLDEN

    z = np.load(os.path.join(GOLDEN, f"grid_{key}.npz"))
    out = zo.grid_number_density(grid_desc(str(z["model"])), z["x"], z["y"], z["z"], z["earth"])
    ref = z["ref_out"]
    assert out.shape == ref.shape == (len(grid_desc(str(z["model"]))["labels"]), z["y"].size, z["x"].size, z["z"].size)
    np.testing.assert_array_equal(np.isnan(out), np.isnan(ref))
    finite = np.isfinite(ref)
    np.testing.assert_array_equal(out[finite], ref[finite])
