"""The CPU side's workload inputs (oracle/workloads.py) equal the GPU side's: the
ring-by-ring HEALPix centres equal the package's per-pixel formula bit for bit, the
Earth position constant equals the package's ephemeris at its epoch, and the oracle
descriptions built from the reference-held fixtures carry the reference's values."""

import numpy as np
import pytest

from conftest import ref_models
from oracle import workloads


@pytest.mark.parametrize("nside", [1, 2, 4, 8, 64, 128])
def test_healpix_centres_equal_package(nside):
    from zodipy_gb300.healpix import pix2vec_ring

    np.testing.assert_array_equal(workloads.healpix_ring_centres(nside), pix2vec_ring(nside))


def test_healpix_centres_are_unit_vectors_in_ring_order():
    v = workloads.healpix_ring_centres(16)
    assert v.shape == (3, 12 * 16 * 16)
    np.testing.assert_allclose(np.linalg.norm(v, axis=0), 1.0, rtol=0, atol=4e-16)
    assert np.all(np.diff(v[2]) <= 0)  # z never increases along RING order


def test_earth_constant_equals_package_ephemeris():
    from zodipy_gb300.ephemeris import earth_position, iso_to_mjd

    e = earth_position(iso_to_mjd(workloads.EARTH_2022_01_01_ISO)).reshape(3)
    np.testing.assert_array_equal(workloads.EARTH_2022_01_01, e)


def test_descriptions_come_from_the_reference_dump():
    d = workloads.oracle_desc("dirbe", "dirbe_bp_80_130", 50)
    m = ref_models()["dirbe"]
    assert d["labels"] == list(m["comps"]) and d["T_0"] == m["T_0"] and d["delta"] == m["delta"]
    assert d["bb_table"].shape == (2, 100) and d["gauss_quad_degree"] == 50
    with pytest.raises(ValueError):
        workloads.oracle_desc("planck18", "dirbe_25um", 50)
