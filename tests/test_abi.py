"""The C ABI: library loads, exports every declared symbol, struct layouts agree,
and the host-only entry points validate and flag exactly like the reference."""

import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "zodigb.h")


def header_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"ZL_API\s+int\s+(zl_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    from zodipy_gb300 import _lib

    syms = header_symbols()
    assert syms, "no declarations found"
    for s in syms:
        assert hasattr(lib, s), f"{s} not exported"
    assert sorted(_lib.declared_symbols()) == syms
    assert lib.zl_abi_version() == _lib.ZL_ABI_VERSION
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = sorted(set(re.findall(r" T (zl_\w+)", out)))
    assert exported == syms, "exported zl_* symbols differ from the header"


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_struct_layout_matches_ctypes(tmp_path):
    from zodipy_gb300 import _lib

    src = tmp_path / "sz.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "zodigb.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(ZlComponent), sizeof(ZlSpectrum),"
        " sizeof(ZlModel), sizeof(ZlObserver), offsetof(ZlModel, comp), offsetof(ZlObserver, pix_begin));return 0;}\n"
    )
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [
        ctypes.sizeof(_lib.ZlComponent),
        ctypes.sizeof(_lib.ZlSpectrum),
        ctypes.sizeof(_lib.ZlModel),
        ctypes.sizeof(_lib.ZlObserver),
        _lib.ZlModel.comp.offset,
        _lib.ZlObserver.pix_begin.offset,
    ]
    assert got == want


def _dirbe_zl():
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    return zg.Model(25 * u.micron).zl_model


def test_model_check_rejects_bad_models(lib):
    from zodipy_gb300 import _lib

    m = _dirbe_zl()
    assert lib.zl_model_check(ctypes.byref(m)) == 0
    for field, bad in (("n_comps", 0), ("n_comps", 9), ("n_nodes", 0), ("n_nodes", 129), ("n_spec", 5), ("abi_version", 99)):
        mm = _lib.ZlModel.from_buffer_copy(m)
        setattr(mm, field, bad)
        assert lib.zl_model_check(ctypes.byref(mm)) != 0
        assert field.split("_")[1] in _lib.last_error() or "abi" in _lib.last_error()
    mm = _lib.ZlModel.from_buffer_copy(m)
    mm.comp[2].range = 7
    assert lib.zl_model_check(ctypes.byref(mm)) == _lib.ZL_ERR_MODEL
    mm = _lib.ZlModel.from_buffer_copy(m)
    mm.temps[3] = mm.temps[2]
    assert lib.zl_model_check(ctypes.byref(mm)) != 0


def test_forward_argument_errors_need_no_gpu(lib):
    """Argument validation happens before any CUDA call."""
    from zodipy_gb300 import _lib

    m = _dirbe_zl()
    obs = (_lib.ZlObserver * 1)()
    rc = lib.zl_forward(ctypes.byref(m), None, 10, obs, 1, 0, None, None, None)
    assert rc == _lib.ZL_ERR_ARG
    rc = lib.zl_forward(ctypes.byref(m), ctypes.c_void_p(8), -1, obs, 1, 0, None, None, None)
    assert rc == -1
    rc = lib.zl_forward(ctypes.byref(m), ctypes.c_void_p(8), 10, obs, 0, 0, ctypes.c_void_p(8), None, None)
    assert rc == -1
    rc = lib.zl_forward(ctypes.byref(m), ctypes.c_void_p(8), 10, obs, 1, 0, None, None, None)
    assert rc == -1 and "NULL" in _lib.last_error()
    rc = lib.zl_forward(ctypes.byref(m), ctypes.c_void_p(8), 10, obs, 1, 7, ctypes.c_void_p(8), None, None)
    assert rc == -1 and "precision" in _lib.last_error()
    # zero pixels is a successful no-op
    assert lib.zl_forward(ctypes.byref(m), None, 0, obs, 1, 0, None, None, None) == _lib.ZL_OK


def test_density_grid_argument_errors_need_no_gpu(lib):
    from zodipy_gb300 import _lib

    m = _dirbe_zl()
    e = (ctypes.c_double * 3)(1.0, 0.0, 0.0)
    p = ctypes.c_void_p(8)
    assert lib.zl_density_grid(ctypes.byref(m), p, -1, p, 2, p, 2, e, p, None) == _lib.ZL_ERR_ARG
    assert lib.zl_density_grid(ctypes.byref(m), None, 2, p, 2, p, 2, e, p, None) == _lib.ZL_ERR_ARG
    assert "NULL" in _lib.last_error()
    assert lib.zl_density_grid(ctypes.byref(m), p, 2, p, 2, p, 2, None, p, None) == _lib.ZL_ERR_ARG
    # an empty mesh is a successful no-op
    assert lib.zl_density_grid(ctypes.byref(m), None, 0, None, 3, None, 3, e, None, None) == _lib.ZL_OK
    bad = _dirbe_zl()
    bad.abi_version = 999
    assert lib.zl_density_grid(ctypes.byref(bad), p, 2, p, 2, p, 2, e, p, None) == _lib.ZL_ERR_MODEL


def test_grid_number_density_rejects_bad_model_type():
    import zodipy_gb300 as zg

    with pytest.raises(TypeError):
        zg.grid_number_density([0.0], [0.0], [0.0], obstime="2022-01-01", model=2)


def test_pack_densities_is_a_valid_model(lib):
    from zodipy_gb300 import packing
    from zodipy_gb300.zodiacal_light_model import model_registry

    for name in ("dirbe", "planck18"):
        m = packing.pack_densities(model_registry.get_model(name))
        assert m.n_comps == len(model_registry.get_model(name).comps)


def test_observer_flags_follow_reference_rule(lib):
    """line_of_sight.py:72-73: a cutoff collapses to eps when r_obs > cutoff (strict)."""
    from zodipy_gb300 import packing

    m = _dirbe_zl()
    cut = [(m.cutoff[r][0], m.cutoff[r][1]) for r in range(m.n_ranges)]
    obs = np.array([[0.9833, 0, 0], [1.25, 0, 0], [0.75, 0, 0], [1.2, 0, 0], [0.0, 0.0, 0.0]]).T
    tab = packing.observer_table(m, obs, obs, np.arange(5), any_mode=False)
    for o in range(5):
        r_obs = np.linalg.norm(obs[:, o])
        want = 0
        for r, (lo, hi) in enumerate(cut):
            want |= (r_obs > lo) << (2 * r)
            want |= (r_obs > hi) << (2 * r + 1)
        assert tab[o].outside == want
    tab = packing.observer_table(m, obs, obs, np.arange(5), any_mode=True)
    assert len({tab[o].outside for o in range(5)}) == 1
