"""ctypes binding of ``libzodigb.so`` (the C ABI declared in ``include/zodigb.h``).

The structures below mirror the header field for field; ``tests/test_abi.py``
checks their sizes against the compiled library's view.  There is no
fallback: if the library cannot be loaded, every GPU entry point raises.
"""

from __future__ import annotations

import ctypes
import os

from ._build import LIB_PATH

ZL_ABI_VERSION = 3
ZL_MAX_COMPS = 8
ZL_MAX_RANGES = 8
ZL_MAX_SPEC = 4
ZL_MAX_NODES = 128
ZL_MAX_TEMPS = 128

ZL_CLOUD, ZL_BAND, ZL_RING, ZL_FEATURE = 0, 1, 2, 3
ZL_FAN, ZL_COMET, ZL_INTERSTELLAR, ZL_NARROW_BAND, ZL_BROAD_BAND, ZL_RING_RRM, ZL_FEATURE_RRM = 4, 5, 6, 7, 8, 9, 10
ZL_KELSALL, ZL_RRM = 0, 1
ZL_SEMB_L2_SCRATCH = 1024
ZL_PREC_F64, ZL_PREC_F32 = 0, 1
ZL_OK, ZL_ERR_ARG, ZL_ERR_CUDA, ZL_ERR_MODEL, ZL_ERR_SPACE = 0, -1, -2, -3, -4
ZL_KERNEL_AUTO, ZL_KERNEL_ONE_PIXEL, ZL_KERNEL_TWO_PIXEL, ZL_KERNEL_PLAIN_GEOMETRY, ZL_KERNEL_WARP_PER_PIXEL = 0, 1, 2, 3, 4

c_double_p = ctypes.POINTER(ctypes.c_double)


class ZlComponent(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32),
        ("range", ctypes.c_int32),
        ("offset", ctypes.c_double * 3),
        ("sin_i", ctypes.c_double),
        ("cos_i", ctypes.c_double),
        ("sin_Omega", ctypes.c_double),
        ("cos_Omega", ctypes.c_double),
        ("n_0", ctypes.c_double),
        ("p", ctypes.c_double * 6),
    ]


class ZlSpectrum(ctypes.Structure):
    _fields_ = [
        ("emissivity", ctypes.c_double * ZL_MAX_COMPS),
        ("albedo", ctypes.c_double * ZL_MAX_COMPS),
        ("C1", ctypes.c_double),
        ("C2", ctypes.c_double),
        ("C3", ctypes.c_double),
        ("solar_irradiance", ctypes.c_double),
        ("calibration", ctypes.c_double),
        ("bb", ctypes.c_double * ZL_MAX_TEMPS),
    ]


class ZlModel(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32),
        ("n_comps", ctypes.c_int32),
        ("n_ranges", ctypes.c_int32),
        ("n_spec", ctypes.c_int32),
        ("n_nodes", ctypes.c_int32),
        ("n_temps", ctypes.c_int32),
        ("family", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("T_0", ctypes.c_double),
        ("delta", ctypes.c_double),
        ("comp_T_0", ctypes.c_double * ZL_MAX_COMPS),
        ("comp_delta", ctypes.c_double * ZL_MAX_COMPS),
        ("cutoff", (ctypes.c_double * 2) * ZL_MAX_RANGES),
        ("temps", ctypes.c_double * ZL_MAX_TEMPS),
        ("gl_x", ctypes.c_double * ZL_MAX_NODES),
        ("gl_w", ctypes.c_double * ZL_MAX_NODES),
        ("comp", ZlComponent * ZL_MAX_COMPS),
        ("spec", ZlSpectrum * ZL_MAX_SPEC),
    ]


class ZlObserver(ctypes.Structure):
    _fields_ = [
        ("obs", ctypes.c_double * 3),
        ("earth", ctypes.c_double * 3),
        ("pix_begin", ctypes.c_int64),
        ("outside", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]


class ZlLaunch(ctypes.Structure):
    """Launch options of one call (include/zodigb.h); all zero = the defaults."""

    _fields_ = [
        ("threads_per_block", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("kernel", ctypes.c_int32),
        ("band_tails", ctypes.c_int32),
        ("tile", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("queue_dev", ctypes.c_void_p),
        ("out_index_dev", ctypes.c_void_p),
    ]


# Every symbol the header declares, with its ctypes signature.
_SIGNATURES = {
    "zl_abi_version": (ctypes.c_int, []),
    "zl_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "zl_model_check": (ctypes.c_int, [ctypes.POINTER(ZlModel)]),
    "zl_observer_flags": (ctypes.c_int, [ctypes.POINTER(ZlModel), ctypes.POINTER(ZlObserver), ctypes.c_int64, ctypes.c_int32]),
    "zl_forward": (
        ctypes.c_int,
        [
            ctypes.POINTER(ZlModel),
            ctypes.c_void_p,
            ctypes.c_int64,
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.c_int32,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
        ],
    ),
    "zl_forward_ex": (
        ctypes.c_int,
        [
            ctypes.POINTER(ZlModel),
            ctypes.c_void_p,
            ctypes.c_int64,
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.c_int32,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.POINTER(ZlLaunch),
            ctypes.c_void_p,
        ],
    ),
    "zl_forward_tod": (
        ctypes.c_int,
        [ctypes.POINTER(ZlModel), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    ),
    "zl_backward_tod": (
        ctypes.c_int,
        [ctypes.POINTER(ZlModel), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "zl_spline_eval": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p],
    ),
    "zl_semb_l2": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
         ctypes.c_void_p, ctypes.c_void_p],
    ),
    "zl_directions": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
         ctypes.c_void_p],
    ),
    "zl_density_grid": (
        ctypes.c_int,
        [
            ctypes.POINTER(ZlModel),
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.POINTER(ctypes.c_double),
            ctypes.c_void_p,
            ctypes.c_void_p,
        ],
    ),
    "zl_backward_static": (
        ctypes.c_int,
        [
            ctypes.POINTER(ZlModel),
            ctypes.c_void_p,
            ctypes.c_int64,
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
        ],
    ),
    "zl_backward_ex": (
        ctypes.c_int,
        [
            ctypes.POINTER(ZlModel),
            ctypes.c_void_p,
            ctypes.c_int64,
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_size_t,
            ctypes.POINTER(ZlLaunch),
            ctypes.c_void_p,
        ],
    ),
    "zl_grad_count": (ctypes.c_int, [ctypes.POINTER(ZlModel), ctypes.POINTER(ctypes.c_int32)]),
    "zl_backward_workspace_bytes": (ctypes.c_int, [ctypes.POINTER(ZlModel), ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    "zl_backward": (
        ctypes.c_int,
        [
            ctypes.POINTER(ZlModel),
            ctypes.c_void_p,
            ctypes.c_int64,
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_size_t,
            ctypes.c_void_p,
        ],
    ),
    "zl_mapped_pointer": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "zl_diag_pipe_probe": (
        ctypes.c_int,
        [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p],
    ),
    "zl_diag_atan2": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "zl_diag_d2f": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "zl_diag_f2d": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
}

_lib = None


class ZodiGBError(RuntimeError):
    """A failure reported by libzodigb (status code and message)."""


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the library once; raise if it is missing or its ABI differs."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("ZODIGB_LIB", LIB_PATH)
    if not os.path.exists(path):
        raise ZodiGBError(
            f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()' "
            "or python -m zodipy_gb300._build)"
        )
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.zl_abi_version() != ZL_ABI_VERSION:
        raise ZodiGBError(f"libzodigb ABI {lib.zl_abi_version()} != {ZL_ABI_VERSION}")
    _lib = lib
    return lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(512)
    load().zl_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise ZodiGBError(f"{what} failed ({rc}): {last_error()}")


def declared_symbols() -> list[str]:
    return list(_SIGNATURES)
