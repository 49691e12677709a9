"""ctypes binding of the C ABI in ``include/fdtd_gb300.h``.

The library is built in-tree (``soundwavesimulation_gb300/libfdtd_gb300.so``)
by ``soundwavesimulation_gb300.build``. There is no fallback: if the library
is missing or a call fails, a RuntimeError says why.
"""

from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_float, c_int32, c_int64, c_size_t, c_void_p
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libfdtd_gb300.so"
ABI_VERSION = 7

STORE_F32, STORE_F16, STORE_BF16 = 0, 1, 2


class Grid(ctypes.Structure):
    _fields_ = [("ny", c_int32), ("nx", c_int32), ("pitch", c_int32),
                ("dx", c_double), ("dy", c_double), ("dt", c_double),
                ("coef", c_void_p), ("mur", c_void_p), ("pml", c_void_p), ("pml_cells", c_int32)]


class Density(ctypes.Structure):
    _fields_ = [("kappa", c_void_p), ("bx", c_void_p), ("by", c_void_p)]


class Receivers(ctypes.Structure):
    _fields_ = [("n", c_int32), ("row0", c_void_p), ("col0", c_void_p), ("w", c_void_p)]


class Sources(ctypes.Structure):
    _fields_ = [("per_shot", c_int32), ("row", c_void_p), ("col", c_void_p), ("w", c_void_p),
                ("wave", c_void_p), ("waveforms", c_void_p), ("n_waves", c_int32),
                ("waveform_len", c_int32)]


class Problem(ctypes.Structure):
    _fields_ = [("grid", Grid), ("n_shots", c_int32), ("n_steps", c_int32),
                ("rx", Receivers), ("src", Sources)]


class Tuning(ctypes.Structure):
    _fields_ = [("rows_per_lane", c_int32), ("warps", c_int32), ("steps_per_launch", c_int32),
                ("ckpt_every", c_int32), ("ckpt_store", c_int32), ("ctas_per_sm", c_int32),
                ("eager", c_int32), ("step_sync", c_int32), ("kept_segments", c_int32)]

    def as_dict(self):
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


_SIGNATURES = {
    "fdtd_abi_version": (c_int32, []),
    "fdtd_last_error": (ctypes.c_char_p, []),
    "fdtd_prepare_medium": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_double, c_double,
                                      c_double, c_void_p, c_void_p, c_void_p]),
    "fdtd_step": (c_int32, [POINTER(Grid), c_int32, c_void_p, c_void_p, c_void_p, c_int32,
                            c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int32,
                            c_void_p, c_int32, c_void_p]),
    "fdtd_step_pml": (c_int32, [POINTER(Grid), c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_int32, c_int32, c_void_p, c_int32, c_void_p]),
    "fdtd_prepare_medium_pml": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_double, c_double, c_double,
                                          c_int32, c_double, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fdtd_gather": (c_int32, [POINTER(Grid), c_int32, c_void_p, c_int32, c_void_p, c_void_p,
                              c_void_p, c_int64, c_int64, c_void_p]),
    "fdtd_scatter": (c_int32, [POINTER(Grid), c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                               c_int64, c_int64, c_void_p, c_void_p]),
    "fdtd_image": (c_int32, [POINTER(Grid), c_int32, c_void_p, c_void_p, c_double, c_void_p,
                             c_void_p]),
    "fdtd_tap_table": (c_int32, [c_int32, c_int32, POINTER(Receivers), c_void_p, c_void_p,
                                 POINTER(c_int32)]),
    "fdtd_plan_create": (c_int32, [POINTER(Problem), POINTER(Tuning), c_int32, POINTER(c_void_p)]),
    "fdtd_plan_destroy": (c_int32, [c_void_p]),
    "fdtd_plan_workspace_bytes": (c_int32, [c_void_p, POINTER(c_size_t)]),
    "fdtd_plan_tuning": (c_int32, [c_void_p, POINTER(Tuning)]),
    "fdtd_plan_bind": (c_int32, [c_void_p, c_void_p, c_size_t, c_void_p]),
    "fdtd_group_workspace_bytes": (c_size_t, [ctypes.POINTER(c_void_p), c_int32]),
    "fdtd_group_forward": (c_int32, [ctypes.POINTER(c_void_p), c_int32, ctypes.POINTER(c_void_p), c_int32,
                                     c_void_p, c_size_t, c_void_p]),
    "fdtd_group_adjoint": (c_int32, [ctypes.POINTER(c_void_p), c_int32, ctypes.POINTER(c_void_p),
                                     ctypes.POINTER(c_void_p), c_void_p, c_size_t, c_void_p]),
    "fdtd_regularization": (c_int32, [c_int32, c_int32, c_void_p, c_void_p, c_double, c_double, c_double,
                                      c_void_p, c_void_p, c_void_p]),
    "fdtd_project": (c_int32, [ctypes.c_int64, c_void_p, c_void_p, c_double, c_double, c_double, c_void_p]),
    "fdtd_resize_slowness": (c_int32, [c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int32, c_int32,
                                       c_void_p, c_void_p, c_double, c_void_p]),
    "fdtd_adam_step": (c_int32, [ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_double,
                                 c_double, c_double, c_double, c_int32, c_double, c_double, c_double,
                                 c_void_p]),
    "fdtd_plan_set_medium": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "fdtd_forward": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_void_p]),
    "fdtd_adjoint": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "fdtd_residual_misfit": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_int64,
                                       c_void_p, c_void_p, c_void_p, c_void_p]),
    "fdtd_chain_rule": (c_int32, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fdtd_forward_plain": (c_int32, [POINTER(Problem), c_void_p, c_void_p, c_size_t, c_void_p]),
    "fdtd_forward_plain_workspace": (c_size_t, [POINTER(Problem)]),
    "fdtd_gradient_plain": (c_int32, [POINTER(Problem), c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_size_t, c_void_p]),
    "fdtd_gradient_plain_workspace": (c_size_t, [POINTER(Problem)]),
    "fdtd_forward_plain_static": (c_int32, [POINTER(Problem), c_void_p, c_void_p]),
    "fdtd_tile_axis": (c_int32, [c_int32, c_int32, c_int32, c_int32, c_int32, c_int32,
                                 c_void_p, POINTER(c_int32)]),
    "fdtd_prepare_density": (c_int32, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_double, c_double, c_double,
                                       c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fdtd_step_density": (c_int32, [POINTER(Grid), POINTER(Density), c_int32, c_void_p, c_void_p, c_void_p, c_int32,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int32,
                                    c_void_p, c_int32, c_void_p]),
    "fdtd_forward_plain_density": (c_int32, [POINTER(Problem), POINTER(Density), c_void_p, c_void_p, c_size_t,
                                             c_void_p]),
    "fdtd_gradient_plain_density": (c_int32, [POINTER(Problem), POINTER(Density), c_void_p, c_void_p, c_void_p,
                                              c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "fdtd_density_chain_rule": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                                          c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fdtd_autotune_workspace_bytes": (c_size_t, [POINTER(Problem), c_int32, c_int32]),
    "fdtd_autotune": (c_int32, [POINTER(Problem), c_int32, c_int32, c_int32, c_void_p, c_size_t,
                                POINTER(Tuning), POINTER(c_double), c_void_p, c_void_p, POINTER(c_int32),
                                c_void_p]),
}

EXPORTED = tuple(_SIGNATURES)

_lib = None


def load():
    """Load the engine library once; raise RuntimeError if it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"GB300 engine library not found at {LIB_PATH}; build it with "
            "`python -c \"import soundwavesimulation_gb300.build as b; b.build()\"`")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.fdtd_abi_version() != ABI_VERSION:
        raise RuntimeError("engine library ABI version mismatch; rebuild it")
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
    """Raise on a non-zero return code, with the library's message."""
    if rc != 0:
        msg = load().fdtd_last_error().decode(errors="replace")
        kinds = {1: ValueError, 3: RuntimeError, 4: ValueError, 5: RuntimeError}
        exc = kinds.get(rc, RuntimeError)
        raise exc(f"{what}: {msg}" if what else msg)


def tile_axis(n, region, align, halo, band, max_tiles=4096):
    """The engine's 1-D tiler: rows of (region origin, owned begin, owned end, flags)."""
    out = np.zeros((max_tiles, 4), dtype=np.int32)
    count = c_int32(0)
    check(load().fdtd_tile_axis(n, region, align, halo, band, max_tiles,
                                out.ctypes.data_as(c_void_p), ctypes.byref(count)), "tile_axis")
    return out[:count.value].copy()


def tap_table(ny, nx, row0, col0, weights):
    """Unique receiver tap nodes: (nodes int32 (n, 10), weights float32 (n, 8))."""
    row0 = np.ascontiguousarray(row0, dtype=np.int32)
    col0 = np.ascontiguousarray(col0, dtype=np.int32)
    w = np.ascontiguousarray(weights, dtype=np.float32).reshape(-1, 4)
    rx = Receivers(len(row0), row0.ctypes.data, col0.ctypes.data, w.ctypes.data)
    cap = max(4 * len(row0), 1)
    nodes = np.zeros((cap, 10), dtype=np.int32)
    tw = np.zeros((cap, 8), dtype=np.float32)
    n = c_int32(cap)
    check(load().fdtd_tap_table(ny, nx, ctypes.byref(rx), nodes.ctypes.data_as(c_void_p),
                                tw.ctypes.data_as(c_void_p), ctypes.byref(n)), "tap_table")
    return nodes[:n.value].copy(), tw[:n.value].copy()


__all__ = ["Grid", "Density", "Receivers", "Sources", "Problem", "Tuning", "load", "check", "tile_axis",
           "tap_table", "EXPORTED", "STORE_F32", "STORE_F16", "STORE_BF16", "c_float"]
