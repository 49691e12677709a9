"""Loader of the float64 C oracle (``oracle/fdtd_oracle.c``): TEST INFRASTRUCTURE ONLY.

``build()`` compiles it with gcc into ``oracle/_build/libfdtd_oracle.so``;
``forward_shots`` runs shots in parallel threads (ctypes releases the GIL during
the call) and returns float64 traces ``(S, R, n_steps)``. Only the tests,
``__graft_entry__`` and bench.py's CPU legs use it, as the checker.
"""

from __future__ import annotations

import concurrent.futures
import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_int
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "fdtd_oracle.c"
LIB = HERE / "_build" / "libfdtd_oracle.so"

_lib = None


def build(force=False):
    """Compile the C oracle if its source is newer than the library."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O3", "-std=c99", "-shared", "-fPIC", str(SRC), "-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(str(LIB))
        ip, dp = POINTER(c_int), POINTER(c_double)
        lib.orc_forward_shot.restype = c_int
        lib.orc_forward_shot.argtypes = [c_int, c_int, c_double, c_double, c_double, dp, c_int, ip, ip, dp, dp,
                                         c_int, c_int, ip, ip, dp, c_int, dp, c_int, c_double]
        lib.orc_gradient_shot.restype = c_int
        lib.orc_gradient_shot.argtypes = [c_int, c_int, c_double, c_double, c_double, dp, c_int, ip, ip, dp, dp,
                                          c_int, c_int, ip, ip, dp, c_int, dp, c_int, c_int, dp, dp, c_int, c_double]
        _lib = lib
    return _lib


def _ip(a):
    return a.ctypes.data_as(POINTER(c_int))


def _dp(a):
    return a.ctypes.data_as(POINTER(c_double))


class _Shots:
    """Shot tables in the C oracle's layout; with a PML of ``pml`` cells the medium
    is padded with its edge values and every index shifted into the padded grid."""

    def __init__(self, c, sources, receivers, wave, pml=0):
        c = np.asarray(c, dtype=np.float64)
        self.pml = int(pml)
        self.shape = c.shape
        self.c = np.ascontiguousarray(np.pad(c, self.pml, mode="edge") if self.pml else c)
        rows, cols, w = (np.asarray(a) for a in sources)
        self.rows = np.ascontiguousarray(rows.reshape(rows.shape[0], -1) + self.pml, dtype=np.int32)
        self.cols = np.ascontiguousarray(cols.reshape(self.rows.shape) + self.pml, dtype=np.int32)
        self.w = np.ascontiguousarray(np.asarray(w, dtype=np.float64).reshape(self.rows.shape))
        r0, c0, rw = receivers
        self.r0 = np.ascontiguousarray(np.asarray(r0) + self.pml, dtype=np.int32)
        self.c0 = np.ascontiguousarray(np.asarray(c0) + self.pml, dtype=np.int32)
        self.rw = np.ascontiguousarray(np.asarray(rw, dtype=np.float64).reshape(-1, 4))
        self.wave = np.ascontiguousarray(wave, dtype=np.float64)
        self.S, self.K = self.rows.shape

    def args(self, s):
        ny, nx = self.c.shape
        return (ny, nx), (_dp(self.c), self.K, _ip(self.rows[s]), _ip(self.cols[s]), _dp(self.w[s]),
                          _dp(self.wave), len(self.wave), len(self.r0), _ip(self.r0), _ip(self.c0), _dp(self.rw))


def _run(fn, n, threads):
    workers = threads or min(n, max(1, len(os.sched_getaffinity(0))))
    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as pool:
        return list(pool.map(fn, range(n)))


def forward_shots(c, dx, dy, dt, sources, receivers, wave, n_steps, threads=None, pml=0, pml_reflection=1e-5):
    """float64 traces (S, R, n_steps) of every shot.

    ``sources``: (rows, cols, weights), each (S, K) — shot s injects
    ``w * wave[step]`` at its K nodes; ``receivers``: (row0, col0, weights (R, 4)).
    ``pml`` > 0 pads a PML of that many cells outside the grid (no Mur edges).
    """
    lib = load()
    sh = _Shots(c, sources, receivers, wave, pml)
    out = np.zeros((sh.S, len(sh.r0), int(n_steps)))

    def one(s):
        (ny, nx), rest = sh.args(s)
        rc = lib.orc_forward_shot(ny, nx, dx, dy, dt, *rest, int(n_steps), _dp(out[s]), sh.pml,
                                  float(pml_reflection))
        if rc != 0:
            raise RuntimeError(f"oracle forward failed ({rc})")

    _run(one, sh.S, threads)
    return out


def gradient_shots(c, dx, dy, dt, sources, receivers, wave, n_steps, observed, mute, ckpt_every=None,
                   threads=None, pml=0, pml_reflection=1e-5):
    """float64 misfit and g_{c^2} (ny, nx) summed over shots (no mask, no chain rule).

    ``observed`` (S, R, n_steps); ``mute[s]`` is the receiver channel of shot s left
    out of the residual (-1: none). With ``pml`` the gradient is returned on the
    physical grid (the layer cropped).
    """
    lib = load()
    sh = _Shots(c, sources, receivers, wave, pml)
    obs = np.ascontiguousarray(observed, dtype=np.float64)
    mute = np.broadcast_to(np.asarray(mute, dtype=np.int64).reshape(-1), (sh.S,))
    C = int(ckpt_every or max(1, int(np.ceil(np.sqrt(2.0 * n_steps)))))
    grads = np.zeros((sh.S,) + sh.c.shape)
    J = np.zeros(sh.S)

    def one(s):
        (ny, nx), rest = sh.args(s)
        j = c_double(0.0)
        rc = lib.orc_gradient_shot(ny, nx, dx, dy, dt, *rest, int(n_steps), _dp(obs[s]), int(mute[s]), C,
                                   ctypes.byref(j), _dp(grads[s]), sh.pml, float(pml_reflection))
        if rc != 0:
            raise RuntimeError(f"oracle gradient failed ({rc})")
        J[s] = j.value

    _run(one, sh.S, threads)
    g = grads.sum(axis=0)
    if sh.pml:
        g = g[sh.pml:sh.pml + sh.shape[0], sh.pml:sh.pml + sh.shape[1]]
    return float(J.sum()), np.ascontiguousarray(g)


def misfit(traces, observed, mute):
    """0.5 * sum((traces - observed)^2) with channel mute[s] of shot s left out, float64."""
    r = np.asarray(traces, dtype=np.float64) - np.asarray(observed, dtype=np.float64)
    for s, ch in enumerate(np.asarray(mute).reshape(-1)):
        if ch >= 0:
            r[s, ch] = 0.0
    return 0.5 * float(np.sum(r * r))
