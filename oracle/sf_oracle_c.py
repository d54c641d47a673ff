"""ctypes binding of the C restatement (oracle/sf_oracle.c).

TEST INFRASTRUCTURE ONLY: used by the tests as a second checker and by
bench.py as the timed CPU baseline (``kind: port``)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from build_oracle import LIB, build


class _Shape(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("C", "F", "Tp", "R", "Rpp", "P", "B")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = ctypes.CDLL(str(LIB))
        P = ctypes.c_void_p
        L.sfo_correlate.argtypes = [ctypes.POINTER(_Shape), P, P, P, ctypes.c_int, P]
        L.sfo_adaptive_chain.argtypes = [ctypes.POINTER(_Shape), P, P, P, P, P, P, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_int, P, P, P, P]
        L.sfo_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def max_threads():
    return int(lib().sfo_max_threads())


def correlate(sh, samples, scales, offsets, nthreads=1):
    shape = _Shape(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    out = np.zeros((sh.C, sh.NBL, 2, 2, 2), np.int64)
    off = np.ascontiguousarray(offsets, np.int32)
    lib().sfo_correlate(ctypes.byref(shape), _p(np.ascontiguousarray(samples)),
                        _p(np.ascontiguousarray(scales)), _p(off), int(nthreads), _p(out))
    return out


def adaptive_chain(sh, samples, scales, offsets, weights, factors, fixed_k=None, k_rule=0,
                   delta=0.0, shrink=False, nthreads=1, want=("vis", "evals", "counts", "beams")):
    shape = _Shape(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    w = np.ascontiguousarray(np.asarray(weights, np.float32).reshape(sh.C, 2, sh.B, sh.R, 2))
    d = np.asarray(factors, np.complex128).reshape(sh.C, 2, sh.R)
    dd = np.ascontiguousarray(np.stack([d.real, d.imag], -1))
    fk = None if fixed_k is None else np.ascontiguousarray(fixed_k, np.int32)
    out = {}
    if "vis" in want:
        out["vis"] = np.zeros((sh.C, sh.NBL, 2, 2, 2), np.int64)
    if "evals" in want:
        out["evals"] = np.zeros((sh.C, 2, sh.R))
    if "counts" in want:
        out["counts"] = np.zeros((sh.C, 2), np.int32)
    if "beams" in want:
        out["beams"] = np.zeros((sh.C, 2, 2 * sh.B, sh.T, 2))
    lib().sfo_adaptive_chain(ctypes.byref(shape), _p(np.ascontiguousarray(samples)),
                             _p(np.ascontiguousarray(scales)), _p(np.ascontiguousarray(offsets, np.int32)),
                             _p(w), _p(dd), _p(fk), int(k_rule), float(delta), int(bool(shrink)),
                             int(nthreads), _p(out.get("vis")), _p(out.get("evals")),
                             _p(out.get("counts")), _p(out.get("beams")))
    if "beams" in out:
        b = out["beams"]
        out["beams"] = b[..., 0] + 1j * b[..., 1]
    return out
