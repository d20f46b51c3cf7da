"""ctypes wrapper of the C oracle (oracle/oakref.c) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
LAPACK's dsyev and BLAS's dgemm are taken from SciPy's exported Cython function pointers
when SciPy is importable (the same routines the reference links, matoper_inc.F90:986-1005,
:420-439); otherwise the C oracle uses its internal Jacobi eigensolver and plain loops.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


class OakrefLoc(ctypes.Structure):
    _fields_ = [("metric", ctypes.c_int), ("loctype", ctypes.c_int), ("kind", ctypes.c_int),
                ("localise", ctypes.c_int), ("rotate", ctypes.c_int)]


def _capsule_pointer(capsule) -> int:
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def lapack_pointers():
    """(dsyev, dgemm) function pointers from SciPy, or (None, None)."""
    try:
        from scipy.linalg import cython_blas, cython_lapack
    except Exception:  # pragma: no cover - SciPy missing
        return None, None
    return (_capsule_pointer(cython_lapack.__pyx_capi__["dsyev"]),
            _capsule_pointer(cython_blas.__pyx_capi__["dgemm"]))


def load(use_lapack: bool = True):
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build_oracle.build())
        lib.oakref_set_lapack.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.oakref_set_lapack.restype = None
        lib.oakref_locfun.argtypes = [ctypes.c_double]
        lib.oakref_locfun.restype = ctypes.c_double
        P = ctypes.c_void_p
        lib.oakref_locanalysis.argtypes = [ctypes.c_int] * 4 + [P] * 14 + [
            ctypes.POINTER(OakrefLoc), P, P, P, P, ctypes.c_int]
        lib.oakref_locanalysis.restype = ctypes.c_int
        lib.oakref_analysis.argtypes = [ctypes.c_int] * 3 + [P] * 9 + [ctypes.c_int]
        lib.oakref_analysis.restype = ctypes.c_int
        _lib = lib
    dsyev, dgemm = lapack_pointers() if use_lapack else (None, None)
    _lib.oakref_set_lapack(dsyev, dgemm)
    return _lib


def _f64(a):
    return np.require(a, dtype=np.float64, requirements=["C"])


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def locanalysis(zone_size, xf, Hxf, yo, Sf, HSf, r_diag, zone_pos, obs_pos, corr_len,
                max_len, metric=0, loctype=1, kind=0, localise_obs=True, rotate=True,
                nthreads=0, want_sa=True, use_lapack=True):
    """locAnalysis with geometric selection. Sf is (n, N) and HSf (m, N), as in the
    reference; they are passed column-major. Returns (xa, Sa, amplitudes, nobs)."""
    lib = load(use_lapack)
    zone_size = np.require(zone_size, dtype=np.int32, requirements=["C"])
    n, N = Sf.shape
    m = yo.size
    Z = zone_size.size
    SfF = np.asfortranarray(Sf, dtype=np.float64)
    HSfF = np.asfortranarray(HSf, dtype=np.float64)
    zpos = _f64(np.asarray(zone_pos, dtype=np.float64).reshape(Z, 4))
    ox, oy, oz, ot = (_f64(np.asarray(c, dtype=np.float64)) for c in obs_pos)
    xa = np.empty(n)
    Sa = np.empty((n, N), order="F") if want_sa else None
    ampl = np.zeros((N, Z), order="F")
    nobs = np.zeros(Z, dtype=np.int32)
    loc = OakrefLoc(metric, loctype, kind, int(bool(localise_obs)), int(bool(rotate)))
    keep = [_f64(xf), _f64(Hxf), _f64(yo), _f64(r_diag), _f64(corr_len), _f64(max_len)]
    rc = lib.oakref_locanalysis(
        n, N, m, Z, _ptr(zone_size), _ptr(keep[0]), _ptr(keep[1]), _ptr(keep[2]),
        SfF.ctypes.data_as(ctypes.c_void_p), HSfF.ctypes.data_as(ctypes.c_void_p),
        _ptr(keep[3]), _ptr(zpos), _ptr(ox), _ptr(oy), _ptr(oz), _ptr(ot),
        _ptr(keep[4]), _ptr(keep[5]), ctypes.byref(loc), _ptr(xa),
        None if Sa is None else Sa.ctypes.data_as(ctypes.c_void_p),
        ampl.ctypes.data_as(ctypes.c_void_p), _ptr(nobs), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oakref_locanalysis failed with status {rc}")
    return xa, Sa, ampl, nobs


def analysis(xf, Hxf, yo, Sf, HSf, r_diag, rotate=True, use_lapack=True):
    lib = load(use_lapack)
    n, N = Sf.shape
    m = yo.size
    SfF = np.asfortranarray(Sf, dtype=np.float64)
    HSfF = np.asfortranarray(HSf, dtype=np.float64)
    xa = np.empty(n)
    Sa = np.empty((n, N), order="F")
    ampl = np.empty(N)
    keep = [_f64(xf), _f64(Hxf), _f64(yo), _f64(r_diag)]
    rc = lib.oakref_analysis(n, N, m, _ptr(keep[0]), _ptr(keep[1]), _ptr(keep[2]),
                             SfF.ctypes.data_as(ctypes.c_void_p),
                             HSfF.ctypes.data_as(ctypes.c_void_p), _ptr(keep[3]),
                             _ptr(xa), Sa.ctypes.data_as(ctypes.c_void_p), _ptr(ampl),
                             int(bool(rotate)))
    if rc != 0:
        raise RuntimeError(f"oakref_analysis failed with status {rc}")
    return xa, Sa, ampl
