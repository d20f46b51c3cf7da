"""GB300-native local ensemble square-root analysis (the analysis path of gher-uliege/OAK).

Python host binding over the C ABI of ``liboakg.so`` (``include/oakg.h``). The functions keep
the argument meaning and order of the reference routines they replace:

* :func:`analysis`      <- ``analysis(xf,Hxf,yo,Sf,HSf,R,xa,Sa,amplitudes)`` (rrsqrt.F90:196-208)
* :func:`loc_analysis`  <- ``locAnalysis(zoneSize,selectObservations,xf,Hxf,yo,Sf,HSf,R,xa,Sa,
  amplitudes,localise_obs)`` (rrsqrt.F90:433-466), with ``selectObservations``
  (assimilation.F90:3683-3771) given as geometry: zone and observation coordinates, the
  per-zone correlation and maximum lengths, a metric and a weight kind.

Arrays are NumPy arrays (host memory; the call copies to and from the GPU) or CUDA
``torch.Tensor`` objects (device memory; nothing is copied). Ensemble matrices are the
reference's Fortran column-major ``(n, N)`` arrays: NumPy arrays are passed in Fortran order,
torch tensors must have strides ``(1, ld)``.

Errors are raised as :class:`OakError` carrying the C status code, where the reference would
stop the program (ERROR_STOP, ppdef.h:22).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

__all__ = ["analysis", "loc_analysis", "loc_analysis_adjoint", "OakError", "lib", "last_timings", "release",
           "PREC_FP64", "PREC_MIXED", "PREC_MIXED_FP64EIG",
           "GAUSS_CUTOFF", "GASPARI_COHN", "CARTESIAN", "SPHERICAL", "SPHERICAL_APPROX",
           "zone_positions", "ensemble_prologue", "ensemble_epilogue", "ens_loc_analysis",
           "ens2sqrt", "sqrt2ens", "ens_analysis", "biased_loc_analysis", "Plan",
           "zone_layout", "partition_compact", "permute_rows", "sea_index", "obsoper_rectilinear",
           "obsoper_to_zone_order"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboakg.so")

# constants of include/oakg.h
OK = 0
ERR_ARGS, ERR_CUDA, ERR_NAN, ERR_EIG, ERR_NOMEM, ERR_TIMEOUT, ERR_INIT, ERR_NOTIMPL = range(1, 9)
MEM_HOST, MEM_DEVICE = 0, 1
GAUSS_CUTOFF, GASPARI_COHN = 0, 1
CARTESIAN, SPHERICAL, SPHERICAL_APPROX = 0, 1, 2
PREC_FP64, PREC_MIXED, PREC_MIXED_FP64EIG = 0, 1, 2
FLAG_AMPL_ALWAYS, FLAG_BRUTE_SEARCH, FLAG_SIMT_UPDATE, FLAG_SIMT_GRAM = 1, 2, 4, 8


class OakError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[oakg status {code}] {msg}")
        self.code = code


class Dims(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("N", ctypes.c_int32), ("pad0", ctypes.c_int32),
                ("m", ctypes.c_int64), ("ldS", ctypes.c_int64), ("ldH", ctypes.c_int64),
                ("mem", ctypes.c_int32), ("pad1", ctypes.c_int32)]


class Loc(ctypes.Structure):
    _fields_ = [("weight", ctypes.c_int32), ("metric", ctypes.c_int32),
                ("loctype", ctypes.c_int32), ("localise_obs", ctypes.c_int32),
                ("rotate", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("flags", ctypes.c_int32), ("pad0", ctypes.c_int32),
                ("cell_size", ctypes.c_double)]


class ObsOper(ctypes.Structure):
    """oakg_obsoper: sparse observation operator, K (index, weight) pairs per observation."""
    _fields_ = [("m", ctypes.c_int64), ("K", ctypes.c_int32), ("pad0", ctypes.c_int32),
                ("index", ctypes.c_void_p), ("weight", ctypes.c_void_p),
                ("shift", ctypes.c_void_p)]


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded ``liboakg.so``; raises if it has not been built (no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OakError(ERR_CUDA, f"{LIB_PATH} is missing: build it with "
                                 "`python -m oak_gb300.build` (there is no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    L.oakg_analysis.argtypes = [ctypes.POINTER(Dims)] + [P] * 9
    L.oakg_analysis.restype = ctypes.c_int
    L.oakg_locanalysis.argtypes = [ctypes.POINTER(Dims), ctypes.POINTER(Loc), ctypes.c_int32] + [P] * 18
    L.oakg_locanalysis.restype = ctypes.c_int
    L.oakg_locanalysis_f32.argtypes = L.oakg_locanalysis.argtypes
    L.oakg_locanalysis_f32.restype = ctypes.c_int
    L.oakg_locanalysis_smw.argtypes = ([ctypes.POINTER(Dims), ctypes.POINTER(Loc),
                                        ctypes.c_int32] + [P] * 7 + [ctypes.c_int32, P,
                                                                     ctypes.c_int64] + [P] * 11)
    L.oakg_locanalysis_smw.restype = ctypes.c_int
    L.oakg_analysis_smw.argtypes = ([ctypes.POINTER(Dims)] + [P] * 6
                                    + [ctypes.c_int32, P, ctypes.c_int64] + [P] * 3)
    L.oakg_analysis_smw.restype = ctypes.c_int
    L.oakg_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.oakg_last_error.restype = ctypes.c_size_t
    L.oakg_last_status.argtypes = []
    L.oakg_last_status.restype = ctypes.c_int
    L.oakg_release.argtypes = []
    L.oakg_release.restype = ctypes.c_int
    L.oakg_last_timings.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    L.oakg_last_timings.restype = ctypes.c_int
    L.oakg_set_stream.argtypes = [P]
    L.oakg_set_stream.restype = ctypes.c_int
    L.oakg_launch_count.argtypes = []
    L.oakg_launch_count.restype = ctypes.c_int64
    L.oakg_fp64_peak.argtypes = [ctypes.POINTER(ctypes.c_double)]
    L.oakg_fp64_peak.restype = ctypes.c_int
    L.oakg_locanalysis_adjoint.argtypes = ([ctypes.POINTER(Dims), ctypes.POINTER(Loc), ctypes.c_int32]
                                           + [P] * 13 + [ctypes.c_double, P, P, P,
                                                          ctypes.POINTER(ctypes.c_double),
                                                          ctypes.POINTER(ctypes.c_double)])
    L.oakg_locanalysis_adjoint.restype = ctypes.c_int
    L.oakg_plan_locanalysis.argtypes = ([ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Dims),
                                         ctypes.POINTER(Loc), ctypes.c_int32] + [P] * 18
                                        + [ctypes.c_int32])
    L.oakg_plan_locanalysis.restype = ctypes.c_int
    L.oakg_plan_execute.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.oakg_plan_execute.restype = ctypes.c_int
    L.oakg_plan_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_double), ctypes.c_int32]
    L.oakg_plan_info.restype = ctypes.c_int
    L.oakg_plan_schedule.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]
    L.oakg_plan_schedule.restype = ctypes.c_int
    L.oakg_plan_destroy.argtypes = [ctypes.c_void_p]
    L.oakg_plan_destroy.restype = None
    L.oakg_ensemble_prologue.argtypes = [ctypes.POINTER(Dims), P, ctypes.c_int64,
                                         ctypes.POINTER(ObsOper), P, P, P, P]
    L.oakg_ensemble_prologue.restype = ctypes.c_int
    L.oakg_ensemble_epilogue.argtypes = [ctypes.POINTER(Dims), P, P, P, ctypes.c_double, P, P,
                                         ctypes.c_int64]
    L.oakg_ensemble_epilogue.restype = ctypes.c_int
    L.oakg_ens_locanalysis.argtypes = ([ctypes.POINTER(Dims), ctypes.POINTER(Loc),
                                        ctypes.c_int32, P, P, ctypes.c_int64,
                                        ctypes.POINTER(ObsOper)] + [P] * 9
                                       + [ctypes.c_double, P, P])
    L.oakg_ens_locanalysis.restype = ctypes.c_int
    L.oakg_ens2sqrt.argtypes = [ctypes.POINTER(Dims), P, ctypes.c_int64, P, P]
    L.oakg_ens2sqrt.restype = ctypes.c_int
    L.oakg_sqrt2ens.argtypes = [ctypes.POINTER(Dims), P, P, P, P, ctypes.c_int64]
    L.oakg_sqrt2ens.restype = ctypes.c_int
    L.oakg_ens_analysis.argtypes = [ctypes.POINTER(Dims), P, ctypes.c_int64, P, ctypes.c_int64,
                                    P, P, P, P, P]
    L.oakg_ens_analysis.restype = ctypes.c_int
    L.oakg_biased_locanalysis.argtypes = ([ctypes.POINTER(Dims), ctypes.POINTER(Loc),
                                           ctypes.c_int32, P, ctypes.c_double,
                                           ctypes.POINTER(ObsOper)] + [P] * 17)
    L.oakg_biased_locanalysis.restype = ctypes.c_int
    L.oakg_zone_layout.argtypes = [ctypes.c_int64, P, ctypes.c_int32, ctypes.c_int32, P, P, P]
    L.oakg_zone_layout.restype = ctypes.c_int
    L.oakg_partition_compact.argtypes = [ctypes.c_int64, P, ctypes.c_int32, P,
                                         ctypes.POINTER(ctypes.c_int32)]
    L.oakg_partition_compact.restype = ctypes.c_int
    L.oakg_permute_rows.argtypes = [ctypes.c_int64, ctypes.c_int32, P, P, ctypes.c_int64, P,
                                    ctypes.c_int64, ctypes.c_int32]
    L.oakg_permute_rows.restype = ctypes.c_int
    L.oakg_sea_index.argtypes = [ctypes.c_int64, P, ctypes.c_int32, P,
                                 ctypes.POINTER(ctypes.c_int64)]
    L.oakg_sea_index.restype = ctypes.c_int
    L.oakg_obsoper_to_zone_order.argtypes = [ctypes.c_int64, P, P, ctypes.c_int64, ctypes.c_int32]
    L.oakg_obsoper_to_zone_order.restype = ctypes.c_int
    L.oakg_obsoper_rectilinear.argtypes = [ctypes.c_int32, P, P, P, ctypes.c_int64,
                                           ctypes.c_int64, P, ctypes.c_int32, P, P]
    L.oakg_obsoper_rectilinear.restype = ctypes.c_int
    L.oakg_read_variable.argtypes = [ctypes.c_char_p, P, ctypes.c_int64,
                                     ctypes.POINTER(ctypes.c_int64), P,
                                     ctypes.POINTER(ctypes.c_int32),
                                     ctypes.POINTER(ctypes.c_double)]
    L.oakg_read_variable.restype = ctypes.c_int
    L.oak_init.argtypes = [ctypes.c_char_p]
    L.oak_init.restype = None
    L.oak_assim.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
    L.oak_assim.restype = None
    L.oak_done.argtypes = []
    L.oak_done.restype = None
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != OK:
        buf = ctypes.create_string_buffer(1024)
        lib().oakg_last_error(buf, len(buf))
        raise OakError(rc, buf.value.decode(errors="replace"))


def last_timings() -> dict:
    """Device time per stage of the last call (CUDA events on the library stream), in ms."""
    arr = (ctypes.c_double * 5)()
    k = lib().oakg_last_timings(arr, 5)
    names = ["obs_prep", "gram", "eig", "update", "total"]
    return {names[i]: arr[i] for i in range(k)}


def release() -> None:
    """Free the device buffers the library keeps between calls."""
    lib().oakg_release()


# ---------------------------------------------------------------------------- array helpers

def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


class _Args:
    """Collects pointers, keeping the backing arrays alive; all host or all device."""

    def __init__(self, device: bool):
        self.device = device
        self.keep = []

    def vec(self, a, dtype=np.float64, name="array", n=None):
        if a is None:
            return None
        if self.device:
            tdt = _torch_dtype(dtype)
            if not (_is_torch(a) and a.is_cuda):
                raise OakError(ERR_ARGS, f"{name}: expected a CUDA tensor")
            if a.dtype != tdt or not a.is_contiguous():
                raise OakError(ERR_ARGS, f"{name}: expected a contiguous {tdt} tensor")
            if n is not None and a.numel() < n:
                raise OakError(ERR_ARGS, f"{name}: needs {n} elements, has {a.numel()}")
            self.keep.append(a)
            return ctypes.c_void_p(a.data_ptr())
        arr = np.ascontiguousarray(np.asarray(a, dtype=dtype)).reshape(-1)
        if n is not None and arr.size < n:
            raise OakError(ERR_ARGS, f"{name}: needs {n} elements, has {arr.size}")
        self.keep.append(arr)
        return ctypes.c_void_p(arr.ctypes.data)

    def mat(self, a, rows, cols, name, dtype=np.float64):
        """Column-major (rows, cols) matrix; returns (pointer, leading dimension)."""
        if self.device:
            if not (_is_torch(a) and a.is_cuda):
                raise OakError(ERR_ARGS, f"{name}: expected a CUDA tensor")
            tdt = _torch_dtype(dtype)
            if a.dtype != tdt or tuple(a.shape) != (rows, cols):
                raise OakError(ERR_ARGS, f"{name}: expected {tdt} of shape ({rows}, {cols})")
            if a.stride(0) != 1 or (cols > 1 and a.stride(1) < rows):
                raise OakError(ERR_ARGS, f"{name}: expected column-major strides (1, ld>=rows)")
            self.keep.append(a)
            return ctypes.c_void_p(a.data_ptr()), (a.stride(1) if cols > 1 else rows)
        arr = np.asfortranarray(np.asarray(a, dtype=dtype))
        if arr.shape != (rows, cols):
            raise OakError(ERR_ARGS, f"{name}: expected shape ({rows}, {cols}), got {arr.shape}")
        self.keep.append(arr)
        return ctypes.c_void_p(arr.ctypes.data), rows


def _torch_dtype(dtype):
    import torch
    return {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
            np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64,
            np.dtype(np.uint8): torch.uint8}[np.dtype(dtype)]


def _is_float32(a) -> bool:
    """True for a float32 array or tensor (FP32 storage at the boundary)."""
    if _is_torch(a):
        import torch
        return a.dtype == torch.float32
    return np.asarray(a).dtype == np.float32


def _device_mode(*arrays) -> bool:
    dev = [_is_torch(a) and a.is_cuda for a in arrays if a is not None]
    if any(dev) and not all(dev):
        raise OakError(ERR_ARGS, "mix of host and device arrays")
    return bool(dev) and all(dev)


def _empty_like_mode(device: bool, shape, dtype=np.float64, order="C", like=None):
    if device:
        import torch
        tdt = _torch_dtype(dtype)
        if order == "F" and len(shape) == 2:
            return torch.empty((shape[1], shape[0]), dtype=tdt, device=like.device).t()
        return torch.empty(shape, dtype=tdt, device=like.device)
    return np.empty(shape, dtype=dtype, order=order)


def _sync_torch(device: bool, ref) -> None:
    if device:
        import torch
        torch.cuda.synchronize(ref.device)


# ----------------------------------------------------------------------------- entry points

def analysis(xf, Hxf, yo, Sf, HSf, r_diag, *, want_sa=True, out=None, smw_B=None):
    """Global analysis (rrsqrt.F90:196-208) with diagonal R = diag(r_diag), or with
    R = diag(r_diag) + B B^T (SMWCovar, covariance.F90:464-570) when ``smw_B`` (m x k) is given.

    Returns ``(xa, Sa, amplitudes)``.
    """
    n = int(xf.shape[0])
    m = int(yo.shape[0])
    N = int(Sf.shape[1])
    device = _device_mode(xf, Hxf, yo, Sf, HSf, r_diag)
    A = _Args(device)
    pSf, ldS = A.mat(Sf, n, N, "Sf")
    pHS, ldH = A.mat(HSf, m, N, "HSf")
    dims = Dims(n=n, N=N, m=m, ldS=ldS, ldH=ldH, mem=MEM_DEVICE if device else MEM_HOST)
    like = Sf
    xa = _empty_like_mode(device, (n,), like=like)
    Sa = None
    if want_sa:
        Sa = _empty_like_mode(device, (n, N), order="F", like=like)
        if device and ldS != n:
            raise OakError(ERR_ARGS, "device Sf with ld != n: pass out arrays explicitly")
    ampl = _empty_like_mode(device, (N,), like=like)
    _sync_torch(device, like)
    if smw_B is not None:
        k = int(smw_B.shape[1])
        pB, ldB = A.mat(smw_B, m, k, "B")
        rc = lib().oakg_analysis_smw(ctypes.byref(dims), A.vec(xf, n=n, name="xf"),
                                     A.vec(Hxf, n=m, name="Hxf"), A.vec(yo, n=m, name="yo"),
                                     pSf, pHS, A.vec(r_diag, n=m, name="r_diag"), k, pB, ldB,
                                     A.vec(xa, name="xa"),
                                     None if Sa is None else A.mat(Sa, n, N, "Sa")[0],
                                     A.vec(ampl, name="ampl"))
        _check(rc)
        return xa, Sa, ampl
    rc = lib().oakg_analysis(ctypes.byref(dims), A.vec(xf, n=n, name="xf"),
                             A.vec(Hxf, n=m, name="Hxf"), A.vec(yo, n=m, name="yo"), pSf, pHS,
                             A.vec(r_diag, n=m, name="r_diag"), A.vec(xa, name="xa"),
                             None if Sa is None else A.mat(Sa, n, N, "Sa")[0],
                             A.vec(ampl, name="ampl"))
    _check(rc)
    return xa, Sa, ampl


def loc_analysis(zone_size, xf, Hxf, yo, Sf, HSf, r_diag, zone_pos, obs_pos, corr_len,
                 max_len, *, weight=GAUSS_CUTOFF, metric=CARTESIAN, loctype=1,
                 localise_obs=True, rotate=True, want_sa=True, want_ampl=True,
                 ampl_always=False, brute_search=False, cell_size=0.0, out=None,
                 precision=PREC_FP64, smw_B=None, simt_update=False, simt_gram=False):
    """Local analysis (rrsqrt.F90:433-466) with geometric observation selection.

    ``zone_pos``: (Z, 4) x, y, z, t of each zone's first state element
    (assimilation.F90:3713-3740); ``obs_pos``: (x, y, z, t) observation coordinate arrays
    (obsGridX/Y/Z/T; unused ones may be None); ``corr_len``, ``max_len``: (Z,) lengths
    (hCorrLengthToObs / hMaxCorrLengthToObs at each zone's first element).

    Returns ``(xa, Sa, amplitudes (N, Z), nobs (Z,))``. As in the reference, amplitudes are
    only written for the non-localised branch unless ``ampl_always`` is set. ``out`` may give
    preallocated ``(xa, Sa)`` arrays of the same memory kind as the inputs (e.g. pinned host
    arrays). ``precision``: PREC_FP64 (plain form), PREC_MIXED (FP32 Gram, eigensolve and
    update; FP64 selection and eigenvalue scalings) or PREC_MIXED_FP64EIG (PREC_MIXED with the
    eigenpairs refined to FP64 accuracy). ``smw_B`` (m x k): the observation error
    covariance R = diag(r_diag) + B B^T (SMWCovar, covariance.F90:464-570; FP64 form).
    ``simt_update``: the mixed form's ensemble update on the CUDA cores instead of the tensor
    cores. ``simt_gram``: the plain form's Gram and square-root-transform products on the FP64
    CUDA cores instead of the tensor cores (exact 8-bit slice products, N <= 64).

    A float32 ``Sf`` selects FP32 storage at the boundary (oakg_locanalysis_f32): xf, Hxf, yo,
    HSf, r_diag are then taken, and xa, Sa, amplitudes returned, in float32; the geometry
    stays float64.
    """
    Z = int(zone_size.shape[0])
    n = int(xf.shape[0])
    m = int(yo.shape[0])
    N = int(Sf.shape[1])
    ox, oy, oz, ot = (tuple(obs_pos) + (None,) * 4)[:4]
    device = _device_mode(zone_size, xf, Hxf, yo, Sf, HSf, r_diag, zone_pos, corr_len, max_len,
                          ox, oy, oz, ot)
    f32 = _is_float32(Sf)
    fdt = np.float32 if f32 else np.float64
    if f32 and smw_B is not None:
        raise OakError(ERR_ARGS, "the SMWCovar form takes float64 arrays")
    A = _Args(device)
    pSf, ldS = A.mat(Sf, n, N, "Sf", fdt)
    pHS, ldH = A.mat(HSf, m, N, "HSf", fdt)
    dims = Dims(n=n, N=N, m=m, ldS=ldS, ldH=ldH, mem=MEM_DEVICE if device else MEM_HOST)
    flags = ((FLAG_AMPL_ALWAYS if ampl_always else 0) | (FLAG_BRUTE_SEARCH if brute_search else 0)
             | (FLAG_SIMT_UPDATE if simt_update else 0) | (FLAG_SIMT_GRAM if simt_gram else 0))
    loc = Loc(weight=weight, metric=metric, loctype=loctype, localise_obs=int(bool(localise_obs)),
              rotate=int(bool(rotate)), precision=int(precision), flags=flags,
              cell_size=float(cell_size))
    like = Sf
    if device:
        zp = zone_pos.reshape(-1)
    else:
        zp = np.ascontiguousarray(np.asarray(zone_pos, dtype=np.float64).reshape(Z, 4))
    if out is not None:
        xa, Sa = out
    else:
        xa = _empty_like_mode(device, (n,), dtype=fdt, like=like)
        Sa = (_empty_like_mode(device, (n, N), dtype=fdt, order="F", like=like) if want_sa
              else None)
    if device and want_sa and ldS != n:
        raise OakError(ERR_ARGS, "device Sf with ld != n is not supported by this wrapper")
    ampl = (_empty_like_mode(device, (N, Z), dtype=fdt, order="F", like=like) if want_ampl
            else None)
    nobs = _empty_like_mode(device, (Z,), dtype=np.int32, like=like)
    _sync_torch(device, like)
    if f32:
        rc = lib().oakg_locanalysis_f32(
            ctypes.byref(dims), ctypes.byref(loc), Z, A.vec(zone_size, np.int32, "zone_size", Z),
            A.vec(xf, fdt, n=n, name="xf"), A.vec(Hxf, fdt, n=m, name="Hxf"),
            A.vec(yo, fdt, n=m, name="yo"), pSf, pHS, A.vec(r_diag, fdt, n=m, name="r_diag"),
            A.vec(zp, n=4 * Z, name="zone_pos"), A.vec(ox, n=m, name="obs_x"),
            A.vec(oy, n=m, name="obs_y"), A.vec(oz, n=m, name="obs_z"),
            A.vec(ot, n=m, name="obs_t"), A.vec(corr_len, n=Z, name="corr_len"),
            A.vec(max_len, n=Z, name="max_len"), A.vec(xa, fdt, name="xa"),
            None if Sa is None else A.mat(Sa, n, N, "Sa", fdt)[0],
            None if ampl is None else A.mat(ampl, N, Z, "ampl", fdt)[0],
            A.vec(nobs, np.int32, "nobs"))
        _check(rc)
        return xa, Sa, ampl, nobs
    if smw_B is not None:
        k = int(smw_B.shape[1])
        pB, ldB = A.mat(smw_B, m, k, "B")
        rc = lib().oakg_locanalysis_smw(
            ctypes.byref(dims), ctypes.byref(loc), Z,
            A.vec(zone_size, np.int32, "zone_size", Z), A.vec(xf, n=n, name="xf"),
            A.vec(Hxf, n=m, name="Hxf"), A.vec(yo, n=m, name="yo"), pSf, pHS,
            A.vec(r_diag, n=m, name="r_diag"), k, pB, ldB,
            A.vec(zp, n=4 * Z, name="zone_pos"), A.vec(ox, n=m, name="obs_x"),
            A.vec(oy, n=m, name="obs_y"), A.vec(oz, n=m, name="obs_z"),
            A.vec(ot, n=m, name="obs_t"), A.vec(corr_len, n=Z, name="corr_len"),
            A.vec(max_len, n=Z, name="max_len"), A.vec(xa, name="xa"),
            None if Sa is None else A.mat(Sa, n, N, "Sa")[0],
            None if ampl is None else A.mat(ampl, N, Z, "ampl")[0],
            A.vec(nobs, np.int32, "nobs"))
        _check(rc)
        return xa, Sa, ampl, nobs
    rc = lib().oakg_locanalysis(
        ctypes.byref(dims), ctypes.byref(loc), Z, A.vec(zone_size, np.int32, "zone_size", Z),
        A.vec(xf, n=n, name="xf"), A.vec(Hxf, n=m, name="Hxf"), A.vec(yo, n=m, name="yo"),
        pSf, pHS, A.vec(r_diag, n=m, name="r_diag"), A.vec(zp, n=4 * Z, name="zone_pos"),
        A.vec(ox, n=m, name="obs_x"), A.vec(oy, n=m, name="obs_y"), A.vec(oz, n=m, name="obs_z"),
        A.vec(ot, n=m, name="obs_t"), A.vec(corr_len, n=Z, name="corr_len"),
        A.vec(max_len, n=Z, name="max_len"), A.vec(xa, name="xa"),
        None if Sa is None else A.mat(Sa, n, N, "Sa")[0],
        None if ampl is None else A.mat(ampl, N, Z, "ampl")[0],
        A.vec(nobs, np.int32, "nobs"))
    _check(rc)
    return xa, Sa, ampl, nobs


def _obsoper(A, H_index, H_weight, H_shift, m):
    """oakg_obsoper from (m, K) index / weight arrays (host or device, as A)."""
    if m == 0:
        return None
    K = int(H_index.shape[1]) if len(H_index.shape) == 2 else 1
    if A.device:
        if H_index.dtype.__str__() != "torch.int64":
            raise OakError(ERR_ARGS, "H_index: expected an int64 CUDA tensor")
        A.keep.append(H_index)
        pidx = ctypes.c_void_p(H_index.contiguous().data_ptr())
    else:
        idx = np.ascontiguousarray(np.asarray(H_index, dtype=np.int64)).reshape(-1)
        A.keep.append(idx)
        pidx = ctypes.c_void_p(idx.ctypes.data)
    H = ObsOper(m=m, K=K, index=pidx, weight=A.vec(H_weight, n=m * K, name="H_weight"),
                shift=A.vec(H_shift, n=m, name="H_shift"))
    A.keep.append(H)
    return H


def ensemble_prologue(Ef, H_index, H_weight, H_shift=None):
    """Mean and scaled anomalies of the ensemble and of H Ef + Hshift
    (assimilation.F90:3110-3134). ``H_index``/``H_weight``: (m, K) sparse rows (index < 0
    unused). Returns ``(xf, Sf, Hxf, HSf)``."""
    n, N = int(Ef.shape[0]), int(Ef.shape[1])
    m = int(H_index.shape[0])
    device = _device_mode(Ef, H_weight, H_shift)
    A = _Args(device)
    pE, ldE = A.mat(Ef, n, N, "Ef")
    H = _obsoper(A, H_index, H_weight, H_shift, m)
    xf = _empty_like_mode(device, (n,), like=Ef)
    Sf = _empty_like_mode(device, (n, N), order="F", like=Ef)
    Hxf = _empty_like_mode(device, (m,), like=Ef)
    HSf = _empty_like_mode(device, (m, N), order="F", like=Ef)
    dims = Dims(n=n, N=N, m=m, ldS=n, ldH=max(m, 1), mem=MEM_DEVICE if device else MEM_HOST)
    _sync_torch(device, Ef)
    rc = lib().oakg_ensemble_prologue(ctypes.byref(dims), pE, ldE,
                                      None if H is None else ctypes.byref(H),
                                      A.vec(xf, name="xf"), A.mat(Sf, n, N, "Sf")[0],
                                      A.vec(Hxf, name="Hxf"), A.mat(HSf, m, N, "HSf")[0])
    _check(rc)
    return xf, Sf, Hxf, HSf


def ensemble_epilogue(xf, xa, Sa, inflation=1.0, max_correction=None):
    """Posterior inflation, correction clip and reconstruction
    (assimilation.F90:3299-3312, 3558-3565). Returns ``Ea`` (n, N)."""
    n, N = int(Sa.shape[0]), int(Sa.shape[1])
    device = _device_mode(xf, xa, Sa, max_correction)
    A = _Args(device)
    pSa, ldS = A.mat(Sa, n, N, "Sa")
    Ea = _empty_like_mode(device, (n, N), order="F", like=Sa)
    dims = Dims(n=n, N=N, m=0, ldS=ldS, ldH=1, mem=MEM_DEVICE if device else MEM_HOST)
    _sync_torch(device, Sa)
    rc = lib().oakg_ensemble_epilogue(ctypes.byref(dims), A.vec(xf, n=n, name="xf"),
                                      A.vec(xa, n=n, name="xa"), pSa, float(inflation),
                                      A.vec(max_correction, n=n, name="max_correction"),
                                      A.mat(Ea, n, N, "Ea")[0], n)
    _check(rc)
    return Ea


def ens_loc_analysis(zone_size, Ef, H_index, H_weight, yo, r_diag, zone_pos, obs_pos, corr_len,
                     max_len, *, H_shift=None, inflation=1.0, max_correction=None,
                     weight=GAUSS_CUTOFF, metric=CARTESIAN, loctype=1, localise_obs=True,
                     rotate=True, precision=PREC_FP64):
    """Local analysis of an ensemble on the device: prologue, :func:`loc_analysis`, epilogue
    (oakg_ens_locanalysis). Returns ``Ea`` (n, N)."""
    Z = int(zone_size.shape[0])
    n, N = int(Ef.shape[0]), int(Ef.shape[1])
    m = int(yo.shape[0])
    ox, oy, oz, ot = (tuple(obs_pos) + (None,) * 4)[:4]
    device = _device_mode(zone_size, Ef, H_weight, yo, r_diag, zone_pos, corr_len, max_len,
                          ox, oy, oz, ot)
    A = _Args(device)
    pE, ldE = A.mat(Ef, n, N, "Ef")
    H = _obsoper(A, H_index, H_weight, H_shift, m)
    dims = Dims(n=n, N=N, m=m, ldS=n, ldH=max(m, 1), mem=MEM_DEVICE if device else MEM_HOST)
    loc = Loc(weight=weight, metric=metric, loctype=loctype, localise_obs=int(bool(localise_obs)),
              rotate=int(bool(rotate)), precision=int(precision), flags=0, cell_size=0.0)
    zp = zone_pos.reshape(-1) if device else np.ascontiguousarray(
        np.asarray(zone_pos, dtype=np.float64).reshape(Z, 4))
    Ea = _empty_like_mode(device, (n, N), order="F", like=Ef)
    _sync_torch(device, Ef)
    rc = lib().oakg_ens_locanalysis(
        ctypes.byref(dims), ctypes.byref(loc), Z, A.vec(zone_size, np.int32, "zone_size", Z), pE,
        ldE, None if H is None else ctypes.byref(H), A.vec(yo, n=m, name="yo"),
        A.vec(r_diag, n=m, name="r_diag"), A.vec(zp, n=4 * Z, name="zone_pos"),
        A.vec(ox, n=m, name="obs_x"), A.vec(oy, n=m, name="obs_y"), A.vec(oz, n=m, name="obs_z"),
        A.vec(ot, n=m, name="obs_t"), A.vec(corr_len, n=Z, name="corr_len"),
        A.vec(max_len, n=Z, name="max_len"), float(inflation),
        A.vec(max_correction, n=n, name="max_correction"), A.mat(Ea, n, N, "Ea")[0])
    _check(rc)
    return Ea


def ens2sqrt(E):
    """Mean and the N - 1 anomaly columns of Pham's reduction (oakg_ens2sqrt,
    rrsqrt.F90:786-806). Returns ``(mean (n,), S (n, N-1))``."""
    n, N = int(E.shape[0]), int(E.shape[1])
    device = _device_mode(E)
    A = _Args(device)
    pE, ldE = A.mat(E, n, N, "E")
    mean = _empty_like_mode(device, (n,), like=E)
    S = _empty_like_mode(device, (n, N - 1), order="F", like=E)
    dims = Dims(n=n, N=N, m=0, ldS=n, ldH=1, mem=MEM_DEVICE if device else MEM_HOST)
    _sync_torch(device, E)
    _check(lib().oakg_ens2sqrt(ctypes.byref(dims), pE, ldE, A.vec(mean, name="mean"),
                               A.mat(S, n, N - 1, "S")[0]))
    return mean, S


def sqrt2ens(mean, S, theta=None):
    """The N-member ensemble with this mean and covariance S S^T (oakg_sqrt2ens,
    rrsqrt.F90:815-839): ``E = mean + S Om^T``, ``Om = sqrt(N-1) perpSpace(1/sqrt(N)) theta``
    with ``theta`` an (N-1) x (N-1) orthogonal matrix (the identity if None; the reference
    draws it at random). Returns ``E (n, N)``."""
    n, K = int(S.shape[0]), int(S.shape[1])
    N = K + 1
    device = _device_mode(mean, S, theta)
    A = _Args(device)
    pS, ldS = A.mat(S, n, K, "S")
    E = _empty_like_mode(device, (n, N), order="F", like=S)
    pT = None if theta is None else A.mat(theta, K, K, "theta")[0]
    dims = Dims(n=n, N=N, m=0, ldS=ldS, ldH=1, mem=MEM_DEVICE if device else MEM_HOST)
    _sync_torch(device, S)
    _check(lib().oakg_sqrt2ens(ctypes.byref(dims), A.vec(mean, n=n, name="mean"), pS, pT,
                               A.mat(E, n, N, "E")[0], n))
    return E


def ens_analysis(Ef, HEf, yo, r_diag):
    """Global analysis of an ensemble (oakg_ens_analysis, ensAnalysis of
    rrsqrt.F90:613-671). Returns ``(Ea (n, N), xa (n,), amplitudes (N,))``."""
    n, N = int(Ef.shape[0]), int(Ef.shape[1])
    m = int(yo.shape[0])
    device = _device_mode(Ef, HEf, yo, r_diag)
    A = _Args(device)
    pE, ldE = A.mat(Ef, n, N, "Ef")
    pH, ldH = A.mat(HEf, m, N, "HEf") if m > 0 else (None, 1)
    Ea = _empty_like_mode(device, (n, N), order="F", like=Ef)
    xa = _empty_like_mode(device, (n,), like=Ef)
    ampl = _empty_like_mode(device, (N,), like=Ef)
    dims = Dims(n=n, N=N, m=m, ldS=n, ldH=max(m, 1), mem=MEM_DEVICE if device else MEM_HOST)
    _sync_torch(device, Ef)
    _check(lib().oakg_ens_analysis(ctypes.byref(dims), pE, ldE, pH, ldH,
                                   A.vec(yo, n=m, name="yo"), A.vec(r_diag, n=m, name="r_diag"),
                                   A.mat(Ea, n, N, "Ea")[0], A.vec(xa, name="xa"),
                                   A.vec(ampl, name="ampl")))
    return Ea, xa, ampl


def biased_loc_analysis(gamma, zone_size, xf, bf, Hxf, yo, Sf, HSf, r_diag, zone_pos, obs_pos,
                        corr_len, max_len, H_index, H_weight, *, H_shift=None,
                        weight=GAUSS_CUTOFF, metric=CARTESIAN, loctype=1, localise_obs=True,
                        rotate=True, precision=PREC_FP64, want_sa=True):
    """Bias-aware local analysis (oakg_biased_locanalysis, biasedLocAnalysis of
    rrsqrt.F90:476-546) with the sparse observation operator (H_index, H_weight, H_shift).
    Returns ``(xa, ba, Sa)`` (Sa = Sf, or None without ``want_sa``)."""
    Z = int(zone_size.shape[0])
    n, N = int(xf.shape[0]), int(Sf.shape[1])
    m = int(yo.shape[0])
    ox, oy, oz, ot = (tuple(obs_pos) + (None,) * 4)[:4]
    device = _device_mode(zone_size, xf, bf, Hxf, yo, Sf, HSf, r_diag, zone_pos, corr_len,
                          max_len, H_weight, ox, oy, oz, ot)
    A = _Args(device)
    pSf, ldS = A.mat(Sf, n, N, "Sf")
    pHS, ldH = A.mat(HSf, m, N, "HSf")
    H = _obsoper(A, H_index, H_weight, H_shift, m)
    dims = Dims(n=n, N=N, m=m, ldS=ldS, ldH=ldH, mem=MEM_DEVICE if device else MEM_HOST)
    loc = Loc(weight=weight, metric=metric, loctype=loctype, localise_obs=int(bool(localise_obs)),
              rotate=int(bool(rotate)), precision=int(precision), flags=0, cell_size=0.0)
    zp = zone_pos.reshape(-1) if device else np.ascontiguousarray(
        np.asarray(zone_pos, dtype=np.float64).reshape(Z, 4))
    xa = _empty_like_mode(device, (n,), like=Sf)
    ba = _empty_like_mode(device, (n,), like=Sf)
    Sa = _empty_like_mode(device, (n, N), order="F", like=Sf) if want_sa else None
    if device and want_sa and ldS != n:
        raise OakError(ERR_ARGS, "device Sf with ld != n is not supported by this wrapper")
    _sync_torch(device, Sf)
    rc = lib().oakg_biased_locanalysis(
        ctypes.byref(dims), ctypes.byref(loc), Z, A.vec(zone_size, np.int32, "zone_size", Z),
        float(gamma), None if H is None else ctypes.byref(H), A.vec(xf, n=n, name="xf"),
        A.vec(bf, n=n, name="bf"), A.vec(Hxf, n=m, name="Hxf"), A.vec(yo, n=m, name="yo"), pSf,
        pHS, A.vec(r_diag, n=m, name="r_diag"), A.vec(zp, n=4 * Z, name="zone_pos"),
        A.vec(ox, n=m, name="obs_x"), A.vec(oy, n=m, name="obs_y"), A.vec(oz, n=m, name="obs_z"),
        A.vec(ot, n=m, name="obs_t"), A.vec(corr_len, n=Z, name="corr_len"),
        A.vec(max_len, n=Z, name="max_len"), A.vec(xa, name="xa"), A.vec(ba, name="ba"),
        None if Sa is None else A.mat(Sa, n, N, "Sa")[0])
    _check(rc)
    return xa, ba, Sa


class Plan:
    """A prepared local analysis over device (torch CUDA) tensors (oakg_plan_locanalysis).

    Takes the arguments of :func:`loc_analysis` (all CUDA tensors). The constructor runs the
    analysis once and captures its device work as one CUDA graph; :meth:`execute` replays it
    against the current contents of the same tensors (update them in place between calls)
    and returns ``(xa, Sa, nobs)`` -- tensors owned by the plan, overwritten by each
    execution. ``tune=True`` picks the observation cell edge by timing candidates on the data
    (see :attr:`info`). The plan keeps references to every tensor it was given.
    """

    def __init__(self, zone_size, xf, Hxf, yo, Sf, HSf, r_diag, zone_pos, obs_pos, corr_len,
                 max_len, *, weight=GAUSS_CUTOFF, metric=CARTESIAN, loctype=1,
                 localise_obs=True, rotate=True, want_sa=True, precision=PREC_FP64, tune=False,
                 cell_size=0.0):
        self._h = None
        Z = int(zone_size.shape[0])
        n = int(xf.shape[0])
        m = int(yo.shape[0])
        N = int(Sf.shape[1])
        ox, oy, oz, ot = (tuple(obs_pos) + (None,) * 4)[:4]
        if not _device_mode(zone_size, xf, Hxf, yo, Sf, HSf, r_diag, zone_pos, corr_len,
                            max_len, ox, oy, oz, ot):
            raise OakError(ERR_ARGS, "a plan binds CUDA tensors")
        A = _Args(True)
        pSf, ldS = A.mat(Sf, n, N, "Sf")
        pHS, ldH = A.mat(HSf, m, N, "HSf")
        dims = Dims(n=n, N=N, m=m, ldS=ldS, ldH=ldH, mem=MEM_DEVICE)
        loc = Loc(weight=weight, metric=metric, loctype=loctype,
                  localise_obs=int(bool(localise_obs)), rotate=int(bool(rotate)),
                  precision=int(precision), flags=0, cell_size=float(cell_size))
        self.xa = _empty_like_mode(True, (n,), like=Sf)
        self.Sa = _empty_like_mode(True, (n, N), order="F", like=Sf) if want_sa else None
        self.nobs = _empty_like_mode(True, (Z,), dtype=np.int32, like=Sf)
        _sync_torch(True, Sf)
        h = ctypes.c_void_p()
        rc = lib().oakg_plan_locanalysis(
            ctypes.byref(h), ctypes.byref(dims), ctypes.byref(loc), Z,
            A.vec(zone_size, np.int32, "zone_size", Z), A.vec(xf, n=n, name="xf"),
            A.vec(Hxf, n=m, name="Hxf"), A.vec(yo, n=m, name="yo"), pSf, pHS,
            A.vec(r_diag, n=m, name="r_diag"), A.vec(zone_pos.reshape(-1), n=4 * Z,
                                                      name="zone_pos"),
            A.vec(ox, n=m, name="obs_x"), A.vec(oy, n=m, name="obs_y"),
            A.vec(oz, n=m, name="obs_z"), A.vec(ot, n=m, name="obs_t"),
            A.vec(corr_len, n=Z, name="corr_len"), A.vec(max_len, n=Z, name="max_len"),
            A.vec(self.xa, name="xa"), None if self.Sa is None else A.mat(self.Sa, n, N, "Sa")[0],
            None, A.vec(self.nobs, np.int32, "nobs"), int(bool(tune)))
        _check(rc)
        self._h = h
        self._keep = A.keep + [zone_pos]

    def execute(self, stream=None):
        """Replay the analysis on ``stream`` (a torch stream, a raw handle or None: the plan's
        own stream, ordered after work on the current torch stream) and wait for it."""
        if self._h is None:
            raise OakError(ERR_ARGS, "plan is closed")
        if stream is None:
            import torch
            torch.cuda.current_stream(self.xa.device).synchronize()
            ptr = None
        else:
            ptr = getattr(stream, "cuda_stream", stream)
        _check(lib().oakg_plan_execute(self._h, None if ptr is None else ctypes.c_void_p(ptr)))
        return self.xa, self.Sa, self.nobs

    @property
    def info(self) -> dict:
        """Chosen cell edge, graph node count, the tuning samples (edge, ms) and the zone
        schedule of the selection + Gram stage (descending observation count or index order,
        with both measured stage times)."""
        cs = ctypes.c_double(0.0)
        nodes = ctypes.c_int64(0)
        tc = (ctypes.c_double * 8)()
        tm = (ctypes.c_double * 8)()
        k = lib().oakg_plan_info(self._h, ctypes.byref(cs), ctypes.byref(nodes), tc, tm, 8)
        t_idx = ctypes.c_double(0.0)
        t_cnt = ctypes.c_double(0.0)
        used = lib().oakg_plan_schedule(self._h, ctypes.byref(t_idx), ctypes.byref(t_cnt))
        return {"cell_size": cs.value, "graph_nodes": nodes.value,
                "tuning": [(tc[i], tm[i]) for i in range(k)],
                "zone_order": "descending observation count" if used else "index",
                "zone_order_ms": {"index": t_idx.value, "count": t_cnt.value}}

    def close(self):
        if self._h is not None:
            lib().oakg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def zone_positions(zone_size, x, y=None, z=None, t=None):
    """(Z, 4) coordinates of each zone's first element, from per-element coordinate arrays
    of the (zone-permuted) state vector -- what selectObservations reads through
    zoneIndex/ind2submv/getCoord (assimilation.F90:3710-3740)."""
    zs = np.asarray(zone_size, dtype=np.int64)
    first = np.concatenate([[0], np.cumsum(zs)[:-1]])
    out = np.zeros((zs.size, 4))
    for k, c in enumerate((x, y, z, t)):
        if c is not None:
            out[:, k] = np.asarray(c, dtype=np.float64)[first]
    return out


def loc_analysis_adjoint(zone_size, Hxf, yo, Sf, HSf, r_diag, zone_pos, obs_pos, corr_len,
                         max_len, dJ_dxa, *, inflation=1.0, weight=GAUSS_CUTOFF,
                         metric=CARTESIAN, loctype=1, localise_obs=True, brute_search=False,
                         cell_size=0.0):
    """Gradients of a scalar cost J(xa) of the local analysis mean (oakg_locanalysis_adjoint).

    ``dJ_dxa`` is dJ/dxa (n,). The analysis is the one of :func:`loc_analysis` with the prior
    anomalies ``inflation * Sf`` and ``inflation * HSf``. Returns ``(dJ_dyo (m,), dJ_dr (m,),
    dJ_dlen, dJ_dinfl)``; ``dJ_dlen`` is the derivative w.r.t. a common factor on
    ``corr_len`` and ``max_len`` at 1, with the selected observations held fixed.
    """
    Z = int(zone_size.shape[0])
    n = int(dJ_dxa.shape[0])
    m = int(yo.shape[0])
    N = int(Sf.shape[1])
    ox, oy, oz, ot = (tuple(obs_pos) + (None,) * 4)[:4]
    device = _device_mode(zone_size, Hxf, yo, Sf, HSf, r_diag, zone_pos, corr_len, max_len,
                          dJ_dxa, ox, oy, oz, ot)
    A = _Args(device)
    pSf, ldS = A.mat(Sf, n, N, "Sf")
    pHS, ldH = A.mat(HSf, m, N, "HSf")
    dims = Dims(n=n, N=N, m=m, ldS=ldS, ldH=ldH, mem=MEM_DEVICE if device else MEM_HOST)
    loc = Loc(weight=weight, metric=metric, loctype=loctype, localise_obs=int(bool(localise_obs)),
              rotate=1, precision=PREC_FP64, flags=FLAG_BRUTE_SEARCH if brute_search else 0,
              cell_size=float(cell_size))
    zp = zone_pos.reshape(-1) if device else np.ascontiguousarray(
        np.asarray(zone_pos, dtype=np.float64).reshape(Z, 4))
    like = Sf
    dyo = _empty_like_mode(device, (m,), like=like)
    dr = _empty_like_mode(device, (m,), like=like)
    dlen = ctypes.c_double(0.0)
    dinfl = ctypes.c_double(0.0)
    _sync_torch(device, like)
    rc = lib().oakg_locanalysis_adjoint(
        ctypes.byref(dims), ctypes.byref(loc), Z, A.vec(zone_size, np.int32, "zone_size", Z),
        A.vec(Hxf, n=m, name="Hxf"), A.vec(yo, n=m, name="yo"), pSf, pHS,
        A.vec(r_diag, n=m, name="r_diag"), A.vec(zp, n=4 * Z, name="zone_pos"),
        A.vec(ox, n=m, name="obs_x"), A.vec(oy, n=m, name="obs_y"), A.vec(oz, n=m, name="obs_z"),
        A.vec(ot, n=m, name="obs_t"), A.vec(corr_len, n=Z, name="corr_len"),
        A.vec(max_len, n=Z, name="max_len"), float(inflation), A.vec(dJ_dxa, n=n, name="dJ_dxa"),
        A.vec(dyo, name="dJ_dyo"), A.vec(dr, name="dJ_dr"), ctypes.byref(dlen),
        ctypes.byref(dinfl))
    _check(rc)
    return dyo, dr, dlen.value, dinfl.value


# ----------------------------------------------------------------------------- layout builders

def zone_layout(partition, nzones=None):
    """initPartition (oakg_zone_layout, assimilation.F90:578-641) of a partition vector of
    1-based zone numbers: ``(zone_size (Z,), zone_index (n,), inv_index (n,))``, int32, the
    indices 0-based (zone_index lists zone 1's elements in ascending order, then zone 2's, ...;
    inv_index is its inverse). ``nzones`` defaults to ``max(partition)``. A zone number outside
    1..nzones or an empty zone raises OakError (ERR_ARGS)."""
    device = _device_mode(partition)
    n = int(partition.numel() if _is_torch(partition) else np.asarray(partition).size)
    if nzones is None:
        nzones = int(partition.max()) if n else 0
    A = _Args(device)
    p = A.vec(partition, dtype=np.int32, name="partition", n=n)
    zs = _empty_like_mode(device, (max(int(nzones), 0),), dtype=np.int32, like=partition)
    zi = _empty_like_mode(device, (n,), dtype=np.int32, like=partition)
    inv = _empty_like_mode(device, (n,), dtype=np.int32, like=partition)
    _sync_torch(device, partition)
    _check(lib().oakg_zone_layout(n, p, int(nzones), MEM_DEVICE if device else MEM_HOST,
                                  A.vec(zs, dtype=np.int32), A.vec(zi, dtype=np.int32),
                                  A.vec(inv, dtype=np.int32)))
    return zs, zi, inv


def partition_compact(labels):
    """The zone numbering of globalInit (oakg_partition_compact, assimilation.F90:416-424):
    ``(partition, nzones)`` with every label replaced by its 1-based rank among the distinct
    labels (int32; gaps and any int32 values allowed)."""
    device = _device_mode(labels)
    n = int(labels.numel() if _is_torch(labels) else np.asarray(labels).size)
    A = _Args(device)
    pl = A.vec(labels, dtype=np.int32, name="labels", n=n)
    out = _empty_like_mode(device, (n,), dtype=np.int32, like=labels)
    nz = ctypes.c_int32(0)
    _sync_torch(device, labels)
    _check(lib().oakg_partition_compact(n, pl, MEM_DEVICE if device else MEM_HOST,
                                        A.vec(out, dtype=np.int32), ctypes.byref(nz)))
    return out, int(nz.value)


def permute_rows(index, X):
    """``X[index]`` for a vector (n,) or a column-major matrix (n, k) (oakg_permute_rows):
    with ``index = zone_index`` the state in zone order, with ``inv_index`` back."""
    device = _device_mode(index, X)
    n = int(X.shape[0])
    k = 1 if X.ndim == 1 else int(X.shape[1])
    A = _Args(device)
    pi = A.vec(index, dtype=np.int32, name="index", n=n)
    if X.ndim == 1:
        px, ldx = A.vec(X, name="X", n=n), n
        Y = _empty_like_mode(device, (n,), like=X)
        py, ldy = A.vec(Y), n
    else:
        px, ldx = A.mat(X, n, k, "X")
        Y = _empty_like_mode(device, (n, k), order="F", like=X)
        py, ldy = A.mat(Y, n, k, "Y")
    _sync_torch(device, X)
    _check(lib().oakg_permute_rows(n, k, pi, px, ldx, py, ldy,
                                   MEM_DEVICE if device else MEM_HOST))
    return Y


def sea_index(mask):
    """Sea packing of a masked grid (oakg_sea_index): ``(sea (npts,) int64, nsea)`` with
    ``sea[i]`` the number of unmasked points before point ``i`` (flat index of ``mask``, which
    callers pass in Fortran order) or -1 where ``mask`` is true."""
    device = _device_mode(mask)
    if device:
        import torch
        mk = mask.reshape(-1)
        mk = (mk != 0).to(torch.uint8).contiguous()
    else:
        mk = np.ascontiguousarray((np.asarray(mask) != 0).reshape(-1, order="F"), dtype=np.uint8)
    npts = int(mk.numel() if device else mk.size)
    A = _Args(device)
    pm = A.vec(mk, dtype=np.uint8, name="mask", n=npts)
    sea = _empty_like_mode(device, (npts,), dtype=np.int64, like=mask)
    cnt = ctypes.c_int64(0)
    _sync_torch(device, mask)
    _check(lib().oakg_sea_index(npts, pm, MEM_DEVICE if device else MEM_HOST,
                                A.vec(sea, dtype=np.int64), ctypes.byref(cnt)))
    return sea, int(cnt.value)


def obsoper_rectilinear(axes, obs_pos, sea=None, offset=0):
    """genObservationOper for one variable on a rectilinear grid (oakg_obsoper_rectilinear,
    assimilation.F90:2471-2656 with cinterp, ndgrid.F90:1183-1257). ``axes``: the 1..4 axis
    coordinate vectors (each strictly monotone, >= 2 points; grid points in Fortran order);
    ``obs_pos``: one coordinate array per axis (m each); ``sea``: the grid's sea packing
    (:func:`sea_index`) or None; ``offset``: the variable's first state row. Returns
    ``(index (m, 2^d) int64, weight (m, 2^d))`` in the oakg_obsoper row form: index -1 for an
    observation outside the grid or next to a masked point, -2 in a cell too small for the
    1e-8 determinant tolerance."""
    d = len(axes)
    device = _device_mode(*axes, *obs_pos, sea)
    shape = np.asarray([int(a.numel() if _is_torch(a) else np.asarray(a).size) for a in axes],
                       dtype=np.int32)
    if len(obs_pos) != d:
        raise OakError(ERR_ARGS, f"obs_pos: expected {d} coordinate arrays")
    m = int(obs_pos[0].numel() if _is_torch(obs_pos[0]) else np.asarray(obs_pos[0]).size)
    K = 1 << d
    if device:
        import torch
        coords = torch.cat([a.reshape(-1).to(torch.float64) for a in axes]).contiguous()
        pos = torch.stack([p.reshape(-1).to(torch.float64) for p in obs_pos]).contiguous()
    else:
        coords = np.concatenate([np.asarray(a, dtype=np.float64).reshape(-1) for a in axes])
        pos = np.ascontiguousarray(np.stack([np.asarray(p, dtype=np.float64).reshape(-1)
                                             for p in obs_pos]))
    A = _Args(device)
    pc = A.vec(coords, name="coords")
    pp = A.vec(pos, name="pos")
    ps = A.vec(sea, dtype=np.int64, name="sea", n=int(np.prod(shape)))
    index = _empty_like_mode(device, (m, K), dtype=np.int64, like=coords)
    weight = _empty_like_mode(device, (m, K), like=coords)
    _sync_torch(device, coords)
    _check(lib().oakg_obsoper_rectilinear(d, shape.ctypes.data_as(ctypes.c_void_p), pc, ps,
                                          int(offset), m, pp,
                                          MEM_DEVICE if device else MEM_HOST,
                                          A.vec(index, dtype=np.int64),
                                          A.vec(weight)))
    return index, weight


def obsoper_to_zone_order(index, inv_index):
    """The operator's state rows mapped to the zone-ordered state (oakg_obsoper_to_zone_order,
    assimilation.F90:2404-2407): ``index`` (int64, any shape, negative entries kept) is updated
    in place and returned."""
    device = _device_mode(index, inv_index)
    n = int(inv_index.numel() if _is_torch(inv_index) else np.asarray(inv_index).size)
    cnt = int(index.numel() if _is_torch(index) else np.asarray(index).size)
    A = _Args(device)
    if not device:
        if not (isinstance(index, np.ndarray) and index.dtype == np.int64
                and index.flags.c_contiguous):
            raise OakError(ERR_ARGS, "index: expected a C-contiguous int64 array (updated in place)")
    pi = A.vec(index, dtype=np.int64, name="index")
    pv = A.vec(inv_index, dtype=np.int32, name="inv_index", n=n)
    _sync_torch(device, index)
    _check(lib().oakg_obsoper_to_zone_order(cnt, pi, pv, n, MEM_DEVICE if device else MEM_HOST))
    return index


# ----------------------------------------------------------------------------- OAK driver

def read_variable(spec):
    """A NetCDF classic-format variable ``"file.nc#var"`` read as the oak_init / oak_assim
    driver reads it (oakg_read_variable): ``(values (Fortran-ordered array), valex)``, the
    missing values left as ``valex``. Host only."""
    L = lib()
    cnt = ctypes.c_int64(0)
    nd = ctypes.c_int32(0)
    vx = ctypes.c_double(0.0)
    shape = (ctypes.c_int64 * 8)()
    _check(L.oakg_read_variable(spec.encode(), None, 0, ctypes.byref(cnt), shape,
                                ctypes.byref(nd), ctypes.byref(vx)))
    out = np.empty(cnt.value)
    _check(L.oakg_read_variable(spec.encode(), out.ctypes.data_as(ctypes.c_void_p), out.size,
                                ctypes.byref(cnt), shape, ctypes.byref(nd), ctypes.byref(vx)))
    return out.reshape([shape[k] for k in range(nd.value)], order="F"), vx.value


def oak_init(fname):
    """oak_init (assimilation.F90:4911-4916): read the init file; raises OakError on failure."""
    L = lib()
    L.oak_init(str(fname).encode())
    _check(L.oakg_last_status())


def oak_assim(ntime, Ef):
    """oak_assim (assimilation.F90:4919-4927) on a host ensemble ``Ef (n, r)``: returns Ea."""
    L = lib()
    E = np.asfortranarray(np.asarray(Ef, dtype=np.float64))
    n, r = E.shape
    Ea = np.empty_like(E, order="F")
    L.oak_assim(int(ntime), int(n), int(r), E.ctypes.data_as(ctypes.c_void_p),
                Ea.ctypes.data_as(ctypes.c_void_p))
    _check(L.oakg_last_status())
    return Ea


def oak_done():
    """oak_done (assimilation.F90:4929-4933)."""
    L = lib()
    L.oak_done()
    _check(L.oakg_last_status())

