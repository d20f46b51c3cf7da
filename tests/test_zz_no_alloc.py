"""oakg_analysis_noalloc -- the global analysis for callers that cannot allocate device memory
(host programs that reserve the whole GPU for their own memory pool, or that must not let
cudaMalloc/cudaFree synchronise the device inside an assimilation cycle).

Called through the C ABI with device arrays, twice in a row on different problems (different
ensemble sizes, so a stale scratch array would show), and compared with oakg_analysis, the
existing entry point, at the tolerance of the other parity tests (1e-10 relative). Also: a call
without observations right after one with observations (nothing stale may leak through the
shared array), and the device's free memory unchanged across calls. This file
sorts last so that a run stopping at the first failure has run every other test first; it
also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from oak_gb300.workloads import global_case, rrsqrt_test_case

pytestmark = pytest.mark.gpu

REL = 1e-10


def _noalloc(oakg):
    L = oakg.lib()
    fn = L.oakg_analysis_noalloc
    fn.argtypes = [ctypes.POINTER(oakg.Dims)] + [ctypes.c_void_p] * 10
    fn.restype = ctypes.c_int
    return fn


def _device_case(torch, xf, Hxf, yo, Sf, HSf, r):
    dev = torch.device("cuda:0")
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
    F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T),
                                  device=dev).t()
    return T(xf), T(Hxf), T(yo), F(Sf), F(HSf), T(r)


def _outputs(torch, args):
    xf, Sf = args[0], args[3]
    n, N = xf.numel(), Sf.shape[1]
    return (torch.empty_like(xf), torch.empty((N, n), dtype=torch.float64, device=xf.device).t(),
            torch.empty(N, dtype=torch.float64, device=xf.device))


def _call(oakg, torch, fn, args, outs):
    """One call into the C ABI on torch's current stream; the outputs are the caller's."""
    xf, Hxf, yo, Sf, HSf, r = args
    xa, Sa, ampl = outs
    n, N, m = xf.numel(), Sf.shape[1], (0 if yo is None else yo.numel())
    dims = oakg.Dims(n=n, N=N, m=m, ldS=n, ldH=m, mem=oakg.MEM_DEVICE)
    p = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    rc = fn(ctypes.byref(dims), p(xf), p(Hxf), p(yo), p(Sf), p(HSf), p(r), p(xa), p(Sa), p(ampl),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, oakg.lib().oakg_last_status()


def _run_noalloc(oakg, torch, fn, args):
    outs = _outputs(torch, args)
    torch.cuda.synchronize()
    _call(oakg, torch, fn, args, outs)
    return tuple(t.cpu().numpy() for t in outs)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_noalloc_matches_analysis_on_two_calls(oakg):
    torch = pytest.importorskip("torch")
    fn = _noalloc(oakg)
    xf, Sf, H, y, r = rrsqrt_test_case()
    cases = [(xf, H @ xf, y, Sf, H @ Sf, r)]
    c = global_case()
    cases.append((c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag))
    for args in cases:  # N = 12, then N = 30
        xa, Sa, ampl = _run_noalloc(oakg, torch, fn, _device_case(torch, *args))
        xa_r, Sa_r, ampl_r = oakg.analysis(*args)
        assert _rel(xa - args[0], xa_r - args[0]) < REL
        assert _rel(Sa, Sa_r) < REL
        assert _rel(ampl, ampl_r) < REL


def test_noalloc_rejects_oversized_ensemble(oakg):
    torch = pytest.importorskip("torch")
    fn = _noalloc(oakg)
    dev = torch.device("cuda:0")
    n, m, N = 50, 10, 113
    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device=dev)
    dims = oakg.Dims(n=n, N=N, m=m, ldS=n, ldH=m, mem=oakg.MEM_DEVICE)
    bufs = [z(n), z(m), z(m), z(n * N), z(m * N), z(m) + 1, z(n), z(n * N), z(N)]
    rc = fn(ctypes.byref(dims), *[ctypes.c_void_p(b.data_ptr()) for b in bufs], None)
    assert rc == oakg.ERR_ARGS
    buf = ctypes.create_string_buffer(256)
    oakg.lib().oakg_last_error(buf, 256)
    assert b"112" in buf.value


def test_noalloc_no_observations_after_observations(oakg):
    """m = 0 right after an m > 0 call: the Gram is skipped, so a stale Gram matrix or stale
    amplitudes left in the shared array by the previous call must not leak into the result;
    the reference returns xa = xf, Sa = Sf and zero amplitudes (rrsqrt.F90:371)."""
    torch = pytest.importorskip("torch")
    fn = _noalloc(oakg)
    c = global_case()
    args = _device_case(torch, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag)
    _run_noalloc(oakg, torch, fn, args)
    xf, _, _, Sf, _, _ = args
    xa, Sa, ampl = _run_noalloc(oakg, torch, fn, (xf, None, None, Sf, None, None))
    assert np.array_equal(xa, c.xf)
    assert np.array_equal(Sa, c.Sf)
    assert np.all(ampl == 0)


def test_noalloc_allocates_no_device_memory(oakg):
    """The free device memory is the same before and after two calls (inputs and outputs made
    beforehand, and oakg_analysis run first since it grows buffers of its own)."""
    torch = pytest.importorskip("torch")
    fn = _noalloc(oakg)
    xf, Sf, H, y, r = rrsqrt_test_case()
    c = global_case()
    cases = [(xf, H @ xf, y, Sf, H @ Sf, r), (c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag)]
    dev_cases = [_device_case(torch, *a) for a in cases]
    outs = [_outputs(torch, a) for a in dev_cases]
    for a in cases:
        oakg.analysis(*a)
    for a, o in zip(dev_cases, outs):   # warm-up: the first call also looks up the array
        _call(oakg, torch, fn, a, o)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for a, o in zip(dev_cases, outs):
        _call(oakg, torch, fn, a, o)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
