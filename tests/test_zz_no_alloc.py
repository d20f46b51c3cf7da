"""oakg_analysis_noalloc -- the global analysis for callers that cannot allocate device memory
(host programs that reserve the whole GPU for their own memory pool, or that must not let
cudaMalloc/cudaFree synchronise the device inside an assimilation cycle).

Called through the C ABI with device arrays, twice in a row on different problems (different
ensemble sizes, so a stale scratch array would show), and compared with oakg_analysis, the
existing entry point, at the tolerance of the other parity tests (1e-10 relative). This file
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


def _run_noalloc(oakg, torch, fn, args):
    xf, Hxf, yo, Sf, HSf, r = args
    n, N, m = xf.numel(), Sf.shape[1], yo.numel()
    xa = torch.empty_like(xf)
    Sa = torch.empty((N, n), dtype=torch.float64, device=xf.device).t()
    ampl = torch.empty(N, dtype=torch.float64, device=xf.device)
    dims = oakg.Dims(n=n, N=N, m=m, ldS=n, ldH=m, mem=oakg.MEM_DEVICE)
    torch.cuda.synchronize()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    rc = fn(ctypes.byref(dims), p(xf), p(Hxf), p(yo), p(Sf), p(HSf), p(r), p(xa), p(Sa), p(ampl),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, oakg.lib().oakg_last_status()
    return xa.cpu().numpy(), Sa.cpu().numpy(), ampl.cpu().numpy()


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
