"""FP32 storage at the boundary (oakg_locanalysis_f32, the reference's single-precision build).

* FP64 form: the FP32 inputs are widened and every product is FP64, so the outputs are exactly
  those of oakg_locanalysis on the widened inputs, rounded once to FP32 (compared bit for bit).
* Mixed form: within 1e-4 of the oracle on the widened inputs (the mixed-form bar), with the
  same selection counts.
Host and device arrays, N in the warp-per-zone (<= 64) and the 128-wide kernel families.
"""
import numpy as np
import pytest

from oracle import cref

from test_gpu_parity import _random_local

pytestmark = pytest.mark.gpu


def _f32(P):
    Q = dict(P)
    for k in ("xf", "Hxf", "yo", "r"):
        Q[k] = P[k].astype(np.float32)
    Q["Sf"] = np.asfortranarray(P["Sf"].astype(np.float32))
    Q["HSf"] = np.asfortranarray(P["HSf"].astype(np.float32))
    return Q


def _wide(Q):
    W = dict(Q)
    for k in ("xf", "Hxf", "yo", "r"):
        W[k] = Q[k].astype(np.float64)
    W["Sf"] = np.asfortranarray(Q["Sf"].astype(np.float64))
    W["HSf"] = np.asfortranarray(Q["HSf"].astype(np.float64))
    return W


def _call(oakg, P, device=False, **kw):
    args = [P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"], P["zone_pos"],
            P["obs_pos"], P["corr"], P["maxl"]]
    if device:
        import torch
        dev = torch.device("cuda:0")
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
        F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device=dev).t()
        args = [T(args[0]), T(args[1]), T(args[2]), T(args[3]), F(args[4]), F(args[5]),
                T(args[6]), T(args[7]), tuple(T(c) for c in args[8]), T(args[9]), T(args[10])]
    out = oakg.loc_analysis(*args, weight=P["kind"], metric=P["metric"], loctype=P["loctype"],
                            ampl_always=True, **kw)
    if device:
        out = tuple(o.cpu().numpy() for o in out)
    return out


@pytest.mark.parametrize("N,device", [(64, False), (64, True), (100, True), (128, False)])
def test_fp64_form_with_fp32_storage_is_fp64_rounded(oakg, N, device):
    Q = _f32(_random_local(300 + N, N=N, nzones=50, m=300, ragged=True))
    xa, Sa, ampl, nobs = _call(oakg, Q, device)
    assert xa.dtype == np.float32 and Sa.dtype == np.float32 and ampl.dtype == np.float32
    xa64, Sa64, ampl64, nobs64 = _call(oakg, _wide(Q), device)
    assert np.array_equal(nobs, nobs64)
    assert np.array_equal(xa, xa64.astype(np.float32))
    assert np.array_equal(Sa, Sa64.astype(np.float32))
    assert np.array_equal(ampl, ampl64.astype(np.float32))


@pytest.mark.parametrize("N,device", [(64, True), (64, False), (100, True), (128, True)])
def test_mixed_form_with_fp32_storage_matches_oracle(oakg, N, device):
    Q = _f32(_random_local(400 + N, N=N, nzones=60, m=400, ragged=True))
    W = _wide(Q)
    xa, Sa, _, nobs = _call(oakg, Q, device, precision=oakg.PREC_MIXED)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(W["zs"], W["xf"], W["Hxf"], W["yo"], W["Sf"],
                                             W["HSf"], W["r"], W["zone_pos"], W["obs_pos"],
                                             W["corr"], W["maxl"], kind=W["kind"])
    assert np.array_equal(nobs, nobs_o)
    inc = np.linalg.norm(xa_o - W["xf"])
    assert np.linalg.norm(xa.astype(np.float64) - xa_o) / inc < 1e-4
    assert np.linalg.norm(Sa.astype(np.float64) - Sa_o) / np.linalg.norm(Sa_o) < 1e-4


def test_fp32_storage_zones_without_observations_copy(oakg):
    Q = _f32(_random_local(8, nzones=50, m=30, dom=200.0, radius=5.0))
    for prec in (oakg.PREC_FP64, oakg.PREC_MIXED):
        xa, Sa, ampl, nobs = _call(oakg, Q, True, precision=prec)
        empty = np.repeat(nobs == 0, Q["zs"])
        assert empty.any()
        assert np.array_equal(xa[empty], Q["xf"][empty])
        assert np.array_equal(Sa[empty], Q["Sf"][empty])
