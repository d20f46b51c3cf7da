"""Adjoint of the local analysis mean (oakg_locanalysis_adjoint) on the GPU.

Checks: (1) against the FP64 reference gradient (torch autograd over oracle/oakref_torch.py)
at 1e-9 relative; (2) against central finite differences of the GPU forward (step 1e-6,
200 random unit directions, seed 4902) at 1e-6 relative; (3) the torch.autograd.Function wrapper; (4) device
pointers. J is the mean squared analysis-minus-truth over a sub-region, as in the benchmark's
adjoint configuration.
"""
import numpy as np
import pytest

from oracle import oakref, oakref_torch

pytestmark = pytest.mark.gpu


def _problem(seed=3, N=16, nx=12, ny=10, nz=3, m=180, kind=1):
    rng = np.random.default_rng(seed)
    Z = nx * ny
    n = Z * nz
    xf, Hxf, Sf, HSf = oakref.ensemble_prologue(rng.standard_normal((n, N)),
                                                rng.standard_normal((m, N)))
    yo = Hxf + 0.3 * rng.standard_normal(m)
    r = rng.uniform(0.05, 0.5, m)
    zc = np.arange(Z)
    zone_pos = np.column_stack([zc % nx, zc // nx, np.zeros(Z), np.zeros(Z)]).astype(float)
    obs_pos = (rng.uniform(0, nx, m), rng.uniform(0, ny, m), np.zeros(m), np.zeros(m))
    corr, maxl = np.full(Z, 2.0), np.full(Z, 4.0)
    xt = xf + rng.standard_normal(n) * 0.2
    # J over a sub-region: zones with x < 6 and y < 5 (all levels)
    sub = np.repeat((zc % nx < 6) & (zc // nx < 5), nz)
    return dict(zs=np.full(Z, nz, np.int32), xf=xf, Hxf=Hxf, Sf=np.asfortranarray(Sf),
                HSf=np.asfortranarray(HSf), yo=yo, r=r, zone_pos=zone_pos, obs_pos=obs_pos,
                corr=corr, maxl=maxl, kind=kind, xt=xt, sub=sub)


def _J_and_seed(xa, P):
    d = (xa - P["xt"]) * P["sub"]
    k = P["sub"].sum()
    return float(np.sum(d * d) / k), 2.0 * d / k


def _forward(oakg, P, yo, r, kappa=1.0, s=1.0):
    xa, _, _, _ = oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], yo, P["Sf"] * s, P["HSf"] * s, r,
                                    P["zone_pos"], P["obs_pos"], P["corr"] * kappa,
                                    P["maxl"] * kappa, weight=P["kind"], want_sa=False,
                                    want_ampl=False)
    return xa


@pytest.mark.parametrize("kind,N", [(0, 16), (1, 16), (1, 128)])
def test_adjoint_matches_reference_gradient(oakg, kind, N):
    import torch
    P = _problem(kind=kind, N=N)
    s = 1.05
    xa = _forward(oakg, P, P["yo"], P["r"], 1.0, s)
    _, seed = _J_and_seed(xa, P)
    dyo, dr, dlen, dinfl = oakg.loc_analysis_adjoint(
        P["zs"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"], P["zone_pos"], P["obs_pos"],
        P["corr"], P["maxl"], seed, inflation=s, weight=kind)
    sels = oakref_torch.selections(P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"], kind=kind)
    yo = torch.tensor(P["yo"], requires_grad=True)
    r = torch.tensor(P["r"], requires_grad=True)
    kap = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(s, dtype=torch.float64, requires_grad=True)
    xa_t = oakref_torch.loc_analysis_mean(P["zs"], P["xf"], P["Hxf"], P["Sf"], P["HSf"],
                                          P["corr"], sels, yo, r, kap, st, kind)
    sub = torch.tensor(P["sub"].astype(float))
    J = torch.sum(((xa_t - torch.tensor(P["xt"])) * sub) ** 2) / sub.sum()
    J.backward()
    rel = lambda a, b: np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
    assert rel(dyo, yo.grad.numpy()) < 1e-9
    assert rel(dr, r.grad.numpy()) < 1e-9
    assert abs(dlen - float(kap.grad)) <= 1e-9 * max(1.0, abs(float(kap.grad)))
    assert abs(dinfl - float(st.grad)) <= 1e-9 * max(1.0, abs(float(st.grad)))


def test_adjoint_matches_finite_differences(oakg):
    P = _problem(kind=1)
    s = 1.05
    xa = _forward(oakg, P, P["yo"], P["r"], 1.0, s)
    _, seed = _J_and_seed(xa, P)
    dyo, dr, dlen, dinfl = oakg.loc_analysis_adjoint(
        P["zs"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"], P["zone_pos"], P["obs_pos"],
        P["corr"], P["maxl"], seed, inflation=s, weight=1)
    # central differences, step 1e-6, on 200 random unit directions of (yo, r, kappa, s)
    rng = np.random.default_rng(4902)
    h = 1e-6
    for _ in range(200):
        u_y = rng.standard_normal(P["yo"].size)
        u_r = rng.standard_normal(P["r"].size)
        u_k, u_s = rng.standard_normal(), rng.standard_normal()
        nrm = np.sqrt(u_y @ u_y + u_r @ u_r + u_k * u_k + u_s * u_s)
        u_y, u_r, u_k, u_s = u_y / nrm, u_r / nrm, u_k / nrm, u_s / nrm
        Jp, _ = _J_and_seed(_forward(oakg, P, P["yo"] + h * u_y, P["r"] + h * u_r, 1 + h * u_k,
                                     s + h * u_s), P)
        Jm, _ = _J_and_seed(_forward(oakg, P, P["yo"] - h * u_y, P["r"] - h * u_r, 1 - h * u_k,
                                     s - h * u_s), P)
        fd = (Jp - Jm) / (2 * h)
        an = dyo @ u_y + dr @ u_r + dlen * u_k + dinfl * u_s
        assert abs(fd - an) <= 1e-6 * max(1e-3, abs(an)), (fd, an)


@pytest.mark.parametrize("device", ["cpu", "cuda"])
def test_autograd_function(oakg, device):
    import torch
    from oak_gb300.autograd import LocAnalysisMean
    P = _problem(kind=1)
    dev = torch.device(device)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device=dev).t()
    prob = dict(zone_size=T(P["zs"]), xf=T(P["xf"]), Hxf=T(P["Hxf"]), Sf=F(P["Sf"]),
                HSf=F(P["HSf"]), zone_pos=T(P["zone_pos"]),
                obs_pos=tuple(T(c) for c in P["obs_pos"]), corr_len=T(P["corr"]),
                max_len=T(P["maxl"]), opts=dict(weight=1))
    if device == "cuda":  # Sf * s keeps strides (1, n) -> column-major on the device
        prob["Sf"] = F(P["Sf"])
    yo = T(P["yo"]).clone().requires_grad_(True)
    r = T(P["r"]).clone().requires_grad_(True)
    kap = torch.tensor(1.0, dtype=torch.float64, device=dev, requires_grad=True)
    s = torch.tensor(1.05, dtype=torch.float64, device=dev, requires_grad=True)
    xa = LocAnalysisMean.apply(yo, r, kap, s, prob)
    sub = T(P["sub"].astype(float))
    J = torch.sum(((xa - T(P["xt"])) * sub) ** 2) / sub.sum()
    J.backward()
    sels = oakref_torch.selections(P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"], kind=1)
    yo2 = torch.tensor(P["yo"], requires_grad=True)
    r2 = torch.tensor(P["r"], requires_grad=True)
    k2 = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    s2 = torch.tensor(1.05, dtype=torch.float64, requires_grad=True)
    xa2 = oakref_torch.loc_analysis_mean(P["zs"], P["xf"], P["Hxf"], P["Sf"], P["HSf"],
                                         P["corr"], sels, yo2, r2, k2, s2, 1)
    J2 = torch.sum(((xa2 - torch.tensor(P["xt"])) * torch.tensor(P["sub"].astype(float))) ** 2) \
        / float(P["sub"].sum())
    J2.backward()
    assert abs(float(J) - float(J2)) < 1e-12
    for a, b in ((yo.grad, yo2.grad), (r.grad, r2.grad)):
        assert torch.linalg.norm(a.cpu() - b) / torch.linalg.norm(b) < 1e-9
    assert abs(float(kap.grad) - float(k2.grad)) <= 1e-9 * max(1.0, abs(float(k2.grad)))
    assert abs(float(s.grad) - float(s2.grad)) <= 1e-9 * max(1.0, abs(float(s2.grad)))
