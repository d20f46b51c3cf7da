"""The FP64 reference gradient (oracle/oakref_torch.py) against central finite differences of
the NumPy oracle's analysis mean, and its forward against the oracle. CPU only."""
import numpy as np
import pytest
import torch

from oracle import oakref, oakref_torch


def _problem(seed=0, N=8, nzones=25, nz=3, m=60, kind=1):
    rng = np.random.default_rng(seed)
    n = nzones * nz
    xf, Hxf, Sf, HSf = oakref.ensemble_prologue(rng.standard_normal((n, N)),
                                                rng.standard_normal((m, N)))
    yo = Hxf + 0.3 * rng.standard_normal(m)
    r = rng.uniform(0.1, 0.5, m)
    zone_pos = np.column_stack([rng.uniform(0, 20, nzones), rng.uniform(0, 20, nzones),
                                np.zeros(nzones), np.zeros(nzones)])
    obs_pos = (rng.uniform(0, 20, m), rng.uniform(0, 20, m), np.zeros(m), np.zeros(m))
    corr, maxl = np.full(nzones, 3.0), np.full(nzones, 6.0)
    return dict(zs=np.full(nzones, nz), xf=xf, Hxf=Hxf, Sf=Sf, HSf=HSf, yo=yo, r=r,
                zone_pos=zone_pos, obs_pos=obs_pos, corr=corr, maxl=maxl, kind=kind)


@pytest.mark.parametrize("kind", [0, 1])
def test_torch_mean_equals_oracle(kind):
    P = _problem(kind=kind)
    sels = oakref_torch.selections(P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"], kind=kind)
    xa_t = oakref_torch.loc_analysis_mean(P["zs"], P["xf"], P["Hxf"], P["Sf"], P["HSf"],
                                          P["corr"], sels, torch.tensor(P["yo"]),
                                          torch.tensor(P["r"]), 1.0, 1.0, kind)
    sel = oakref.geometric_selector(P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"], kind=kind)
    xa_o, _, _, _ = oakref.loc_analysis(P["zs"], sel, P["xf"], P["Hxf"], P["yo"], P["Sf"],
                                        P["HSf"], P["r"])
    assert np.max(np.abs(xa_t.numpy() - xa_o)) < 1e-12


def test_reference_gradient_matches_finite_differences():
    P = _problem(kind=1)
    sels = oakref_torch.selections(P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"], kind=1)
    rng = np.random.default_rng(9)
    wgt = torch.tensor(rng.standard_normal(P["xf"].size))
    yo = torch.tensor(P["yo"], requires_grad=True)
    r = torch.tensor(P["r"], requires_grad=True)
    kap = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    s = torch.tensor(1.05, dtype=torch.float64, requires_grad=True)

    def J(yo_, r_, k_, s_):
        xa = oakref_torch.loc_analysis_mean(P["zs"], P["xf"], P["Hxf"], P["Sf"], P["HSf"],
                                            P["corr"], sels, yo_, r_, k_, s_, 1)
        return torch.sum(wgt * xa)

    J(yo, r, kap, s).backward()
    h = 1e-6
    for _ in range(5):
        dy = torch.tensor(rng.standard_normal(P["yo"].size))
        dr = torch.tensor(rng.standard_normal(P["r"].size)) * 0.01
        dk, ds = float(rng.standard_normal()), float(rng.standard_normal())
        with torch.no_grad():
            fd = (J(yo + h * dy, r + h * dr, kap + h * dk, s + h * ds)
                  - J(yo - h * dy, r - h * dr, kap - h * dk, s - h * ds)) / (2 * h)
        an = (yo.grad @ dy + r.grad @ dr + kap.grad * dk + s.grad * ds)
        assert abs(float(fd) - float(an)) <= 1e-6 * max(1.0, abs(float(an)))
