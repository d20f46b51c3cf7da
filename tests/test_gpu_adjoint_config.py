"""The adjoint of the local analysis on the full local configuration: 360 x 180 x 20 grid,
N = 64, 50,000 observations, Gaspari-Cohn radius 12, prior inflation 1.05, and
J = mean over the 60 x 40 column sub-region (all levels) of (xa - x_true)^2.

* Reference gradient: torch float64 autograd through oracle/oakref_torch.py over the 2,400
  zones of the sub-region (the zones outside it do not enter J), with every observation:
  dJ/dyo and dJ/dr (50,000 each), dJ/d(length factor) and dJ/d(inflation) at 1e-9.
* Central finite differences of the GPU forward, step 1e-6 (FP64), on 200 random unit
  directions of (yo, r, length factor, inflation), seed 4902, at 1e-6. The forward of the
  differences runs on the sub-region's zones with all observations; it is first checked to be
  bit-identical, on those zones, to the forward over all 64,800 zones.
"""
import numpy as np
import pytest

from oak_gb300.workloads import local_case
from oracle import oakref_torch

pytestmark = pytest.mark.gpu

INFL = 1.05


@pytest.fixture(scope="module")
def case():
    c = local_case(scale=1.0)
    nx = 360
    zc = np.arange(c.Z)
    subz = ((zc % nx) >= nx // 3) & ((zc % nx) < nx // 3 + 60) & \
           ((zc // nx) >= 60) & ((zc // nx) < 100)
    zsel = np.flatnonzero(subz)
    starts = np.concatenate([[0], np.cumsum(c.zone_size)[:-1]])
    rows = np.concatenate([np.arange(starts[z], starts[z] + c.zone_size[z]) for z in zsel])
    return c, zsel, rows


def _fwd(oakg, c, zsel, rows, yo, r, kappa, s):
    xa, _, _, _ = oakg.loc_analysis(c.zone_size[zsel], c.xf[rows], c.Hxf, yo, c.Sf[rows] * s,
                                    c.HSf * s, r, c.zone_pos[zsel], c.obs_pos,
                                    c.corr_len[zsel] * kappa, c.max_len[zsel] * kappa,
                                    weight=c.weight, want_sa=False, want_ampl=False)
    return xa


def _J(xa, xt):
    d = xa - xt
    return float(np.sum(d * d) / d.size), 2.0 * d / d.size


def test_config_adjoint_reference_gradient_and_finite_differences(oakg, case):
    import torch
    c, zsel, rows = case
    assert zsel.size == 2400
    # forward over all zones; the sub-region's forward alone gives the same rows bit for bit
    xa_all, _, _, _ = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf * INFL,
                                        c.HSf * INFL, c.r_diag, c.zone_pos, c.obs_pos,
                                        c.corr_len, c.max_len, weight=c.weight, want_sa=False,
                                        want_ampl=False)
    xa = _fwd(oakg, c, zsel, rows, c.yo, c.r_diag, 1.0, INFL)
    assert np.array_equal(xa, xa_all[rows])
    xt = c.x_true[rows]
    J0, seed = _J(xa, xt)
    dyo, dr, dlen, dinfl = oakg.loc_analysis_adjoint(
        c.zone_size[zsel], c.Hxf, c.yo, c.Sf[rows], c.HSf, c.r_diag, c.zone_pos[zsel],
        c.obs_pos, c.corr_len[zsel], c.max_len[zsel], seed, inflation=INFL, weight=c.weight)

    # FP64 reference gradient: torch autograd through the restatement, same zones
    sels = oakref_torch.selections(c.zone_pos[zsel], c.obs_pos, c.corr_len[zsel],
                                   c.max_len[zsel], kind=c.weight)
    yo = torch.tensor(c.yo, requires_grad=True)
    r = torch.tensor(c.r_diag, requires_grad=True)
    kap = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(INFL, dtype=torch.float64, requires_grad=True)
    xa_t = oakref_torch.loc_analysis_mean(c.zone_size[zsel], c.xf[rows], c.Hxf, c.Sf[rows],
                                          c.HSf, c.corr_len[zsel], sels, yo, r, kap, st,
                                          c.weight)
    J = torch.sum((xa_t - torch.tensor(xt)) ** 2) / xt.size
    assert abs(float(J) - J0) <= 1e-10 * J0
    J.backward()
    rel = lambda a, b: np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
    assert np.count_nonzero(yo.grad.numpy()) > 1000
    assert rel(dyo, yo.grad.numpy()) < 1e-9
    assert rel(dr, r.grad.numpy()) < 1e-9
    assert abs(dlen - float(kap.grad)) <= 1e-9 * max(1.0, abs(float(kap.grad)))
    assert abs(dinfl - float(st.grad)) <= 1e-9 * max(1.0, abs(float(st.grad)))

    # central differences of the GPU forward on 200 random unit directions
    rng = np.random.default_rng(4902)
    h = 1e-6
    worst = 0.0
    for _ in range(200):
        u_y = rng.standard_normal(c.m)
        u_r = rng.standard_normal(c.m)
        u_k, u_s = rng.standard_normal(), rng.standard_normal()
        nrm = np.sqrt(u_y @ u_y + u_r @ u_r + u_k * u_k + u_s * u_s)
        u_y, u_r, u_k, u_s = u_y / nrm, u_r / nrm, u_k / nrm, u_s / nrm
        Jp, _ = _J(_fwd(oakg, c, zsel, rows, c.yo + h * u_y, c.r_diag + h * u_r, 1 + h * u_k,
                        INFL + h * u_s), xt)
        Jm, _ = _J(_fwd(oakg, c, zsel, rows, c.yo - h * u_y, c.r_diag - h * u_r, 1 - h * u_k,
                        INFL - h * u_s), xt)
        fd = (Jp - Jm) / (2 * h)
        an = dyo @ u_y + dr @ u_r + dlen * u_k + dinfl * u_s
        err = abs(fd - an) / max(1e-3, abs(an))
        worst = max(worst, err)
        assert err <= 1e-6, (fd, an)
    print(f"config adjoint: J={J0:.6e} dJ/dlen={dlen:.6e} dJ/dinfl={dinfl:.6e} "
          f"worst FD rel err {worst:.2e}")
