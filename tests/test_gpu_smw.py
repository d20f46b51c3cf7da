"""Non-diagonal observation error covariance R = diag(C) + B B^T (SMWCovar,
covariance.F90:464-570) on the GPU, against the oracle (pinned to the SMW cases of
test/test_rrsqrt.F90:326-340 in tests/test_oracle_golden.py): the augmented zone Gram and the
per-zone Woodbury reduction (zone_smw.cu)."""
import numpy as np
import pytest

from oak_gb300.workloads import local_case, rrsqrt_test_case
from oracle import oakref

pytestmark = pytest.mark.gpu

REL = 1e-10


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _B(m, k):
    return np.sin(3.0 * np.arange(1, m * k + 1)).reshape(k, m).T.copy()


def test_smw_reference_case(oakg):
    """test_rrsqrt.F90's case (n = 10, m = 5, N = 12) with R = SMWCovar(2 I, sin(3 i)):
    global analysis == Kalman; Gaspari-Cohn local analysis with and without observation
    localisation == the oracle."""
    xf, Sf, H, y, r = rrsqrt_test_case()
    HSf, Hxf = H @ Sf, H @ xf
    n, m = xf.size, y.size
    B = _B(m, 12)
    xa_k, Pa_k = oakref.kalman_reference(xf, Sf, H, y, np.diag(r) + B @ B.T)
    xa, Sa, _ = oakg.analysis(xf, Hxf, y, Sf, HSf, r, smw_B=B)
    assert np.max(np.abs(xa - xa_k)) < 1e-8 and np.max(np.abs(Sa @ Sa.T - Pa_k)) < 1e-8
    xmod, xobs = np.arange(n) / (n - 1.0), np.arange(m) / (m - 1.0)
    zone_pos = np.zeros((n, 4))
    zone_pos[:, 0] = xmod
    obs_pos = (xobs, np.zeros(m), np.zeros(m), np.zeros(m))
    corr, maxl = np.full(n, 0.21), np.full(n, 1e30)
    sel = oakref.geometric_selector(zone_pos, obs_pos, corr, maxl, kind=oakref.GASPARI_COHN)
    zs = np.ones(n, dtype=np.int32)
    for localise in (False, True):
        xa, Sa, _, _ = oakg.loc_analysis(zs, xf, Hxf, y, Sf, HSf, r, zone_pos, obs_pos, corr,
                                         maxl, weight=oakg.GASPARI_COHN, localise_obs=localise,
                                         smw_B=B)
        xa_o, Sa_o, _, _ = oakref.loc_analysis(zs, sel, xf, Hxf, y, Sf, HSf, r,
                                               localise_obs=localise, smw_B=B)
        assert _rel(xa - xf, xa_o - xf) < REL and _rel(Sa, Sa_o) < REL


@pytest.mark.parametrize("device", [False, True])
def test_smw_local_case(oakg, device):
    """The local workload at 1/10 scale (N = 32) with a rank-6 B: zones select hundreds of
    observations, so each zone packs its own Woodbury matrix."""
    c = local_case(scale=1 / 10, N=32)
    rng = np.random.default_rng(31)
    B = np.asfortranarray(0.05 * rng.standard_normal((c.m, 6)))
    sel = oakref.geometric_selector(c.zone_pos, c.obs_pos, c.corr_len, c.max_len, kind=c.weight)
    xa_o, Sa_o, _, nobs_o = oakref.loc_analysis(c.zone_size, sel, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                                c.r_diag, smw_B=B)
    args = (c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag, c.zone_pos, c.obs_pos,
            c.corr_len, c.max_len)
    if device:
        import torch
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")
        F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device="cuda:0").t()
        args = tuple(F(a) if (isinstance(a, np.ndarray) and a.ndim == 2 and a.shape[1] == c.N)
                     else (tuple(T(x) for x in a) if isinstance(a, tuple) else T(a))
                     for a in args)
        xa, Sa, _, nobs = oakg.loc_analysis(*args, weight=c.weight, smw_B=F(B))
        xa, Sa, nobs = xa.cpu().numpy(), Sa.cpu().numpy(), nobs.cpu().numpy()
    else:
        xa, Sa, _, nobs = oakg.loc_analysis(*args, weight=c.weight, smw_B=B)
    assert np.array_equal(nobs, nobs_o) and nobs_o.max() > 100
    assert _rel(xa - c.xf, xa_o - c.xf) < REL and _rel(Sa, Sa_o) < REL


def test_smw_limits(oakg):
    xf, Sf, H, y, r = rrsqrt_test_case()
    B = _B(y.size, 4)
    with pytest.raises(oakg.OakError) as ei:
        oakg.loc_analysis(np.array([xf.size], np.int32), xf, H @ xf, y, Sf, H @ Sf, r,
                          np.zeros((1, 4)), (np.zeros(y.size), np.zeros(y.size)),
                          np.ones(1), np.ones(1), precision=oakg.PREC_MIXED, smw_B=B)
    assert "OAKG_PREC_FP64" in str(ei.value)
