"""Ensemble prologue / epilogue and the whole-ensemble local analysis on the GPU, against the
oracle (assimilation.F90:3110-3134, 3299-3312, 3558-3565 restated in oracle/oakref.py)."""
import numpy as np
import pytest

from oak_gb300.workloads import local_case
from oracle import cref, oakref

pytestmark = pytest.mark.gpu


def _sparse_operator(c, rng):
    """Two non-zeros per observation (observed level and its neighbour), some rows with one."""
    idx2 = np.where(c.obs_index % 20 > 0, c.obs_index - 1, c.obs_index + 1)
    index = np.stack([c.obs_index, idx2], axis=1).astype(np.int64)
    w = rng.uniform(0.2, 0.8, c.m)
    weight = np.stack([w, 1 - w], axis=1)
    index[::7, 1] = -1  # unused pair
    shift = 0.01 * rng.standard_normal(c.m)
    H = np.zeros((c.m, c.n))
    for t in range(2):
        ok = index[:, t] >= 0
        np.add.at(H, (np.nonzero(ok)[0], index[ok, t]), weight[ok, t])
    return index, weight, shift, H


def test_prologue_matches_oracle(oakg):
    rng = np.random.default_rng(11)
    c = local_case(scale=1 / 10, N=24, keep_ensemble=True)
    index, weight, shift, H = _sparse_operator(c, rng)
    xf, Sf, Hxf, HSf = oakg.ensemble_prologue(c.Ef, index, weight, shift)
    xf_o, Hxf_o, Sf_o, HSf_o = oakref.ensemble_prologue(c.Ef, H @ c.Ef + shift[:, None])
    for a, b in ((xf, xf_o), (Sf, Sf_o), (Hxf, Hxf_o), (HSf, HSf_o)):
        assert np.allclose(a, b, rtol=1e-13, atol=1e-13 * np.abs(b).max())


def test_epilogue_matches_oracle(oakg):
    rng = np.random.default_rng(12)
    n, N = 5000, 16
    xf = rng.standard_normal(n)
    xa = xf + rng.standard_normal(n)
    Sa = np.asfortranarray(rng.standard_normal((n, N)))
    mc = np.full(n, 0.8)
    for infl, m in ((1.0, None), (1.05, mc)):
        Ea = oakg.ensemble_epilogue(xf, xa, Sa, inflation=infl, max_correction=m)
        Ea_o = oakref.ensemble_epilogue(xf, xa, Sa, inflation=infl, max_correction=m)
        assert np.allclose(Ea, Ea_o, rtol=1e-15, atol=1e-15)


@pytest.mark.parametrize("device", [False, True])
def test_ensemble_local_analysis_matches_oracle(oakg, device):
    import torch
    rng = np.random.default_rng(13)
    c = local_case(scale=1 / 10, N=24, keep_ensemble=True)
    index, weight, shift, H = _sparse_operator(c, rng)
    mc = np.full(c.n, 0.5)
    args = (c.zone_size, c.Ef, index, weight, c.yo, c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
            c.max_len)
    kw = dict(H_shift=shift, inflation=1.05, max_correction=mc, weight=c.weight)
    if device:
        dev = torch.device("cuda", 0)
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
        F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device=dev).t()
        args = (T(c.zone_size), F(c.Ef), T(index), T(weight), T(c.yo), T(c.r_diag),
                T(c.zone_pos), tuple(T(x) for x in c.obs_pos), T(c.corr_len), T(c.max_len))
        kw.update(H_shift=T(shift), max_correction=T(mc))
    Ea = oakg.ens_loc_analysis(*args, **kw)
    if device:
        Ea = Ea.cpu().numpy()
    xf, Hxf, Sf, HSf = oakref.ensemble_prologue(c.Ef, H @ c.Ef + shift[:, None])
    xa, Sa, _, _ = cref.locanalysis(c.zone_size, xf, Hxf, c.yo, Sf, HSf, c.r_diag, c.zone_pos,
                                    c.obs_pos, c.corr_len, c.max_len, kind=c.weight)
    Ea_o = oakref.ensemble_epilogue(xf, xa, Sa, inflation=1.05, max_correction=mc)
    assert np.linalg.norm(Ea - Ea_o) <= 1e-10 * np.linalg.norm(Ea_o - c.Ef)


@pytest.mark.parametrize("device", [False, True])
def test_ens2sqrt_sqrt2ens_match_oracle(oakg, device):
    rng = np.random.default_rng(21)
    n, N = 3000, 33
    E = np.asfortranarray(rng.standard_normal((n, N)))
    theta, _ = np.linalg.qr(rng.standard_normal((N - 1, N - 1)))
    theta = np.asfortranarray(theta)
    mean_o, S_o = oakref.ens2sqrt(E)
    if device:
        import torch
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")
        F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device="cuda:0").t()
        mean, S = oakg.ens2sqrt(F(E))
        mean, S = mean.cpu().numpy(), S.cpu().numpy()
        E2 = oakg.sqrt2ens(T(mean_o), F(S_o), F(theta)).cpu().numpy()
    else:
        mean, S = oakg.ens2sqrt(E)
        E2 = oakg.sqrt2ens(mean_o, S_o, theta)
    assert np.allclose(mean, mean_o, rtol=1e-14, atol=1e-14)
    assert np.allclose(S, S_o, rtol=1e-13, atol=1e-13)
    E2_o = oakref.sqrt2ens(mean_o, S_o, theta)
    assert np.allclose(E2, E2_o, rtol=1e-12, atol=1e-12)
    if not device:  # theta = identity
        assert np.allclose(oakg.sqrt2ens(mean_o, S_o), oakref.sqrt2ens(mean_o, S_o),
                           rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("N", [2, 33, 65, 100])
def test_sqrt2ens_identity_and_general_theta(oakg, N):
    """Theta = I takes the closed form (row sums of S, one FMA an element), a general Theta the
    library GEMM; both against the oracle's N x (N-1) product, on device arrays with padded
    leading dimensions; ens2sqrt gives back the mean and S S^T."""
    import torch
    rng = np.random.default_rng(200 + N)
    n = 2500
    dev = torch.device("cuda:0")
    S_full = torch.as_tensor(rng.standard_normal((N - 1, n + 7)), device=dev)
    S = S_full.t()[:n]  # column-major, ldS = n + 7
    mean = torch.as_tensor(rng.standard_normal(n), device=dev)
    S_np, mean_np = S.cpu().numpy(), mean.cpu().numpy()
    E = oakg.sqrt2ens(mean, S).cpu().numpy()
    assert np.allclose(E, oakref.sqrt2ens(mean_np, S_np), rtol=1e-12, atol=1e-12)
    theta, _ = np.linalg.qr(rng.standard_normal((N - 1, N - 1)))
    th = torch.as_tensor(np.ascontiguousarray(theta.T), device=dev).t()
    E2 = oakg.sqrt2ens(mean, S, th).cpu().numpy()
    assert np.allclose(E2, oakref.sqrt2ens(mean_np, S_np, theta), rtol=1e-12, atol=1e-12)
    # ens2sqrt inverts it: the same mean and covariance S S^T (the same S for Theta = I)
    Edev = lambda E_: torch.as_tensor(np.ascontiguousarray(E_.T), device=dev).t()
    m2, S2 = (t.cpu().numpy() for t in oakg.ens2sqrt(Edev(E)))
    assert np.allclose(m2, mean_np, rtol=1e-12, atol=1e-12)
    assert np.allclose(S2, S_np, rtol=1e-12, atol=1e-12)
    m3, S3 = (t.cpu().numpy() for t in oakg.ens2sqrt(Edev(E2)))
    assert np.allclose(m3, mean_np, rtol=1e-12, atol=1e-12)
    assert np.allclose(S3 @ S3.T, S_np @ S_np.T, rtol=1e-11, atol=1e-11)


def test_ens_analysis_matches_oracle(oakg):
    rng = np.random.default_rng(22)
    n, N, m = 4000, 30, 300
    Ef = np.asfortranarray(rng.standard_normal((n, N)))
    idx = rng.choice(n, m, replace=False)
    HEf = np.asfortranarray(Ef[idx] + 0.01 * rng.standard_normal((m, N)))
    yo = HEf.mean(axis=1) + 0.3 * rng.standard_normal(m)
    r = rng.uniform(0.05, 0.2, m)
    Ea, xa, ampl = oakg.ens_analysis(Ef, HEf, yo, r)
    Ea_o, xa_o, ampl_o = oakref.ens_analysis(Ef, HEf, yo, r)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(xa, xa_o) < 1e-10 and rel(Ea, Ea_o) < 1e-10 and rel(ampl, ampl_o) < 1e-10


@pytest.mark.parametrize("gamma", [0.0, 0.35])
def test_biased_local_analysis_matches_oracle(oakg, gamma):
    rng = np.random.default_rng(23)
    c = local_case(scale=1 / 12, N=24, keep_ensemble=True)
    index, weight, shift, H = _sparse_operator(c, rng)
    Hxf = H @ c.xf + shift
    HSf = np.asfortranarray(H @ c.Sf)
    bf = 0.05 * rng.standard_normal(c.n)
    xa, ba, Sa = oakg.biased_loc_analysis(gamma, c.zone_size, c.xf, bf, Hxf, c.yo, c.Sf, HSf,
                                          c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                          c.max_len, index, weight, H_shift=shift,
                                          weight=c.weight)
    sel = oakref.geometric_selector(c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                    kind=c.weight)
    xa_o, ba_o, _ = oakref.biased_loc_analysis(gamma, c.zone_size, sel, index, weight, shift,
                                               c.xf, bf, Hxf, c.yo, c.Sf, HSf, c.r_diag)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(ba, ba_o) < 1e-10 and rel(xa, xa_o) < 1e-10
    assert np.array_equal(Sa, c.Sf)
