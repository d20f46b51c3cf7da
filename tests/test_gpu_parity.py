"""Parity of the CUDA path (through the C ABI) with the oracle.

FP64 tolerance: 1e-10 relative (analysis mean increment and anomalies), the bar of the
north-star specification; eigenvectors are never compared (sign freedom), only xa, Sa and the
amplitudes, which do not depend on it. Selection counts are integer and compared exactly.
"""
import numpy as np
import pytest

from oak_gb300.workloads import global_case, local_case, rrsqrt_test_case
from oracle import cref, oakref

pytestmark = pytest.mark.gpu

REL = 1e-10


def rel_err(a, b, ref_scale=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.linalg.norm(b) if ref_scale is None else ref_scale
    return np.linalg.norm(a - b) / max(s, 1e-300)


def check_local(xa, Sa, xa_r, Sa_r, xf, tol=REL):
    inc = np.linalg.norm(xa_r - xf)
    assert rel_err(xa, xa_r, max(inc, 1e-300)) < tol, "xa increment"
    assert rel_err(Sa, Sa_r) < tol, "Sa"


def check_local_on_zones(xa, Sa, xa_r, Sa_r, xf, zone_size, keep, tol=REL):
    """check_local restricted to the rows of the zones where `keep` is true (zones are
    consecutive row blocks of zone_size rows, rrsqrt.F90:328-335)."""
    rows = np.repeat(np.asarray(keep, bool), np.asarray(zone_size))
    assert rows.any()
    check_local(xa[rows], Sa[rows], xa_r[rows], Sa_r[rows], xf[rows], tol)


# ------------------------------------------------------------------ reference known answers

def test_analysis_rrsqrt_case_kalman(oakg):
    xf, Sf, H, y, r = rrsqrt_test_case()
    HSf, Hxf = H @ Sf, H @ xf
    xa, Sa, ampl = oakg.analysis(xf, Hxf, y, Sf, HSf, r)
    xa_k, Pa_k = oakref.kalman_reference(xf, Sf, H, y, np.diag(r))
    assert np.max(np.abs(xa - xa_k)) < 1e-8
    assert np.max(np.abs(Sa @ Sa.T - Pa_k)) < 1e-8
    xa_o, Sa_o, ampl_o = oakref.analysis(xf, Hxf, y, Sf, HSf, r)
    assert rel_err(xa, xa_o) < REL and rel_err(Sa, Sa_o) < REL and rel_err(ampl, ampl_o) < REL


@pytest.mark.parametrize("zones", ["one", "per-element"])
def test_local_all_obs_equals_global(oakg, zones):
    """test_rrsqrt.F90:140-159 with a selection that keeps every observation at weight 1:
    Gaussian weights with an infinite correlation length and maximum length."""
    xf, Sf, H, y, r = rrsqrt_test_case()
    HSf, Hxf = H @ Sf, H @ xf
    n, m = xf.size, y.size
    zs = np.array([n], np.int32) if zones == "one" else np.ones(n, np.int32)
    Z = zs.size
    xa, Sa, _, nobs = oakg.loc_analysis(zs, xf, Hxf, y, Sf, HSf, r, np.zeros((Z, 4)),
                                        (np.zeros(m), np.zeros(m)), np.full(Z, np.inf),
                                        np.full(Z, np.inf), weight=oakg.GAUSS_CUTOFF)
    xa_k, Pa_k = oakref.kalman_reference(xf, Sf, H, y, np.diag(r))
    assert np.all(nobs == m)
    assert np.max(np.abs(xa - xa_k)) < 1e-8
    assert np.max(np.abs(Sa @ Sa.T - Pa_k)) < 1e-8


@pytest.mark.parametrize("localise", [True, False])
def test_gc_local_rrsqrt_case(oakg, localise):
    """test_rrsqrt.F90:163-236 (GC weights locfun(|xmod - xobs| / 0.21))."""
    xf, Sf, H, y, r = rrsqrt_test_case()
    HSf, Hxf = H @ Sf, H @ xf
    n, m = xf.size, y.size
    zone_pos = np.zeros((n, 4))
    zone_pos[:, 0] = np.arange(n) / (n - 1.0)
    obs_pos = (np.arange(m) / (m - 1.0), np.zeros(m))
    corr, maxl = np.full(n, 0.21), np.full(n, 1e30)
    zs = np.ones(n, np.int32)
    xa, Sa, ampl, nobs = oakg.loc_analysis(zs, xf, Hxf, y, Sf, HSf, r, zone_pos, obs_pos, corr,
                                           maxl, weight=oakg.GASPARI_COHN,
                                           localise_obs=localise)
    sel = oakref.geometric_selector(zone_pos, obs_pos + (np.zeros(m), np.zeros(m)), corr, maxl,
                                    kind=oakref.GASPARI_COHN)
    xa_o, Sa_o, ampl_o, nobs_o = oakref.loc_analysis(zs, sel, xf, Hxf, y, Sf, HSf, r,
                                                     localise_obs=localise)
    assert np.array_equal(nobs, nobs_o)
    check_local(xa, Sa, xa_o, Sa_o, xf)
    assert rel_err(ampl, ampl_o) < REL or (localise and np.all(ampl == 0) and np.all(ampl_o == 0))


# ------------------------------------------------------------------ random local problems

def _random_local(seed, N=16, nzones=150, nz=4, m=400, metric=0, loctype=1, kind=1,
                  dom=40.0, radius=8.0, ragged=False):
    rng = np.random.default_rng(seed)
    zs = rng.integers(1, 2 * nz, nzones).astype(np.int32) if ragged else np.full(nzones, nz, np.int32)
    n = int(zs.sum())
    E = rng.standard_normal((n, N))
    HE = rng.standard_normal((m, N))
    xf, Hxf, Sf, HSf = oakref.ensemble_prologue(E, HE)
    yo = Hxf + rng.standard_normal(m) * 0.3
    r = rng.uniform(0.05, 0.5, m)
    if metric == 0:
        zone_pos = np.column_stack([rng.uniform(0, dom, nzones), rng.uniform(0, dom, nzones),
                                    rng.uniform(0, dom, nzones), rng.uniform(0, dom, nzones)])
        obs_pos = tuple(rng.uniform(0, dom, m) for _ in range(4))
        corr, maxl = np.full(nzones, radius / 2), np.full(nzones, radius)
    else:
        zone_pos = np.column_stack([rng.uniform(-180, 180, nzones), rng.uniform(-80, 80, nzones),
                                    np.zeros(nzones), np.zeros(nzones)])
        obs_pos = (rng.uniform(-180, 360, m), rng.uniform(-89, 89, m), np.zeros(m), np.zeros(m))
        corr, maxl = np.full(nzones, 1.5e6), np.full(nzones, 3e6)
    return dict(zs=zs, xf=xf, Hxf=Hxf, yo=yo, Sf=np.asfortranarray(Sf),
                HSf=np.asfortranarray(HSf), r=r, zone_pos=zone_pos, obs_pos=obs_pos, corr=corr,
                maxl=maxl, metric=metric, loctype=loctype, kind=kind)


def _run_both(oakg, P, localise=True, brute=False, rotate=True):
    xa, Sa, ampl, nobs = oakg.loc_analysis(
        P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"], P["zone_pos"],
        P["obs_pos"], P["corr"], P["maxl"], weight=P["kind"], metric=P["metric"],
        loctype=P["loctype"], localise_obs=localise, rotate=rotate, ampl_always=True,
        brute_search=brute)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(
        P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"], P["zone_pos"],
        P["obs_pos"], P["corr"], P["maxl"], metric=P["metric"], loctype=P["loctype"],
        kind=P["kind"], localise_obs=localise, rotate=rotate)
    return (xa, Sa, ampl, nobs), (xa_o, Sa_o, nobs_o)


@pytest.mark.parametrize("metric,loctype,kind", [(0, 1, 0), (0, 1, 1), (1, 1, 0), (2, 1, 1),
                                                 (0, 2, 0), (0, 3, 1)])
def test_random_local_matches_oracle(oakg, metric, loctype, kind):
    P = _random_local(11 + metric * 7 + loctype * 3 + kind, metric=metric, loctype=loctype,
                      kind=kind)
    (xa, Sa, _, nobs), (xa_o, Sa_o, nobs_o) = _run_both(oakg, P)
    same = nobs == nobs_o
    if metric == 0:
        assert same.all()
    else:  # CUDA's sin/cos/acos may differ from the host's by an ulp at the cut-off radius
        assert np.sum(~same) <= 1
    assert nobs.max() > 0
    # the numbers are compared on every zone whose selection agrees (all of them, or all but
    # the one zone an ulp at the cut-off moved)
    check_local_on_zones(xa, Sa, xa_o, Sa_o, P["xf"], P["zs"], same)


@pytest.mark.parametrize("N", [2, 7, 30, 64, 100, 113, 128])
def test_ensemble_sizes(oakg, N):
    P = _random_local(100 + N, N=N, nzones=40, m=250, ragged=True)
    (xa, Sa, _, nobs), (xa_o, Sa_o, nobs_o) = _run_both(oakg, P)
    assert np.array_equal(nobs, nobs_o)
    check_local(xa, Sa, xa_o, Sa_o, P["xf"])


def test_non_localised_branch_and_amplitudes(oakg):
    P = _random_local(5, nzones=30, m=120)
    (xa, Sa, ampl, nobs), (xa_o, Sa_o, nobs_o) = _run_both(oakg, P, localise=False)
    assert np.array_equal(nobs, nobs_o)
    check_local(xa, Sa, xa_o, Sa_o, P["xf"])
    _, _, ampl_o, _ = cref.locanalysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"],
                                       P["r"], P["zone_pos"], P["obs_pos"], P["corr"],
                                       P["maxl"], kind=P["kind"], localise_obs=False)
    assert rel_err(ampl, ampl_o) < REL


def test_no_rotation(oakg):
    P = _random_local(6, nzones=30, m=200)
    (xa, Sa, _, _), (xa_o, Sa_o, _) = _run_both(oakg, P, rotate=False)
    check_local(xa, Sa, xa_o, Sa_o, P["xf"])


def test_binned_search_equals_brute_force(oakg):
    """ndgrid near == checknear (test/test_cellgrid.F90) for the cell-grid selection."""
    for metric in (0, 1, 2):
        P = _random_local(21 + metric, metric=metric, nzones=120, m=600)
        a = oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"],
                              P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"],
                              weight=P["kind"], metric=metric)
        b = oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"],
                              P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"],
                              weight=P["kind"], metric=metric, brute_search=True)
        assert np.array_equal(a[3], b[3])
        assert rel_err(a[0], b[0]) < 1e-13 and rel_err(a[1], b[1]) < 1e-13


def test_zones_without_observations_copy_forecast(oakg):
    P = _random_local(8, nzones=50, m=30, dom=200.0, radius=5.0)
    xa, Sa, ampl, nobs = oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"],
                                           P["HSf"], P["r"], P["zone_pos"], P["obs_pos"],
                                           P["corr"], P["maxl"], weight=1, ampl_always=True)
    empty = np.repeat(nobs == 0, P["zs"])
    assert empty.any()
    assert np.array_equal(xa[empty], P["xf"][empty])
    assert np.array_equal(Sa[empty], P["Sf"][empty])
    assert np.all(ampl[:, nobs == 0] == 0)


def test_no_observations_at_all(oakg):
    P = _random_local(9, nzones=10, m=1)
    m0 = np.zeros(0)
    xa, Sa, _, nobs = oakg.loc_analysis(P["zs"], P["xf"], m0, m0, P["Sf"], np.zeros((0, 16)),
                                        m0, P["zone_pos"], (m0, m0), P["corr"], P["maxl"])
    assert np.all(nobs == 0)
    assert np.array_equal(xa, P["xf"]) and np.array_equal(Sa, P["Sf"])


def test_device_pointers_match_host(oakg):
    import torch
    P = _random_local(12, nzones=60, m=300)
    h = oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"],
                          P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"], weight=1)
    dev = torch.device("cuda:0")
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device=dev).t()
    d = oakg.loc_analysis(T(P["zs"]), T(P["xf"]), T(P["Hxf"]), T(P["yo"]), F(P["Sf"]),
                          F(P["HSf"]), T(P["r"]), T(P["zone_pos"]),
                          tuple(T(c) for c in P["obs_pos"]), T(P["corr"]), T(P["maxl"]),
                          weight=1)
    assert np.array_equal(h[3], d[3].cpu().numpy())
    assert np.array_equal(h[0], d[0].cpu().numpy())
    assert np.array_equal(h[1], d[1].cpu().numpy())


def test_nan_observation_is_reported(oakg):
    P = _random_local(13, nzones=20, m=100)
    yo = P["yo"].copy()
    yo[3] = np.nan
    with pytest.raises(oakg.OakError) as ei:
        oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], yo, P["Sf"], P["HSf"], P["r"],
                          P["zone_pos"], P["obs_pos"], P["corr"], np.full(20, 1e9),
                          weight=0)
    assert ei.value.code == 3  # OAKG_ERR_NAN
    # the library stays usable after the error
    oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"],
                      P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"])


def test_bad_arguments_are_rejected(oakg):
    P = _random_local(14, nzones=20, m=100)
    with pytest.raises(oakg.OakError) as ei:
        oakg.loc_analysis(P["zs"][:-1], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"],
                          P["zone_pos"][:-1], P["obs_pos"], P["corr"][:-1], P["maxl"][:-1])
    assert ei.value.code == 1


# ------------------------------------------------------------------ benchmark configurations

def test_global_config_matches_oracle(oakg):
    c = global_case()
    xa, Sa, ampl = oakg.analysis(c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag)
    xa_o, Sa_o, ampl_o = cref.analysis(c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag)
    check_local(xa, Sa, xa_o, Sa_o, c.xf)
    assert rel_err(ampl, ampl_o) < REL


def test_local_config_scaled_matches_oracle(oakg):
    """The 360x180x20 / N=64 / GC-12 configuration at 1/6 horizontal scale (same density)."""
    c = local_case(scale=1 / 6)
    xa, Sa, _, nobs = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                        weight=c.weight)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                             c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                             c.max_len, kind=c.weight)
    assert np.array_equal(nobs, nobs_o)
    check_local(xa, Sa, xa_o, Sa_o, c.xf)


def test_zero_weight_zone_keeps_forecast(oakg):
    """Gaussian weights that underflow to 0 (d >> L but d <= maxLength) give G = 0: the
    reference then returns xa = xf, Sa = Sf for the zone (lambda = 0, T = I, Omega = I)."""
    P = _random_local(15, nzones=12, m=40)
    corr = np.full(12, 1e-3)       # exp(-(d/L)^2) underflows for every d > ~0.03
    maxl = np.full(12, 1e9)        # every observation relevant
    xa, Sa, _, nobs = oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"],
                                        P["HSf"], P["r"], P["zone_pos"], P["obs_pos"], corr,
                                        maxl, weight=oakg.GAUSS_CUTOFF)
    assert np.all(nobs == 40)
    xa_o, Sa_o, _, _ = cref.locanalysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"],
                                        P["r"], P["zone_pos"], P["obs_pos"], corr, maxl, kind=0)
    assert np.allclose(xa, P["xf"], atol=1e-14) and np.allclose(Sa, P["Sf"], atol=1e-14)
    assert np.allclose(xa_o, P["xf"], atol=1e-14) and np.allclose(Sa_o, P["Sf"], atol=1e-14)


@pytest.mark.parametrize("N", [16, 64])
def test_rank_deficient_zones(oakg, N):
    """Few observations per zone (p < N): G has a large cluster of zero eigenvalues, which the
    eigensolver must still turn into an orthonormal basis (complement fill)."""
    P = _random_local(31 + N, N=N, nzones=60, m=12, dom=20.0, radius=10.0)
    (xa, Sa, _, nobs), (xa_o, Sa_o, nobs_o) = _run_both(oakg, P)
    assert np.array_equal(nobs, nobs_o)
    assert nobs.max() < N
    check_local(xa, Sa, xa_o, Sa_o, P["xf"])


@pytest.mark.parametrize("pinned", [False, True])
def test_host_pipeline_matches_device(oakg, pinned):
    """Host-memory calls copy Sf in on a copy stream while the selection, Gram and eigensolve
    stages run, and Sa / xa out per zone chunk; the kernels are those of device-memory calls,
    so both forms must agree bit for bit, with pageable and with pinned host buffers."""
    import torch
    from oak_gb300.workloads import local_case
    c = local_case(scale=1 / 6, N=64)
    dev = torch.device("cuda:0")
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device=dev).t()

    def host(a, fortran=False):
        a = np.asarray(a)
        if not pinned:
            return np.asfortranarray(a) if fortran else np.ascontiguousarray(a)
        if fortran:
            t = torch.empty((a.shape[1], a.shape[0]), dtype=torch.float64, pin_memory=True)
            t.numpy()[...] = a.T
            return t.numpy().T
        t = torch.empty(a.shape, dtype=torch.from_numpy(a[:0].copy()).dtype, pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    for prec in (oakg.PREC_FP64, oakg.PREC_MIXED):
        kw = dict(weight=c.weight, precision=prec)
        h = oakg.loc_analysis(host(c.zone_size), host(c.xf), host(c.Hxf), host(c.yo),
                              host(c.Sf, True), host(c.HSf, True), host(c.r_diag),
                              host(c.zone_pos), tuple(host(x) for x in c.obs_pos),
                              host(c.corr_len), host(c.max_len), **kw)
        d = oakg.loc_analysis(T(c.zone_size), T(c.xf), T(c.Hxf), T(c.yo), F(c.Sf), F(c.HSf),
                              T(c.r_diag), T(c.zone_pos), tuple(T(x) for x in c.obs_pos),
                              T(c.corr_len), T(c.max_len), **kw)
        assert np.array_equal(h[3], d[3].cpu().numpy())
        assert np.array_equal(h[0], d[0].cpu().numpy())
        assert np.array_equal(h[1], d[1].cpu().numpy())
