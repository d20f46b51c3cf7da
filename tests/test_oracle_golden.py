"""The oracle (oracle/oakref.py and oracle/oakref.c) against the reference's own
known-answer tests -- this is what pins the oracle before it judges the CUDA path.

* test/test_covariance.F90:612-617  locfun values
* test/test_rrsqrt.F90:27-77        analysis == Kalman formulas (tol 1e-8 in double)
* test/test_rrsqrt.F90:140-159      locAnalysis with one zone / one zone per element and
                                    all observations == global Kalman formulas
* test/test_rrsqrt.F90:163-236      locAnalysis with Gaspari-Cohn weights, with and without
                                    observation localisation, == explicit per-zone formula
* test/test_assim.F90:59-172        ensemble prologue + analysis + epilogue: ensemble mean
                                    and covariance == Kalman (tol 1e-5)
* test/test_rrsqrt.F90:326-340      the same analyses with R = SMWCovar(2 I, B), B = sin(3 i)
                                    (m x dim_ens, column-major)
"""
import numpy as np
import pytest

from oak_gb300.workloads import rrsqrt_test_case
from oracle import cref, oakref

TOL = 1e-8  # test_rrsqrt.F90:20


@pytest.mark.parametrize("impl", ["numpy", "c"])
def test_locfun_known_values(impl):
    f = oakref.locfun if impl == "numpy" else (lambda r: np.array([cref.load().oakref_locfun(x) for x in r]))
    r = np.array([0.0, 0.4, 1.5, 2.5])
    v = np.asarray(f(r), dtype=float)
    assert abs(v[0] - 1.0) < 1e-7
    assert abs(v[1] - 0.783573333333333) < 1e-6
    assert abs(v[2] - 0.0164930555555556) < 1e-6
    assert abs(v[3] - 0.0) < 1e-7
    # support ends at 2 (continuity at 1 and 2)
    assert abs(oakref.locfun(np.array([2.0]))[0]) < 1e-15
    lo = oakref.locfun(np.array([1.0 - 1e-12, 1.0 + 1e-12]))
    assert abs(lo[0] - lo[1]) < 1e-10


def _kalman_case():
    xf, Sf, H, y, r = rrsqrt_test_case()
    return xf, Sf, H, y, r, H @ Sf, H @ xf


@pytest.mark.parametrize("impl", ["numpy", "c-lapack", "c-internal"])
def test_analysis_equals_kalman(impl):
    xf, Sf, H, y, r, HSf, Hxf = _kalman_case()
    xa_k, Pa_k = oakref.kalman_reference(xf, Sf, H, y, np.diag(r))
    if impl == "numpy":
        xa, Sa, _ = oakref.analysis(xf, Hxf, y, Sf, HSf, r)
    else:
        xa, Sa, _ = cref.analysis(xf, Hxf, y, Sf, HSf, r, use_lapack=(impl == "c-lapack"))
    assert np.max(np.abs(xa - xa_k)) < TOL
    assert np.max(np.abs(Sa @ Sa.T - Pa_k)) < TOL


def test_local_all_obs_equals_global():
    xf, Sf, H, y, r, HSf, Hxf = _kalman_case()
    xa_k, Pa_k = oakref.kalman_reference(xf, Sf, H, y, np.diag(r))
    n, m = xf.size, y.size
    sel_all = lambda zi, start: (np.ones(m), np.ones(m, dtype=bool))  # selectAllObservations
    for zs in (np.array([n]), np.ones(n, dtype=int)):
        xa, Sa, _, _ = oakref.loc_analysis(zs, sel_all, xf, Hxf, y, Sf, HSf, r)
        assert np.max(np.abs(xa - xa_k)) < TOL
        assert np.max(np.abs(Sa @ Sa.T - Pa_k)) < TOL


def _gc_geometry(n, m):
    """test_rrsqrt.F90:254-271: xmod, xobs on [0, 1], c = locfun(|xmod - xobs| / 0.21)."""
    xmod = np.arange(n) / (n - 1.0)
    xobs = np.arange(m) / (m - 1.0)
    zone_pos = np.zeros((n, 4))
    zone_pos[:, 0] = xmod
    obs_pos = (xobs, np.zeros(m), np.zeros(m), np.zeros(m))
    return zone_pos, obs_pos, np.full(n, 0.21), np.full(n, 1e30)


def _explicit_local(xf, Sf, H, y, r, weights_rel, localise):
    """Explicit per-zone formula of test_rrsqrt.F90:189-231 (one zone per element)."""
    Pf = Sf @ Sf.T
    R = np.diag(r)
    xa = np.empty_like(xf)
    for i, (w, rel) in enumerate(weights_rel):
        if not localise:
            rel = np.ones_like(rel)
        iloc = np.nonzero(rel)[0]
        Hloc = H[iloc]
        invRloc = np.linalg.inv(R[np.ix_(iloc, iloc)]) * np.outer(w[iloc], w[iloc])
        Pa = np.linalg.inv(np.linalg.inv(Pf) + Hloc.T @ invRloc @ Hloc)
        xa[i] = xf[i] + (Pa[i] @ (Hloc.T @ (invRloc @ (y[iloc] - Hloc @ xf))))
    return xa


@pytest.mark.parametrize("localise", [False, True])
@pytest.mark.parametrize("impl", ["numpy", "c"])
def test_gc_local_equals_explicit_formula(localise, impl):
    xf, Sf, H, y, r, HSf, Hxf = _kalman_case()
    n, m = xf.size, y.size
    zone_pos, obs_pos, corr, maxl = _gc_geometry(n, m)
    sel = oakref.geometric_selector(zone_pos, obs_pos, corr, maxl, kind=oakref.GASPARI_COHN)
    wr = [sel(i, i) for i in range(n)]
    xa_x = _explicit_local(xf, Sf, H, y, r, wr, localise)
    zs = np.ones(n, dtype=np.int32)
    if impl == "numpy":
        xa, Sa, ampl, nobs = oakref.loc_analysis(zs, sel, xf, Hxf, y, Sf, HSf, r,
                                                 localise_obs=localise)
    else:
        xa, Sa, ampl, nobs = cref.locanalysis(zs, xf, Hxf, y, Sf, HSf, r, zone_pos, obs_pos,
                                              corr, maxl, kind=1, localise_obs=localise)
    assert np.max(np.abs(xa - xa_x)) < TOL
    # amplitudes are written only in the non-localised branch (rrsqrt.F90:375-384)
    assert (np.abs(ampl).max() > 0) == (not localise)


def test_ensemble_driver_equals_kalman():
    """test_assim.F90: 3x3 grid, 2 variables (n = 18), N = 10, one observation of var1 at
    cell (2,2) (state index 5), yo = 1, R = 2; Ef = sin(3 i)."""
    n, N, m = 18, 10, 1
    i = np.arange(1, n * N + 1, dtype=np.float64)
    Ef = np.sin(3.0 * i).reshape(N, n).T.copy()
    H = np.zeros((m, n))
    H[0, 4] = 1.0
    yo = np.ones(m)
    R = 2.0 * np.eye(m)
    xf_m = Ef.mean(axis=1)
    Efp = Ef - xf_m[:, None]
    Pf = Efp @ Efp.T / (N - 1)
    K = Pf @ H.T @ np.linalg.inv(H @ Pf @ H.T + R)
    Pa_check = Pf - K @ H @ Pf
    xa_check = xf_m + K @ (yo - H @ xf_m)
    xf, Hxf, Sf, HSf = oakref.ensemble_prologue(Ef, H @ Ef)
    xa, Sa, _ = oakref.analysis(xf, Hxf, yo, Sf, HSf, np.diag(R))
    Ea = oakref.ensemble_epilogue(xf, xa, Sa)
    xa_e = Ea.mean(axis=1)
    Eap = Ea - xa_e[:, None]
    assert np.max(np.abs(xa_e - xa_check)) < 1e-5
    assert np.max(np.abs(Eap @ Eap.T / (N - 1.0) - Pa_check)) < 1e-5


def test_c_oracle_matches_numpy_oracle_random_local():
    """Both restatements agree on a random local problem (all metrics / weight kinds)."""
    rng = np.random.default_rng(7)
    n_z, nz, N, m = 40, 3, 9, 60
    n = n_z * nz
    Sf = rng.standard_normal((n, N)) * 0.3
    Sf -= Sf.mean(axis=1, keepdims=True)
    HSf = rng.standard_normal((m, N)) * 0.3
    HSf -= HSf.mean(axis=1, keepdims=True)
    xf, Hxf, yo = rng.standard_normal(n), rng.standard_normal(m), rng.standard_normal(m)
    r = rng.uniform(0.05, 0.2, m)
    zs = np.full(n_z, nz, dtype=np.int32)
    for metric, loctype, kind, scale in [(0, 1, 0, 1.0), (0, 1, 1, 1.0), (2, 1, 0, 1e5),
                                         (1, 1, 1, 1e5), (0, 2, 0, 1.0), (0, 3, 1, 1.0)]:
        zone_pos = np.column_stack([rng.uniform(0, 10, n_z), rng.uniform(-60, 60, n_z),
                                    rng.uniform(0, 10, n_z), rng.uniform(0, 10, n_z)])
        obs_pos = (rng.uniform(0, 10, m), rng.uniform(-60, 60, m), rng.uniform(0, 10, m),
                   rng.uniform(0, 10, m))
        corr = np.full(n_z, 2.0 * scale)
        maxl = np.full(n_z, 4.0 * scale)
        sel = oakref.geometric_selector(zone_pos, obs_pos, corr, maxl, metric, loctype, kind)
        xa1, Sa1, _, nobs1 = oakref.loc_analysis(zs, sel, xf, Hxf, yo, Sf, HSf, r)
        xa2, Sa2, _, nobs2 = cref.locanalysis(zs, xf, Hxf, yo, Sf, HSf, r, zone_pos, obs_pos,
                                              corr, maxl, metric=metric, loctype=loctype,
                                              kind=kind)
        assert np.array_equal(nobs1, nobs2)
        assert np.max(np.abs(xa1 - xa2)) < 1e-11
        assert np.max(np.abs(Sa1 - Sa2)) < 1e-11


def test_rotation_preserves_zero_sum_anomalies():
    """doc/oak.tex:492-517: with Sf columns summing to zero, Sa's rows still sum to zero."""
    rng = np.random.default_rng(3)
    n, N, m = 30, 11, 20
    E = rng.standard_normal((n, N))
    HE = rng.standard_normal((m, N))
    xf, Hxf, Sf, HSf = oakref.ensemble_prologue(E, HE)
    xa, Sa, _ = oakref.analysis(xf, Hxf, rng.standard_normal(m), Sf, HSf, np.full(m, 0.5))
    assert np.max(np.abs(Sa.sum(axis=1))) < 1e-12


def test_ens2sqrt_sqrt2ens_identities():
    """test/assimtest2.F90:65-103: Ef(jmax = 5, kmax + 1 = 3) = sin(1..15) (column-major);
    ens2sqrt gives S with S S^T = enscov(Ef) and the ensemble mean; sqrt2ens gives back an
    ensemble with that covariance and mean (for any orthogonal theta: the reference draws it
    at random)."""
    jmax, N = 5, 3
    Ef = np.sin(np.arange(1, jmax * N + 1, dtype=np.float64)).reshape(N, jmax).T.copy()
    cov = np.cov(Ef)
    mean, S = oakref.ens2sqrt(Ef)
    assert S.shape == (jmax, N - 1)
    assert np.max(np.abs(S @ S.T - cov)) < 1e-14
    assert np.max(np.abs(mean - Ef.mean(axis=1))) < 1e-15
    rng = np.random.default_rng(7)
    theta, _ = np.linalg.qr(rng.standard_normal((N - 1, N - 1)))
    for th in (None, theta):
        Ea = oakref.sqrt2ens(mean, S, th)
        assert np.max(np.abs(np.cov(Ea) - cov)) < 1e-14
        assert np.max(np.abs(Ea.mean(axis=1) - mean)) < 1e-14


def test_ens_analysis_equals_kalman():
    """ensAnalysis (rrsqrt.F90:613-671) on the test_assim.F90 case: the analysed ensemble's mean
    and covariance are the Kalman ones."""
    n, N, m = 18, 10, 1
    i = np.arange(1, n * N + 1, dtype=np.float64)
    Ef = np.sin(3.0 * i).reshape(N, n).T.copy()
    H = np.zeros((m, n))
    H[0, 4] = 1.0
    yo, R = np.ones(m), 2.0 * np.eye(m)
    Pf = np.cov(Ef)
    K = Pf @ H.T @ np.linalg.inv(H @ Pf @ H.T + R)
    xf = Ef.mean(axis=1)
    Ea, xa, _ = oakref.ens_analysis(Ef, H @ Ef, yo, np.diag(R))
    assert np.max(np.abs(xa - (xf + K @ (yo - H @ xf)))) < 1e-12
    assert np.max(np.abs(Ea.mean(axis=1) - xa)) < 1e-12
    assert np.max(np.abs(np.cov(Ea) - (Pf - K @ H @ Pf))) < 1e-12


def test_biased_analysis_reduces_to_plain_and_scales_r():
    """biasedLocAnalysis (rrsqrt.F90:476-546): with gamma = 0 and no prior bias it is the plain
    local analysis (H xf + Hshift = Hxf); with gamma > 0 the second pass is the plain analysis
    of the unbiased forecast with R (1 - gamma), and ba = bf - gamma (first-pass increment)."""
    rng = np.random.default_rng(5)
    n, N, m, Z = 40, 8, 25, 10
    zone_size = np.full(Z, n // Z)
    idx = np.stack([rng.integers(0, n, m), rng.integers(0, n, m)], 1)
    idx[::4, 1] = -1
    w = rng.uniform(0.2, 0.8, (m, 2))
    shift = 0.1 * rng.standard_normal(m)
    xf = rng.standard_normal(n)
    Sf = rng.standard_normal((n, N))
    Hxf = oakref.sparse_apply(idx, w, xf, shift)
    HSf = np.stack([oakref.sparse_apply(idx, w, Sf[:, k]) for k in range(N)], 1)
    yo = Hxf + rng.standard_normal(m)
    r = rng.uniform(0.5, 2.0, m)
    zone_pos = np.column_stack([np.arange(Z), np.zeros(Z), np.zeros(Z), np.zeros(Z)]) * 1.0
    obs_pos = (rng.uniform(0, Z, m), np.zeros(m), np.zeros(m), np.zeros(m))
    sel = oakref.geometric_selector(zone_pos, obs_pos, np.full(Z, 2.0), np.full(Z, 4.0),
                                    kind=oakref.GASPARI_COHN)
    xa0, Sa0, _, _ = oakref.loc_analysis(zone_size, sel, xf, Hxf, yo, Sf, HSf, r)
    xa, ba, Sa = oakref.biased_loc_analysis(0.0, zone_size, sel, idx, w, shift, xf,
                                            np.zeros(n), Hxf, yo, Sf, HSf, r)
    assert np.max(np.abs(xa - xa0)) < 1e-12 and np.max(np.abs(ba)) == 0.0
    assert np.array_equal(Sa, Sf)
    g, bf = 0.3, 0.2 * rng.standard_normal(n)
    xa, ba, _ = oakref.biased_loc_analysis(g, zone_size, sel, idx, w, shift, xf, bf, Hxf, yo, Sf,
                                           HSf, r)
    inc = oakref.loc_analysis(zone_size, sel, np.zeros(n), Hxf, yo, Sf, HSf, r)[0]
    assert np.max(np.abs(ba - (bf - g * inc))) < 1e-14
    ux = xf - ba
    xa2 = oakref.loc_analysis(zone_size, sel, ux, oakref.sparse_apply(idx, w, ux, shift), yo, Sf,
                              HSf, (1 - g) * r)[0]
    assert np.max(np.abs(xa - xa2)) < 1e-12


def _smw_B(m, k=12):
    """test_rrsqrt.F90:329-332: B = reshape(sin(3 i), [m, dim_ens]), i = 1..m*dim_ens."""
    return np.sin(3.0 * np.arange(1, m * k + 1)).reshape(k, m).T.copy()


def test_smw_analysis_equals_kalman():
    xf, Sf, H, y, r, HSf, Hxf = _kalman_case()
    B = _smw_B(y.size)
    R = np.diag(r) + B @ B.T
    xa_k, Pa_k = oakref.kalman_reference(xf, Sf, H, y, R)
    xa, Sa, _ = oakref.analysis(xf, Hxf, y, Sf, HSf, r, smw_B=B)
    assert np.max(np.abs(xa - xa_k)) < TOL
    assert np.max(np.abs(Sa @ Sa.T - Pa_k)) < TOL
    n = xf.size
    sel_all = lambda zi, start: (np.ones(y.size), np.ones(y.size, dtype=bool))
    for zs in (np.array([n]), np.ones(n, dtype=int)):
        xa, Sa, _, _ = oakref.loc_analysis(zs, sel_all, xf, Hxf, y, Sf, HSf, r, smw_B=B)
        assert np.max(np.abs(xa - xa_k)) < TOL
        assert np.max(np.abs(Sa @ Sa.T - Pa_k)) < TOL


@pytest.mark.parametrize("localise", [False, True])
def test_smw_gc_local_equals_explicit_formula(localise):
    """test_rrsqrt.F90:163-236 with R = SMWCovar: the zone's inverse covariance is
    inv(R(iloc, iloc)) .* (w w^T) (R(iloc, iloc) is the packed SMWCovar)."""
    xf, Sf, H, y, r, HSf, Hxf = _kalman_case()
    n, m = xf.size, y.size
    B = _smw_B(m)
    R = np.diag(r) + B @ B.T
    zone_pos, obs_pos, corr, maxl = _gc_geometry(n, m)
    sel = oakref.geometric_selector(zone_pos, obs_pos, corr, maxl, kind=oakref.GASPARI_COHN)
    Pf = Sf @ Sf.T
    xa_x = np.empty_like(xf)
    for i in range(n):
        w, rel = sel(i, i)
        if not localise:
            rel = np.ones_like(rel)
        iloc = np.nonzero(rel)[0]
        Hloc = H[iloc]
        invRloc = np.linalg.inv(R[np.ix_(iloc, iloc)]) * np.outer(w[iloc], w[iloc])
        Pa = np.linalg.inv(np.linalg.inv(Pf) + Hloc.T @ invRloc @ Hloc)
        xa_x[i] = xf[i] + (Pa[i] @ (Hloc.T @ (invRloc @ (y[iloc] - Hloc @ xf))))
    xa, _, _, _ = oakref.loc_analysis(np.ones(n, dtype=np.int32), sel, xf, Hxf, y, Sf, HSf, r,
                                      localise_obs=localise, smw_B=B)
    assert np.max(np.abs(xa - xa_x)) < TOL
