"""Mixed-precision form (OAKG_PREC_MIXED) against the FP64 oracle.

Tolerance: 1e-4 relative analysis error (the spec bar): increment-relative for the mean,
Frobenius-relative for the anomalies. The observation selection is FP64 in both forms, so the
relevant-observation counts must be identical.
"""
import numpy as np
import pytest

from oak_gb300.workloads import batched_case, large_case, local_case
from oracle import cref

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _errs(xa, Sa, xa_o, Sa_o, xf):
    return (np.linalg.norm(xa - xa_o) / np.linalg.norm(xa_o - xf),
            np.linalg.norm(Sa - Sa_o) / np.linalg.norm(Sa_o))


# 64: the warp-per-zone FP32 eigensolve at its full width; 32 and 37: padded inside it (37 is
# not a multiple of 4); 65, 97, 100 and 128: the block-per-zone FP32 eigensolve (97 leaves a
# partial 16-component group and a partial 8-column block of the update)
@pytest.mark.parametrize("N,scale", [(64, 1 / 6), (32, 1 / 8), (37, 1 / 8), (65, 1 / 10),
                                     (97, 1 / 10), (100, 1 / 10), (128, 1 / 10)])
def test_mixed_local_matches_fp64_oracle(oakg, N, scale):
    c = local_case(scale=scale, N=N)
    xa, Sa, _, nobs = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                        weight=c.weight, precision=oakg.PREC_MIXED)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                             c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                             c.max_len, kind=c.weight)
    assert np.array_equal(nobs, nobs_o)
    e_mean, e_anom = _errs(xa, Sa, xa_o, Sa_o, c.xf)
    assert e_mean < TOL and e_anom < TOL, (e_mean, e_anom)


def test_mixed_gaussian_weights_and_amplitudes(oakg):
    c = local_case(scale=1 / 8, N=48)
    kw = dict(weight=oakg.GAUSS_CUTOFF, ampl_always=True)
    xa, Sa, ampl, _ = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                        precision=oakg.PREC_MIXED, **kw)
    xa6, Sa6, ampl6, _ = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                           c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                           c.max_len, **kw)
    e_mean, e_anom = _errs(xa, Sa, xa6, Sa6, c.xf)
    assert e_mean < TOL and e_anom < TOL
    assert np.linalg.norm(ampl - ampl6) / np.linalg.norm(ampl6) < TOL


def test_mixed_empty_zones_copy_forecast(oakg):
    c = local_case(scale=1 / 8, N=16, m=400)
    xa, Sa, _, nobs = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                        weight=c.weight, precision=oakg.PREC_MIXED)
    empty = np.repeat(nobs == 0, c.zone_size)
    assert empty.any()
    assert np.array_equal(xa[empty], c.xf[empty]) and np.array_equal(Sa[empty], c.Sf[empty])


def test_mixed_rank_deficient_zones(oakg):
    c = local_case(scale=1 / 8, N=64, m=2000)
    xa, Sa, _, nobs = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                        weight=c.weight, precision=oakg.PREC_MIXED)
    xa_o, Sa_o, _, _ = cref.locanalysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                        kind=c.weight)
    assert (nobs[nobs > 0] < 64).any()
    e_mean, e_anom = _errs(xa, Sa, xa_o, Sa_o, c.xf)
    assert e_mean < TOL and e_anom < TOL, (e_mean, e_anom)


def test_dense_clusters_fill_many_tiles(oakg):
    """Observations packed on a few tracks: zones select well over the 512-entry staging ring
    of the tensor-core Gram (many K-tiles, ring wrap-around); both forms against the oracle."""
    c = local_case(scale=1 / 8, N=64, m=300000, track_frac=0.95, ntracks=3)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                             c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                             c.max_len, kind=c.weight)
    assert nobs_o.max() > 1500
    for prec, tol in ((oakg.PREC_FP64, 1e-10), (oakg.PREC_MIXED, TOL)):
        xa, Sa, _, nobs = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                            c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                            c.max_len, weight=c.weight, precision=prec)
        assert np.array_equal(nobs, nobs_o)
        e_mean, e_anom = _errs(xa, Sa, xa_o, Sa_o, c.xf)
        assert e_mean < tol and e_anom < tol, (prec, e_mean, e_anom)


def test_mixed_batched_bilinear_case(oakg):
    """The 5-variable batched case (121-element columns, N = 100, bilinear observations
    clustered on track segments) against the oracle."""
    c = batched_case(scale=1 / 16)
    xa, Sa, _, nobs = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                        weight=c.weight, precision=oakg.PREC_MIXED)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                             c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                             c.max_len, kind=c.weight)
    assert np.array_equal(nobs, nobs_o) and nobs_o.max() > 300
    e_mean, e_anom = _errs(xa, Sa, xa_o, Sa_o, c.xf)
    assert e_mean < TOL and e_anom < TOL, (e_mean, e_anom)


def test_large_case_both_forms(oakg):
    """The 2-variable large case (100-element columns, N = 128, clustered bilinear
    observations with error sd ~ U(0.05, 0.5)) at 1/16 of its grid: the FP64 form at 1e-10 and
    the mixed form at 1e-4 against the oracle."""
    c = large_case(scale=1 / 16)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                             c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                             c.max_len, kind=c.weight)
    assert nobs_o.max() > 500
    for prec, tol in ((oakg.PREC_FP64, 1e-10), (oakg.PREC_MIXED, TOL)):
        xa, Sa, _, nobs = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                            c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                            c.max_len, weight=c.weight, precision=prec)
        assert np.array_equal(nobs, nobs_o)
        e_mean, e_anom = _errs(xa, Sa, xa_o, Sa_o, c.xf)
        assert e_mean < tol and e_anom < tol, (prec, e_mean, e_anom)


def test_ensemble_size_limits(oakg):
    """Both forms take N <= 128; N = 129 is rejected with an argument error."""
    c = local_case(scale=1 / 16, N=129, m=300)
    for prec in (oakg.PREC_FP64, oakg.PREC_MIXED):
        with pytest.raises(oakg.OakError) as ei:
            oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                              c.zone_pos, c.obs_pos, c.corr_len, c.max_len, weight=c.weight,
                              precision=prec)
        assert ei.value.code == oakg.ERR_ARGS and "128" in str(ei.value)


# the tensor-core update (3xTF32, the default) against the CUDA-core FP32 update: both give
# FP32-level products, so they agree far below the mixed-form bar; ragged zones longer than a
# 128-row tile, N not a multiple of 8 or 32, FP64 and FP32 storage
@pytest.mark.parametrize("N,f32", [(16, False), (37, False), (64, True), (100, True),
                                   (113, False), (128, True)])
def test_tensor_core_update_matches_cuda_core_update(oakg, N, f32):
    rng = np.random.default_rng(700 + N)
    Z = 40
    zs = rng.integers(1, 300, Z).astype(np.int32)   # some zones span up to three row tiles
    n, m = int(zs.sum()), 500
    Sf = np.asfortranarray(rng.standard_normal((n, N)) * 0.1)
    HSf = np.asfortranarray(rng.standard_normal((m, N)) * 0.1)
    xf, Hxf = rng.standard_normal(n), rng.standard_normal(m) * 0.1
    yo = Hxf + rng.standard_normal(m) * 0.1
    r = rng.uniform(0.01, 0.1, m)
    zone_pos = np.column_stack([rng.uniform(0, 30, Z), rng.uniform(0, 30, Z), np.zeros(Z),
                                np.zeros(Z)])
    zone_pos[:4, :2] = 100.0   # far from every observation: copied zones
    obs_pos = (rng.uniform(0, 30, m), rng.uniform(0, 30, m), np.zeros(m), np.zeros(m))
    corr, maxl = np.full(Z, 4.0), np.full(Z, 8.0)
    dt = np.float32 if f32 else np.float64
    args = (zs, xf.astype(dt), Hxf.astype(dt), yo.astype(dt), np.asfortranarray(Sf.astype(dt)),
            np.asfortranarray(HSf.astype(dt)), r.astype(dt), zone_pos, obs_pos, corr, maxl)
    kw = dict(weight=1, precision=oakg.PREC_MIXED)
    xa_t, Sa_t, _, nobs = oakg.loc_analysis(*args, **kw)
    xa_s, Sa_s, _, nobs_s = oakg.loc_analysis(*args, simt_update=True, **kw)
    assert np.array_equal(nobs, nobs_s) and (nobs > 0).any() and (nobs == 0).any()
    xa_t, Sa_t, xa_s, Sa_s = (a.astype(np.float64) for a in (xa_t, Sa_t, xa_s, Sa_s))
    e_mean = np.linalg.norm(xa_t - xa_s) / np.linalg.norm(xa_s - xf.astype(dt))
    e_anom = np.linalg.norm(Sa_t - Sa_s) / np.linalg.norm(Sa_s)
    assert e_mean < 1e-5 and e_anom < 1e-5, (e_mean, e_anom)
    empty = np.repeat(nobs == 0, zs)
    assert np.array_equal(Sa_t[empty], Sf.astype(dt)[empty].astype(np.float64))


# ---------------------------------------------------------------- FP64-accurate eigensolve

@pytest.mark.parametrize("N,scale", [(64, 1 / 6), (37, 1 / 8), (100, 1 / 10), (128, 1 / 10)])
def test_refined_eigensolve_matches_oracle(oakg, N, scale):
    """OAKG_PREC_MIXED_FP64EIG (the FP32 eigenpairs refined to FP64 accuracy) on the local
    configuration, at the mixed-form bar."""
    c = local_case(scale=scale, N=N)
    xa, Sa, _, nobs = oakg.loc_analysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                        weight=c.weight, precision=oakg.PREC_MIXED_FP64EIG)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf,
                                             c.r_diag, c.zone_pos, c.obs_pos, c.corr_len,
                                             c.max_len, kind=c.weight)
    assert np.array_equal(nobs, nobs_o)
    e_mean, e_anom = _errs(xa, Sa, xa_o, Sa_o, c.xf)
    assert e_mean < TOL and e_anom < TOL, (e_mean, e_anom)


def _exact_gram_case(N, dmax, seed=1, Z=16, nz=3):
    """Zones whose Gram matrix and innovation projection are exact in FP32: p = N integer
    observation rows d_q (+-1, ...) with d_q from 1 to dmax (geometric), weight 1 (every
    observation at its zone's position), r = 1, integer innovations. The eigenvalues spread
    over ~5 decades (dmax 1-8), so an FP32 eigensolve misses the small ones by ~eps_32 ||G||
    while the eigensolve is the only FP32 error source besides the transform and update."""
    rng = np.random.default_rng(seed)
    p, m = N, Z * N
    rows = []
    for _ in range(Z):
        M = rng.choice([-1.0, 1.0], size=(p, N))
        rows.append(np.round(np.geomspace(1.0, dmax, p))[:, None] * M)
    HSf = np.asfortranarray(np.vstack(rows))
    yo = rng.integers(-3, 4, m).astype(np.float64)
    Sf = np.asfortranarray(rng.standard_normal((Z * nz, N)) * 0.1)
    xf = rng.standard_normal(Z * nz)
    zone_pos = np.zeros((Z, 4))
    zone_pos[:, 0] = 100.0 * np.arange(Z)
    obs_pos = (np.repeat(zone_pos[:, 0], p), np.zeros(m), np.zeros(m), np.zeros(m))
    return (np.full(Z, nz, np.int32), xf, np.zeros(m), yo, Sf, HSf, np.ones(m), zone_pos,
            obs_pos, np.full(Z, 10.0), np.full(Z, 1.0))


# spectra that one refinement step separates (eigenvalue gaps above its threshold delta)
@pytest.mark.parametrize("N,dmax", [(32, 8.0), (100, 2.0), (128, 1.0)])
def test_refined_eigensolve_is_fp64_accurate(oakg, N, dmax):
    """With G exact in FP32, the refined eigenpairs leave only the FP32 rounding of T and of
    the update (~1e-6 of the oracle), several times closer than the FP32 eigensolve."""
    args = _exact_gram_case(N, dmax)
    xa_o, Sa_o, _, nobs_o = cref.locanalysis(*args, kind=0)
    out = {}
    for prec in (oakg.PREC_MIXED, oakg.PREC_MIXED_FP64EIG):
        xa, Sa, _, nobs = oakg.loc_analysis(*args, weight=oakg.GAUSS_CUTOFF, precision=prec)
        assert np.array_equal(nobs, nobs_o) and np.all(nobs == N)
        out[prec] = _errs(xa, Sa, xa_o, Sa_o, args[1])
    e32, e64 = out[oakg.PREC_MIXED], out[oakg.PREC_MIXED_FP64EIG]
    assert e64[0] < 1e-5 and e64[1] < 1e-5, (e64, e32)
    assert e64[0] < 0.2 * e32[0] and e64[1] < 0.4 * e32[1], (e64, e32)
