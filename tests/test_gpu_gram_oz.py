"""The plain form's tensor-core products (zone_gram_oz.cu: exact 8-bit slice products on BF16
tensor cores, N <= 64) against the FP64 CUDA-core ones (OAKG_FLAG_SIMT_GRAM) and the oracle:
the Gram of X = diag(|w| / sqrt(r)) HS_sel and the square-root transform
T_sym = U (I + L)^-1/2 U^T (the Gram of diag((1 + lambda)^-1/4) U^T).

* Both forms select the same observations and agree to 1e-12 on xa and Sa, 1e-11 on the
  amplitudes;
  each matches the oracle at the plain form's 1e-10.
* Zones selecting more than 256 observations (several accumulator reads) and more than 512 (the
  ring of selected observations wraps), every metric / selection kind, localise_obs = false.
* Columns of HS spanning six orders of magnitude and r spanning four: as close to the oracle as
  the FP64 CUDA-core products (to a factor 30) on that ill-conditioned case.
* A NaN in one observation row fails the call with the same status as the CUDA-core products
  (only the zones that select it see it).
* The transform without the mean-preserving rotation (rotate = false), and the one-zone global
  analysis.
"""
import numpy as np
import pytest

from oracle import cref

from test_gpu_parity import REL, _random_local, check_local, rel_err

pytestmark = pytest.mark.gpu


def _call(oakg, P, simt, localise=True, **kw):
    return oakg.loc_analysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"],
                             P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"],
                             weight=P["kind"], metric=P["metric"], loctype=P["loctype"],
                             localise_obs=localise, ampl_always=True, simt_gram=simt, **kw)


def _oracle(P, localise=True, rotate=True):
    return cref.locanalysis(P["zs"], P["xf"], P["Hxf"], P["yo"], P["Sf"], P["HSf"], P["r"],
                            P["zone_pos"], P["obs_pos"], P["corr"], P["maxl"],
                            metric=P["metric"], loctype=P["loctype"], kind=P["kind"],
                            localise_obs=localise, rotate=rotate)


def _both_agree(oakg, P, localise=True, tol=1e-12, **kw):
    a = _call(oakg, P, False, localise, **kw)
    b = _call(oakg, P, True, localise, **kw)
    assert np.array_equal(a[3], b[3])
    inc = np.linalg.norm(b[0] - P["xf"])
    assert rel_err(a[0], b[0], max(inc, 1e-300)) < tol
    assert rel_err(a[1], b[1]) < tol
    # the amplitudes are the increment in ensemble coordinates, before Sf averages their errors
    assert rel_err(a[2], b[2]) < 10 * tol
    return a, b


@pytest.mark.parametrize("N,metric,loctype,kind", [(64, 0, 1, 1), (37, 0, 1, 0), (20, 1, 1, 0),
                                                   (64, 2, 1, 1), (48, 0, 2, 0), (9, 0, 3, 1)])
def test_tensor_core_gram_matches_cuda_core_and_oracle(oakg, N, metric, loctype, kind):
    P = _random_local(700 + N + 10 * metric + loctype, N=N, nzones=80, m=500, metric=metric,
                      loctype=loctype, kind=kind, ragged=True)
    a, b = _both_agree(oakg, P)
    xa_o, Sa_o, _, nobs_o = _oracle(P)
    same = a[3] == nobs_o
    assert same.mean() > 0.95
    rows = np.repeat(same, P["zs"])
    check_local(a[0][rows], a[1][rows], xa_o[rows], Sa_o[rows], P["xf"][rows], REL)


def test_long_zones(oakg):
    """Zones selecting ~300 to ~3000 observations: several reads of the tensor-memory
    accumulators (every 256 observations) and a wrapping ring of selected observations."""
    P = _random_local(92, N=64, nzones=40, m=4000, dom=40.0, radius=30.0)
    a, b = _both_agree(oakg, P)
    assert a[3].max() > 1000 and a[3].min() > 200
    xa_o, Sa_o, _, nobs_o = _oracle(P)
    assert np.array_equal(a[3], nobs_o)
    check_local(a[0], a[1], xa_o, Sa_o, P["xf"], REL)


def test_wide_column_and_error_scales(oakg):
    """HS columns scaled by 10^-3 .. 10^3 and r by 10^-2 .. 10^2: every column keeps its own
    exponent (max_q |HS_qa| / sqrt(r_q)). The problem is then ill-conditioned (the largest
    eigenvalues of G near 10^8), so no FP64 evaluation agrees with another to 1e-10; the
    tensor-core form is held to the FP64 CUDA-core form's own distance from the oracle."""
    rng = np.random.default_rng(91)
    P = _random_local(95, N=64, nzones=60, m=800, radius=10.0)
    P["HSf"] = np.asfortranarray(P["HSf"] * (10.0 ** rng.uniform(-3, 3, 64))[None, :])
    P["r"] = 10.0 ** rng.uniform(-2, 2, P["r"].size)
    a = _call(oakg, P, False)
    b = _call(oakg, P, True)
    xa_o, Sa_o, _, nobs_o = _oracle(P)
    assert np.array_equal(a[3], nobs_o) and np.array_equal(b[3], nobs_o)
    inc = np.linalg.norm(xa_o - P["xf"])
    e_tc = max(rel_err(a[0], xa_o, inc), rel_err(a[1], Sa_o))
    e_cc = max(rel_err(b[0], xa_o, inc), rel_err(b[1], Sa_o))
    print(f"wide scales: tensor-core {e_tc:.2e}, CUDA-core {e_cc:.2e} from the oracle")
    assert e_tc <= max(REL, 30.0 * e_cc)


def test_every_observation_selected(oakg):
    P = _random_local(93, N=32, nzones=20, m=700)
    a, _ = _both_agree(oakg, P, localise=False)
    xa_o, Sa_o, _, _ = _oracle(P, localise=False)
    check_local(a[0], a[1], xa_o, Sa_o, P["xf"], REL)


def test_nan_row_marks_the_zones_that_select_it(oakg):
    P = _random_local(94, N=16, nzones=60, m=400, radius=6.0)
    P["HSf"] = np.array(P["HSf"])
    P["HSf"][17, 3] = np.nan
    codes = []
    for simt in (False, True):
        with pytest.raises(oakg.OakError) as ei:
            _call(oakg, P, simt)
        codes.append(ei.value.code)
    assert codes[0] == codes[1] and codes[0] in (oakg.ERR_NAN, oakg.ERR_EIG)


@pytest.mark.parametrize("N", [64, 23])
def test_transform_without_rotation(oakg, N):
    P = _random_local(96 + N, N=N, nzones=60, m=500)
    a, _ = _both_agree(oakg, P, rotate=False)
    xa_o, Sa_o, _, nobs_o = _oracle(P, rotate=False)
    assert np.array_equal(a[3], nobs_o)
    check_local(a[0], a[1], xa_o, Sa_o, P["xf"], REL)


def test_global_analysis_transform(oakg):
    """One zone (the global analysis): the transform's grid is a single CTA."""
    rng = np.random.default_rng(97)
    n, m, N = 300, 120, 40
    Sf = np.asfortranarray(rng.standard_normal((n, N)))
    HSf = np.asfortranarray(rng.standard_normal((m, N)))
    xf, Hxf, yo = rng.standard_normal(n), rng.standard_normal(m), rng.standard_normal(m)
    r = rng.uniform(0.5, 2.0, m)
    xa, Sa, ampl = oakg.analysis(xf, Hxf, yo, Sf, HSf, r)
    xa_o, Sa_o, ampl_o = cref.analysis(xf, Hxf, yo, Sf, HSf, r)
    check_local(xa, Sa, xa_o, Sa_o, xf, REL)
    assert rel_err(ampl, ampl_o) < REL
