"""NumPy restatement of OAK's local ensemble square-root analysis (test oracle).

This module is TEST INFRASTRUCTURE. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it, and only as the checker: the product path
(``oak_gb300`` + ``liboakg.so``) never calls into it.

Every function restates one routine of the reference (gher-uliege/OAK 1.7, Fortran), in the
reference's own argument order, with 0-based indices where the reference is 1-based.
Arrays follow the reference layout: state/observation vectors are 1-D, ensembles are
``(n, N)`` matrices (members are columns).

Pinned against the reference's own known-answer tests:
- ``test/test_rrsqrt.F90`` Kalman-formula identities and its SMWCovar cases,
  ``test/test_covariance.F90:612-617`` ``locfun`` values, ``test/assimtest2.F90`` identities
  and ``test/test_assim.F90``'s Kalman case, by ``tests/test_oracle_golden.py``;
- ``test/test_ndgrid.F90``'s linear-function checks for ``split`` / ``cinterp`` and the
  ``initPartition`` error cases, by ``tests/test_oracle_layout.py``.
"""
from __future__ import annotations

import math

import numpy as np

# Metric codes (assimilation.F90:108-112)
CARTESIAN = 0
SPHERICAL = 1
SPHERICAL_APPROX = 2

# Weight kinds: the reference Gaussian with cut-off (assimilation.F90:3756-3767) and the
# Gaspari-Cohn function (covariance.F90:645-667) as used by test/test_rrsqrt.F90:254-271.
GAUSS_CUTOFF = 0
GASPARI_COHN = 1

EARTH_RADIUS = 6378137.0  # m, assimilation.F90:3643
PI = 3.141592653589793238462643383279502884197


def locfun(r):
    """Gaspari-Cohn 5th-order piecewise rational function (covariance.F90:645-667)."""
    r = np.asarray(r, dtype=np.float64)
    out = np.zeros_like(r)
    a = r <= 1.0
    b = (r > 1.0) & (r <= 2.0)
    ra = r[a]
    out[a] = (((-ra / 4.0 + 1.0 / 2.0) * ra + 5.0 / 8.0) * ra - 5.0 / 3.0) * ra**2 + 1.0
    rb = r[b]
    out[b] = ((((rb / 12.0 - 1.0 / 2.0) * rb + 5.0 / 8.0) * rb + 5.0 / 3.0) * rb - 5.0) * rb \
        + 4.0 - 2.0 / (3.0 * rb)
    return out


def distance(x0, y0, x1, y1, metric):
    """Distance between p0 = (x0, y0) and p1 = (x1, y1) (assimilation.F90:3635-3672),
    elementwise with NumPy broadcasting."""
    x0 = np.asarray(x0, dtype=np.float64)
    y0 = np.asarray(y0, dtype=np.float64)
    x1 = np.asarray(x1, dtype=np.float64)
    y1 = np.asarray(y1, dtype=np.float64)
    if metric == CARTESIAN:
        dx = x1 - x0
        dy = y1 - y0
        return np.sqrt(dx * dx + dy * dy)
    if metric == SPHERICAL_APPROX:
        coeff = PI * EARTH_RADIUS / 180.0
        a = coeff * np.cos((y0 + y1) * (PI / 360.0)) * (x1 - x0)
        b = coeff * (y1 - y0)
        return np.sqrt(a * a + b * b)
    if metric == SPHERICAL:
        d2r = PI / 180.0
        a = y0 * d2r
        b = y1 * d2r
        c = (x1 - x0) * d2r
        coeff = np.sin(b) * np.sin(a) + np.cos(b) * np.cos(a) * np.cos(c)
        coeff = np.clip(coeff, -1.0, 1.0)
        return EARTH_RADIUS * np.arccos(coeff)
    raise ValueError(f"unsupported metric {metric}")


def select_observations(zone_pos, obs_pos, corr_len, max_len, metric=CARTESIAN,
                        loctype=1, kind=GAUSS_CUTOFF):
    """Per-zone observation selection (assimilation.F90:3683-3771).

    ``zone_pos`` = (x, y, z, t) of the zone's first element (assimilation.F90:3713-3740);
    ``obs_pos`` = (obsGridX, obsGridY, obsGridZ, obsGridT) arrays.
    Returns ``(weight, relevant)`` over all m observations.

    GAUSS_CUTOFF: relevant = d <= maxLength (:3756), weight = exp(-(d/L)^2) (:3767).
    GASPARI_COHN: weight = locfun(d/L) (covariance.F90:645), relevant = d <= maxLength and
    weight /= 0 (the selection rule of test/test_rrsqrt.F90:268-269).
    """
    if loctype == 1:
        # p0 = observation, p1 = zone position, as in assimilation.F90:3749
        d = distance(obs_pos[0], obs_pos[1], zone_pos[0], zone_pos[1], metric)
    elif loctype == 2:
        d = np.abs(np.asarray(obs_pos[2], dtype=np.float64) - zone_pos[2])
    else:
        d = np.abs(np.asarray(obs_pos[3], dtype=np.float64) - zone_pos[3])
    if kind == GAUSS_CUTOFF:
        relevant = d <= max_len
        if relevant.any():
            weight = np.exp(-((d / corr_len) ** 2))
        else:
            weight = d
    else:
        weight = locfun(d / corr_len)
        relevant = (d <= max_len) & (weight != 0)
    return weight, relevant


def perp_space(w):
    """n-1 orthonormal vectors perpendicular to w (matoper.F90:509-535, Hoteit et al. 2002)."""
    w = np.asarray(w, dtype=np.float64)
    n = w.size
    alpha = -1.0 / (abs(w[n - 1]) + 1.0)
    H = np.zeros((n, n - 1))
    H[: n - 1, :] = alpha * np.outer(w[: n - 1], w[: n - 1]) + np.eye(n - 1)
    sgn = 1.0 if w[n - 1] >= 0 else -1.0  # Fortran sign(1., x) with x = +0 or -0 -> +1 for +0
    if w[n - 1] == 0.0 and math.copysign(1.0, w[n - 1]) < 0:
        sgn = -1.0
    H[n - 1, :] = alpha * (w[n - 1] + sgn) * w[: n - 1]
    return H


def normate(v):
    """v / ||v|| (rrsqrt.F90:748-756)."""
    v = np.asarray(v, dtype=np.float64)
    return v / np.sqrt(np.sum(v**2))


def rotate_vector(w, v):
    """Orthogonal matrix Omega with Omega w = v (rrsqrt.F90:737-742)."""
    return np.outer(v, w) + perp_space(v) @ perp_space(w).T


def analysis_increment(Hxf, yo, Sf, HSf, rinv_eff, rotate=True):
    """Analysis increment and anomalies (rrsqrt.F90:100-190).

    ``rinv_eff`` is the diagonal of the (localised) inverse observation error covariance,
    i.e. ``R%mldivide`` for DiagCovar (covariance.F90:425-432) or DCDCovar with D = w
    (covariance.F90:612-619): ``w**2 / r``; or the full matrix of a non-diagonal one (SMWCovar).
    Returns ``(xa_xf, Sa, ampl)``.
    """
    HSf = np.asarray(HSf, dtype=np.float64)
    Sf = np.asarray(Sf, dtype=np.float64)
    N = Sf.shape[1]
    rinv_eff = np.asarray(rinv_eff, dtype=np.float64)
    mld = (lambda x: rinv_eff @ x) if rinv_eff.ndim == 2 else (
        lambda x: (rinv_eff[:, None] * x) if x.ndim == 2 else rinv_eff * x)
    temp = HSf.T @ mld(HSf)  # :135 (HSf .tx. R%mldivide(HSf))
    lam, U = np.linalg.eigh(temp, UPLO="L")  # :136 symeig -> dsyev('V','L')
    lam = np.where(lam < 0, 0.0, lam)  # :137
    lam = 1.0 / (1.0 + lam)  # :140
    ampl = U @ (lam * (U.T @ (HSf.T @ mld(yo - Hxf))))  # :142
    if np.any(ampl != ampl):  # :145-149
        raise FloatingPointError("NaN in analysis amplitudes")
    xa_xf = Sf @ ampl  # :151
    sqrt_lam = np.sqrt(lam)  # :162
    if rotate:  # ROTATE_ENSEMBLE (:24, :165-185)
        w = np.full(N, 1.0 / np.sqrt(1.0 * N))
        v = U @ (np.sum(U, axis=0) / sqrt_lam)
        v = normate(v)
        Sa = Sf @ (U @ (sqrt_lam[:, None] * (U.T @ rotate_vector(w, v))))
    else:
        Sa = Sf @ (U @ (sqrt_lam[:, None] * U.T))
    return xa_xf, Sa, ampl


def smw_rinv(C, B):
    """Inverse of the SMWCovar R = diag(C) + B B^T (covariance.F90:464-570) as its mldivide
    computes it: C^-1 - C^-1 B D B^T C^-1 with D = (B^T C^-1 B + I)^-1 (SMWCovar_init :475-483,
    SMWCovar_mldivide_vec :525-535)."""
    C = np.asarray(C, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    CiB = B / C[:, None]
    D = np.linalg.inv(B.T @ CiB + np.eye(B.shape[1]))
    return np.diag(1.0 / C) - CiB @ D @ CiB.T


def analysis(xf, Hxf, yo, Sf, HSf, r_diag, rotate=True, smw_B=None):
    """Global analysis with diagonal R (rrsqrt.F90:196-208), or R = diag(r_diag) + B B^T
    (SMWCovar) when ``smw_B`` is given. Returns ``(xa, Sa, ampl)``."""
    if smw_B is not None:
        xa_xf, Sa, ampl = analysis_increment(Hxf, yo, Sf, HSf, smw_rinv(r_diag, smw_B), rotate)
        return xf + xa_xf, Sa, ampl
    rinv = 1.0 / np.asarray(r_diag, dtype=np.float64)
    xa_xf, Sa, ampl = analysis_increment(Hxf, yo, Sf, HSf, rinv, rotate)
    return xf + xa_xf, Sa, ampl


def loc_analysis(zone_size, select, xf, Hxf, yo, Sf, HSf, r_diag, localise_obs=True,
                 rotate=True, smw_B=None):
    """Local analysis (rrsqrt.F90:258-466) with a selection callback.

    With ``smw_B`` (m x k) the observation error covariance is R = diag(r_diag) + B B^T
    (SMWCovar): the zone uses DCDCovar(w, R) (rrsqrt.F90:385-391) or, with observation
    localisation and not every observation relevant, DCDCovar(w_sel, R%pack(sel)) (:395,
    SMWCovar_pack covariance.F90:540-570: the Woodbury matrix of the packed rows).

    ``select(zi, start_index) -> (weight(m), relevant(m))`` plays the role of
    ``selectObservations`` (called with the zone's first state index, :368).
    Returns ``(xa, Sa, amplitudes(N, Z), nobs(Z))``. As in the reference, ``amplitudes`` is
    only filled in the non-localised branch (:375-384); zones without relevant
    observations keep ``xa_xf = 0`` and ``Sa = Sf`` (:322-326, :371).
    """
    xf = np.asarray(xf, dtype=np.float64)
    Sf = np.asarray(Sf, dtype=np.float64)
    HSf = np.asarray(HSf, dtype=np.float64)
    yo = np.asarray(yo, dtype=np.float64)
    Hxf = np.asarray(Hxf, dtype=np.float64)
    r_diag = np.asarray(r_diag, dtype=np.float64)
    m = yo.size
    N = Sf.shape[1]
    Z = len(zone_size)
    xa_xf = np.zeros_like(xf)
    Sa = Sf.copy()
    amplitudes = np.zeros((N, Z))
    nobs = np.zeros(Z, dtype=np.int64)
    ends = np.cumsum(zone_size)
    starts = ends - np.asarray(zone_size)
    for zi in range(Z):
        i1, i2 = int(starts[zi]), int(ends[zi])
        weight, relevant = select(zi, i1)
        nb = int(np.count_nonzero(relevant))
        nobs[zi] = nb
        if nb == 0:
            continue
        if smw_B is None:
            full_rinv = lambda: weight**2 / r_diag
            sel_rinv = lambda s: weight[s] ** 2 / r_diag[s]
        else:
            Bm = np.asarray(smw_B, dtype=np.float64)
            full_rinv = lambda: np.outer(weight, weight) * smw_rinv(r_diag, Bm)
            sel_rinv = lambda s: np.outer(weight[s], weight[s]) * smw_rinv(r_diag[s], Bm[s])
        if not localise_obs:
            dxa, dSa, ampl = analysis_increment(Hxf, yo, Sf[i1:i2], HSf, full_rinv(), rotate)
            amplitudes[:, zi] = ampl
        elif nb == m:
            dxa, dSa, _ = analysis_increment(Hxf, yo, Sf[i1:i2], HSf, full_rinv(), rotate)
        else:
            sel = np.nonzero(relevant)[0]
            dxa, dSa, _ = analysis_increment(Hxf[sel], yo[sel], Sf[i1:i2], HSf[sel],
                                             sel_rinv(sel), rotate)
        xa_xf[i1:i2] = dxa
        Sa[i1:i2] = dSa
    return xf + xa_xf, Sa, amplitudes, nobs


def geometric_selector(zone_pos, obs_pos, corr_len, max_len, metric=CARTESIAN, loctype=1,
                       kind=GAUSS_CUTOFF):
    """Selection callback built from zone/observation geometry, as the C ABI takes it.

    ``zone_pos`` is ``(Z, 4)``; ``corr_len``/``max_len`` are per-zone ``(Z,)`` arrays
    (hCorrLengthToObs / hMaxCorrLengthToObs at the zone's first element,
    assimilation.F90:3756-3767).
    """
    def select(zi, _start):
        return select_observations(zone_pos[zi], obs_pos, corr_len[zi], max_len[zi],
                                   metric, loctype, kind)
    return select


def ensemble_prologue(Ef, HEf):
    """Mean and scaled anomalies of an ensemble (assimilation.F90:3127-3134, ASSIM_SCALING=1).

    Returns ``(xf, Hxf, Sf, HSf)`` with ``Sf = (Ef - xf) / sqrt(N-1)``.
    """
    N = Ef.shape[1]
    scaling = math.sqrt(N - 1.0)
    xf = Ef.sum(axis=1) / N
    Hxf = HEf.sum(axis=1) / N
    Sf = (Ef - xf[:, None]) / scaling
    HSf = (HEf - Hxf[:, None]) / scaling
    return xf, Hxf, Sf, HSf


def ensemble_epilogue(xf, xa, Sa, inflation=1.0, max_correction=None):
    """Inflation, correction clip and ensemble reconstruction (assimilation.F90:3299-3312,
    3558-3565). Returns ``Ea``."""
    N = Sa.shape[1]
    if inflation != 1:
        Sa = inflation * Sa
    xa = xa.copy()
    if max_correction is not None:
        mc = np.asarray(max_correction, dtype=np.float64)
        xa = np.where(xa - mc > xf, xf + mc, xa)
        xa = np.where(xa < xf - mc, xf - mc, xa)
    return xa[:, None] + Sa * math.sqrt(N - 1.0)


def kalman_reference(xf, Sf, H, yo, R):
    """Explicit Kalman formulas of test/test_rrsqrt.F90:49-56 (the reference's check)."""
    Pf = Sf @ Sf.T
    K = (Pf @ H.T) @ np.linalg.inv(H @ Pf @ H.T + R)
    Pa = Pf - K @ (H @ Pf)
    xa = xf + K @ (yo - H @ xf)
    return xa, Pa


def ens2sqrt(E):
    """Mean and N - 1 anomaly columns of an ensemble (ens2sqrt, rrsqrt.F90:786-806, Pham 2001).

    Returns ``(mean, S)`` with ``S S^T`` the ensemble covariance.
    """
    E = np.asarray(E, dtype=np.float64)
    N = E.shape[1]
    mean = E.sum(axis=1) / N
    alpha = (-1.0 + math.sqrt(1.0 * N)) / (N - 1)
    shift = (1.0 - alpha) * mean + alpha * E[:, N - 1]
    S = (E[:, : N - 1] - shift[:, None]) / math.sqrt(N - 1.0)
    return mean, S


def sqrt2ens(mean, S, theta=None):
    """Ensemble with the given mean and covariance ``S S^T`` (sqrt2ens, rrsqrt.F90:815-839):
    ``E = mean + S Om^T``, ``Om = sqrt(N-1) perpSpace(w) theta``, ``w = 1/sqrt(N)``.

    The reference draws ``theta`` with ``randOrthMatrix(N-1)``; it is an argument here (the
    identity if None).
    """
    S = np.asarray(S, dtype=np.float64)
    K = S.shape[1]
    N = K + 1
    w = np.full(N, 1.0 / math.sqrt(1.0 * N))
    th = np.eye(K) if theta is None else np.asarray(theta, dtype=np.float64)
    Om = math.sqrt(N - 1.0) * (perp_space(w) @ th)
    return np.asarray(mean, dtype=np.float64)[:, None] + S @ Om.T


def ens_analysis(Ef, HEf, yo, r_diag, rotate=True):
    """Global analysis of an ensemble (ensAnalysis, rrsqrt.F90:613-671): mean and scaled
    anomalies of Ef and HEf, ``analysis``, ``Ea = xa + sqrt(N-1) Sa``.

    Returns ``(Ea, xa, amplitudes)``.
    """
    xf, Hxf, Sf, HSf = ensemble_prologue(np.asarray(Ef, dtype=np.float64),
                                         np.asarray(HEf, dtype=np.float64))
    xa, Sa, ampl = analysis(xf, Hxf, yo, Sf, HSf, r_diag, rotate)
    N = Sf.shape[1]
    return xa[:, None] + math.sqrt(N - 1.0) * Sa, xa, ampl


def sparse_apply(H_index, H_weight, x, shift=None):
    """``H x + shift`` for the operator given as K (index, weight) pairs per row (a negative
    index marks an unused pair): the SparseMatrix product of matoper_inc.F90:220-242."""
    idx = np.asarray(H_index)
    w = np.asarray(H_weight, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    y = np.where(idx >= 0, w * x[np.maximum(idx, 0)], 0.0).sum(axis=1)
    return y if shift is None else y + np.asarray(shift, dtype=np.float64)


def biased_loc_analysis(gamma, zone_size, select, H_index, H_weight, Hshift, xf, bf, Hxf, yo,
                        Sf, HSf, r_diag, localise_obs=True, rotate=True):
    """Bias-aware local analysis (biasedLocAnalysis, rrsqrt.F90:476-546).

    The bias increment is the local analysis increment of (Hxf, yo, Sf, HSf, R);
    ``ba = bf - gamma inc``; the unbiased forecast ``xf - ba`` is analysed with
    ``H (xf - ba) + Hshift`` and R scaled by (1 - gamma) (``DCDCovar`` with
    ``D = 1/sqrt(1 - gamma)``: ``mldivide(x) = D C^-1 (D x)``, covariance.F90:611-618);
    ``Sa = Sf``. Returns ``(xa, ba, Sa)``.
    """
    zeros = np.zeros_like(np.asarray(xf, dtype=np.float64))
    inc, _, _, _ = loc_analysis(zone_size, select, zeros, Hxf, yo, Sf, HSf, r_diag,
                                localise_obs, rotate)
    ba = np.asarray(bf, dtype=np.float64) - gamma * inc
    ux = np.asarray(xf, dtype=np.float64) - ba
    uHx = sparse_apply(H_index, H_weight, ux, Hshift)
    inc2, _, _, _ = loc_analysis(zone_size, select, zeros, uHx, yo, Sf, HSf,
                                 (1.0 - gamma) * np.asarray(r_diag, dtype=np.float64),
                                 localise_obs, rotate)
    return ux + inc2, ba, np.asarray(Sf, dtype=np.float64).copy()


# ---------------------------------------------------------------------------- layout builders

def init_partition(partition):
    """initPartition (assimilation.F90:578-641): zone sizes, zoneIndex and invZoneIndex of a
    partition vector of 1-based zone numbers (indices 0-based here). Counting pass, start
    offsets, then every element appended to its zone in element order. Raises ValueError where
    the reference stops (a zone number < 1, an empty zone)."""
    p = np.asarray(partition, dtype=np.int64).reshape(-1)
    if p.size and p.min() < 1:
        raise ValueError("partition values must be >= 1")
    nz = int(p.max()) if p.size else 0
    size = np.bincount(p - 1, minlength=nz).astype(np.int32)
    if (size == 0).any():
        raise ValueError("empty zone")
    start = np.concatenate([[0], np.cumsum(size)[:-1]])
    cur = start.copy()
    zone_index = np.empty(p.size, dtype=np.int32)
    inv = np.empty(p.size, dtype=np.int32)
    for j, zi in enumerate(p - 1):
        zone_index[cur[zi]] = j
        inv[j] = cur[zi]
        cur[zi] += 1
    return size, zone_index, inv


def sea_index(mask):
    """Sea packing of a flat mask: running count of the unmasked points, -1 on masked ones."""
    mk = np.asarray(mask).reshape(-1) != 0
    sea = np.cumsum(~mk) - 1
    sea[mk] = -1
    return sea.astype(np.int64), int((~mk).sum())


def split(n):
    """split (ndgrid.F90:357-435) called as in initgrid (:892): the simplices of the n-cube.
    Returns T (nbth, n+1, 2^n): vertex v of simplex l as shares of the cube corners (corner c:
    bit k set = upper side of axis k), nbth = n! 2^(n-1)."""
    K = 1 << n
    nbth = math.factorial(n) << (n - 1)
    T = np.zeros((nbth, n + 1, K))

    def rec(subn, fixed, sel, l0):
        if subn == 1:
            T[l0, 0:2, :] = 0.0
            j = 0
            for c in range(K):
                if sel[c]:
                    T[l0, j, c] = 1.0
                    j += 1
            return
        nb = math.factorial(subn) << (subn - 1)
        sub_nb = math.factorial(subn - 1) << (subn - 2)
        cnt = sum(sel)
        for l in range(l0, l0 + nb):
            T[l, subn, :] = [1.0 / cnt if s else 0.0 for s in sel]
        m = l0
        for i in range(n):
            if fixed[i]:
                continue
            fd = list(fixed)
            fd[i] = True
            for j in (0, 1):
                sub = [sel[c] and (((c >> i) & 1) == j) for c in range(K)]
                rec(subn - 1, fd, sub, m)
                m += sub_nb

    rec(n, [False] * n, [True] * K, 0)
    return T


def interp_tetrahedron(X, xi, tol=1e-8):
    """interp_tetrahedron (ndgrid.F90:464-629), non-degenerate branch: barycentric
    coordinates c of xi in the simplex X (n, n+1) from [1; X - xc] c = [1; xi - xc] (xc the
    vertex mean). Returns (out, c, det); det <= tol in magnitude marks the degenerate case
    (the reference's SVD branch, not restated)."""
    n = X.shape[0]
    xc = X.mean(axis=1)
    M = np.ones((n + 1, n + 1))
    M[1:, :] = X - xc[:, None]
    d = np.ones(n + 1)
    d[1:] = np.asarray(xi) - xc
    det = np.linalg.det(M)
    if not abs(det) > tol:
        return True, None, det
    c = np.linalg.solve(M, d)
    out = not bool(np.all((c >= -tol) & (c <= 1 + tol)))
    return out, c, det


def cinterp_rectilinear(axes, xi, sea=None, T=None):
    """cinterp (ndgrid.F90:1183-1257) on a rectilinear grid: the cell [c(i), c(i+1)] of every
    axis holding xi (the largest i <= len - 2 with c(i) on the lower side; axes ascending or
    descending), its 2^n corners (Fortran-order linear index, then the sea packing), out if one
    is masked, else interp_cube (:636-665): the first simplex of split(n) accepting xi.
    Returns (status, corner indices (2^n), weights (2^n)); status 'in', 'out' or
    'degenerate'."""
    n = len(axes)
    K = 1 << n
    if T is None:
        T = split(n)
    lo = []
    for k, c in enumerate(axes):
        c = np.asarray(c, dtype=np.float64)
        x = xi[k]
        asc = c[-1] > c[0]
        if not (min(c[0], c[-1]) <= x <= max(c[0], c[-1])):
            return "out", None, None
        i, hi = 0, len(c) - 1
        while hi - i > 1:
            mid = (i + hi) // 2
            if (c[mid] <= x) if asc else (c[mid] >= x):
                i = mid
            else:
                hi = mid
        lo.append(i)
    shape = [len(c) for c in axes]
    stride = np.cumprod([1] + shape[:-1])
    px = np.zeros((n, K))
    idx = np.zeros(K, dtype=np.int64)
    for cc in range(K):
        lin = 0
        for k in range(n):
            ik = lo[k] + ((cc >> k) & 1)
            lin += ik * stride[k]
            px[k, cc] = axes[k][ik]
        idx[cc] = lin if sea is None else sea[lin]
    if sea is not None and (idx < 0).any():
        return "out", None, None
    for l in range(T.shape[0]):
        out, c, det = interp_tetrahedron(px @ T[l].T, xi)
        if c is None:
            return "degenerate", None, None
        if not out:
            return "in", idx, T[l].T @ c
    return "out", None, None


def obsoper_rectilinear(axes, obs_pos, sea=None, offset=0):
    """genObservationOper (assimilation.F90:2471-2656) for one variable on a rectilinear grid,
    in the fixed-width row form: (index (m, 2^n), weight (m, 2^n)), index = offset + packed
    corner index, -1 and weight 0 for an observation outside the grid or next to a masked
    point, -2 in a degenerate cell."""
    n = len(axes)
    K = 1 << n
    T = split(n)
    pos = [np.asarray(p, dtype=np.float64).reshape(-1) for p in obs_pos]
    m = pos[0].size
    index = np.full((m, K), -1, dtype=np.int64)
    weight = np.zeros((m, K))
    for j in range(m):
        st, idx, w = cinterp_rectilinear(axes, [p[j] for p in pos], sea, T)
        if st == "in":
            index[j] = offset + idx
            weight[j] = w
        elif st == "degenerate":
            index[j] = -2
    return index, weight


def partition_compact(labels):
    """globalInit's zone numbering (assimilation.F90:416-424): unique(..., ind2 = partition)
    (matoper.F90:1821-1882), every label replaced by its 1-based rank among the distinct labels
    in ascending order. Returns (partition, number of distinct labels)."""
    lab = np.asarray(labels).reshape(-1)
    u, inv = np.unique(lab, return_inverse=True)
    return (inv + 1).astype(np.int32), int(u.size)
