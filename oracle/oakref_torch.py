"""Differentiable torch (FP64, CPU) restatement of the local analysis mean -- TEST
INFRASTRUCTURE, the reference gradient for the adjoint kernels.

Per zone (rrsqrt.F90:100-190, :258-466; selection assimilation.F90:3683-3771):
    xa_z = xf_z + s Sf_z (I + s^2 G)^-1 s g,  G = HS^T diag(c) HS,  g = HS^T diag(c) (yo - Hxf),
    c = w^2 / r,  w = exp(-(d/(kappa L))^2) (Gaussian) or locfun(d/(kappa L)) (Gaspari-Cohn).
The mean equals the reference's U diag(1/(1+max(lambda,0))) U^T g form up to rounding. The
selected observation set is computed once at kappa = 1 with the NumPy oracle and held fixed.
Autograd gives dJ/dyo, dJ/dr, dJ/dkappa and dJ/ds for any scalar J(xa).
"""
from __future__ import annotations

import numpy as np
import torch

from . import oakref


def _locfun_t(r):
    r1 = (((-r / 4.0 + 0.5) * r + 5.0 / 8.0) * r - 5.0 / 3.0) * r * r + 1.0
    # the 1 < r <= 2 branch is evaluated at a safe argument elsewhere: torch.where passes the
    # gradient through both branches, and 2/(3r) at r = 0 (an observation at the zone's own
    # position) would make it NaN
    rs = torch.where(r > 1.0, r, torch.ones_like(r))
    r2 = ((((rs / 12.0 - 0.5) * rs + 5.0 / 8.0) * rs + 5.0 / 3.0) * rs - 5.0) * rs + 4.0 \
        - 2.0 / (3.0 * rs)
    return torch.where(r <= 1.0, r1, torch.where(r <= 2.0, r2, torch.zeros_like(r)))


def selections(zone_pos, obs_pos, corr_len, max_len, metric=0, loctype=1, kind=0,
               localise=True):
    """Per zone: (indices, distances) of the selected observations (NumPy oracle rules)."""
    out = []
    for z in range(len(corr_len)):
        w, rel = oakref.select_observations(zone_pos[z], obs_pos, corr_len[z], max_len[z], metric,
                                            loctype, kind)
        if not rel.any():
            out.append((np.zeros(0, dtype=np.int64), np.zeros(0)))
            continue
        idx = np.nonzero(rel)[0] if localise else np.arange(len(w))
        if loctype == 1:
            d = oakref.distance(obs_pos[0][idx], obs_pos[1][idx], zone_pos[z][0], zone_pos[z][1],
                                metric)
        else:
            k = 2 if loctype == 2 else 3
            d = np.abs(np.asarray(obs_pos[k])[idx] - zone_pos[z][k])
        out.append((idx, np.asarray(d, dtype=np.float64)))
    return out


def loc_analysis_mean(zone_size, xf, Hxf, Sf, HSf, corr_len, sels, yo, r_diag, kappa, s,
                      kind=0):
    """xa (torch, FP64) as a differentiable function of yo, r_diag, kappa, s."""
    xf = torch.as_tensor(xf, dtype=torch.float64)
    Hxf = torch.as_tensor(Hxf, dtype=torch.float64)
    Sf = torch.as_tensor(np.asarray(Sf), dtype=torch.float64)
    HSf = torch.as_tensor(np.asarray(HSf), dtype=torch.float64)
    N = Sf.shape[1]
    eye = torch.eye(N, dtype=torch.float64)
    out = []
    start = 0
    for z, nz in enumerate(np.asarray(zone_size)):
        rows = slice(start, start + int(nz))
        start += int(nz)
        idx, d = sels[z]
        if idx.size == 0:
            out.append(xf[rows])
            continue
        t = torch.as_tensor(d) / (kappa * float(corr_len[z]))
        w = torch.exp(-t * t) if kind == 0 else _locfun_t(t)
        it = torch.as_tensor(idx)
        c = w * w / r_diag[it]
        H = HSf[it] * s
        G = H.T @ (c[:, None] * H)
        g = H.T @ (c * (yo[it] - Hxf[it]))
        ampl = torch.linalg.solve(eye + G, g)
        out.append(xf[rows] + (Sf[rows] * s) @ ampl)
    return torch.cat(out)
