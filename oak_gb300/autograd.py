"""torch.autograd.Function over the local analysis mean.

    xa = LocAnalysisMean.apply(yo, r_diag, kappa, inflation, problem)

The forward runs oakg_locanalysis (FP64) on the anomalies ``inflation * Sf`` and
``inflation * HSf`` with localisation lengths ``kappa * corr_len`` and ``kappa * max_len``; the
backward runs oakg_locanalysis_adjoint and returns dJ/dyo, dJ/dr_diag, dJ/dkappa and
dJ/dinflation for the incoming dJ/dxa. ``problem`` holds the remaining (constant) inputs:
zone_size, xf, Hxf, Sf, HSf, zone_pos, obs_pos, corr_len, max_len and the loc options.
All tensors are float64, on the CPU (the library copies to and from the GPU) or on a CUDA
device (used in place).
"""
from __future__ import annotations

import torch

import oak_gb300 as oak


def _np_or_tensor(t: torch.Tensor):
    return t if t.is_cuda else t.detach().numpy()


def _wrap(a, like: torch.Tensor) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a
    return torch.as_tensor(a, dtype=like.dtype, device=like.device)


class LocAnalysisMean(torch.autograd.Function):
    @staticmethod
    def forward(ctx, yo, r_diag, kappa, inflation, problem):
        p = problem
        k = float(kappa)
        s = float(inflation)
        Sf = p["Sf"] * s
        HSf = p["HSf"] * s
        corr = p["corr_len"] * k
        maxl = p["max_len"] * k
        opts = p.get("opts", {})
        xa, _, _, _ = oak.loc_analysis(
            _np_or_tensor(p["zone_size"]), _np_or_tensor(p["xf"]), _np_or_tensor(p["Hxf"]),
            _np_or_tensor(yo.detach()), _np_or_tensor(Sf), _np_or_tensor(HSf),
            _np_or_tensor(r_diag.detach()), _np_or_tensor(p["zone_pos"]),
            tuple(_np_or_tensor(c) for c in p["obs_pos"]), _np_or_tensor(corr),
            _np_or_tensor(maxl), want_sa=False, want_ampl=False, **opts)
        ctx.problem = p
        ctx.kappa = k
        ctx.inflation = s
        ctx.save_for_backward(yo.detach(), r_diag.detach())
        return _wrap(xa, yo)

    @staticmethod
    def backward(ctx, gxa):
        yo, r_diag = ctx.saved_tensors
        p = ctx.problem
        k = ctx.kappa
        opts = {kk: v for kk, v in p.get("opts", {}).items()
                if kk in ("weight", "metric", "loctype", "localise_obs", "brute_search",
                          "cell_size")}
        seed = gxa.contiguous()
        dyo, dr, dlen, dinfl = oak.loc_analysis_adjoint(
            _np_or_tensor(p["zone_size"]), _np_or_tensor(p["Hxf"]), _np_or_tensor(yo),
            _np_or_tensor(p["Sf"]), _np_or_tensor(p["HSf"]), _np_or_tensor(r_diag),
            _np_or_tensor(p["zone_pos"]), tuple(_np_or_tensor(c) for c in p["obs_pos"]),
            _np_or_tensor(p["corr_len"] * k), _np_or_tensor(p["max_len"] * k),
            _np_or_tensor(seed), inflation=ctx.inflation, **opts)
        # lengths are kappa * L0: dJ/dkappa = (dJ/d factor on kappa * L0 at 1) / kappa
        dk = torch.tensor(dlen / k, dtype=gxa.dtype, device=gxa.device)
        ds = torch.tensor(dinfl, dtype=gxa.dtype, device=gxa.device)
        return _wrap(dyo, gxa), _wrap(dr, gxa), dk, ds, None
