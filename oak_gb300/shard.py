"""Zone-sharded local analysis over several processes, one GPU each.

The zone loop of locAnalysisIncrement (rrsqrt.F90:357-424) has no dependency between zones once
every zone can see the observations, so the path shards by contiguous zone ranges:

* ``partition`` splits the zones into contiguous ranges of nearly equal cost, the role of
  parallPartion (parall.F90:166-186), with the cost of a zone taken from its work on this path
  (p N^2 for the Gram plus 9 N^3 for the eigensolve when it has observations, a copy of nz N
  values otherwise) instead of a processor speed.
* Each process owns the state rows of its zones. The observed ensemble is the only exchange:
  every process applies the observation operator to its own rows and the partial H x_f and
  H S_f are summed over the processes (the partial H E allreduce of assimilation.F90:2881-2894).
* Each process then analyses its own zones with every observation; there is no exchange after.

The observation operator is the reference's sparse interpolation (H(m, n) with a few non-zeros
per observation: nearest cell, bilinear, ...), given as (index, weight) arrays of shape (m, K).

Everything here is host orchestration over ``torch.distributed`` (NCCL between GPUs, gloo in the
CPU tests); the analysis itself is ``oak_gb300.loc_analysis`` unless another callable with the
same signature is given.
"""
from __future__ import annotations

import numpy as np


def zone_cost(zone_size, nobs, N):
    """Work of each zone on this path (flop-like units)."""
    zone_size = np.asarray(zone_size, dtype=np.float64)
    nobs = np.asarray(nobs, dtype=np.float64)
    return np.where(nobs > 0, nobs * N * N + 9.0 * N ** 3, zone_size * N)


def partition(cost, world):
    """Contiguous zone ranges of nearly equal total cost.

    Returns ``bounds`` (world + 1,): process r owns zones [bounds[r], bounds[r+1]). Boundary r
    is the first zone whose cost prefix reaches r/world of the total, so every range is
    within one zone's cost of its share.
    """
    cost = np.asarray(cost, dtype=np.float64)
    Z = cost.size
    if world < 1:
        raise ValueError("world must be >= 1")
    if Z == 0:
        return np.zeros(world + 1, dtype=np.int64)
    prefix = np.concatenate([[0.0], np.cumsum(cost)])
    total = prefix[-1]
    bounds = np.empty(world + 1, dtype=np.int64)
    bounds[0], bounds[world] = 0, Z
    for r in range(1, world):
        bounds[r] = np.searchsorted(prefix, total * r / world, side="left")
    return np.maximum.accumulate(np.clip(bounds, 0, Z))


def zone_rows(zone_size):
    """First state row of every zone, and the total (n)."""
    zs = np.asarray(zone_size, dtype=np.int64)
    return np.concatenate([[0], np.cumsum(zs)])


def partial_observed(obs_index, obs_weight, row0, row1, xf_local, Sf_local):
    """This process's share of H x_f and H S_f (rows [row0, row1) of the state).

    ``obs_index``/``obs_weight``: (m, K) torch tensors on the same device as the state;
    ``xf_local`` (row1 - row0,), ``Sf_local`` (row1 - row0, N). Returns (Hxf_part (m,),
    HSf_part (m, N)), zero where no non-zero of an observation falls in these rows.
    """
    import torch
    own = (obs_index >= row0) & (obs_index < row1)
    local = torch.where(own, obs_index - row0, torch.zeros_like(obs_index))
    w = torch.where(own, obs_weight, torch.zeros_like(obs_weight))
    Hx = (w * xf_local[local]).sum(dim=1)
    HS = (w.unsqueeze(-1) * Sf_local[local]).sum(dim=1)
    return Hx, HS


def sharded_loc_analysis(zone_size, zone_pos, corr_len, max_len, bounds, xf_local, Sf_local,
                         obs_index, obs_weight, yo, r_diag, obs_pos, *, group=None,
                         analysis=None, **opts):
    """Local analysis of this process's zones.

    ``zone_size``, ``zone_pos``, ``corr_len``, ``max_len`` describe all Z zones (host or
    device); ``bounds`` comes from :func:`partition`; ``xf_local`` / ``Sf_local`` are the state
    rows of this process's zones. The observed ensemble is summed over the group (one
    all-reduce of m (N + 1) values), then ``analysis`` (default ``oak_gb300.loc_analysis``) runs
    on the local zones. Returns ``(xa_local, Sa_local, ampl_local, nobs_local)``.
    """
    import torch
    import torch.distributed as dist
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    if len(bounds) != world + 1:
        raise ValueError(f"bounds has {len(bounds)} entries for {world} processes")
    z0, z1 = int(bounds[rank]), int(bounds[rank + 1])
    zs_host = np.asarray(zone_size.cpu() if hasattr(zone_size, "cpu") else zone_size)
    rows = zone_rows(zs_host)
    row0, row1 = int(rows[z0]), int(rows[z1])
    if xf_local.shape[0] != row1 - row0 or Sf_local.shape[0] != row1 - row0:
        raise ValueError(f"process {rank} owns rows [{row0}, {row1}) but was given "
                         f"{xf_local.shape[0]} rows")
    Hx, HS = partial_observed(obs_index, obs_weight, row0, row1, xf_local, Sf_local)
    N = Sf_local.shape[1]
    m = Hx.shape[0]
    buf = torch.cat([Hx.reshape(m, 1), HS], dim=1).contiguous()
    if world > 1:
        dist.all_reduce(buf, group=group)
    Hxf = buf[:, 0].contiguous()
    HSf = buf[:, 1:].t().contiguous().t()  # column-major (m, N), as the reference stores it
    if analysis is None:
        from . import loc_analysis as analysis
    return analysis(zone_size[z0:z1], xf_local, Hxf, yo, Sf_local, HSf, r_diag,
                    zone_pos[z0:z1], obs_pos, corr_len[z0:z1], max_len[z0:z1], **opts)
