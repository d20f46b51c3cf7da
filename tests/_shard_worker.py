"""Rank bodies for the zone-sharding tests (imported by spawned gloo processes).

The per-rank analysis is the oracle (CPU); what is under test is the host logic of
oak_gb300.shard: the partition, the partial observation operator and its all-reduce, the
per-rank slicing, and failure propagation between ranks."""
import os
import traceback
from datetime import timedelta

import numpy as np


def problem(seed=7):
    from oak_gb300.workloads import local_case
    c = local_case(scale=1 / 12, N=16)
    rng = np.random.default_rng(seed)
    m = c.m
    # two non-zeros per observation (the observed level and the one below it, weights 0.7 /
    # 0.3), so that observations near a range boundary draw on two processes' rows
    idx2 = np.where(c.obs_index % 20 > 0, c.obs_index - 1, c.obs_index + 1)
    index = np.stack([c.obs_index, idx2], axis=1).astype(np.int64)
    weight = np.tile(np.array([0.7, 0.3]), (m, 1))
    Hxf = (weight * c.xf[index]).sum(1)
    HSf = np.asfortranarray((weight[:, :, None] * c.Sf[index]).sum(1))
    yo = Hxf + 0.1 * rng.standard_normal(m)
    return c, index, weight, Hxf, HSf, yo


def oracle_analysis(zone_size, xf, Hxf, yo, Sf, HSf, r_diag, zone_pos, obs_pos, corr_len,
                    max_len, **opts):
    from oracle import cref
    a = lambda t: t.detach().cpu().numpy() if hasattr(t, "detach") else np.asarray(t)
    return cref.locanalysis(a(zone_size), a(xf), a(Hxf), a(yo), np.asfortranarray(a(Sf)),
                            np.asfortranarray(a(HSf)), a(r_diag), a(zone_pos),
                            tuple(a(x) for x in obs_pos), a(corr_len), a(max_len),
                            kind=opts.get("weight", 1), metric=opts.get("metric", 0),
                            loctype=opts.get("loctype", 1), nthreads=2)


def run_rank(rank, world, port, mode, queue):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    try:
        import torch
        import torch.distributed as dist
        from oak_gb300 import shard
        dist.init_process_group("gloo", rank=rank, world_size=world,
                                timeout=timedelta(seconds=6))
        c, index, weight, Hxf, HSf, yo = problem()
        # costs from the relevant-observation counts of a previous analysis (here: the oracle)
        _, _, _, nobs = oracle_analysis(c.zone_size, c.xf, Hxf, yo, c.Sf, HSf, c.r_diag,
                                        c.zone_pos, c.obs_pos, c.corr_len, c.max_len)
        bounds = shard.partition(shard.zone_cost(c.zone_size, nobs, c.N), world)
        rows = shard.zone_rows(c.zone_size)
        r0, r1 = rows[bounds[rank]], rows[bounds[rank + 1]]
        T = torch.as_tensor
        if mode == "fail" and rank == world - 1:
            raise RuntimeError("rank failed before the exchange")
        xa, Sa, _, nobs_l = shard.sharded_loc_analysis(
            T(c.zone_size), T(c.zone_pos), T(c.corr_len), T(c.max_len), bounds,
            T(c.xf[r0:r1]), T(np.ascontiguousarray(c.Sf[r0:r1])), T(index), T(weight), T(yo),
            T(c.r_diag), tuple(T(x) for x in c.obs_pos), analysis=oracle_analysis, weight=1)
        queue.put((rank, "ok", (int(r0), int(r1), xa, Sa, nobs_l, bounds)))
        dist.destroy_process_group()
    except Exception as exc:  # reported to the parent, which decides what is expected
        queue.put((rank, "error", f"{type(exc).__name__}: {exc}\n{traceback.format_exc()}"))
