"""Zone sharding across processes (oak_gb300.shard) on CPU with gloo, world size 2.

Sharded == monolithic (the partitioned-equals-serial check of matlab/test_oakassim_local.m,
restated for zone ranges), the cost partition, the partial observation operator, and a rank
that fails between steps: the surviving rank's exchange ends with an error within the
process-group timeout instead of hanging.
"""
import multiprocessing as mp
import socket
import time

import numpy as np
import pytest

import _shard_worker as W
from oak_gb300 import shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _launch(world, mode, timeout=120):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=W.run_rank, args=(r, world, port, mode, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    t0 = time.time()
    while len(out) < world and time.time() - t0 < timeout:
        try:
            rank, status, payload = q.get(timeout=1.0)
            out[rank] = (status, payload)
        except Exception:
            if all(not p.is_alive() for p in procs) and q.empty():
                break
    for p in procs:
        p.join(timeout=10)
        if p.is_alive():
            p.kill()
    return out, time.time() - t0


def test_partition_contiguous_and_balanced():
    rng = np.random.default_rng(1)
    cost = rng.gamma(2.0, 1.0, 1000)
    for world in (1, 2, 3, 8):
        b = shard.partition(cost, world)
        assert b[0] == 0 and b[-1] == cost.size and np.all(np.diff(b) >= 0)
        share = cost.sum() / world
        parts = np.array([cost[b[r]:b[r + 1]].sum() for r in range(world)])
        assert np.all(np.abs(parts - share) <= cost.max() + 1e-9)
    assert np.array_equal(shard.partition(np.zeros(0), 2), [0, 0, 0])


def test_partial_observed_sums_to_full():
    import torch
    c, index, weight, Hxf, HSf, yo = W.problem()
    rows = shard.zone_rows(c.zone_size)
    cut = int(rows[c.zone_size.size // 3])
    T = torch.as_tensor
    parts = [shard.partial_observed(T(index), T(weight), a, b, T(c.xf[a:b]),
                                    T(np.ascontiguousarray(c.Sf[a:b])))
             for a, b in ((0, cut), (cut, c.n))]
    assert np.allclose(sum(p[0] for p in parts).numpy(), Hxf, rtol=0, atol=1e-13)
    assert np.allclose(sum(p[1] for p in parts).numpy(), HSf, rtol=0, atol=1e-13)


def test_sharded_equals_monolithic():
    out, _ = _launch(2, "ok")
    assert set(out) == {0, 1}, out
    for r in (0, 1):
        assert out[r][0] == "ok", out[r][1]
    c, index, weight, Hxf, HSf, yo = W.problem()
    xa_m, Sa_m, _, nobs_m = W.oracle_analysis(c.zone_size, c.xf, Hxf, yo, c.Sf, HSf, c.r_diag,
                                              c.zone_pos, c.obs_pos, c.corr_len, c.max_len)
    xa = np.empty(c.n)
    Sa = np.empty((c.n, c.N))
    covered = np.zeros(c.n, bool)
    for r in (0, 1):
        r0, r1, xa_r, Sa_r, nobs_r, bounds = out[r][1]
        xa[r0:r1], Sa[r0:r1], covered[r0:r1] = xa_r, Sa_r, True
        assert np.array_equal(nobs_r, nobs_m[bounds[r]:bounds[r + 1]])
    assert covered.all()
    assert np.linalg.norm(xa - xa_m) <= 1e-12 * np.linalg.norm(xa_m - c.xf)
    assert np.linalg.norm(Sa - Sa_m) <= 1e-12 * np.linalg.norm(Sa_m)


def test_failed_rank_is_detected_by_the_other():
    out, elapsed = _launch(2, "fail", timeout=90)
    assert out[1][0] == "error" and "failed before the exchange" in out[1][1]
    # the surviving rank leaves its all-reduce with an error (peer gone or timeout), not a hang
    assert out[0][0] == "error", out[0]
    assert elapsed < 90
