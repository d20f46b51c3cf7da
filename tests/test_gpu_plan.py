"""Prepared local analyses (oakg_plan_locanalysis / oakg_plan_execute): the CUDA-graph replay
equals a direct oakg_locanalysis call, follows in-place updates of the bound tensors
(observation values and positions, including positions outside the grid the plan was built
on), and the tuned plan gives the same analysis."""
import numpy as np
import pytest

from oak_gb300.workloads import local_case

pytestmark = pytest.mark.gpu


def _dev(c):
    import torch
    dev = torch.device("cuda", 0)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device=dev).t()
    return dict(zone_size=T(c.zone_size), xf=T(c.xf), Hxf=T(c.Hxf), yo=T(c.yo), Sf=F(c.Sf),
                HSf=F(c.HSf), r_diag=T(c.r_diag), zone_pos=T(c.zone_pos),
                obs_pos=tuple(T(x) for x in c.obs_pos), corr_len=T(c.corr_len),
                max_len=T(c.max_len))


def _direct(oakg, d, **kw):
    xa, Sa, _, nobs = oakg.loc_analysis(d["zone_size"], d["xf"], d["Hxf"], d["yo"], d["Sf"],
                                        d["HSf"], d["r_diag"], d["zone_pos"], d["obs_pos"],
                                        d["corr_len"], d["max_len"], want_ampl=False, **kw)
    return xa.cpu().numpy(), Sa.cpu().numpy(), nobs.cpu().numpy()


def _plan(oakg, d, **kw):
    return oakg.Plan(d["zone_size"], d["xf"], d["Hxf"], d["yo"], d["Sf"], d["HSf"], d["r_diag"],
                     d["zone_pos"], d["obs_pos"], d["corr_len"], d["max_len"], **kw)


@pytest.mark.parametrize("precision", [0, 1])
def test_plan_replay_equals_direct_call(oakg, precision):
    c = local_case(scale=1 / 8, N=32)
    d = _dev(c)
    kw = dict(weight=c.weight, precision=precision)
    ref = _direct(oakg, d, **kw)
    pl = _plan(oakg, d, **kw)
    assert pl.info["graph_nodes"] > 5
    for _ in range(2):
        xa, Sa, nobs = (t.cpu().numpy() for t in pl.execute())
        assert np.array_equal(nobs, ref[2])
        assert np.array_equal(xa, ref[0]) and np.array_equal(Sa, ref[1])
    pl.close()


def test_plan_follows_in_place_updates(oakg):
    import torch
    c = local_case(scale=1 / 8, N=24)
    d = _dev(c)
    kw = dict(weight=c.weight)
    pl = _plan(oakg, d, **kw)
    # new observation values
    d["yo"].add_(0.05 * torch.randn_like(d["yo"]))
    xa, Sa, nobs = (t.cpu().numpy() for t in pl.execute())
    ref = _direct(oakg, d, **kw)
    assert np.array_equal(nobs, ref[2])
    assert np.array_equal(xa, ref[0]) and np.array_equal(Sa, ref[1])
    # observations moved, some beyond the grid the plan was built on (they fall in its edge
    # cells); the direct call bins on a grid fitted to the new positions
    ox, oy = d["obs_pos"][0], d["obs_pos"][1]
    k = ox.numel()
    ox[: k // 10].add_(7.5)
    oy[k // 10: k // 5].sub_(9.0)
    xa, Sa, nobs = (t.cpu().numpy() for t in pl.execute())
    ref = _direct(oakg, d, **kw)
    assert np.array_equal(nobs, ref[2])
    assert np.linalg.norm(xa - ref[0]) <= 1e-10 * np.linalg.norm(ref[0] - c.xf)
    assert np.linalg.norm(Sa - ref[1]) <= 1e-10 * np.linalg.norm(ref[1])
    pl.close()


def test_tuned_plan(oakg):
    c = local_case(scale=1 / 8, N=32)
    d = _dev(c)
    kw = dict(weight=c.weight, precision=1)
    ref = _direct(oakg, d, **kw)
    pl = _plan(oakg, d, tune=True, **kw)
    info = pl.info
    assert len(info["tuning"]) == 5
    assert info["cell_size"] == min(info["tuning"], key=lambda t: t[1])[0]
    # the zone schedule is the faster of the two measured orders
    t = info["zone_order_ms"]
    assert t["index"] > 0 and t["count"] > 0
    assert info["zone_order"] == ("descending observation count" if t["count"] < t["index"]
                                  else "index")
    xa, Sa, nobs = (t.cpu().numpy() for t in pl.execute())
    assert np.array_equal(nobs, ref[2])
    # another cell edge changes the order of the FP32 Gram sums only
    assert np.linalg.norm(xa - ref[0]) <= 1e-5 * np.linalg.norm(ref[0] - c.xf)
    assert np.linalg.norm(Sa - ref[1]) <= 1e-5 * np.linalg.norm(ref[1])
    pl.close()


def test_tuned_plan_fp64(oakg):
    """The tuned FP64 plan (edge and zone schedule chosen on the data) against the direct
    call: selection identical, products summed in another order only."""
    c = local_case(scale=1 / 8, N=24)
    d = _dev(c)
    kw = dict(weight=c.weight, precision=0)
    ref = _direct(oakg, d, **kw)
    pl = _plan(oakg, d, tune=True, **kw)
    assert pl.info["zone_order"] in ("index", "descending observation count")
    xa, Sa, nobs = (t.cpu().numpy() for t in pl.execute())
    assert np.array_equal(nobs, ref[2])
    assert np.linalg.norm(xa - ref[0]) <= 1e-12 * np.linalg.norm(ref[0] - c.xf)
    assert np.linalg.norm(Sa - ref[1]) <= 1e-12 * np.linalg.norm(ref[1])
    pl.close()


def test_plan_needs_device_tensors(oakg):
    c = local_case(scale=1 / 12, N=8)
    with pytest.raises(oakg.OakError):
        oakg.Plan(c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag, c.zone_pos, c.obs_pos,
                  c.corr_len, c.max_len)
