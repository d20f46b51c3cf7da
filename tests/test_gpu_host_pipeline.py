"""Host-memory calls large enough to be split into chunks (the Sa / xa rows of a chunk copied
out while the next chunk computes) give the device-memory call's results bit for bit, for both
forms, with and without the amplitudes."""
import numpy as np
import pytest

from oak_gb300.workloads import local_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_chunked_host_call_equals_device_call(oakg, precision):
    import torch
    c = local_case(scale=0.56, N=32)  # 202 x 101 = 20,402 zones: four chunks
    assert c.Z >= 4 * 4096
    args = (c.zone_size, c.xf, c.Hxf, c.yo, c.Sf, c.HSf, c.r_diag, c.zone_pos, c.obs_pos,
            c.corr_len, c.max_len)
    kw = dict(weight=c.weight, precision=precision, ampl_always=True)
    xa_h, Sa_h, am_h, nobs_h = oakg.loc_analysis(*args, **kw)
    dev = torch.device("cuda", 0)
    T = lambda x: torch.as_tensor(np.ascontiguousarray(x), device=dev)
    F = lambda x: torch.as_tensor(np.ascontiguousarray(np.asarray(x).T), device=dev).t()
    xa_d, Sa_d, am_d, nobs_d = oakg.loc_analysis(
        T(c.zone_size), T(c.xf), T(c.Hxf), T(c.yo), F(c.Sf), F(c.HSf), T(c.r_diag),
        T(c.zone_pos), tuple(T(x) for x in c.obs_pos), T(c.corr_len), T(c.max_len), **kw)
    assert np.array_equal(nobs_h, nobs_d.cpu().numpy())
    assert np.array_equal(xa_h, xa_d.cpu().numpy())
    assert np.array_equal(Sa_h, Sa_d.cpu().numpy())
    assert np.array_equal(am_h, am_d.cpu().numpy())
