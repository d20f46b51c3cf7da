"""oak_gb300.shard on one GPU: the sharded entry (world size 1, no process group) runs the
CUDA library on device tensors and equals a direct call; the partial observation operator on
the device equals the host one."""
import numpy as np
import pytest

import _shard_worker as W
from oak_gb300 import shard

pytestmark = pytest.mark.gpu


def test_single_process_sharded_equals_direct(oakg):
    import torch
    dev = torch.device("cuda", 0)
    c, index, weight, Hxf, HSf, yo = W.problem()
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    F = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), device=dev).t()
    bounds = np.array([0, c.zone_size.size])
    xa, Sa, _, nobs = shard.sharded_loc_analysis(
        T(c.zone_size), T(c.zone_pos), T(c.corr_len), T(c.max_len), bounds, T(c.xf), F(c.Sf),
        T(index), T(weight), T(yo), T(c.r_diag), tuple(T(x) for x in c.obs_pos), weight=1)
    xa_d, Sa_d, _, nobs_d = oakg.loc_analysis(c.zone_size, c.xf, Hxf, yo, c.Sf, HSf, c.r_diag,
                                              c.zone_pos, c.obs_pos, c.corr_len, c.max_len,
                                              weight=1)
    assert np.array_equal(nobs.cpu().numpy(), nobs_d)
    xa, Sa = xa.cpu().numpy(), Sa.cpu().numpy()
    assert np.linalg.norm(xa - xa_d) <= 1e-10 * np.linalg.norm(xa_d - c.xf)
    assert np.linalg.norm(Sa - Sa_d) <= 1e-10 * np.linalg.norm(Sa_d)
