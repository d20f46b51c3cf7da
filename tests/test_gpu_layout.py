"""Layout builders on the GPU against the oracle: initPartition (zone sizes, zoneIndex,
invZoneIndex; bit-exact), the sea packing (bit-exact), and the rectilinear-grid observation
operator of genObservationOper / cinterp (indices bit-exact, weights to 1e-12 absolute: the
device solves the barycentric system by its own elimination). At full sizes: linear functions
reproduced to 1e-10, weights summing to 1."""
import numpy as np
import pytest

from oracle import oakref as R

pytestmark = pytest.mark.gpu


def _dev(x):
    import torch
    return torch.as_tensor(np.ascontiguousarray(x), device="cuda")


@pytest.mark.parametrize("n,Z", [(1000, 7), (100000, 256), (100000, 3000), (300000, 70000)])
def test_zone_layout_matches_init_partition(oakg, n, Z):
    rng = np.random.default_rng(n + Z)
    part = rng.integers(1, Z + 1, size=n).astype(np.int32)
    part[:Z] = np.arange(1, Z + 1)  # every zone non-empty
    rng.shuffle(part)
    size_o, zi_o, inv_o = R.init_partition(part)
    for device in (False, True):
        p = _dev(part) if device else part
        zs, zi, inv = oakg.zone_layout(p, Z)
        if device:
            zs, zi, inv = zs.cpu().numpy(), zi.cpu().numpy(), inv.cpu().numpy()
        assert np.array_equal(zs, size_o)
        assert np.array_equal(zi, zi_o) and np.array_equal(inv, inv_o)


def test_zone_layout_large_zones_stay_in_element_order(oakg):
    """Three zones of ~10^6 elements each: the order inside a zone is the element order."""
    rng = np.random.default_rng(5)
    part = rng.integers(1, 4, size=3_000_000).astype(np.int32)
    zs, zi, inv = oakg.zone_layout(_dev(part))
    zi = zi.cpu().numpy()
    assert np.array_equal(zi, np.argsort(part, kind="stable"))
    assert np.array_equal(zs.cpu().numpy(), np.bincount(part)[1:])


def test_zone_layout_errors(oakg):
    for part, Z, what in (([1, 0, 2], 2, "1..2"), ([1, 3, 2], 2, "1..2"),
                          ([1, 3, 3], 3, "at least one")):
        with pytest.raises(oakg.OakError) as ei:
            oakg.zone_layout(np.array(part, dtype=np.int32), Z)
        assert ei.value.code == oakg.ERR_ARGS and what in str(ei.value)


def test_permute_rows_round_trip(oakg):
    rng = np.random.default_rng(8)
    part = rng.integers(1, 40, size=5000).astype(np.int32)
    part[:39] = np.arange(1, 40)
    _, zi, inv = oakg.zone_layout(part)
    X = np.asfortranarray(rng.normal(size=(5000, 6)))
    Y = oakg.permute_rows(zi, X)
    assert np.array_equal(Y, X[zi])
    assert np.array_equal(oakg.permute_rows(inv, Y), X)
    v = rng.normal(size=5000)
    assert np.array_equal(oakg.permute_rows(_dev(zi), _dev(v)).cpu().numpy(), v[zi])


@pytest.mark.parametrize("npts", [1, 4095, 4096, 4097, 3_000_001])
def test_sea_index(oakg, npts):
    rng = np.random.default_rng(npts)
    mask = rng.random(npts) < 0.3
    sea_o, n_o = R.sea_index(mask)
    sea, n = oakg.sea_index(mask)
    assert n == n_o and np.array_equal(sea, sea_o)
    sea_d, n_d = oakg.sea_index(_dev(mask))
    assert n_d == n_o and np.array_equal(sea_d.cpu().numpy(), sea_o)


def _axes(rng, n, sizes):
    axes = []
    for k in range(n):
        a = np.cumsum(rng.uniform(0.2, 1.5, size=sizes[k]))
        axes.append(a[::-1].copy() if k % 2 else a)
    return axes


@pytest.mark.parametrize("n,m", [(1, 400), (2, 400), (3, 200), (4, 60)])
def test_rectilinear_operator_matches_oracle(oakg, n, m):
    rng = np.random.default_rng(100 + n)
    sizes = [7, 6, 5, 4][:n]
    axes = _axes(rng, n, sizes)
    # points inside, a margin outside, and some exactly on grid nodes
    pos = [rng.uniform(min(a) - 0.3, max(a) + 0.3, size=m) for a in axes]
    for k in range(n):
        pos[k][:10] = axes[k][rng.integers(0, sizes[k], size=10)]
    mask = rng.random(int(np.prod(sizes))) < 0.04
    sea, _ = R.sea_index(mask)
    idx_o, w_o = R.obsoper_rectilinear(axes, pos, sea=sea, offset=17)
    for device in (False, True):
        if device:
            idx, w = oakg.obsoper_rectilinear([_dev(a) for a in axes], [_dev(p) for p in pos],
                                              sea=_dev(sea), offset=17)
            idx, w = idx.cpu().numpy(), w.cpu().numpy()
        else:
            idx, w = oakg.obsoper_rectilinear(axes, pos, sea=sea, offset=17)
        assert np.array_equal(idx, idx_o)
        assert np.abs(w - w_o).max() < 1e-12
    assert (idx_o[:, 0] >= 0).sum() > m // 5 and (idx_o[:, 0] == -1).sum() > 0


def test_rectilinear_unit_square_hand_case(oakg):
    idx, w = oakg.obsoper_rectilinear([np.array([0.0, 1.0]), np.array([0.0, 1.0])],
                                      [np.array([0.5, 0.5]), np.array([0.25, 0.5])])
    assert np.array_equal(idx, [[0, 1, 2, 3], [0, 1, 2, 3]])
    assert np.abs(w - [[0.375, 0.375, 0.125, 0.125], [0.25] * 4]).max() < 1e-15


def test_rectilinear_degenerate_cell(oakg):
    """Cells of 1e-5 x 1e-5 have |det| = 5e-11 <= 1e-8: the reference leaves its plain solve;
    both the oracle and the device mark the observation -2."""
    ax = [np.array([0.0, 1e-5, 2e-5]), np.array([0.0, 1e-5])]
    pos = [np.array([0.5e-5]), np.array([0.5e-5])]
    idx_o, _ = R.obsoper_rectilinear(ax, pos)
    idx, w = oakg.obsoper_rectilinear(ax, pos)
    assert (idx_o == -2).all() and (idx == -2).all() and (w == 0).all()


def test_rectilinear_linear_reproduction_full_size(oakg):
    """10^6 observations on a 3-D 720 x 360 x 20 rectilinear grid with a land mask: every
    in-grid observation reproduces an affine field to 1e-10, weights sum to 1, no weight below
    -1e-8; the out-of-grid / next-to-land rows are the masked cells' neighbours only."""
    import torch
    rng = np.random.default_rng(3)
    x = np.linspace(-180, 179.5, 720)
    y = np.linspace(-89.75, 89.75, 360)
    z = np.cumsum(rng.uniform(1, 50, size=20))
    mask = np.zeros((720, 360, 20), dtype=bool)
    mask[100:200, 50:120, :] = True
    mask[:, :, 15:] |= (np.arange(720)[:, None, None] % 7 == 0)
    sea, nsea = oakg.sea_index(_dev(mask.reshape(-1, order="F")))
    m = 1_000_000
    pos = [rng.uniform(-181, 181, m), rng.uniform(-90, 90, m), rng.uniform(0, z[-1] + 5, m)]
    idx, w = oakg.obsoper_rectilinear([_dev(x), _dev(y), _dev(z)], [_dev(p) for p in pos],
                                      sea=sea)
    X, Y, Zg = np.meshgrid(x, y, z, indexing="ij")
    f = (1.5 + 0.01 * X - 0.02 * Y + 0.003 * Zg).reshape(-1, order="F")
    keep = ~mask.reshape(-1, order="F")
    f_sea = torch.as_tensor(f[keep], device="cuda")
    ref = torch.as_tensor(1.5 + 0.01 * pos[0] - 0.02 * pos[1] + 0.003 * pos[2], device="cuda")
    inside = idx[:, 0] >= 0
    assert nsea == int(keep.sum()) and inside.float().mean() > 0.7
    val = (w[inside] * f_sea[idx[inside]]).sum(dim=1)
    assert (val - ref[inside]).abs().max().item() < 1e-10
    assert (w[inside].sum(dim=1) - 1).abs().max().item() < 1e-12
    assert w[inside].min().item() >= -1e-8


def test_operator_to_zone_order(oakg):
    rng = np.random.default_rng(11)
    part = rng.integers(1, 30, size=2000).astype(np.int32)
    part[:29] = np.arange(1, 30)
    _, _, inv = oakg.zone_layout(part)
    idx = rng.integers(-1, 2000, size=(300, 4)).astype(np.int64)
    exp = np.where(idx >= 0, inv[np.maximum(idx, 0)], idx)
    got = oakg.obsoper_to_zone_order(idx.copy(), inv)
    assert np.array_equal(got, exp)
    d = _dev(idx)
    assert np.array_equal(oakg.obsoper_to_zone_order(d, _dev(inv)).cpu().numpy(), exp)
    bad = idx.copy()
    bad[0, 0] = 2000
    with pytest.raises(oakg.OakError):
        oakg.obsoper_to_zone_order(bad, inv)


@pytest.mark.parametrize("n", [1, 5000, 2_000_000])
def test_partition_compact_matches_unique(oakg, n):
    """Labels over the whole int32 range, with gaps and repeats, host and device memory."""
    rng = np.random.default_rng(n)
    pool = rng.integers(-2**31, 2**31 - 1, size=max(1, n // 7), dtype=np.int64)
    labels = pool[rng.integers(0, pool.size, size=n)].astype(np.int32)
    part_o, nz_o = R.partition_compact(labels)
    part, nz = oakg.partition_compact(labels)
    assert nz == nz_o and np.array_equal(part, part_o)
    part_d, nz_d = oakg.partition_compact(_dev(labels))
    assert nz_d == nz_o and np.array_equal(part_d.cpu().numpy(), part_o)
    # the compacted partition feeds the zone layout directly
    zs, zi, _ = oakg.zone_layout(part, nz)
    assert np.array_equal(zs, np.bincount(part_o)[1:])
