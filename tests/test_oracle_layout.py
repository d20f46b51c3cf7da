"""The layout-builder oracle (initPartition, sea packing, split / cinterp on rectilinear grids)
pinned against the reference's own checks: test/test_ndgrid.F90 (linear functions reproduced
at the domain centre to 1e-6 on the 10, 10x20, 2x2x2 and 2x2x2x2 grids and on the 2-D grids of
test_ndgrid_2d / test_regular_ndgrid_2d), a hand-derived unit-square case, the split counts
n! 2^(n-1) and the simplex volumes filling the cell, and the initPartition error cases."""
import math

import numpy as np
import pytest

from oracle import oakref as R


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_split_fills_the_cube(n):
    T = R.split(n)
    assert T.shape == (math.factorial(n) << (n - 1), n + 1, 1 << n)
    assert np.allclose(T.sum(axis=2), 1.0)
    # corner coordinates of the unit cube; simplex volume |det [1; X]| / n!
    K = 1 << n
    P = np.array([[(c >> k) & 1 for c in range(K)] for k in range(n)], dtype=float)
    vols = []
    for l in range(T.shape[0]):
        X = P @ T[l].T
        M = np.vstack([np.ones(n + 1), X])
        vols.append(abs(np.linalg.det(M)) / math.factorial(n))
    vols = np.array(vols)
    assert np.allclose(vols, vols[0]) and abs(vols.sum() - 1.0) < 1e-12


def test_unit_square_hand_case():
    """(0.5, 0.25) lies in the triangle (0,0), (1,0), centroid with barycentric coordinates
    (1/4, 1/4, 1/2); the centroid spreads 1/4 to every corner: weights 3/8, 3/8, 1/8, 1/8."""
    ax = [np.array([0.0, 1.0]), np.array([0.0, 1.0])]
    st, idx, w = R.cinterp_rectilinear(ax, [0.5, 0.25])
    assert st == "in" and list(idx) == [0, 1, 2, 3]
    assert np.allclose(w, [0.375, 0.375, 0.125, 0.125], atol=1e-15)
    st, idx, w = R.cinterp_rectilinear(ax, [0.5, 0.5])
    assert np.allclose(w, 0.25, atol=1e-15)


def _fun_nd(x):
    # test_ndgrid.F90 fun_nd: sum_i 2 i x_i (1-based i)
    return sum(2 * (i + 1) * x[i] for i in range(len(x)))


@pytest.mark.parametrize("sz", [(10,), (10, 20), (2, 2, 2), (2, 2, 2, 2)])
def test_ndgrid_nd_centre(sz):
    """test_ndgrid_nd: integer coordinates 0..sz-1 per axis, f = fun_nd on the grid points,
    interpolated at the mean coordinate; |ref - fi| <= 1e-6."""
    axes = [np.arange(s, dtype=float) for s in sz]
    xi = [a.mean() for a in axes]
    grid = np.meshgrid(*axes, indexing="ij")
    f = _fun_nd(grid).reshape(-1, order="F")
    idx, w = R.obsoper_rectilinear(axes, [[x] for x in xi])
    assert (idx >= 0).all()
    assert abs(np.dot(w[0], f[idx[0]]) - _fun_nd(xi)) <= 1e-6


@pytest.mark.parametrize("regular", [False, True])
def test_ndgrid_2d_centre(regular):
    """test_ndgrid_2d(10, 20) (x = i + 1, y = j + 2) and test_regular_ndgrid_2d (the same
    points as a regular grid): fun = 2x + 4y at the domain mean, to 1e-6."""
    m, n = 10, 20
    x = np.arange(1, m + 1) + 1.0
    y = np.arange(1, n + 1) + 2.0
    X, Y = np.meshgrid(x, y, indexing="ij")
    f = (2 * X + 4 * Y).reshape(-1, order="F")
    xi, yi = X.mean(), Y.mean()
    idx, w = R.obsoper_rectilinear([x, y], [[xi], [yi]])
    assert abs(np.dot(w[0], f[idx[0]]) - (2 * xi + 4 * yi)) <= 1e-6


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_linear_functions_reproduced(n):
    """Interpolation on simplices is exact for affine functions: random non-uniform axes
    (some descending), random points, weights in [0, 1] summing to 1."""
    rng = np.random.default_rng(40 + n)
    axes = []
    for k in range(n):
        a = np.cumsum(rng.uniform(0.2, 1.5, size=rng.integers(2, 7)))
        axes.append(a[::-1].copy() if k % 2 else a)
    m = 40 if n < 4 else 12
    pos = [rng.uniform(min(a), max(a), size=m) for a in axes]
    idx, w = R.obsoper_rectilinear(axes, pos)
    grid = np.meshgrid(*axes, indexing="ij")
    coef = rng.normal(size=n)
    f = (3.0 + sum(coef[k] * grid[k] for k in range(n))).reshape(-1, order="F")
    for j in range(m):
        assert (idx[j] >= 0).all()
        assert abs(w[j].sum() - 1) < 1e-12 and (w[j] >= -1e-8).all()
        ref = 3.0 + sum(coef[k] * pos[k][j] for k in range(n))
        assert abs(np.dot(w[j], f[idx[j]]) - ref) < 1e-10


def test_masked_corner_and_outside():
    x = np.arange(4.0)
    y = np.arange(3.0)
    mask = np.zeros((4, 3), dtype=bool)
    mask[2, 1] = True
    sea, nsea = R.sea_index(mask.reshape(-1, order="F"))
    assert nsea == 11 and sea[2 + 4 * 1] == -1 and sea[3 + 4 * 1] == 6
    idx, w = R.obsoper_rectilinear([x, y], [[0.5, 2.5, 5.0, 1.5], [0.5, 0.5, 1.0, 1.5]],
                                   sea=sea, offset=100)
    assert (idx[0] >= 100).all() and abs(w[0].sum() - 1) < 1e-12
    assert (idx[1] == -1).all() and (w[1] == 0).all()   # corner (2, 1) masked
    assert (idx[2] == -1).all()                          # outside
    assert (idx[3] == -1).all()                          # corner (2, 1) masked


def test_init_partition():
    part = np.array([2, 1, 3, 2, 1, 1, 3, 2])
    size, zi, inv = R.init_partition(part)
    assert list(size) == [3, 3, 2]
    assert list(zi) == [1, 4, 5, 0, 3, 7, 2, 6]
    assert (zi[inv] == np.arange(8)).all()
    with pytest.raises(ValueError):
        R.init_partition(np.array([1, 0, 2]))
    with pytest.raises(ValueError):
        R.init_partition(np.array([1, 3, 3]))


def test_partition_compact_hand_case():
    """unique(..., ind2 = partition): labels replaced by their rank among the distinct ones."""
    part, nz = R.partition_compact(np.array([5, -3, 5, 100, -3, 7]))
    assert nz == 4 and list(part) == [2, 1, 2, 4, 1, 3]


def _locate(p, n):
    """The operator kernel's direct simplex location (zone_layout.cu, locate_simplex) restated:
    per level, the free axis of largest |p - 1/2| and its side pick the block of split's
    numbering; the point is projected from the centroid onto that face."""
    p = list(p)
    fixed, l = 0, 0
    for subn in range(n, 1, -1):
        sub = math.factorial(subn - 1) << (subn - 2)
        best, best_rank, rank, dev = 0, 0, 0, -1.0
        for k in range(n):
            if (fixed >> k) & 1:
                continue
            d = abs(p[k] - 0.5)
            if d > dev:
                dev, best, best_rank = d, k, rank
            rank += 1
        side = 1 if p[best] > 0.5 else 0
        l += (2 * best_rank + side) * sub
        if dev > 0:
            t = 0.5 / dev
            for k in range(n):
                if not (fixed >> k) & 1 and k != best:
                    p[k] = 0.5 + (p[k] - 0.5) * t
        p[best] = float(side)
        fixed |= 1 << best
    return l


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_direct_location_is_the_first_accepting_simplex(n):
    """For points in general position the located simplex is the one interp_cube's ordered
    search accepts first; for corners, centres and half-integer points it accepts the point."""
    rng = np.random.default_rng(70 + n)
    T = R.split(n)
    K = 1 << n
    P = np.array([[(c >> k) & 1 for c in range(K)] for k in range(n)], dtype=float)
    for u in rng.random((300, n)):
        l = _locate(u, n)
        first = next(q for q in range(T.shape[0])
                     if not R.interp_tetrahedron(P @ T[q].T, u)[0])
        assert l == first
    special = [np.full(n, 0.5), np.zeros(n), np.ones(n)]
    special += [rng.integers(0, 3, n) / 2.0 for _ in range(60)]
    for u in special:
        assert not R.interp_tetrahedron(P @ T[_locate(u, n)].T, u)[0]
