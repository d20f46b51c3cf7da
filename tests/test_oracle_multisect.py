"""The few-zone eigenvalue kernel's arithmetic (zone_eig.cu, k_eig_values_multisect) restated in
NumPy and checked against LAPACK (numpy.linalg.eigvalsh) on tridiagonal matrices of the kinds
the eigensolve meets: random, graded over many orders, with clustered pairs (Wilkinson), and
rank-deficient (blocks of zeros). Sturm counts come from the division-free three-term recurrence
of the leading minors with power-of-two rescaling; 32 interior points per step (33-fold
narrowing) until the interval is at the rounding level of the matrix."""
import numpy as np
import pytest

EPS = 1.1102230246251565e-16


def sturm_counts(d, e2, x):
    """Number of eigenvalues below each x (array): sign changes of p_0 = 1, p_1, ..., p_N."""
    p0 = np.ones_like(x)
    p1 = d[0] - x
    s1 = ~(p1 > 0)
    c = s1.astype(np.int64)
    for i in range(1, d.size):
        p2 = (d[i] - x) * p1 - e2[i - 1] * p0
        s2 = np.where(p2 == 0, ~s1, p2 < 0)
        c += s2 != s1
        s1 = s2
        p0, p1 = p1, p2
        if i % 8 == 0:
            mx = np.maximum(np.abs(p0), np.abs(p1))
            big = (mx > 1e150) | ((mx < 1e-150) & (mx > 0))
            if big.any():
                _, ex = np.frexp(np.where(big, mx, 1.0))
                sc = np.where(big, np.ldexp(1.0, -ex), 1.0)
                p0, p1 = p0 * sc, p1 * sc
    return c


def multisect(d, e):
    N = d.size
    r = np.abs(np.concatenate([e, [0.0]])) + np.abs(np.concatenate([[0.0], e]))
    onenrm = np.max(np.abs(d) + r)
    pad = 2 * EPS * onenrm + 1e-300
    a = np.full(N, np.min(d - r) - pad)
    b = np.full(N, np.max(d + r) + pad)
    e2 = np.concatenate([e * e, [0.0]])
    k = np.arange(N)
    frac = np.arange(1, 33) / 33.0
    for _ in range(64):
        x = a[:, None] + (b - a)[:, None] * frac[None, :]
        cnt = sturm_counts(d, e2, x.ravel()).reshape(N, 32)
        past = cnt > k[:, None]
        ss = np.where(past.any(axis=1), past.argmax(axis=1), 32)
        xl = np.where(ss == 0, a, a + (b - a) * ss / 33.0)
        xu = np.where(ss == 32, b, a + (b - a) * (ss + 1) / 33.0)
        a, b = xl, xu
        if np.all(b - a <= 2 * EPS * np.maximum(np.abs(a), np.abs(b)) + EPS * onenrm):
            break
    return 0.5 * (a + b), onenrm


def _check(d, e):
    lam, onenrm = multisect(d, e)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    ref = np.linalg.eigvalsh(T)
    assert np.all(np.diff(lam) >= 0)
    assert np.abs(lam - ref).max() <= 8 * EPS * onenrm * d.size ** 0.5


@pytest.mark.parametrize("N", [2, 30, 64, 128])
def test_random_tridiagonals(N):
    rng = np.random.default_rng(N)
    for _ in range(5):
        _check(rng.uniform(-1, 1, N), rng.uniform(-1, 1, N - 1))


def test_graded_and_clustered():
    # graded over 12 orders of magnitude
    N = 64
    d = np.logspace(0, -12, N)
    e = 0.5 * np.sqrt(d[:-1] * d[1:])
    _check(d, e)
    # Wilkinson W+ (pairs of eigenvalues agreeing to many digits)
    m = 10
    d = np.abs(np.arange(-m, m + 1, dtype=float))
    _check(d / d.max(), np.ones(2 * m) / d.max())


def test_rank_deficient_blocks():
    """A Gram matrix of rank p < N gives a zero block after tridiagonalisation."""
    rng = np.random.default_rng(9)
    for N, p in ((64, 20), (128, 5)):
        X = rng.normal(size=(p, N))
        G = X.T @ X
        G /= np.abs(G).max()
        # Householder tridiagonalisation (LAPACK via SciPy) of the Gram matrix
        scipy_linalg = pytest.importorskip("scipy.linalg")
        H = scipy_linalg.hessenberg(G)
        d = np.diag(H).copy()
        e = np.diag(H, -1).copy()
        _check(d, e)
