"""The slice budget of an exact FP64 Gram on TF32 tensor-core arithmetic, emulated on the CPU.
Each column of X is scaled by a power of two and split into 8-bit integer slices: exact in
TF32, with FP32 sums of 256 rows exact. The slice-pair products are summed in FP64. Six slices
(21 products) must reach the Gram's FP64 value to better than 1e-12 relative, well inside the
1e-10 parity bar of the analysis; five must not (the budget is tight)."""
import numpy as np


def _split(X, b, S):
    E = np.ceil(np.log2(np.abs(X).max(axis=0)))
    R = X / 2.0 ** E
    out = []
    for s in range(S):
        sc = 2.0 ** (b * (s + 1))
        q = np.trunc(R * sc)
        out.append(q)
        R = R - q / sc
    return out, E


def _gram(X, b=8, S=6, kc=256):
    sl, E = _split(X, b, S)
    G = np.zeros((X.shape[1], X.shape[1]))
    for s in range(S):
        for t in range(S - s):
            acc = np.zeros_like(G)
            for k0 in range(0, X.shape[0], kc):
                a = sl[s][k0:k0 + kc].astype(np.float32)
                c = sl[t][k0:k0 + kc].astype(np.float32)
                part = a.T @ c
                # the FP32 sums are exact: integers below 2^24
                assert np.abs(part).max() < 2.0 ** 24
                acc += part.astype(np.float64)
            G += acc / 2.0 ** (b * (s + t + 2))
    return G * np.outer(2.0 ** E, 2.0 ** E)


def test_six_slices_reach_fp64():
    rng = np.random.default_rng(0)
    X = rng.normal(size=(900, 64)) * rng.uniform(0.1, 3.0, size=(900, 1))
    G = X.T @ X
    err = lambda S: np.abs(_gram(X, S=S) - G).max() / np.abs(G).max()
    assert err(6) < 1e-12
    assert err(5) > 1e-12
