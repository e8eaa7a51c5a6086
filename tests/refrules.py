"""Closed-form structural rules the oracle's literal assembly is checked against,
and small numeric helpers shared by the tests."""
import numpy as np


def support(L, c):
    """Closed support of the 1-based level L, cell c hierarchical function."""
    w = 1.0 / (1 << max(0, L - 2))
    return (c - 1) * w, c * w


def touch(a, b):
    (a0, a1), (b0, b1) = a, b
    if a0 <= b1 and b0 <= a1:
        return True
    return (a0 == 0 and b1 == 1) or (b0 == 0 and a1 == 1)


def pattern_1d(k, n):
    """Stored pattern of the 1D hierarchical DLF operator: dense k x k blocks for
    every pair of level/cell blocks whose closed supports meet (periodically)."""
    blocks = []
    for L in range(1, n + 2):
        for c in range(1, (1 << max(0, L - 2)) + 1):
            blocks.append((L, c))
    rows, cols = [], []
    for bj, (L2, c2) in enumerate(blocks):
        for bi, (L1, c1) in enumerate(blocks):
            if touch(support(L1, c1), support(L2, c2)):
                for mi in range(k):
                    for mj in range(k):
                        rows.append(bi * k + mi)
                        cols.append(bj * k + mj)
    return set(zip(rows, cols))


def l2_error_1d(O, k, n, coeffs, exact, q=8, scheme="full"):
    """int_0^1 (reconstruct - exact)^2 by Gauss-Legendre on each finest cell."""
    gx, gw = np.polynomial.legendre.leggauss(q)
    h = 1.0 / (1 << n)
    xs = np.concatenate([(i + 0.5) * h + 0.5 * h * gx for i in range(1 << n)])
    ws = np.tile(0.5 * h * gw, 1 << n)
    vals = O.reconstruct(1, k, n, coeffs, xs[:, None], scheme)
    return float(np.sum(ws * (vals - exact(xs)) ** 2))


def l2_error_2d(O, k, n, coeffs, exact, q=4, scheme="full"):
    gx, gw = np.polynomial.legendre.leggauss(q)
    h = 1.0 / (1 << n)
    xs = np.concatenate([(i + 0.5) * h + 0.5 * h * gx for i in range(1 << n)])
    ws = np.tile(0.5 * h * gw, 1 << n)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    W = np.outer(ws, ws)
    pts = np.stack([X.ravel(), Y.ravel()], axis=1)
    vals = O.reconstruct(2, k, n, coeffs, pts, scheme)
    return float(np.sum(W.ravel() * (vals - exact(pts[:, 0], pts[:, 1])) ** 2))


def spectral_radius(matvec, N, iters=300, seed=0):
    """Power iteration on A^T A style growth: returns an estimate of max |lambda|."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(N)
    x /= np.linalg.norm(x)
    lam = 0.0
    for _ in range(iters):
        y = matvec(matvec(x))
        nrm = np.linalg.norm(y)
        lam = np.sqrt(nrm)
        x = y / nrm
    return lam
