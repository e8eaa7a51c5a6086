"""Seeded inputs of the Vlasov workload: collocation-point coordinates of the
point basis, a sinusoidal force field and a Maxwellian initial density.

Phase space [0,1]^(2D) is ordered x_1..x_D, p_1..p_D; the velocity is
v = 2 p - 1 (the reference's get_xi_modal, src/basic_function_exact_coeffs.jl:
11-17), so a Maxwellian centred at v = 0 sits at p = 1/2."""
import numpy as np


def point_coords_1d(k, n):
    """Collocation point of every 1D point-basis index (level-major, k per
    cell: k-1 new nodes, then the cell's last point), src/1d_nodal_basis.jl:
    183-213."""
    out = []
    for l in range(0, n + 1):
        nc = 1 << max(0, l - 1)
        for c in range(1, nc + 1):
            for t in range(k - 1):
                node = t / (k - 1) if l == 0 else (2 * t + 1) / (2 * (k - 1))
                out.append((c - 1 + node) / nc)
            out.append(1.0 if l == 0 else (c - 0.5) / nc)
    return np.array(out)


def point_coords(sg, D, k, n, scheme="sparse"):
    """(N, D) coordinates of the point basis on the sparse grid."""
    L, C, M = sg.index_map(D, k, n, scheme)
    x1 = point_coords_1d(k, n)
    idx = k * (np.where(L >= 2, 1 << np.maximum(L - 2, 0), 0) + C - 1) + M - 1
    return x1[idx]


def vlasov_case(sg, D, k, n, seed=0, amplitude=0.1, sigma=0.15, perturb=0.05, nmodes=2):
    """(F_point (D, N), f0 modal coefficients) of the Vlasov workload: a fixed
    force E(x) = amplitude * sum of seeded sin/cos modes of x (one field per
    velocity component), and f0 = (1 + perturb cos(2 pi x_1)) *
    exp(-|v|^2 / (2 sigma^2)), projected dimension by dimension."""
    rng = np.random.default_rng(seed)
    P = 2 * D
    X = point_coords(sg, P, k, n)
    F = np.zeros((D, X.shape[0]))
    for d in range(D):
        for _ in range(nmodes):
            a = rng.integers(1, 3, D)
            ph = rng.uniform(0, 2 * np.pi)
            F[d] += amplitude / nmodes * np.sin(2 * np.pi * (X[:, :D] @ a) + ph)
    one = lambda x: np.ones_like(x)
    fx1 = lambda x: 1.0 + perturb * np.cos(2 * np.pi * x)
    maxw = lambda p: np.exp(-((2 * p - 1) ** 2) / (2 * sigma ** 2))
    fac = [fx1 if d == 0 else one for d in range(D)] + [maxw] * D
    q = max(12, k + 8)
    f0 = sg.tensor_construct(P, k, n, [sg.vcoeffs_1d(k, n, f, q=q) for f in fac])
    return F, f0
