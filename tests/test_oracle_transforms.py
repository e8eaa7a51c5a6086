"""The oracle's nodal-basis transforms pinned against the reference's own
tests (test/transformations.jl) and known answers: the maps are inverses of
each other in 1D and on the 2D sparse grid, triangular in the level, and
carry the modal coefficients of 2 x - 1 to its values at the collocation
points."""
import numpy as np
import pytest
import scipy.sparse as sp

LEVEL_DIR = {("modal", "nodal"): -1, ("nodal", "modal"): -1, ("nodal", "points"): +1, ("points", "nodal"): +1}


def threshold(A, atol=1e-12):
    A = A.tocsc(copy=True)
    A.data[np.abs(A.data) < atol] = 0.0
    A.eliminate_zeros()
    return A


@pytest.mark.parametrize("k", [2, 3, 5])
def test_1d_maps_are_inverses(O, k):
    # test/transformations.jl:16-43: norm(A*B - I) < 1e-15 * 10^k, n = 5
    n = 5
    I = np.eye(k << n)
    for a, b in [(("points", "nodal"), ("nodal", "points")), (("nodal", "modal"), ("modal", "nodal"))]:
        A = O.transform_1D(k, n, *a).toarray()
        B = O.transform_1D(k, n, *b).toarray()
        assert np.linalg.norm(A @ B - I) < 1e-15 * 10 ** k
        assert np.linalg.norm(B @ A - I) < 1e-15 * 10 ** k
    # points <-> modal through nodal (transform_1D's threshold(T2 * T1))
    p2m = threshold(sp.csc_matrix(O.transform_1D(k, n, "nodal", "modal") @ O.transform_1D(k, n, "points", "nodal")))
    m2p = threshold(sp.csc_matrix(O.transform_1D(k, n, "nodal", "points") @ O.transform_1D(k, n, "modal", "nodal")))
    assert np.linalg.norm((p2m @ m2p).toarray() - I) < 1e-15 * 10 ** k
    assert np.linalg.norm((m2p @ p2m).toarray() - I) < 1e-15 * 10 ** k


def test_2d_sparse_maps_are_inverses(O):
    # test/transformations.jl:55-78: D=2, k=3, n=5, norm(A*B - I) < 1e-10
    D, k, n = 2, 3, 5
    T = {w: O.transform(D, k, n, *w) for w in LEVEL_DIR}
    I = np.eye(T[("points", "nodal")].shape[0])
    for a, b in [(("points", "nodal"), ("nodal", "points")), (("nodal", "modal"), ("modal", "nodal"))]:
        assert np.linalg.norm((T[a] @ T[b]).toarray() - I) < 1e-10
        assert np.linalg.norm((T[b] @ T[a]).toarray() - I) < 1e-10
    p2m = threshold(T[("nodal", "modal")] @ T[("points", "nodal")])
    m2p = threshold(T[("nodal", "points")] @ T[("modal", "nodal")])
    assert np.linalg.norm((p2m @ m2p).toarray() - I) < 1e-10
    assert np.linalg.norm((m2p @ p2m).toarray() - I) < 1e-10


@pytest.mark.parametrize("k", [2, 3, 5])
def test_1d_maps_are_level_triangular(O, k):
    n = 4
    lev = np.concatenate([[0] * k] + [[l] * (k << max(0, l - 1)) for l in range(1, n + 1)])
    for w, sign in LEVEL_DIR.items():
        A = O.transform_1D(k, n, *w).tocoo()
        dl = lev[A.row] - lev[A.col]  # output level - input level
        assert np.all(sign * dl >= 0), w


def collocation_points(O, D, k, n):
    """Coordinates of the point basis: per level, k-1 new nodes of each cell
    then its last point (src/1d_nodal_basis.jl:183-213)."""
    x1 = []
    for l in range(n + 1):
        nc = 1 << max(0, l - 1)
        for c in range(1, nc + 1):
            x1 += [(c - 1 + (t / (k - 1) if l == 0 else (2 * t + 1) / (2 * (k - 1)))) / nc for t in range(k - 1)]
            x1.append(1.0 if l == 0 else (c - 0.5) / nc)
    L, C, M = O.index_map(D, k, n)
    i1 = k * (np.where(L >= 2, 1 << np.maximum(L - 2, 0), 0) + C - 1) + M - 1
    return np.array(x1)[i1]


@pytest.mark.parametrize("D,k,n", [(2, 2, 4), (2, 3, 4), (3, 2, 3), (2, 5, 3)])
def test_xi_modal_to_points_known_answer(O, D, k, n):
    # get_xi_point (src/basic_function_exact_coeffs.jl:39-43): the values of 2 x_i - 1
    X = collocation_points(O, D, k, n)
    m2n = O.transform(D, k, n, "modal", "nodal")
    n2p = O.transform(D, k, n, "nodal", "points")
    for i in range(1, D + 1):
        vals = n2p @ (m2n @ O.get_xi_modal(D, i, k, n))
        assert np.max(np.abs(vals - (2 * X[:, i - 1] - 1))) < 1e-13
