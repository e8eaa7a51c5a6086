"""Pins the oracle's derivative operator against the reference's tests
(test/differentiation.jl, test/hier_DG.jl) and against the structural rule the
reference's sparse algebra produces."""
import numpy as np
import pytest

import refrules as R


@pytest.mark.parametrize("k,n", [(1, 2), (1, 4), (2, 2), (2, 4), (3, 2), (3, 5), (4, 4), (5, 3), (6, 2)])
def test_1d_pattern_is_support_touch_rule(O, k, n):
    A = O.periodic_DLF_matrix(k, n).tocoo()
    got = set(zip(A.row.tolist(), A.col.tolist()))
    assert got == R.pattern_1d(k, n)


@pytest.mark.parametrize("k", [1, 2, 3, 4])
@pytest.mark.parametrize("n", [0, 1])
def test_1d_pattern_degenerate_below_two_levels(O, k, n):
    # With <= 2 finest cells both periodic neighbours of a cell are the same
    # cell, their central fluxes cancel and the reference stores fewer entries
    # (which ones depends on exact cancellation).  The product rejects n < 2.
    A = O.periodic_DLF_matrix(k, n).tocoo()
    got = set(zip(A.row.tolist(), A.col.tolist()))
    assert got < R.pattern_1d(k, n)


@pytest.mark.parametrize("k,n", [(1, 3), (2, 4), (3, 5), (4, 3)])
def test_1d_operator_is_skew(O, k, n):
    A = O.periodic_DLF_matrix(k, n)
    # central flux on a periodic domain is skew-adjoint; the reference's
    # +-5e-16 edge offsets (src/1d_derivative.jl:56-64) leave ~1e-13 relative.
    assert abs(A + A.T).max() <= 1e-12 * abs(A).max()


@pytest.mark.parametrize("D,d,k,n", [(2, 1, 3, 5), (2, 2, 3, 5), (3, 2, 2, 4), (3, 3, 3, 3)])
def test_dd_pattern_is_lines_of_1d_pattern(O, D, d, k, n):
    # src/multidim_derivative.jl:32-55: column j copies the 1D column of its
    # dim-d triple into dim d, skipping cut rows.
    Dd = O.D_matrix(D, d, k, n).tocoo()
    L, C, M = O.index_map(D, k, n)
    p1 = R.pattern_1d(k, n)
    from oracle import index_literal as IL
    i1 = np.array([IL.get_index_1D(k, L[j, d - 1], C[j, d - 1], M[j, d - 1]) - 1 for j in range(L.shape[0])])
    others = [tuple(np.r_[np.delete(L[j], d - 1), np.delete(C[j], d - 1), np.delete(M[j], d - 1)])
              for j in range(L.shape[0])]
    got = set(zip(Dd.row.tolist(), Dd.col.tolist()))
    for i, j in got:
        assert others[i] == others[j] and (i1[i], i1[j]) in p1
    # every admissible line pair present
    byline = {}
    for j, o in enumerate(others):
        byline.setdefault(o, []).append(j)
    count = sum(1 for line in byline.values() for i in line for j in line if (i1[i], i1[j]) in p1)
    assert count == len(got)


@pytest.mark.parametrize("l", [2, 3, 4, 5])
def test_1d_differentiation_bound(O, l):
    # test/differentiation.jl:13-26 (k=3, full): ||D f - f'||^2 < 1/2^(k+l-2)
    k = 3
    Dop = O.D_matrix(1, 1, k, l, "full")
    vc = O.vcoeffs_1d(k, l, lambda x: np.cos(2 * np.pi * x))
    err = R.l2_error_1d(O, k, l, Dop @ vc, lambda x: -2 * np.pi * np.sin(2 * np.pi * x))
    assert err < 1.0 / (1 << (k + l - 2))
    assert err < 0.06 * 50.0 ** (2 - l)  # observed k-th order: err^2 falls ~64x per level


@pytest.mark.parametrize("l", [2, 3, 4, 5])
def test_2d_full_differentiation_bound(O, l):
    # test/differentiation.jl:28-40 (D=2, k=3, full scheme, dim 1)
    k = 3
    Dop = O.D_matrix(2, 1, k, l, "full")
    c1 = O.vcoeffs_1d(k, l, lambda x: np.cos(2 * np.pi * x))
    vc = O.tensor_construct(2, k, l, [c1, c1], "full")
    err = R.l2_error_2d(O, k, l, Dop @ vc,
                        lambda x, y: -2 * np.pi * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y))
    assert err < 1.0 / (1 << (k + l - 2))


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("l", [1, 3, 6])
def test_1d_reconstruction_bound(O, k, l):
    # test/hier_DG.jl:14-30 and test/vhier_DG.jl:15-27: ||f - P f||^2 < 1/2^(l+k-1)
    vc = O.vcoeffs_1d(k, l, lambda x: np.sin(4 * x))
    err = R.l2_error_1d(O, k, l, vc, lambda x: np.sin(4 * x), scheme="sparse")
    assert err < 1.0 / (1 << (l + k - 1))


@pytest.mark.parametrize("k", [1, 3, 5])
@pytest.mark.parametrize("l", [1, 3, 5])
def test_2d_sparse_reconstruction_bound(O, k, l):
    # test/hier_DG.jl:45-54: 2D sparse, sin(4x+y), bound 1/2^(l+k-2)
    s4 = O.vcoeffs_1d(k, l, lambda x: np.sin(4 * x))
    c4 = O.vcoeffs_1d(k, l, lambda x: np.cos(4 * x))
    s1 = O.vcoeffs_1d(k, l, np.sin)
    c1 = O.vcoeffs_1d(k, l, np.cos)
    vc = O.tensor_construct(2, k, l, [s4, c1]) + O.tensor_construct(2, k, l, [c4, s1])
    err = R.l2_error_2d(O, k, l, vc, lambda x, y: np.sin(4 * x + y), scheme="sparse")
    assert err < 1.0 / (1 << (l + k - 2))


def test_fourier_coeffs_match_tensor_construct(O):
    k, n = 3, 4
    s = O.vcoeffs_1d(k, n, lambda x: np.sin(2 * np.pi * x))
    c = O.vcoeffs_1d(k, n, lambda x: np.cos(4 * np.pi * x))
    ref = 0.7 * O.tensor_construct(2, k, n, [s, c])
    # sin(2 pi x) cos(4 pi y) = (sin(2pi(x+2y)) + sin(2pi(x-2y)))/2
    got = O.fourier_coeffs(2, k, n, [((1, 2), 0.35, "sin", 0.0), ((1, -2), 0.35, "sin", 0.0)])
    assert np.max(np.abs(got - ref)) < 1e-13
