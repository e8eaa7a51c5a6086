"""Pins the oracle's basis and index map against the reference's own tests:
test/basis_constructor.jl, test/elementary.jl, test/vhier_DG.jl (round trips)."""
import numpy as np
import pytest

from oracle import index_literal as IL


def _poly_inner(p, q):
    """Exact <p, q> on [-1, 1] for 'x^i (+) sgn(x) x^i' coefficient arrays."""
    n = len(p)
    k = n // 2

    def integ(a, b, sa, sb):
        e = a + b
        odd = (sa + sb) % 2  # number of sgn factors mod 2
        if odd == 0:
            return (1 + (-1) ** e) / (1 + e)
        return (1 - (-1) ** e) / (1 + e)

    s = 0.0
    for i in range(n):
        for j in range(n):
            s += p[i] * q[j] * integ(i % k, j % k, i // k, j // k)
    return s


@pytest.mark.parametrize("k", range(1, 7))
def test_dg_basis_orthonormal_vanishing_moments(O, k):
    # test/basis_constructor.jl:14-19 (dg_basis builds, right shape, k=1..5) plus
    # the defining properties of dg_basis (src/dg_basis.jl:104-190).  Beyond k~8
    # the reference's monomial Gram-Schmidt loses orthogonality (1e-6 at k=9),
    # which the oracle reproduces; workloads use k <= 5.
    Q = O.dg_coeffs(k)
    assert Q.shape == (2 * k, k)
    G = np.array([[_poly_inner(Q[:, a], Q[:, b]) for b in range(k)] for a in range(k)])
    assert np.allclose(G, np.eye(k), atol=1e-9 * 10 ** (k / 3))
    for m in range(k):
        for j in range(k):  # orthogonal to every polynomial of degree < k
            mono = np.zeros(2 * k)
            mono[j] = 1.0
            assert abs(_poly_inner(Q[:, m], mono)) < 1e-9 * 10 ** (k / 3)


def test_dg_basis_known_answer_k1(O):
    assert np.array_equal(O.dg_coeffs(1)[:, 0], [0.0, 1.0 / np.sqrt(2.0)])


def test_legendre_orthonormal(O):
    L = O.leg_coeffs()
    G = np.array([[_poly_inner(L[a], L[b]) for b in range(11)] for a in range(11)])
    assert np.allclose(G, np.eye(11), atol=1e-9)
    assert L[1][1] == pytest.approx(np.sqrt(1.5), rel=1e-15)


def test_cell_index_known_answers(O):
    # test/elementary.jl:15-30
    for l in range(1, 6):
        assert O.cell_index(1.3, l) == 1 << (l - 1)
        assert O.cell_index(0.01, l) == 1
    assert [O.cell_index(0.3, l) for l in range(1, 6)] == [1, 1, 2, 3, 5]


def test_inner_product_known_answers():
    # test/elementary.jl:32-45: inner products on the unit cell, atol 2 eps.
    gx, gw = np.polynomial.legendre.leggauss(12)
    x = 0.5 * (gx + 1)
    w = 0.5 * gw
    eps = np.finfo(float).eps
    assert abs(np.sum(w * x ** 2 * x ** 3) - 1 / 6) < 2 * eps
    X, Y = np.meshgrid(x, x, indexing="ij")
    W2 = np.outer(w, w)
    assert abs(np.sum(W2 * (X ** 2 + Y ** 2) * X ** 3) - 0.25) < 2 * eps
    X3, Y3, Z3 = np.meshgrid(x, x, x, indexing="ij")
    W3 = np.einsum("i,j,k->ijk", w, w, w)
    val = np.sum(W3 * (X3 ** 2 + Y3 ** 2 - Z3 ** 2) * (X3 ** 3 + Y3 + Z3))
    assert abs(val - 0.5) < 2 * eps


@pytest.mark.parametrize("D,k,n,N", [(2, 3, 5, 1008), (3, 3, 7, 45792), (4, 2, 8, 167936), (3, 4, 7, 108544),
                                     (5, 3, 8, 5684256), (2, 2, 4, 192), (1, 3, 5, 96)])
def test_get_size_known(O, D, k, n, N):
    assert O.get_size(D, k, n) == N
    if N < 200000:
        assert IL.get_size(D, k, n) == N


@pytest.mark.parametrize("scheme", ["full", "sparse"])
@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("k", [1, 2, 3, 4])
@pytest.mark.parametrize("l", [1, 2, 3])
def test_index_map_matches_literal_and_round_trips(O, scheme, D, k, l):
    # test/vhier_DG.jl:30-68: V2D(D2V(dict)) == dict and D2V(V2D(v)) == v,
    # plus the oracle's C index map equal to the literal V2Dref.
    ref = IL.V2Dref(D, k, l, scheme)
    L, C, M = O.index_map(D, k, l, scheme)
    assert len(ref) == L.shape[0] == O.get_size(D, k, l, scheme)
    for j, (lv, cl, md) in enumerate(ref):
        assert tuple(L[j]) == lv and tuple(C[j]) == cl and tuple(M[j]) == md
    rng = np.random.default_rng(D * 100 + k * 10 + l)
    vect = list(rng.standard_normal(len(ref)))
    dct = IL.V2D(D, k, l, vect, scheme)
    assert IL.D2V(D, k, l, dct, scheme) == vect
    assert IL.V2D(D, k, l, IL.D2V(D, k, l, dct, scheme), scheme) == dct
    dv = IL.D2Vref(D, k, l, scheme)
    assert all(dv[ref[j]] == j + 1 for j in range(len(ref)))


def test_get_index_1D_matches_1d_order():
    for k in (1, 3):
        ref = IL.V2Dref(1, k, 5)
        for j, (lv, cl, md) in enumerate(ref, start=1):
            assert IL.get_index_1D(k, lv[0], cl[0], md[0]) == j
