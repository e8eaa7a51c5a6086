"""Frozen oracle outputs (tests/golden/oracle_small.npz, written by
tests/golden/make_golden.py): the oracle must keep reproducing them, and the
product must match them -- index map and stored patterns bit for bit, values
to roundoff, and on the GPU the evolutions within each form's tolerance."""
import os

import numpy as np
import pytest
import scipy.sparse as sp

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_small.npz")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLD)


def csr(G, prefix, n):
    return sp.csr_matrix((G[prefix + "_data"], G[prefix + "_indices"], G[prefix + "_indptr"]), shape=(n, n))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def same_pattern(A, B):
    A = A.tocsr()
    B = B.tocsr()
    A.sort_indices()
    B.sort_indices()
    return np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)


def maxrel(A, B):
    return float(np.max(np.abs((A - B).toarray())) / np.max(np.abs(B.toarray())))


def modes(D, seed, count=3):
    rng = np.random.default_rng(seed)
    return [(tuple(int(v) for v in rng.integers(1, 4, D)), float(rng.uniform(-1, 1)),
             "sin" if rng.random() < 0.5 else "cos", 0.0) for _ in range(count)]


# ----------------------------------------------------------- the oracle ----
def test_oracle_reproduces_golden(O, G):
    L, C, M = O.index_map(3, 2, 3)
    assert np.array_equal(L, G["index_L"]) and np.array_equal(C, G["index_C"]) and np.array_equal(M, G["index_M"])
    for prefix, A in [("dlf_k3_n3", O.periodic_DLF_matrix(3, 3)), ("d2_D2k2n3", O.D_matrix(2, 2, 2, 3)),
                      ("lap_D2k2n3", O.laplacian_matrix(2, 2, 3)),
                      ("m2n_1d_k2n3", O.transform_1D(2, 3, "modal", "nodal")),
                      ("n2p_D2k3n2", O.transform(2, 3, 2, "nodal", "points"))]:
        B = csr(G, prefix, A.shape[0])
        assert same_pattern(A, B), prefix
        assert maxrel(A, B) < 1e-14, prefix
    y = O.CSR(O.wave_rhs_raw(2, 3, 3)).rk4(G["wave_y0"], 2e-3, 40, nthreads=1)
    assert rel(y, G["wave_y40"]) < 1e-14
    y = O.CSR(O.advection_matrix_raw(3, 2, 3, G["adv_a"])).rk4(G["adv_y0"], 2e-3, 40, nthreads=1)
    assert rel(y, G["adv_y40"]) < 1e-14
    r = O.vlasov_rhs(1, 2, 3, O.vlasov_operators(1, 2, 3), G["vlasov_F"], G["vlasov_f"])
    assert rel(r, G["vlasov_rhs"]) < 1e-14


def test_initial_states_match_golden(sgdg, G):
    f0 = sgdg.fourier_coeffs(2, 3, 3, modes(2, 1))
    assert rel(f0, G["wave_y0"][:f0.size]) < 1e-13
    g0 = sgdg.fourier_coeffs(3, 2, 3, modes(3, 3))
    assert rel(g0, G["adv_y0"]) < 1e-13


# ---------------------------------------------------------- the product ----
def test_product_host_matches_golden(sgdg, G):
    L, C, M = sgdg.index_map(3, 2, 3)
    assert np.array_equal(L, G["index_L"]) and np.array_equal(C, G["index_C"]) and np.array_equal(M, G["index_M"])
    # the 1D operator, D_d and the Laplacian (whose map(+) drops the sums that
    # cancel to exactly 0.0) hold the oracle's entries bit for bit
    for prefix, A in [("dlf_k3_n3", sgdg.periodic_DLF_matrix(3, 3)), ("d2_D2k2n3", sgdg.D_matrix(2, 2, 2, 3)),
                      ("lap_D2k2n3", sgdg.laplacian_matrix(2, 2, 3))]:
        B = csr(G, prefix, A.shape[0])
        assert same_pattern(A, B) and maxrel(A, B) == 0.0, prefix
    for prefix, A in [("m2n_1d_k2n3", sgdg.transform_1D(2, 3, "modal", "nodal")),
                      ("n2p_D2k3n2", sgdg.transform(2, 3, 2, "nodal", "points"))]:
        B = csr(G, prefix, A.shape[0])
        assert same_pattern(A, B) and maxrel(A, B) < 1e-13, prefix


@pytest.mark.gpu
def test_product_evolutions_match_golden(sgdg, G):
    y0 = G["wave_y0"]
    N = y0.size // 2
    for method, tol in (("plain", 1e-10), ("matfree", 1e-6)):
        _, st = sgdg.wave_evolve(2, 3, 3, y0[:N], y0[N:], 0.0, 40 * 2e-3, nsteps=40, method=method)
        assert rel(st[-1], G["wave_y40"]) < tol, method
        _, st = sgdg.advect_evolve(3, 2, 3, G["adv_a"], G["adv_y0"], 0.0, 40 * 2e-3, nsteps=40, method=method)
        assert rel(st[-1], G["adv_y40"]) < tol, method
    op = sgdg.VlasovOperator(1, 2, 3)
    assert rel(op.rhs(G["vlasov_F"], G["vlasov_f"]), G["vlasov_rhs"]) < 1e-10
