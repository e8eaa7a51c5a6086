"""libsgdg host-side logic against the oracle (no GPU needed): the C ABI loads
and exports every declared symbol, the index map, the basis and the assembled
CSR operators (pattern bit-exact, values within roundoff)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    src = open(os.path.join(ROOT, "include", "sgdg.h")).read()
    return sorted(set(re.findall(r"\bint\s+(sgdg_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(sgdg):
    L = sgdg.lib()
    names = _declared_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
    from galerkinsparsegrids_gb300 import _lib
    assert sorted(_lib.EXPORTS) == names


def test_version_and_error_reporting(sgdg):
    buf = ctypes.create_string_buffer(64)
    assert sgdg.lib().sgdg_version(buf, 64) == 0 and b"sm_103a" in buf.value
    with pytest.raises(sgdg.SGDGError) as e:
        sgdg.SparseGridOperator(2, 3, 1)
    assert e.value.code == 1 and "n must be >= 2" in str(e.value)
    with pytest.raises(sgdg.SGDGError) as e:
        sgdg.SparseGridOperator(2, 11, 4)
    assert e.value.code == 1
    assert sgdg.lib().sgdg_get_size(2, 3, 4, 0, None) == 1  # SGDG_EINVAL for a NULL output
    with pytest.raises(sgdg.SGDGError, match="must not be NULL"):
        sgdg.check(sgdg.lib().sgdg_get_size(2, 3, 4, 0, None))
    with pytest.raises(ValueError):
        sgdg.get_size(2, 3, 4, "energy")


@pytest.mark.parametrize("D,k,n,scheme", [(1, 3, 5, "sparse"), (2, 3, 5, "sparse"), (3, 2, 4, "sparse"),
                                          (2, 2, 3, "full"), (4, 2, 4, "sparse")])
def test_index_map_matches_oracle(sgdg, O, D, k, n, scheme):
    assert sgdg.get_size(D, k, n, scheme) == O.get_size(D, k, n, scheme)
    for a, b in zip(sgdg.index_map(D, k, n, scheme), O.index_map(D, k, n, scheme)):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
def test_dg_coeffs_match_oracle(sgdg, O, k):
    assert np.max(np.abs(sgdg.dg_coeffs(k) - O.dg_coeffs(k))) < 1e-12


def _csr_equal_pattern(A, B):
    A = A.tocsr()
    B = B.tocsr()
    A.sort_indices()
    B.sort_indices()
    return A.shape == B.shape and np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)


def _csr_same_bits(A, B):
    """Same stored entries and bit-identical values (numerical zeros count)."""
    A = A.tocsr()
    B = B.tocsr()
    A.sort_indices()
    B.sort_indices()
    return _csr_equal_pattern(A, B) and np.array_equal(A.data.view(np.int64), B.data.view(np.int64))


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("n", [2, 3, 5, 6, 8])
def test_1d_operator_bit_identical(sgdg, O, k, n):
    # periodic_DLF_matrix (src/1d_derivative.jl:113-117): the product builds
    # Q' (A Q) by the reference's route, so the stored entries (numerical
    # zeros included) and every value equal the oracle's
    assert _csr_same_bits(sgdg.periodic_DLF_matrix(k, n), O.periodic_DLF_matrix(k, n))


@pytest.mark.parametrize("D,k,n,scheme", [(2, 3, 5, "sparse"), (3, 2, 4, "sparse"), (3, 3, 3, "sparse"),
                                          (2, 2, 3, "full"), (4, 2, 4, "sparse"), (1, 4, 4, "sparse")])
def test_dd_csr_bit_exact(sgdg, O, D, k, n, scheme):
    op = sgdg.SparseGridOperator(D, k, n, scheme)
    for d in range(1, D + 1):
        P = op.csr(d)
        Q = O.D_matrix(D, d, k, n, scheme)
        assert P.nnz == Q.nnz == op.nnz(d)
        assert _csr_same_bits(P, Q)


# laplacian_matrix (src/multidim_derivative.jl:71-79) adds the products
# D_d * D_d with map(+), which drops every sum that is exactly 0.0; the
# shapes below lose 0.2-1.2 % of the structural entries that way
@pytest.mark.parametrize("D,k,n,scheme", [(2, 3, 4, "sparse"), (3, 2, 3, "sparse"), (2, 2, 5, "sparse"),
                                          (2, 3, 5, "sparse"), (3, 3, 4, "sparse"), (1, 4, 5, "sparse"),
                                          (2, 1, 4, "sparse"), (2, 5, 4, "sparse"), (2, 2, 3, "full"),
                                          (3, 2, 2, "full"), (4, 2, 3, "sparse")])
def test_laplacian_and_wave_rhs_equal_oracle(sgdg, O, D, k, n, scheme):
    op = sgdg.SparseGridOperator(D, k, n, scheme)
    lap = O.laplacian_matrix(D, k, n, scheme)
    assert op.nnz(0) == lap.nnz
    assert _csr_same_bits(op.csr(0), lap)
    W = op.csr(-1)
    N = op.N
    assert W.shape == (2 * N, 2 * N)
    assert np.array_equal(W[:N].indices, np.arange(N, 2 * N)) and np.all(W[:N].data == 1.0)
    assert _csr_same_bits(W, O.wave_rhs_raw(D, k, n, scheme).csc())
    op.close()


def test_vcoeffs_DG_matches_oracle_projection(sgdg, O):
    D, k, n = 2, 3, 4
    f = lambda p: np.sin(2 * np.pi * p[:, 0]) * np.cos(4 * np.pi * p[:, 1]) + p[:, 0] ** 2
    got = sgdg.vcoeffs_DG(D, k, n, f)
    s = O.vcoeffs_1d(k, n, lambda x: np.sin(2 * np.pi * x))
    c = O.vcoeffs_1d(k, n, lambda x: np.cos(4 * np.pi * x))
    x2 = O.vcoeffs_1d(k, n, lambda x: x ** 2)
    one = O.vcoeffs_1d(k, n, lambda x: np.ones_like(x))
    ref = O.tensor_construct(D, k, n, [s, c]) + O.tensor_construct(D, k, n, [x2, one])
    assert np.max(np.abs(got - ref)) < 1e-12


def test_fourier_and_tensor_construct_match_oracle(sgdg, O):
    D, k, n = 3, 2, 4
    modes = [((1, 2, -1), 0.7, "sin", 0.3), ((3, 0, 1), -0.4, "cos", 0.0)]
    assert np.max(np.abs(sgdg.fourier_coeffs(D, k, n, modes) - O.fourier_coeffs(D, k, n, modes))) < 1e-13
    v = [np.random.default_rng(q).standard_normal(k << n) for q in range(D)]
    assert np.array_equal(sgdg.tensor_construct(D, k, n, v), O.tensor_construct(D, k, n, v))


def test_round_trips(sgdg):
    D, k, n = 2, 2, 3
    v = np.random.default_rng(0).standard_normal(sgdg.get_size(D, k, n))
    d = sgdg.V2D(D, k, n, v)
    assert np.array_equal(sgdg.D2V(D, k, n, d), v)
    ref = sgdg.D2Vref(D, k, n)
    assert all(ref[t] == i + 1 for i, t in enumerate(sgdg.V2Dref(D, k, n)))


def test_evolve_argument_errors(sgdg):
    N = sgdg.get_size(2, 2, 3)
    z = np.zeros(N)
    with pytest.raises(ValueError, match="rk4"):
        sgdg.wave_evolve(2, 2, 3, z, z, 0.0, 1.0, order="45", dt=0.1)
    with pytest.raises(ValueError):
        sgdg.wave_evolve(2, 2, 3, z, z, 0.0, 1.0, dt=0.3)
    with pytest.raises(ValueError):
        sgdg.advect_evolve(2, 2, 3, [1.0], z, 0.0, 1.0, dt=0.1)


def test_compute_without_gpu_fails_loudly(sgdg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    op = sgdg.SparseGridOperator(2, 2, 3)
    with pytest.raises(sgdg.SGDGError) as e:
        op.apply(np.zeros(op.N), 1)
    assert e.value.code == 6  # SGDG_ENOGPU: no CPU fallback


@pytest.mark.parametrize("k,n", [(1, 5), (2, 8), (3, 7), (4, 6), (5, 6), (3, 2)])
def test_zero_blocks_are_separated_from_genuine_ones(sgdg, k, n):
    # The matrix-free form skips the k x k blocks whose largest entry is below
    # 1e-10 of the operator's largest: those vanish mathematically (vanishing
    # moments of the finer wavelet) and sit at roundoff, far from every genuine
    # block.
    A = sgdg.periodic_DLF_matrix(k, n).tocoo()
    mx = np.abs(A.data).max()
    bm = {}
    for r, c, v in zip(A.row // k, A.col // k, np.abs(A.data)):
        bm[(r, c)] = max(bm.get((r, c), 0.0), v)
    rel = np.array(list(bm.values())) / mx
    assert not np.any((rel > 1e-12) & (rel < 1e-4))
    assert np.sum(rel > 1e-10) < len(rel) or n <= 2
