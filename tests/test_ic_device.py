"""Initial conditions built on the GPU (sgdg_tensor_sum): tensor_construct
(src/tensor_construct.jl:19-62) and sums of Fourier modes from host 1D
projections must equal the host construction -- exactly for a real product
(the same products in the same order), to roundoff for complex modes (the
host's numpy complex product may fuse its multiply-adds)."""
import numpy as np
import pytest


@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n,scheme", [(2, 3, 5, "sparse"), (3, 3, 4, "sparse"), (4, 2, 3, "sparse"),
                                          (2, 2, 3, "full")])
def test_tensor_construct_device_equals_host(sgdg, D, k, n, scheme):
    rng = np.random.default_rng(D + 10 * k + 100 * n)
    vs = [rng.standard_normal(k << n) for _ in range(D)]
    host = sgdg.tensor_construct(D, k, n, vs, scheme)
    dev = sgdg.tensor_construct(D, k, n, vs, scheme, device=True)
    assert np.array_equal(host, dev)


@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n", [(2, 3, 5), (3, 3, 4), (4, 2, 3)])
def test_fourier_device_matches_host(sgdg, D, k, n):
    rng = np.random.default_rng(7 * D + k)
    modes = [(tuple(int(v) for v in rng.integers(1, 4, D)), float(rng.uniform(-1, 1)),
              "sin" if rng.random() < 0.5 else "cos", float(rng.uniform(0, 2 * np.pi))) for _ in range(5)]
    host = sgdg.fourier_coeffs(D, k, n, modes)
    dev = sgdg.fourier_coeffs(D, k, n, modes, device=True)
    assert np.max(np.abs(host - dev)) <= 1e-14 * np.max(np.abs(host))


def test_tensor_sum_argument_checks(sgdg):
    with pytest.raises(ValueError):
        sgdg._tensor_sum(2, 2, 3, np.zeros((1, 3, 16)), [[1, 1, 0, 0]], "sparse")


# vcoeffs_DG (src/dg_vmethods.jl:149-179) of a general (non-separable) f:
# host samples at the quadrature nodes, GPU contraction over the level blocks
# (sgdg_vcoeffs_contract); the same quadrature as the host path, summed in
# another order, and against the oracle's separable projections
@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n,scheme", [(1, 3, 5, "sparse"), (2, 3, 4, "sparse"), (3, 2, 4, "sparse"),
                                          (2, 2, 3, "full")])
def test_vcoeffs_DG_device_matches_host(sgdg, D, k, n, scheme):
    f = lambda p: np.sin(2 * np.pi * (p @ np.arange(1, D + 1))) * np.exp(p[:, 0]) + p[:, -1] ** 2
    host = sgdg.vcoeffs_DG(D, k, n, f, scheme)
    dev = sgdg.vcoeffs_DG(D, k, n, f, scheme, device=True)
    assert np.max(np.abs(host - dev)) <= 1e-13 * np.max(np.abs(host))


@pytest.mark.gpu
def test_vcoeffs_DG_device_matches_oracle(sgdg, O):
    D, k, n = 2, 3, 4
    f = lambda p: np.sin(2 * np.pi * p[:, 0]) * np.cos(4 * np.pi * p[:, 1]) + p[:, 0] ** 2
    got = sgdg.vcoeffs_DG(D, k, n, f, device=True)
    s = O.vcoeffs_1d(k, n, lambda x: np.sin(2 * np.pi * x))
    c = O.vcoeffs_1d(k, n, lambda x: np.cos(4 * np.pi * x))
    x2 = O.vcoeffs_1d(k, n, lambda x: x ** 2)
    one = O.vcoeffs_1d(k, n, lambda x: np.ones_like(x))
    ref = O.tensor_construct(D, k, n, [s, c]) + O.tensor_construct(D, k, n, [x2, one])
    assert np.max(np.abs(got - ref)) < 1e-12
