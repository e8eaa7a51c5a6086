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
