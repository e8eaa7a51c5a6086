"""Plain-form operators assembled on the GPU (gpu_assemble.cu) against the
host assembly (assemble.cpp, whose stored pattern the golden and oracle
tests pin to the reference): D_d (src/multidim_derivative.jl:19-58), the
Laplacian (src/multidim_derivative.jl:71-79) and the wave right-hand side
(src/pdes.jl:22-49) must hold the same stored entries with bit-identical
values; the plain advection evolution, which now sums -a_d D_d on the GPU,
must match the oracle as before."""
import numpy as np
import pytest

CASES = [(1, 3, 5, "sparse"), (2, 3, 4, "sparse"), (3, 2, 3, "sparse"), (2, 2, 3, "full"), (4, 2, 3, "sparse"),
         (3, 3, 3, "sparse"), (2, 5, 3, "sparse"), (3, 2, 2, "full")]


def same_bits(A, B):
    A = A.tocsr()
    B = B.tocsr()
    A.sort_indices()
    B.sort_indices()
    return (A.shape == B.shape and np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)
            and np.array_equal(A.data.view(np.int64), B.data.view(np.int64)))


@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n,scheme", CASES)
def test_device_operators_equal_host(sgdg, D, k, n, scheme):
    op = sgdg.SparseGridOperator(D, k, n, scheme)
    for which in list(range(1, D + 1)) + [0, -1]:
        assert same_bits(op.device_csr(which), op.csr(which)), which
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n,scheme", [(2, 3, 5, "sparse"), (3, 3, 4, "sparse"), (2, 2, 5, "sparse"),
                                          (3, 2, 2, "full")])
def test_device_laplacian_and_wave_rhs_equal_oracle(sgdg, O, D, k, n, scheme):
    # the device merge drops the sums that cancel to exactly 0.0, as
    # SparseArrays' map(+) does in laplacian_matrix (src/multidim_derivative.jl:71-79)
    op = sgdg.SparseGridOperator(D, k, n, scheme)
    assert same_bits(op.device_csr(0), O.laplacian_matrix(D, k, n, scheme))
    assert same_bits(op.device_csr(-1), O.wave_rhs_raw(D, k, n, scheme).csc())
    op.close()


@pytest.mark.gpu
def test_plain_advection_uses_the_same_operator(sgdg, O):
    D, k, n = 3, 2, 3
    a = np.array([0.7, -0.3, 0.5])
    rng = np.random.default_rng(4)
    f0 = rng.standard_normal(sgdg.get_size(D, k, n))
    dt, steps = 2e-3, 30
    _, st = sgdg.advect_evolve(D, k, n, a, f0, 0.0, steps * dt, nsteps=steps, method="plain")
    ref = O.CSR(O.advection_matrix_raw(D, k, n, a)).rk4(f0, dt, steps, nthreads=1)
    assert np.linalg.norm(st[-1] - ref) <= 1e-10 * np.linalg.norm(ref)  # FP64 SpMV with FMA on the GPU


WHICH = [("modal", "nodal"), ("nodal", "points"), ("points", "nodal"), ("nodal", "modal")]


@pytest.mark.gpu
# (6, 2, 3): the coarse modal rows of n2m and m2n have 4^6 = 4096 level
# tuples, above the 1,024 from which a row gets a whole block
# (k_transform_long); the other cases stay in the warp-per-row kernel
@pytest.mark.parametrize("D,k,n,scheme", [(1, 3, 4, "sparse"), (2, 2, 3, "sparse"), (2, 3, 4, "sparse"),
                                          (3, 2, 3, "sparse"), (4, 2, 3, "sparse"), (2, 5, 3, "sparse"),
                                          (2, 2, 3, "full"), (6, 2, 3, "sparse")])
def test_device_transforms_equal_host(sgdg, D, k, n, scheme):
    # the restricted Kronecker products (src/multidim_nodal_basis.jl:40-109)
    for w in WHICH:
        assert same_bits(sgdg.transform(D, k, n, *w, scheme=scheme, device=True),
                         sgdg.transform(D, k, n, *w, scheme=scheme)), w
