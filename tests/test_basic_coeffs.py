"""The exact coefficient vectors of src/basic_function_exact_coeffs.jl and the
transform pairs of src/multidim_nodal_basis.jl:127-141 on the host: the
constant and the coordinate functions against the oracle and against the
projection of the function itself, and the transform pairs against the
single transforms and as a round trip to roundoff (the reference's own
invertibility check of the nodal maps)."""
import numpy as np
import pytest


@pytest.mark.parametrize("D,k,n", [(2, 2, 3), (3, 3, 2), (1, 4, 4)])
def test_get_one_modal_and_xi_modal(sgdg, O, D, k, n):
    one = sgdg.get_one_modal(D, k, n)
    assert np.array_equal(one, O.get_one_modal(D, k, n))
    # the projection of f = 1 is exactly the first basis coefficient
    proj = sgdg.vcoeffs_DG(D, k, n, lambda x: np.ones(len(x)))
    assert np.max(np.abs(proj - one)) < 1e-12
    for i in range(1, D + 1):
        xi = sgdg.get_xi_modal(D, i, k, n)
        assert np.max(np.abs(xi - O.get_xi_modal(D, i, k, n))) <= 1e-15
        proj = sgdg.vcoeffs_DG(D, k, n, lambda x, i=i: 2.0 * x[:, i - 1] - 1.0)
        assert np.max(np.abs(proj - xi)) < 1e-12


@pytest.mark.parametrize("D,k,n", [(2, 2, 3), (2, 3, 2)])
def test_transform_pairs(sgdg, D, k, n):
    m2n, n2p = sgdg.make_modal2point_matrices(D, k, n)
    p2n, n2m = sgdg.make_point2modal_matrices(D, k, n)
    for A, (f, t) in ((m2n, ("modal", "nodal")), (n2p, ("nodal", "points")), (p2n, ("points", "nodal")),
                      (n2m, ("nodal", "modal"))):
        B = sgdg.transform(D, k, n, f, t)
        assert (A != B).nnz == 0
    x = np.random.default_rng(3).standard_normal(m2n.shape[1])
    back = n2m @ (p2n @ (n2p @ (m2n @ x)))
    assert np.max(np.abs(back - x)) < 1e-10 * np.max(np.abs(x))
    # the point values of 2 x_i - 1 through the pair, as the Vlasov operator builds its velocities
    for i in range(1, D + 1):
        pts = sgdg.get_xi_point(D, i, k, n, m2n, n2p)
        assert np.max(np.abs(n2m @ (p2n @ pts) - sgdg.get_xi_modal(D, i, k, n))) < 1e-10
