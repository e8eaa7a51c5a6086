"""The Vlasov evolver (src/pdes.jl:131-227): the product's nodal transforms
against the oracle (same stored pattern, values to roundoff), the velocity
points, argument errors, and on the GPU the right-hand side and the RK4
evolution against the oracle's FP64 restatement."""
import importlib

import numpy as np
import pytest

WHICH = [("modal", "nodal"), ("nodal", "points"), ("points", "nodal"), ("nodal", "modal")]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def same_sparse(A, B, tol):
    A = A.tocsr()
    B = B.tocsr()
    A.sort_indices()
    B.sort_indices()
    assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)
    scale = max(np.abs(B.data).max(), 1e-300)
    assert np.max(np.abs(A.data - B.data)) <= tol * scale


@pytest.fixture(scope="module")
def W(sgdg):
    return importlib.import_module(sgdg.__name__ + ".workloads")


@pytest.mark.parametrize("k", [2, 3, 5])
def test_1d_transforms_match_oracle(sgdg, O, k):
    for n in (2, 4, 6):
        for w in WHICH:
            same_sparse(sgdg.transform_1D(k, n, *w), O.transform_1D(k, n, *w), 1e-13)


@pytest.mark.parametrize("D,k,n", [(2, 3, 5), (2, 2, 4), (3, 2, 3), (4, 2, 3), (2, 5, 3), (3, 3, 2)])
def test_dd_transforms_match_oracle(sgdg, O, D, k, n):
    for w in WHICH:
        same_sparse(sgdg.transform(D, k, n, *w), O.transform(D, k, n, *w), 1e-13)


def test_full_scheme_transform_matches_oracle(sgdg, O):
    for w in WHICH:
        same_sparse(sgdg.transform(2, 2, 3, *w, scheme="full"), O.transform(2, 2, 3, *w, scheme="full"), 1e-13)


@pytest.mark.parametrize("D,k,n", [(1, 2, 4), (2, 2, 3), (1, 3, 4), (1, 5, 3)])
def test_vlasov_operator_holds_the_reference_operators(sgdg, O, W, D, k, n):
    op = sgdg.VlasovOperator(D, k, n)
    P = 2 * D
    assert op.N == sgdg.get_size(P, k, n)
    for w in WHICH:
        same_sparse(op.transform(*w), sgdg.transform(P, k, n, *w), 0.0)
    # v_point: the velocity 2 p_d - 1 at the collocation points
    X = W.point_coords(sgdg, P, k, n)
    vp = op.v_point()
    for d in range(D):
        assert np.max(np.abs(vp[d] - (2 * X[:, D + d] - 1))) < 1e-13
    op.close()


def test_vlasov_argument_errors(sgdg):
    with pytest.raises(sgdg.SGDGError) as e:
        sgdg.VlasovOperator(1, 4, 3)  # no nodal basis for k = 4
    assert e.value.code == 1
    with pytest.raises(sgdg.SGDGError):
        sgdg.VlasovOperator(5, 2, 3)  # phase space of 10 dimensions
    with pytest.raises(ValueError):
        sgdg.transform(2, 2, 3, "modal", "points")


def test_vlasov_case_inputs(sgdg, W):
    F, f0 = W.vlasov_case(sgdg, 2, 2, 3, seed=4)
    N = sgdg.get_size(4, 2, 3)
    assert F.shape == (2, N) and f0.shape == (N,)
    assert np.max(np.abs(F)) <= 0.1 + 1e-12
    # F depends on x only: equal on points that share their x coordinates
    X = W.point_coords(sgdg, 4, 2, 3)
    key = {tuple(r): v for r, v in zip(np.round(X[:, :2], 12), F[0])}
    assert all(abs(key[tuple(r)] - v) < 1e-15 for r, v in zip(np.round(X[:, :2], 12), F[0]))


# ------------------------------------------------------------------- GPU ----
def oracle_ops(O, D, k, n):
    return O.vlasov_operators(D, k, n)


# D = 3: six phase-space derivatives, carried by the transform pass as a
# 4-vector and a 2-vector chunk of a 6-wide interleaved set; at n = 3, 256 m2n
# rows are longer than the 2,048-entry split (segment sums on 4 and 2 vectors)
@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n", [(1, 2, 5), (2, 2, 3), (1, 3, 4), (1, 5, 3), (3, 2, 3)])
def test_vlasov_rhs_matches_oracle(sgdg, O, W, D, k, n):
    F, f0 = W.vlasov_case(sgdg, D, k, n, seed=7)
    op = sgdg.VlasovOperator(D, k, n)
    got = op.rhs(F, f0)
    ref = O.vlasov_rhs(D, k, n, oracle_ops(O, D, k, n), F, f0)
    assert rel(got, ref) < 1e-10  # FP64, chained SpMVs with cancellation; GPU uses FMA


@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n,steps", [(2, 2, 3, 20), (1, 3, 4, 30), (3, 2, 2, 10)])
def test_vlasov_evolve_matches_oracle(sgdg, O, W, D, k, n, steps):
    F, f0 = W.vlasov_case(sgdg, D, k, n, seed=8)
    dt = 2e-3
    times, states = sgdg.vlasov_evolve(D, k, n, F, f0, 0.0, steps * dt, nout=3, nsteps=steps)
    assert np.allclose(times, [0.0, steps * dt / 2, steps * dt])
    assert np.array_equal(states[0], f0)
    ref = O.vlasov_rk4(D, k, n, oracle_ops(O, D, k, n), F, f0, dt, steps)
    assert rel(states[-1], ref) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n,steps", [(1, 2, 4, 20), (2, 2, 3, 20), (1, 3, 4, 15), (1, 5, 3, 10), (3, 2, 2, 10)])
def test_vlasov_matfree_matches_oracle(sgdg, O, W, D, k, n, steps):
    F, f0 = W.vlasov_case(sgdg, D, k, n, seed=9)
    dt = 2e-3
    _, st = sgdg.vlasov_evolve(D, k, n, F, f0, 0.0, steps * dt, nsteps=steps, method="matfree")
    ref = O.vlasov_rk4(D, k, n, oracle_ops(O, D, k, n), F, f0, dt, steps)
    assert rel(st[-1], ref) < 1e-6
    _, sp = sgdg.vlasov_evolve(D, k, n, F, f0, 0.0, steps * dt, nsteps=steps, method="plain")
    assert rel(st[-1], sp[-1]) < 1e-6


@pytest.mark.gpu
def test_vlasov_in_a_mixed_batch_equals_alone(sgdg, W):
    F1, f1 = W.vlasov_case(sgdg, 1, 2, 4, seed=1)
    F2, f2 = W.vlasov_case(sgdg, 2, 2, 3, seed=2)
    a0 = np.zeros(sgdg.get_size(2, 2, 4))
    a0[:10] = 0.3
    b = sgdg.Batch()
    i1 = b.add_vlasov(1, 2, 4, f1, F1, 1e-3)
    i2 = b.add_vlasov(2, 2, 3, f2, F2, 1e-3)
    i3 = b.add("advect", 2, 2, 4, a0, 1e-3, a=[0.4, -0.2])
    b.step(6)
    for i, (Dx, k, n, f, F) in [(i1, (1, 2, 4, f1, F1)), (i2, (2, 2, 3, f2, F2))]:
        alone = sgdg.Batch()
        j = alone.add_vlasov(Dx, k, n, f, F, 1e-3)
        alone.step(6)
        assert np.array_equal(b.state(i), alone.state(j))
    alone = sgdg.Batch()
    j = alone.add("advect", 2, 2, 4, a0, 1e-3, a=[0.4, -0.2])
    alone.step(6)
    assert np.array_equal(b.state(i3), alone.state(j))
