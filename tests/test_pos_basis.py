"""The position-basis route of wave_evolve_1D (src/pdes.jl:89-121 with
basis = "pos"): D_op = periodic_pos_DLF_matrix (src/1d_derivative.jl:108-111),
laplac = D_op * D_op, wave_data around it, functions projected with
pos_vcoeffs_DG (src/1d_dg_functions.jl:103-117).  The reference's own test is
test/solvers.jl:20-31 (k = 4, level = 4, sqrt(energy) = 2 pi to 1e-7)."""
import numpy as np
import pytest

SHAPES = [(1, 2), (2, 3), (3, 4), (4, 4), (5, 5), (2, 7), (4, 8)]


def _same(P, M):
    rp, ci, v = M.csr_arrays()
    return np.array_equal(P.indptr, rp) and np.array_equal(P.indices, ci) and np.array_equal(P.data, v)


@pytest.mark.parametrize("k,n", SHAPES)
def test_pos_operators_equal_oracle_bitwise(sgdg, O, k, n):
    # host assembly, no GPU: stored pattern and values of D_op, D_op * D_op
    # (structural zeros kept) and the wave right-hand side equal the oracle's
    op = sgdg.SparseGridOperator(1, k, n, basis="pos")
    A, lap, W = O.pos_wave_rhs_raw(k, n)
    assert _same(op.csr(1), A)
    assert _same(op.csr(0), lap)
    assert _same(op.csr(-1), W)
    P = sgdg.periodic_DLF_matrix(k, n, basis="pos")
    assert _same(P, A)


def test_pos_operator_is_the_hierarchical_one_in_the_other_basis(sgdg, O):
    # periodic_hier_DLF_matrix = Q' A Q with Q = hier2pos orthogonal
    # (src/1d_derivative.jl:113-117), so A = Q H Q'
    for k, n in [(2, 4), (3, 5), (4, 4)]:
        A = sgdg.periodic_DLF_matrix(k, n, basis="pos").toarray()
        H = sgdg.periodic_DLF_matrix(k, n).toarray()
        Q = O.hier2pos(k, n).toarray()
        assert np.allclose(Q.T @ Q, np.eye(Q.shape[0]), rtol=0, atol=1e-12)
        assert np.max(np.abs(Q @ H @ Q.T - A)) <= 1e-11 * np.max(np.abs(A))


@pytest.mark.parametrize("k,level", [(1, 3), (3, 4), (4, 4), (5, 6)])
def test_pos_vcoeffs_match_oracle_and_hier2pos(sgdg, O, k, level):
    f = lambda x: np.sin(2 * np.pi * x) + 0.3 * np.cos(6 * np.pi * x) + x ** 2
    c = sgdg.pos_vcoeffs_DG(k, level, lambda p: f(p[:, 0]))
    assert c.shape == (k << level,)
    ref = O.pos_vcoeffs_1d(k, level, f)
    assert np.max(np.abs(c - ref)) <= 1e-13 * np.max(np.abs(ref))
    # the same function in the hierarchical basis, carried over by hier2pos
    h = sgdg.vcoeffs_DG(1, k, level, lambda p: f(p[:, 0]))
    Q = O.hier2pos(k, level)
    assert np.max(np.abs(Q @ h - c)) <= 1e-11 * np.max(np.abs(c))


def test_pos_vcoeffs_reproduce_piecewise_polynomials(sgdg):
    # a polynomial of degree < k on every cell is represented exactly: its
    # L2 norm equals the norm of its coefficients (orthonormal basis)
    k, level = 3, 4
    f = lambda p: 1.0 + 2.0 * p[:, 0] - 3.0 * p[:, 0] ** 2
    c = sgdg.pos_vcoeffs_DG(k, level, f)
    xs, ws = np.polynomial.legendre.leggauss(12)
    xs, ws = 0.5 * (xs + 1), 0.5 * ws
    exact = float(np.sum(ws * (1.0 + 2.0 * xs - 3.0 * xs ** 2) ** 2))
    assert sgdg.norm_squared(c, basis="pos") == pytest.approx(exact, rel=1e-14)


def test_pos_basis_arguments(sgdg):
    with pytest.raises(ValueError):
        sgdg.SparseGridOperator(2, 3, 4, basis="pos")
    with pytest.raises(ValueError):
        sgdg.wave_evolve_1D(3, 4, np.zeros(48), np.zeros(48), 0.0, 1.0, nsteps=10, basis="nodal")
    with pytest.raises(ValueError):
        sgdg.wave_evolve_1D(3, 4, np.zeros(48), np.zeros(48), 0.0, 1.0, nsteps=10, basis="pos", method="matfree")
    op = sgdg.SparseGridOperator(1, 3, 4, basis="pos")
    with pytest.raises(sgdg.SGDGError):
        op.csr(2)
    with pytest.raises(NotImplementedError):
        sgdg.energy_func_1D(3, 4, (np.zeros(1), [np.zeros(96)]), basis="point")


def test_pos_energy_matches_oracle_operator(sgdg, O):
    k, level = 3, 5
    n1 = k << level
    rng = np.random.default_rng(4)
    states = [rng.standard_normal(2 * n1) for _ in range(3)]
    _, E = sgdg.energy_func_1D(k, level, (np.array([0.0, 0.5, 1.0]), states), basis="pos")
    A = O.periodic_pos_DLF_matrix(k, level)
    for s, e in zip(states, E):
        want = np.sum((A @ s[:n1]) ** 2) + np.sum(s[n1:] ** 2)
        assert abs(e - want) <= 1e-12 * want


@pytest.mark.gpu
def test_pos_wave_1d_energy_known_answer(sgdg):
    # test/solvers.jl:20-31: k = 4, level = 4, f0 = sin(2 pi x),
    # v0 = 2 pi cos(2 pi x), t in [0, 1], basis = "pos": sqrt(energy) = 2 pi
    # to 1e-7 at every stored state
    f0 = lambda x: np.sin(2 * np.pi * x[:, 0])
    v0 = lambda x: 2 * np.pi * np.cos(2 * np.pi * x[:, 0])
    soln = sgdg.wave_evolve_1D(4, 4, f0, v0, 0.0, 1.0, basis="pos", nsteps=2000, nout=5)
    _, E = sgdg.energy_func_1D(4, 4, soln, basis="pos")
    assert len(E) == 5
    assert np.max(np.abs(np.sqrt(E) - 2 * np.pi)) < 1e-7


@pytest.mark.gpu
@pytest.mark.parametrize("k,n", [(2, 5), (3, 6), (4, 4)])
def test_pos_wave_evolution_matches_oracle(sgdg, O, k, n):
    # plain FP64 CSR RK4 on the GPU against the oracle's RK4 on its own
    # position-basis right-hand side, same seeded state, same steps
    N = k << n
    rng = np.random.default_rng(k * 10 + n)
    f0, v0 = rng.standard_normal(N), rng.standard_normal(N)
    _, _, W = O.pos_wave_rhs_raw(k, n)
    dt, steps = 2e-4, 500
    ref = O.CSR(W).rk4(np.concatenate([f0, v0]), dt, steps, nthreads=4)
    _, st = sgdg.wave_evolve_1D(k, n, f0, v0, 0.0, dt * steps, basis="pos", nsteps=steps)
    err = np.linalg.norm(st[-1] - ref) / np.linalg.norm(ref)
    print("pos k=%d n=%d: rel L2 vs oracle %.2e" % (k, n, err))
    assert err <= 1e-10


@pytest.mark.gpu
def test_pos_and_hier_evolutions_agree(sgdg, O):
    # why the reference has a 1D wave evolver (src/pdes.jl:86-88): the
    # position and hierarchical bases agree; Q carries one solution onto
    # the other at every stored time
    k, n = 3, 5
    f = lambda x: np.sin(2 * np.pi * x[:, 0]) + 0.5 * np.cos(4 * np.pi * x[:, 0])
    g = lambda x: np.zeros(x.shape[0])
    _, sp = sgdg.wave_evolve_1D(k, n, f, g, 0.0, 0.5, basis="pos", nsteps=1000, nout=3)
    _, sh = sgdg.wave_evolve_1D(k, n, f, g, 0.0, 0.5, basis="hier", nsteps=1000, nout=3)
    Q = O.hier2pos(k, n)
    N = k << n
    for a, b in zip(sp, sh):
        mapped = np.concatenate([Q @ b[:N], Q @ b[N:]])
        assert np.linalg.norm(a - mapped) <= 1e-10 * np.linalg.norm(a)
