"""Point evaluation (reconstruct_DG, src/dg_methods.jl:150-165) and the
Monte Carlo error measures (src/error_measure.jl:12-45): the host logic on
CPU; on the GPU the batched FP64 evaluator against the oracle's restatement
(or_reconstruct) at random, boundary and midpoint coordinates, against the
basis products for unit coefficient vectors, and the argument errors; the
energy functions of src/pdes.jl:228-273 against a direct computation and the
reference's 1D energy known answer (test/solvers.jl:34-41)."""
import numpy as np
import pytest


def edge_points(D, n, rng, count=64):
    """Coordinates on cell boundaries j / 2^m, cell midpoints, 0 and 1."""
    m = rng.integers(0, n + 1, size=(count, D))
    j = rng.integers(0, 2 ** m + 1)
    pts = j / 2.0 ** m
    mid = (rng.integers(0, 2 ** m) + 0.5) / 2.0 ** m
    pts = np.where(rng.random((count, D)) < 0.3, mid, pts)
    pts[0] = 0.0
    pts[1] = 1.0
    return np.clip(pts, 0.0, 1.0)


# ------------------------------------------------------------------ CPU ----
def test_mcerr_host_logic(sgdg):
    rng = np.random.default_rng(0)
    f = lambda x: np.sum(x, axis=1)  # vectorised
    g = lambda x: sum(x)             # one point as a tuple, as in the reference
    assert sgdg.mcerr(f, g, 3, count=200, rng=rng) < 1e-14
    one = lambda x: np.ones(x.shape[0])
    zero = lambda x: 0.0
    assert abs(sgdg.mcerr(one, zero, 2, count=50, rng=rng) - 1.0) < 1e-15
    # mean of x1 over [0,1]^2 is 1/2; the estimate converges like count^-1/2
    assert abs(sgdg.monte_carlo(lambda x: x[:, 0], 2, count=20000, rng=rng) - 0.5) < 0.02


def test_mcerr2_batches(sgdg):
    # a constant difference: every batch mean is equal, so the stopping rule
    # (|new - mean| / std < Z) needs a nonzero spread; use noise of known size
    rng = np.random.default_rng(1)
    f = lambda x: np.zeros(x.shape[0])
    g = lambda x: 0.1 * np.sin(40 * x[:, 0])
    e = sgdg.mcerr2(f, g, 1, batch=50, Z=1.0, rng=rng)
    assert 0.05 < e < 0.1  # rms of 0.1 sin over many periods is 0.1 / sqrt(2)


def test_reconstruct_argument_checks(sgdg):
    N = sgdg.get_size(2, 2, 3)
    with pytest.raises(ValueError):
        sgdg.reconstruct_DG(2, 2, 3, np.zeros(N + 1), [0.5, 0.5])
    with pytest.raises(ValueError):
        sgdg.reconstruct_DG(2, 2, 3, np.zeros(N), [0.5, 0.5, 0.5])


# ------------------------------------------------------------------ GPU ----
CASES = [(1, 3, 5, "sparse"), (2, 3, 4, "sparse"), (3, 2, 3, "sparse"), (2, 5, 3, "sparse"), (4, 2, 3, "sparse"),
         (2, 2, 3, "full"), (3, 1, 4, "sparse")]


@pytest.mark.gpu
@pytest.mark.parametrize("D,k,n,scheme", CASES)
def test_evaluate_matches_oracle(sgdg, O, D, k, n, scheme):
    rng = np.random.default_rng(D * 100 + k * 10 + n)
    N = sgdg.get_size(D, k, n, scheme)
    c = rng.standard_normal(N)
    pts = np.concatenate([rng.random((300, D)), edge_points(D, n, rng)])
    got = sgdg.reconstruct_DG(D, k, n, c, pts, scheme)
    ref = O.reconstruct(D, k, n, c, pts, scheme)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    # a single point gives a float
    assert abs(sgdg.reconstruct_DG(D, k, n, c, pts[3], scheme) - ref[3]) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_unit_vectors_are_basis_products(sgdg, O):
    # coefficient vector e_i evaluates to prod_d v(k, L_d - 1, C_d, M_d, x_d)
    # inside the support of basis function i and to 0 outside it
    D, k, n = 2, 3, 3
    L, C, M = O.index_map(D, k, n)
    rng = np.random.default_rng(3)
    pts = rng.random((40, D))
    for i in rng.choice(L.shape[0], 12, replace=False):
        e = np.zeros(L.shape[0])
        e[i] = 1.0
        got = sgdg.reconstruct_DG(D, k, n, e, pts)
        for p, x in enumerate(pts):
            want = 1.0
            for d in range(D):
                l = int(L[i, d]) - 1
                inside = O.cell_index(x[d], l) == C[i, d]
                want *= O.v(k, l, int(C[i, d]), int(M[i, d]), x[d]) if inside else 0.0
            assert abs(got[p] - want) <= 1e-12 * max(1.0, abs(want))


@pytest.mark.gpu
def test_fourier_projection_reconstructs_the_function(sgdg):
    D, k, n = 2, 3, 6
    modes = [((1, 2), 0.7, "sin", 0.0), ((2, 1), -0.4, "cos", 0.0)]
    c = sgdg.fourier_coeffs(D, k, n, modes)
    f = sgdg.DGFunction(D, k, n, c)

    def exact(x):
        return 0.7 * np.sin(2 * np.pi * (x[:, 0] + 2 * x[:, 1])) - 0.4 * np.cos(2 * np.pi * (2 * x[:, 0] + x[:, 1]))

    e = sgdg.mcerr(f, exact, D, count=4000, rng=np.random.default_rng(5))
    assert e < 2e-3  # sparse k=3, n=6 projection error of these modes
    assert sgdg.mcerr(f, f, D, count=100) == 0.0


@pytest.mark.gpu
def test_points_outside_the_domain(sgdg, O):
    D, k, n = 2, 2, 3
    N = sgdg.get_size(D, k, n)
    c = np.random.default_rng(7).standard_normal(N)
    # above 1: the last cell, where the basis vanishes beyond its support (as the reference)
    pts = np.array([[1.25, 0.5], [0.5, 2.0], [1.0, 1.0]])
    got = sgdg.reconstruct_DG(D, k, n, c, pts)
    ref = O.reconstruct(D, k, n, c, pts)
    assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
    # below 0 or NaN: no cell (the reference raises an index error)
    for bad in ([-0.1, 0.5], [0.5, np.nan]):
        with pytest.raises(sgdg.SGDGError) as e:
            sgdg.reconstruct_DG(D, k, n, c, np.array([[0.3, 0.3], bad]))
        assert e.value.code == 1
    # an empty batch is a no-op
    assert sgdg.reconstruct_DG(D, k, n, c, np.zeros((0, D))).shape == (0,)


# ------------------------------------------------- energies (pdes.jl) ----
def test_norm_squared_and_energy_1d_host(sgdg, O):
    assert sgdg.norm_squared([3.0, 4.0]) == 25.0
    with pytest.raises(NotImplementedError):
        sgdg.norm_squared([1.0], basis="nodal")
    k, level = 3, 4
    rng = np.random.default_rng(8)
    n1 = k << level
    states = [rng.standard_normal(2 * n1) for _ in range(3)]
    times, E = sgdg.energy_func_1D(k, level, (np.array([0.0, 0.5, 1.0]), states))
    D = O.periodic_DLF_matrix(k, level)
    for s, e in zip(states, E):
        want = np.sum((D @ s[:n1]) ** 2) + np.sum(s[n1:] ** 2)
        assert abs(e - want) <= 1e-12 * want
    with pytest.raises(NotImplementedError):
        sgdg.energy_func_1D(k, level, (times, states), basis="nodal")


@pytest.mark.gpu
def test_wave_1d_energy_known_answer(sgdg):
    # test/solvers.jl:34-41: k = 4, level = 4, u = sin(2 pi x), u_t = 2 pi cos(2 pi x):
    # sqrt(energy) = 2 pi to 1e-7 at every stored time
    f0 = lambda x: np.sin(2 * np.pi * x[:, 0])
    v0 = lambda x: 2 * np.pi * np.cos(2 * np.pi * x[:, 0])
    soln = sgdg.wave_evolve_1D(4, 4, f0, v0, 0.0, 1.0, nsteps=2000, nout=5)
    _, E = sgdg.energy_func_1D(4, 4, soln)
    assert np.max(np.abs(np.sqrt(E) - 2 * np.pi)) < 1e-7
