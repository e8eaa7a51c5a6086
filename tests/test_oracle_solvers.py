"""Pins the oracle's RHS assembly and fixed-step RK4 against test/solvers.jl
(wave energy conservation) and exact transport of a Fourier mode."""
import numpy as np
import pytest

import refrules as R


def _wave_run(O, D, k, n, f0, v0, t1, dt, nout):
    rhs = O.wave_rhs_raw(D, k, n)
    A = O.CSR(rhs)
    y = np.concatenate([f0, v0])
    steps = int(round(t1 / dt))
    per = steps // (nout - 1)
    states = [y.copy()]
    for _ in range(nout - 1):
        y = A.rk4(y, dt, per, nthreads=4)
        states.append(y.copy())
    return states, rhs


def test_wave_1d_hier_energy(O):
    # test/solvers.jl:35-47: k=4, level=4, f0=sin(2 pi x), v0=2 pi cos(2 pi x):
    # sqrt(E) = 2 pi within 1e-7 at every stored state.
    k, n = 4, 4
    f0 = O.vcoeffs_1d(k, n, lambda x: np.sin(2 * np.pi * x))
    v0 = O.vcoeffs_1d(k, n, lambda x: 2 * np.pi * np.cos(2 * np.pi * x))
    states, rhs = _wave_run(O, 1, k, n, f0, v0, 1.0, 1e-3, 11)
    A = O.CSR(rhs)
    rho = R.spectral_radius(lambda x: A.spmv(x), 2 * f0.size)
    assert rho * 1e-3 < 2.8  # RK4 stability on the imaginary axis
    grads = O.grad_matrix(1, k, n)
    for s in states:
        assert np.sqrt(O.energy(1, k, n, s, grads=grads)) == pytest.approx(2 * np.pi, abs=1e-7)


def test_wave_2d_sparse_energy(O):
    # test/solvers.jl:51-75: D=2, k=3, n=5 sparse, f0=sin(2pi x)sin(2pi y), v0=0,
    # t in [0,1]: sqrt(E) = sqrt(2) pi within 1e-4; energy decreases by < 1e-8.
    D, k, n = 2, 3, 5
    s = O.vcoeffs_1d(k, n, lambda x: np.sin(2 * np.pi * x))
    f0 = O.tensor_construct(D, k, n, [s, s])
    v0 = np.zeros_like(f0)
    states, rhs = _wave_run(O, D, k, n, f0, v0, 1.0, 1e-3, 6)
    grads = O.grad_matrix(D, k, n)
    E = [O.energy(D, k, n, st, grads=grads) for st in states]
    assert E[0] - E[-1] > 0
    assert abs(E[0] - E[-1]) < 1e-8
    for e in E:
        assert np.sqrt(e) == pytest.approx(np.sqrt(2) * np.pi, abs=1e-4)


def _advect_err(O, D, k, n, scheme, a, wv, t1):
    f0 = O.fourier_coeffs(D, k, n, [(wv, 1.0, "sin", 0.0)], scheme)
    ph = -2 * np.pi * float(np.dot(wv, a)) * t1
    exact = O.fourier_coeffs(D, k, n, [(wv, 1.0, "sin", ph)], scheme)
    A = O.CSR(O._Mat(O.lib().or_advection(D, k, n, O.SCHEMES[scheme], np.ascontiguousarray(a))))
    y = A.rk4(f0, 1e-3, int(round(t1 / 1e-3)), nthreads=4)
    return np.linalg.norm(y - exact) / np.linalg.norm(exact)


def test_advection_translates_fourier_mode(O):
    # f_t = -a . grad f, periodic: f(x,t) = f0(x - a t).  2D k=3, diagonal mode.
    a, wv, t1 = np.array([0.3, -0.7]), (1, 2), 0.5
    errs = [_advect_err(O, 2, 3, n, "sparse", a, wv, t1) for n in (4, 5, 6)]
    assert errs[0] > 5 * errs[1] > 25 * errs[2]
    assert errs[2] < 2e-3
    assert _advect_err(O, 2, 3, 5, "full", a, wv, t1) < 1e-4


def test_rk4_csc_and_csr_products_agree(O):
    D, k, n = 2, 2, 4
    rhs = O.wave_rhs_raw(D, k, n)
    A = O.CSR(rhs)
    x = np.random.default_rng(1).standard_normal(2 * O.get_size(D, k, n))
    assert np.allclose(A.spmv(x, nthreads=3), O.spmv_csc(rhs, x), rtol=0, atol=1e-11)
