"""The configurations at their full sizes against the FP64 oracle.

- Uneven batch: all 256 advection solves (D in {2,3}, k in {2,3,4}, n in
  {4..7}, seeded velocities and 3-mode Fourier data) after the 50 RK4 steps
  the bench runs, every solve against the oracle's FP64 CSR RK4.
- Vlasov 2x2v (D = 2 space dimensions), sparse k = 2, n = 8 (167,936
  coefficients), seeded force E(x) of amplitude 0.1, Maxwellian sigma 0.15:
  plain FP64 and matrix-free against the oracle's Vlasov RK4
  (src/pdes.jl:131-227) after 100 steps at the bench's dt (the oracle takes
  about a second per step on the host, so 100 of the 500 steps); the error
  trend to 500 steps is the matrix-free form against the plain FP64 form.
- The matrix-free form with its 1D table in global memory (k = 3, n = 10)
  against the oracle's assembled operators.

Tolerances as in test_gpu_parity.py: plain FP64 1e-10, matrix-free 1e-6
(evolved) and 5e-7 (one application), relative L2."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_all_256_uneven_solves_after_50_steps(sgdg, O):
    serving = importlib.import_module(sgdg.__name__ + ".serving")
    specs = serving.uneven_batch(256, seed=33)
    dt, steps = 1e-3, 50
    b = sgdg.Batch()
    ids, y0s = [], []
    for D, k, n, a, modes in specs:
        y0 = sgdg.fourier_coeffs(D, k, n, modes)
        ids.append(b.add("advect", D, k, n, y0, dt, a=a))
        y0s.append(y0)
    b.autotune()
    b.step(steps)
    # the oracle's D_d of each (D, k, n), combined as -sum_d a_d D_d per solve
    dd = {}
    worst = 0.0
    for i, (D, k, n, a, _) in enumerate(specs):
        if (D, k, n) not in dd:
            dd[(D, k, n)] = [O.D_matrix_raw(D, d, k, n).csc() for d in range(1, D + 1)]
        A = sum(-a[d] * dd[(D, k, n)][d] for d in range(D))
        ref = O.CSR(O.from_csc(A)).rk4(y0s[i], dt, steps, nthreads=O.max_threads())
        e = rel(b.state(ids[i]), ref)
        worst = max(worst, e)
        assert e < 1e-6, (i, D, k, n, e)
    print("256 uneven solves, 50 steps: worst rel L2 vs oracle %.3e" % worst)
    b.close()


@pytest.fixture(scope="module")
def vlasov2x2v(sgdg, O):
    W = importlib.import_module(sgdg.__name__ + ".workloads")
    serving = importlib.import_module(sgdg.__name__ + ".serving")
    Dx, k, n = 2, 2, 8
    F, f0 = W.vlasov_case(sgdg, Dx, k, n, seed=11)
    rho = serving.spectral_radius_1d(sgdg, k, n)
    dt = 1.0 / (rho * (Dx * 1.0 + float(np.sum(np.max(np.abs(F), axis=1)))))  # the bench's step
    steps = 100
    ref = O.vlasov_rk4(Dx, k, n, O.vlasov_operators(Dx, k, n), F, f0, dt, steps)
    return Dx, k, n, F, f0, dt, steps, ref


def test_vlasov_2x2v_k2_n8_plain_and_matfree(sgdg, vlasov2x2v):
    Dx, k, n, F, f0, dt, steps, ref = vlasov2x2v
    _, sp = sgdg.vlasov_evolve(Dx, k, n, F, f0, 0.0, steps * dt, nsteps=steps, method="plain")
    ep = rel(sp[-1], ref)
    _, sm = sgdg.vlasov_evolve(Dx, k, n, F, f0, 0.0, steps * dt, nsteps=steps, method="matfree")
    em = rel(sm[-1], ref)
    einf = float(np.max(np.abs(sm[-1] - ref)) / np.max(np.abs(ref)))
    # the trend to the full 500 steps: matrix-free against plain FP64
    _, sp5 = sgdg.vlasov_evolve(Dx, k, n, F, f0, 0.0, 5 * steps * dt, nsteps=5 * steps, method="plain")
    _, sm5 = sgdg.vlasov_evolve(Dx, k, n, F, f0, 0.0, 5 * steps * dt, nsteps=5 * steps, method="matfree")
    e5 = rel(sm5[-1], sp5[-1])
    print("2x2v k=2 n=8, %d steps vs oracle: plain %.3e, matfree %.3e (Linf %.3e); 500 steps matfree vs plain %.3e"
          % (steps, ep, em, einf, e5))
    assert ep < 1e-10
    assert em < 1e-6
    assert e5 < 1e-6


def test_matfree_table_in_global_memory_vs_oracle(sgdg, O):
    # k=3, n=10: the pruned 1D table (~82 KB) exceeds the shared-memory copy
    # limit, so the pass tiles read it from global memory
    D, k, n = 2, 3, 10
    op = sgdg.SparseGridOperator(D, k, n)
    x = np.random.default_rng(1).standard_normal(op.N)
    for d in (1, 2):
        assert rel(op.apply(x, d, "matfree"), O.spmv_csc(O.D_matrix_raw(D, d, k, n), x)) < 5e-7
    assert rel(op.apply(x, 0, "matfree"), O.spmv_csc(O.laplacian_matrix_raw(D, k, n), x)) < 1e-6
    op.close()
