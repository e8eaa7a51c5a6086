"""More GPU coverage: the device-side bounded wait gives up as designed
(failure detection without a fault), the matrix-free form on a grid whose
operator table is read from global memory (n = 10), and a mixed served
stream with wave and advection requests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_bounded_wait_gives_up_and_context_survives(sgdg):
    secs = ctypes.c_double()
    code = sgdg.lib().sgdg_selftest_bounded_wait(ctypes.byref(secs))
    assert code == 3  # SGDG_ETIMEOUT: the wait ran out, raised the flag and returned
    assert 0.0 < secs.value < 30.0
    # the context is still usable: a normal application right after
    op = sgdg.SparseGridOperator(2, 2, 4)
    x = np.random.default_rng(0).standard_normal(op.N)
    assert rel(op.apply(x, 1, "matfree"), op.apply(x, 1, "plain")) < 5e-7


def test_matfree_with_table_in_global_memory(sgdg):
    # k=3, n=10: the pruned 1D table (~82 KB) exceeds the shared-memory copy limit
    D, k, n = 2, 3, 10
    op = sgdg.SparseGridOperator(D, k, n)
    x = np.random.default_rng(1).standard_normal(op.N)
    for d in (1, 2):
        assert rel(op.apply(x, d, "matfree"), op.apply(x, d, "plain")) < 5e-7
    assert rel(op.apply(x, 0, "matfree"), op.apply(x, 0, "plain")) < 5e-7


def test_served_wave_and_advection_requests(sgdg):
    srv = sgdg.Server(max_chunk_steps=4)
    rng = np.random.default_rng(2)
    specs = [("wave", 2, 3, 4), ("advect", 3, 2, 4), ("wave", 3, 2, 3), ("advect", 2, 3, 5)]
    ids, inputs = [], []
    for kind, D, k, n in specs:
        N = sgdg.get_size(D, k, n)
        y0 = rng.standard_normal(2 * N if kind == "wave" else N) * 1e-2
        a = rng.uniform(-1, 1, D)
        steps = int(rng.integers(5, 15))
        ids.append(srv.submit(kind, D, k, n, y0, 1e-3, steps, a=a if kind == "advect" else None))
        inputs.append((kind, D, k, n, y0, a, steps))
    while srv.counts()[0] + srv.counts()[1] > 0:
        srv.tick()
    for rid, (kind, D, k, n, y0, a, steps) in zip(ids, inputs):
        got = srv.result(rid, y0.size)
        b = sgdg.Batch()
        j = b.add(kind, D, k, n, y0, 1e-3, a=a if kind == "advect" else None)
        b.step(steps)
        assert np.array_equal(got, b.state(j)), (kind, D, k, n)
