"""Failure isolation without a GPU fault: a NaN planted in one solve's host
initial state stays in that solve.  Tiles take columns from several solves
of a class but never mix columns' arithmetic, so every other solve of a
mixed batch comes out bit for bit as without the NaN, and the request loop
reports the poisoned request as failed (SGDG_ENONFINITE) while the others
finish normally."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECS = [("advect", 2, 3, 4), ("advect", 2, 3, 4), ("advect", 2, 3, 4), ("advect", 3, 2, 3), ("advect", 3, 2, 3),
         ("wave", 2, 2, 4)]
POISONED = 1  # a solve that shares its class (and its tiles) with two others


def _inputs(sgdg):
    rng = np.random.default_rng(31)
    out = []
    for kind, D, k, n in SPECS:
        N = sgdg.get_size(D, k, n)
        y0 = rng.standard_normal(2 * N if kind == "wave" else N) * 1e-2
        out.append((kind, D, k, n, y0, rng.uniform(-1, 1, D)))
    return out


def _run_batch(sgdg, inputs, steps):
    b = sgdg.Batch()
    ids = [b.add(kind, D, k, n, y0, 1e-3, a=a if kind == "advect" else None) for kind, D, k, n, y0, a in inputs]
    b.step(steps)
    states = [b.state(i) for i in ids]
    b.close()
    return states


def test_nan_in_one_solve_leaves_the_batch_unchanged(sgdg):
    clean = _inputs(sgdg)
    poisoned = [list(x) for x in clean]
    y = poisoned[POISONED][4].copy()
    y[5] = np.nan
    poisoned[POISONED][4] = y
    ref = _run_batch(sgdg, clean, 12)
    got = _run_batch(sgdg, [tuple(x) for x in poisoned], 12)
    for i, (a, b) in enumerate(zip(got, ref)):
        if i == POISONED:
            assert not np.all(np.isfinite(a))
        else:
            assert np.all(np.isfinite(a)) and np.array_equal(a, b), i


def test_server_fails_the_nan_request_alone(sgdg):
    inputs = _inputs(sgdg)
    srv = sgdg.Server(max_chunk_steps=5)
    ids = []
    for i, (kind, D, k, n, y0, a) in enumerate(inputs):
        if i == POISONED:
            y0 = y0.copy()
            y0[5] = np.inf
        ids.append(srv.submit(kind, D, k, n, y0, 1e-3, 12, a=a if kind == "advect" else None))
    while srv.counts()[0] + srv.counts()[1] > 0:
        srv.tick()
    alone = _run_batch(sgdg, inputs, 12)
    for i, rid in enumerate(ids):
        st = srv.status(rid)[0]
        if i == POISONED:
            assert st == srv.FAILED
            with pytest.raises(sgdg.SGDGError) as e:
                srv.result(rid, inputs[i][4].size)
            assert e.value.code == 9 and "not finite" in str(e.value)
        else:
            assert st == srv.DONE
            assert np.array_equal(srv.result(rid, inputs[i][4].size), alone[i]), i
    srv.close()
