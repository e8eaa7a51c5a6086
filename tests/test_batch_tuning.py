"""Batches of uneven advection solves (256 solves, D in {2,3}, k in {2,3,4},
n in {4..7}) in one persistent launch per stage, with the tile shapes chosen
by the autotuner: the shapes it picks, and results against the FP64 oracle."""
import numpy as np
import pytest


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_tile_shape_defaults_and_validation(sgdg):
    w, c, tuned = sgdg.tile_shape(7, 5)
    assert (w, c) == (0, 4) and not tuned
    with pytest.raises(sgdg.SGDGError):
        sgdg.set_tile_shape(2, 3, 4, 4)  # width factor 2^4 out of range
    with pytest.raises(sgdg.SGDGError):
        sgdg.set_tile_shape(9, 3, 1, 4)  # no such D


@pytest.mark.gpu
def test_autotuned_uneven_batch_matches_oracle(sgdg, O):
    import importlib
    serving = importlib.import_module(sgdg.__name__ + ".serving")
    sgdg.clear_tile_shapes()
    specs = serving.uneven_batch(256, seed=33)
    dt = 1e-3
    b = sgdg.Batch()
    ids, y0s = [], []
    for D, k, n, a, modes in specs:
        y0 = sgdg.fourier_coeffs(D, k, n, modes)
        ids.append(b.add("advect", D, k, n, y0, dt, a=a))
        y0s.append(y0)
    ntuned = b.autotune()
    dks = {(D, k) for D, k, _, _, _ in specs}
    assert ntuned == len(dks)
    for D, k in dks:
        w, c, tuned = sgdg.tile_shape(D, k)
        assert tuned and -2 <= w <= 3 and c in (3, 4, 5, 6)
    assert b.autotune() == 0  # already tuned
    steps = 20
    b.step(steps)
    # a sample of solves against the oracle (one per (D, k) and the largest)
    picks = {}
    for i, (D, k, n, a, _) in enumerate(specs):
        picks.setdefault((D, k), i)
    picks["largest"] = int(np.argmax([y.size for y in y0s]))
    for i in picks.values():
        D, k, n, a, _ = specs[i]
        ref = O.CSR(O.advection_matrix_raw(D, k, n, a)).rk4(y0s[i], dt, steps, nthreads=8)
        assert rel(b.state(ids[i]), ref) < 1e-6, (D, k, n)
