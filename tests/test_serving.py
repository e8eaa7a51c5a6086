"""The request loop (sgdg_server_*): stream generation and latency accounting
on the host, and on the GPU that every request's result is the same alone and
in the mix, under an HBM budget that forces requests to wait, and against the
FP64 oracle."""
import numpy as np
import pytest



def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def serving(sgdg):
    import importlib
    return importlib.import_module(sgdg.__name__ + ".serving")


# ------------------------------------------------------------------ host ----
def test_stream_is_seeded_and_in_range(sgdg, serving):
    a = serving.poisson_stream(sgdg, 40, rate=50.0, seed=3)
    b = serving.poisson_stream(sgdg, 40, rate=50.0, seed=3)
    assert [(r.D, r.k, r.n, r.nsteps, r.t_arrival) for r in a] == [(r.D, r.k, r.n, r.nsteps, r.t_arrival) for r in b]
    for r in a:
        assert 2 <= r.D <= 5 and r.k in (2, 3) and 4 <= r.n <= 8 and 100 <= r.nsteps <= 1000
        assert r.a.shape == (r.D,) and np.all(np.abs(r.a) <= 1.0)
        assert 2 <= len(r.modes) <= 4
        assert all(1 <= v <= 3 for m in r.modes for v in m[0])
    t = np.array([r.t_arrival for r in a])
    assert np.all(np.diff(t) > 0)
    # mean inter-arrival time near 1/rate (40 samples: loose)
    assert 0.3 / 50.0 < np.mean(np.diff(t)) < 3.0 / 50.0


def test_spectral_radius_matches_dense_eigenvalues(sgdg, serving):
    for k, n in [(2, 4), (3, 4), (2, 5)]:
        A = sgdg.periodic_DLF_matrix(k, n).toarray()
        exact = np.max(np.abs(np.linalg.eigvals(A)))
        assert abs(serving.spectral_radius_1d(sgdg, k, n) - exact) < 1e-6 * exact


def test_stable_dt_keeps_rk4_amplification_below_one(sgdg, serving):
    # RK4 amplification on the imaginary axis: |1 + z + z^2/2 + z^3/6 + z^4/24|, z = i w
    a = np.array([0.7, -0.4])
    dt = serving.stable_dt(sgdg, 3, 4, a)
    w = np.sum(np.abs(a)) * serving.spectral_radius_1d(sgdg, 3, 4) * dt
    z = 1j * np.linspace(0, w, 200)
    g = np.abs(1 + z + z ** 2 / 2 + z ** 3 / 6 + z ** 4 / 24)
    assert np.all(g <= 1.0 + 1e-12)


def test_fifo_latencies_known_answer(serving):
    lat = serving.fifo_latencies([0.0, 1.0, 1.5, 10.0], [2.0, 1.0, 0.5, 1.0])
    # starts 0, 2, 3, 10 -> ends 2, 3, 3.5, 11
    assert np.allclose(lat, [2.0, 2.0, 2.0, 1.0])
    p = serving.percentiles([1, 2, 3, 4, 100])
    assert p["p50"] == 3.0 and 4.0 < p["p99"] <= 100.0


def test_server_needs_a_gpu(sgdg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sgdg.SGDGError) as e:
        sgdg.Server()
    assert e.value.code == 6  # SGDG_ENOGPU


# ------------------------------------------------------------------- GPU ----
def _small_stream(sgdg, serving, count=10, seed=11):
    # small problems so the oracle finishes in seconds; arrivals over ~0.2 s
    reqs = serving.poisson_stream(sgdg, count, rate=50.0, seed=seed, D_range=(2, 3), n_range=(4, 5),
                                  steps_range=(15, 60))
    y0s = [serving.initial_state(sgdg, r) for r in reqs]
    return reqs, y0s


def _alone(sgdg, r, y0):
    b = sgdg.Batch()
    i = b.add(r.kind, r.D, r.k, r.n, y0, r.dt, a=r.a)
    b.step(r.nsteps)
    return b.state(i)


@pytest.mark.gpu
def test_served_results_equal_alone_and_oracle(sgdg, serving, O):
    reqs, y0s = _small_stream(sgdg, serving)
    srv = sgdg.Server(max_chunk_steps=7)  # several chunks per request: joins and leaves mid-run
    times, results, dof, makespan = serving.run_stream(sgdg, srv, reqs, y0s)
    assert all(t[3] == srv.DONE for t in times)
    assert dof == pytest.approx(sum(4.0 * y.size * r.nsteps for r, y in zip(reqs, y0s)))
    overlapped = 0
    for i, (r, y0, got) in enumerate(zip(reqs, y0s, results)):
        ta, tb, tc, _ = times[i]
        assert ta <= tb <= tc
        assert np.array_equal(got, _alone(sgdg, r, y0)), "request %d differs alone vs in the mix" % i
        ref = O.CSR(O.advection_matrix_raw(r.D, r.k, r.n, r.a)).rk4(y0, r.dt, r.nsteps, nthreads=8)
        assert rel(got, ref) < 1e-6
        # did this request share the GPU with another one?
        overlapped += any(j != i and times[j][1] < tc and tb < times[j][2] for j in range(len(reqs)))
    assert overlapped >= 2


def _max_concurrency(times):
    ev = sorted([(t[1], 1) for t in times] + [(t[2], -1) for t in times])
    c = m = 0
    for _, d in ev:
        c += d
        m = max(m, c)
    return m


@pytest.mark.gpu
def test_budget_makes_requests_wait_not_fail(sgdg, serving):
    # eight requests of one size (D=3, k=3, n=5: 7,344 coefficients), so the
    # budget below holds two of them at a time
    reqs = serving.poisson_stream(sgdg, 8, rate=50.0, seed=12, D_range=(3, 3), k_choices=(3,), n_range=(5, 5),
                                  steps_range=(15, 60))
    y0s = [serving.initial_state(sgdg, r) for r in reqs]
    # every request arrives at once (speed up the arrival clock)
    free = sgdg.Server(max_chunk_steps=5)
    ftimes, ref_results, _, _ = serving.run_stream(sgdg, free, reqs, y0s, speed=1e6)
    free.close()
    sgdg.sync()
    base = sgdg.hbm_in_use()
    need = 36 * y0s[0].size  # FP64 y, acc + FP32 u[4], rhs per coefficient
    # room for two requests at a time (tables and work lists take < 64 KB)
    sgdg.set_hbm_budget(base + int(2.5 * need) + (64 << 10))
    try:
        srv = sgdg.Server(max_chunk_steps=5)
        times, results, _, _ = serving.run_stream(sgdg, srv, reqs, y0s, speed=1e6)
        assert all(t[3] == srv.DONE for t in times)
        for got, ref in zip(results, ref_results):
            assert np.array_equal(got, ref)
        assert _max_concurrency(ftimes) == 8
        assert 1 <= _max_concurrency(times) <= 2
        # a request that cannot fit even alone fails; the server keeps going
        D, k, n = 3, 3, 7
        big = np.zeros(sgdg.get_size(D, k, n))
        rid = srv.submit("advect", D, k, n, big, 1e-3, 2, a=[1.0, 0.0, 0.0])
        srv.tick()
        assert srv.status(rid)[0] == srv.FAILED
        with pytest.raises(sgdg.SGDGError) as e:
            srv.result(rid, big.size)
        assert e.value.code == 2  # SGDG_ENOMEM_BUDGET
    finally:
        sgdg.set_hbm_budget(0)


@pytest.mark.gpu
def test_cancel_queued_and_running(sgdg, serving):
    reqs, y0s = _small_stream(sgdg, serving, count=2, seed=13)
    srv = sgdg.Server(max_chunk_steps=3)
    r0, r1 = reqs
    i0 = srv.submit("advect", r0.D, r0.k, r0.n, y0s[0], r0.dt, r0.nsteps, a=r0.a)
    i1 = srv.submit("advect", r1.D, r1.k, r1.n, y0s[1], r1.dt, r1.nsteps, a=r1.a, t_arrival=srv.clock() + 3600)
    srv.tick()
    assert srv.status(i0)[0] == srv.RUNNING and srv.status(i1)[0] == srv.QUEUED
    srv.cancel(i0)
    srv.cancel(i1)
    for i in (i0, i1):
        assert srv.status(i)[0] == srv.CANCELLED
        with pytest.raises(sgdg.SGDGError) as e:
            srv.result(i, 1)
        assert e.value.code == 5  # SGDG_ECANCELLED
    assert srv.counts()[:2] == (0, 0)


@pytest.mark.gpu
def test_snapshot_and_resume_equals_uninterrupted(sgdg):
    # checkpoint/resume of a served request: its state after some ticks,
    # submitted again for the remaining steps, ends with the same bits as the
    # uninterrupted solve (wave and advection, a neighbour request in the mix)
    rng = np.random.default_rng(21)
    for kind, D, k, n in (("wave", 3, 2, 4), ("advect", 2, 3, 5)):
        N = sgdg.get_size(D, k, n)
        y0 = rng.standard_normal(2 * N if kind == "wave" else N) * 1e-2
        a = rng.uniform(-1, 1, D) if kind == "advect" else None
        dt, nsteps = 1e-3, 23
        other = rng.standard_normal(sgdg.get_size(2, 2, 4)) * 1e-2

        full = sgdg.Server(max_chunk_steps=5)
        i_full = full.submit(kind, D, k, n, y0, dt, nsteps, a=a)
        full.submit("advect", 2, 2, 4, other, dt, 40, a=[0.3, -0.7])
        while full.status(i_full)[0] != full.DONE:
            full.tick()
        ref = full.result(i_full, y0.size)
        full.close()

        srv = sgdg.Server(max_chunk_steps=5)
        rid = srv.submit(kind, D, k, n, y0, dt, nsteps, a=a)
        y_q, done_q = srv.snapshot(rid, y0.size)  # queued: the initial state
        assert done_q == 0 and np.array_equal(y_q, y0)
        srv.submit("advect", 2, 2, 4, other, dt, 40, a=[0.3, -0.7])
        srv.tick()
        srv.tick()
        y_mid, done = srv.snapshot(rid, y0.size)
        assert srv.status(rid)[0] == srv.RUNNING and done == 10
        srv.cancel(rid)
        rid2 = srv.submit(kind, D, k, n, y_mid, dt, nsteps - done, a=a)
        while srv.status(rid2)[0] != srv.DONE:
            srv.tick()
        y_end, done_end = srv.snapshot(rid2, y0.size)  # finished: the result
        assert done_end == nsteps - done
        assert np.array_equal(srv.result(rid2, y0.size), ref)
        assert np.array_equal(y_end, ref)
        with pytest.raises(sgdg.SGDGError) as e:  # the cancelled request has no state to give
            srv.snapshot(rid, y0.size)
        assert e.value.code == 5
        srv.close()
