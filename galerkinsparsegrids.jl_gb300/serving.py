"""Request streams for the matrix-free request loop (``Server``): a seeded
Poisson stream of advection solves of uneven (D, k, n), its initial states, a
driver that replays the stream against a ``Server`` in real time, and the
latency statistics reported next to the per-request plain FP64 path.

Stream parameters follow the serving workload: D in {2..5}, k in {2, 3},
n in {4..8}, velocities U(-1, 1)^D, 2-4 Fourier modes with integer wave
vectors in [1, 3]^D and amplitudes U(-1, 1), 100-1000 RK4 steps, dt at a
fixed fraction (cfl / 2.83) of the RK4 stability limit.

Precision note: the FP32 sweeps accumulate each row's products in FP32, and
the partial sums of a DG derivative cancel (entries grow like 2^n while the
result stays O(|u|)), so each apply carries a rounding error of ~1e-7 of the
state; its effect on the solution grows like dt sqrt(steps).  At cfl = 0.5 a
1000-step request stays near 1e-6 relative to the FP64 path; at cfl = 2 it
reaches a few 1e-6."""
import dataclasses
import functools
import time

import numpy as np


@dataclasses.dataclass
class Request:
    D: int
    k: int
    n: int
    a: np.ndarray          # velocity (D,)
    modes: list            # [(wave vector, amplitude, "sin"|"cos", phase)]
    nsteps: int
    dt: float
    t_arrival: float       # seconds after the stream starts
    kind: str = "advect"


@functools.lru_cache(maxsize=64)
def spectral_radius_1d(sg, k, n):
    """Largest |eigenvalue| of the 1D periodic derivative: the matrix is
    skew-symmetric, so this is its 2-norm (dense SVD; k 2^n <= a few
    thousand rows)."""
    return float(np.linalg.norm(sg.periodic_DLF_matrix(k, n).toarray(), 2))


def stable_dt(sg, k, n, a, cfl=0.5):
    """dt with |lambda| dt <= cfl for f_t = -sum_d a_d D_d f.  Each D_d acts on
    a line as a leading block of the skew 1D operator, so its norm is at most
    the 1D spectral radius; classical RK4 is stable on the imaginary axis up
    to 2 sqrt(2)."""
    return cfl / (float(np.sum(np.abs(a))) * spectral_radius_1d(sg, k, n))


def poisson_stream(sg, count, rate, seed=0, D_range=(2, 5), k_choices=(2, 3), n_range=(4, 8),
                   steps_range=(100, 1000), modes_range=(2, 4), cfl=0.5):
    """``count`` requests with exponential inter-arrival times of mean 1/rate."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        D = int(rng.integers(D_range[0], D_range[1] + 1))
        k = int(rng.choice(k_choices))
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        a = rng.uniform(-1.0, 1.0, D)
        nm = int(rng.integers(modes_range[0], modes_range[1] + 1))
        modes = [(tuple(int(v) for v in rng.integers(1, 4, D)), float(rng.uniform(-1.0, 1.0)),
                  "sin" if rng.random() < 0.5 else "cos", 0.0) for _ in range(nm)]
        nsteps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        out.append(Request(D, k, n, a, modes, nsteps, stable_dt(sg, k, n, a, cfl), t))
    return out


def uneven_batch(count, seed, D_range=(2, 3), k_range=(2, 4), n_range=(4, 7), nmodes=3):
    """Seeded solves of the uneven-batch workload: (D, k, n, velocity, modes)
    with D, k, n uniform in their ranges, velocity U(-1, 1)^D and nmodes
    Fourier modes (wave vectors in [1, 3]^D, amplitudes U(-1, 1))."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        D = int(rng.integers(D_range[0], D_range[1] + 1))
        k = int(rng.integers(k_range[0], k_range[1] + 1))
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        a = rng.uniform(-1, 1, D)
        modes = [(tuple(int(v) for v in rng.integers(1, 4, D)), float(rng.uniform(-1, 1)),
                  "sin" if rng.random() < 0.5 else "cos", 0.0) for _ in range(nmodes)]
        out.append((D, k, n, a, modes))
    return out


def initial_state(sg, r):
    return sg.fourier_coeffs(r.D, r.k, r.n, r.modes)


def run_stream(sg, server, reqs, y0s, speed=1.0):
    """Replays ``reqs`` against ``server`` in real time (arrival times divided
    by ``speed``): every request is submitted up front with its arrival time
    and the server holds it back until then.  Returns per-request
    (t_arrival, t_admit, t_done) on the server clock, the results, the
    DOF-updates executed and the wall time from the first arrival to the
    last completion."""
    t0 = server.clock() + 0.05
    ids = []
    for r, y0 in zip(reqs, y0s):
        ids.append(server.submit(r.kind, r.D, r.k, r.n, y0, r.dt, r.nsteps, a=r.a,
                                 t_arrival=t0 + r.t_arrival / speed))
    pending = set(range(len(ids)))
    times = [None] * len(ids)
    results = [None] * len(ids)
    while pending:
        server.tick()
        q, running, _, _ = server.counts()
        for i in list(pending):
            st, _, ta, tb, tc = server.status(ids[i])
            if st in (server.DONE, server.FAILED, server.CANCELLED):
                times[i] = (ta, tb, tc, st)
                try:
                    results[i] = server.result(ids[i], y0s[i].size)
                except Exception as e:  # failed or cancelled: keep the error
                    results[i] = e
                pending.discard(i)
        if pending and running == 0:
            # nothing on the GPU: sleep until the next arrival
            wait = min(t0 + reqs[i].t_arrival / speed for i in pending) - server.clock()
            if wait > 0:
                time.sleep(min(wait, 0.05))
    dof = server.counts()[3]
    first = min(t[0] for t in times)
    last = max(t[2] for t in times)
    return times, results, dof, last - first


def fifo_latencies(arrivals, service):
    """Latencies of a single first-in-first-out server that serves requests
    one at a time with the given service times."""
    free = -np.inf
    lat = []
    for ta, s in zip(arrivals, service):
        start = max(ta, free)
        free = start + s
        lat.append(free - ta)
    return np.array(lat)


def percentiles(x, ps=(50, 99)):
    x = np.asarray(x, np.float64)
    return {"p%d" % p: float(np.percentile(x, p)) for p in ps}
