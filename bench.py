#!/usr/bin/env python
"""Benchmark of the sparse-grid DG derivative operator inside RK4 time stepping.

Workload (one GPU): the 3D wave equation as a first-order system on the
periodic unit cube, sparse grid k=3, n=7 (N = 45,792 coefficients per field,
state 2N = 91,584), seeded 6-mode Fourier initial conditions, classical RK4
with dt = 2.5e-3 (spectral radius 1034, rho*dt = 2.58).  A batch of
independent solves of that problem (different seeds) advances together; one
bench step = one RK4 step (4 stages) of every solve in the batch.  The batch
working set (~0.6 GB at 256 solves) exceeds the 126 MB L2, so no L2 flush is
needed between steps.

value:  DOF-updates/s = state coefficients x RK stages / time, FP32
        matrix-free apply with FP64 RK state, inputs resident in HBM.
e2e:    the same metric through the C ABI with host buffers: every timed step
        uploads all states from page-locked host memory, advances one RK4
        step and downloads all states.
plain_fp64_batch: the drop-in form (assembled FP64 CSR SpMV + FP64 RK4) on the
        same batch of solves, device-resident, at equal work.
uneven_batch: 256 advection solves of uneven (D, k, n) in the same launches,
        with default and with autotuned tile shapes.
vlasov: Vlasov transport in 2x2v phase space (k=2, n=8), FP64 sparse form.
cpu_baseline: the FP64 CPU oracle (OpenMP, all host threads) on a bounded
        sample; it also checks the error of solve 0 against the GPU result.
serving: a seeded Poisson stream of advection requests of uneven (D, k, n)
        through the request loop (continuous batching), p50/p99 latency and
        DOF-updates/s, beside the plain per-request FP64 path (FIFO).

--impl reference times the reference's CPU implementation of the path: the
Julia package cannot run here (no julia), so its C restatement (oracle/) runs
with all host threads on the same workload, a bounded sample per step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

D, K, NLEV, DT = 3, 3, 7, 2.5e-3
METRIC = "DOF-updates/s per RK stage"
UNIT = "DOF-updates/s"
BYTES_PER_DOF_UPDATE = 32.0  # read u fp32 + write u fp32 + read y fp64 + r/w acc fp64


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--solves", type=int, default=256)
    p.add_argument("--e2e-steps", type=int, default=50, help="calls per repeat of the end-to-end leg (3 repeats)")
    p.add_argument("--e2e-chunks", type=int, default=16, help="pipeline chunks of the end-to-end leg")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--vlasov-steps", type=int, default=500, help="RK4 steps of the 2x2v Vlasov leg (0: skip)")
    p.add_argument("--serve-requests", type=int, default=32, help="requests in the serving stream (0: skip)")
    p.add_argument("--eval-points", type=int, default=1 << 20, help="points of the evaluation leg (0: skip)")
    p.add_argument("--assembly", type=int, default=1, help="time GPU vs host operator assembly (0: skip)")
    p.add_argument("--serve-rate", type=float, default=20.0, help="Poisson arrival rate of the stream, 1/s")
    p.add_argument("--serve-chunk", type=int, default=25, help="max RK4 steps between admissions")
    return p.parse_args()


def max_over_ranks(x, dist, device):
    """The maximum of a per-rank scalar over all ranks (a job takes as long as
    its slowest rank); x itself when running alone."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank_step, steps, world, seconds):
    """Whole-job units per second: each rank advances its own replica of the
    workload (no exchange), so the job's units are world times one rank's."""
    return units_per_rank_step * steps * world / seconds


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def wave_modes(seed):
    """Seeded 6-mode Fourier f0 and v0 of one solve, wave vectors in [1,3]^3,
    amplitudes U(-1,1) (the shape of the reference's traveling-wave inputs)."""
    rng = np.random.default_rng(seed)
    fields = []
    for _ in range(2):
        modes = []
        for _ in range(6):
            a = tuple(int(v) for v in rng.integers(1, 4, size=D))
            modes.append((a, float(rng.uniform(-1, 1)), "sin" if rng.random() < 0.5 else "cos", 0.0))
        fields.append(modes)
    return fields


def initial_states(fourier_coeffs, nsolves, seed0):
    """[f0; v0] per solve from the seeded modes; fourier_coeffs is the
    package's (the timed arms) or the oracle's (the reference arm)."""
    return [np.concatenate([fourier_coeffs(D, K, NLEV, m) for m in wave_modes(seed0 + s)]) for s in range(nsolves)]


def workload_config(solves, state_dofs):
    """The workload both arms time: the same dict in both JSON lines."""
    return {"workload": "wave3d_sparse_k3_n7_batch", "D": D, "k": K, "n": NLEV, "dt": DT,
            "solves_per_gpu": solves, "state_dofs_per_solve": int(state_dofs),
            "l2": "working set > 126 MB L2, no flush"}


class Clocks:
    """nvidia-smi samples (20 ms apart, time-stamped) from before the batch is
    built to after the timed region; stop() keeps the samples taken inside the
    timed region or in the 0.5 s of warm-up steps right before it (the same
    kernel under load), since the timed region alone can be shorter than one
    sample interval."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self, t0=None, t1=None):
        """t0, t1: the timed region (time.time())."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        import datetime
        sm, smax, reasons, inside = [], [], set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                mhz, mx = float(parts[1]), float(parts[2])
            except ValueError:
                continue
            if t0 is not None and not (t0 - 0.5 <= ts <= t1 + 0.05):
                continue
            inside += 1 if t0 is None or ts >= t0 else 0
            sm.append(mhz)
            smax.append(mx)
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "samples_in_timed_region": inside,
                "window": "timed region and the 0.5 s of warm-up before it", "reasons": sorted(reasons)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_mf_stage_wave3d.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def cpu_oracle_leg(y0, gpu_state, steps, nthreads):
    """Times the oracle's FP64 CSR RK4 on one solve and returns (DOF-updates/s,
    seconds, threads, (rel L2, rel Linf) error of the GPU state)."""
    from oracle import oracle as O
    A = O.CSR(O.wave_rhs_raw(D, K, NLEV))
    A.rk4(y0, DT, 1, nthreads=nthreads)  # warm
    t = time.perf_counter()
    ref = A.rk4(y0, DT, steps, nthreads=nthreads)
    el = time.perf_counter() - t
    err = None
    if gpu_state is not None:
        err = (float(np.linalg.norm(gpu_state - ref) / np.linalg.norm(ref)),
               float(np.max(np.abs(gpu_state - ref)) / np.max(np.abs(ref))))
    return y0.size * 4.0 * steps / el, el, nthreads, err


def timed_steps(b, stream, steps, warmup):
    import torch
    for _ in range(warmup):
        b.step(1)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        b.step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def uneven_batch_leg(sg, stream, steps=50, warmup=5):
    """256 independent advection solves, D in {2,3}, k in {2,3,4}, n in
    {4..7}, one persistent launch per RK4 step: default tile shapes, then the
    autotuned ones."""
    import importlib
    sv = importlib.import_module(sg.__name__ + ".serving")
    specs = sv.uneven_batch(256, seed=33)
    saved = {(d, k): sg.tile_shape(d, k) for d in (2, 3) for k in (2, 3, 4)}
    sg.clear_tile_shapes()
    b = sg.Batch()
    b.set_stream(stream.cuda_stream)
    for d, k, n, a, modes in specs:
        b.add("advect", d, k, n, sg.fourier_coeffs(d, k, n, modes), 1e-3, a=a)
    _, dofs = b.step_info()
    ms_default = timed_steps(b, stream, steps, warmup)
    b.autotune()
    ms_tuned = timed_steps(b, stream, steps, warmup)
    shapes = {"D%d_k%d" % (d, k): list(sg.tile_shape(d, k)[:2]) for d in (2, 3) for k in (2, 3, 4)}
    total = b.total_size()
    b.close()
    for (d, k), (w, c, tuned) in saved.items():
        if tuned:
            sg.set_tile_shape(d, k, w, c)
    return {"workload": "256 advection solves, D 2-3, k 2-4, n 4-7, dt 1e-3", "state_dofs": int(total),
            "working_set_bytes": int(36 * total), "steps": steps,
            "default_tiles": {"value": dofs / (ms_default / 1e3), "ms_per_step": ms_default},
            "autotuned_tiles": {"value": dofs / (ms_tuned / 1e3), "ms_per_step": ms_tuned},
            "shapes_wlog_coop": shapes}


def vlasov_leg(sg, stream, steps, batch=16):
    """Vlasov-type transport in 2x2v phase space (D = 2 space dimensions),
    sparse k=2, n=8: seeded force E(x) of amplitude 0.1, Maxwellian in v
    (sigma 0.15) times (1 + 0.05 cos 2 pi x_1), RK4.  Two forms: FP64 sparse
    operators on the GPU (derivatives, nodal transforms, point products), and
    the matrix-free FP32 form (pencil sweeps of the transforms, FP64 RK state)
    for one solve and for a batch of independent solves in one launch per
    RK4 step; the two forms' results after the same steps are compared."""
    import importlib
    W = importlib.import_module(sg.__name__ + ".workloads")
    sv = importlib.import_module(sg.__name__ + ".serving")
    Dx, k, n = 2, 2, 8
    t0 = time.perf_counter()
    op = sg.VlasovOperator(Dx, k, n)
    op.v_point()  # builds the device operators (derivatives, transforms) on the GPU
    setup = time.perf_counter() - t0
    F, f0 = W.vlasov_case(sg, Dx, k, n, seed=11)
    rho = sv.spectral_radius_1d(sg, k, n)
    dt = 1.0 / (rho * (Dx * 1.0 + float(np.sum(np.max(np.abs(F), axis=1)))))
    sg.vlasov_evolve(Dx, k, n, F, f0, 0.0, dt, nsteps=1, op=op)  # warm: device copies, graph
    t1 = time.perf_counter()
    sg.vlasov_evolve(Dx, k, n, F, f0, 0.0, dt, nsteps=1, op=op)
    one = time.perf_counter() - t1
    t1 = time.perf_counter()
    _, st = sg.vlasov_evolve(Dx, k, n, F, f0, 0.0, steps * dt, nsteps=steps, op=op)
    total = time.perf_counter() - t1
    per_step = max(total - one, 1e-9) / max(steps - 1, 1)
    op.close()
    N = int(f0.size)
    out = {"workload": "Vlasov 2x2v (D=4 phase space), sparse k=2, n=8, RK4", "state_dofs": N,
           "steps": steps, "dt": dt, "unit": UNIT,
           "plain_fp64": {"form": "FP64 sparse operators (CSR SpMV), graph per RK4 step",
                          "value": N * 4.0 / per_step, "ms_per_step": 1e3 * per_step,
                          "wall_s_end_to_end": total, "setup_s": setup},
           "rel_l2_change_of_f": float(np.linalg.norm(st[-1] - f0) / np.linalg.norm(f0))}
    # matrix-free, one solve: same steps, then the difference to the FP64 result
    b = sg.Batch()
    b.set_stream(stream.cuda_stream)
    b.add_vlasov(Dx, k, n, f0, F, dt)
    b.autotune()  # the tile shape of (4, 2) is kept for the batches below
    b.close()
    b = sg.Batch()
    b.set_stream(stream.cuda_stream)
    i = b.add_vlasov(Dx, k, n, f0, F, dt)
    b.step(steps)
    mf = b.state(i)
    ms_one = timed_steps(b, stream, 20, 3)
    b.close()
    out["matfree_one"] = {"form": "FP32 pencil sweeps, FP64 RK state, graph per RK4 step",
                          "value": N * 4.0 / (ms_one / 1e3), "ms_per_step": ms_one,
                          "rel_l2_vs_plain_fp64": float(np.linalg.norm(mf - st[-1]) / np.linalg.norm(st[-1]))}
    # matrix-free, a batch of independent solves (different seeded forces and data)
    b = sg.Batch()
    b.set_stream(stream.cuda_stream)
    for s in range(batch):
        Fs, fs = W.vlasov_case(sg, Dx, k, n, seed=100 + s)
        b.add_vlasov(Dx, k, n, fs, Fs, dt)
    b.autotune()
    ms_b = timed_steps(b, stream, 20, 3)
    b.close()
    rate = batch * N * 4.0 / (ms_b / 1e3)
    # algorithmic bytes per DOF-update: the RK state's 32 B (as for the wave)
    # and the point weights of the 2 Dx products, an FP32 hi/lo pair each
    bpd = BYTES_PER_DOF_UPDATE + 2 * (2 * Dx) * 4.0
    peak, peak_kind = measured_peak_hbm()
    out["matfree_batch"] = {"solves": batch, "value": rate, "ms_per_step": ms_b,
                            "roofline": {"bound": "hbm", "achieved": rate * bpd / 1e9, "peak": peak, "unit": "GB/s",
                                         "frac": rate * bpd / 1e9 / peak, "peak_kind": peak_kind,
                                         "bytes_per_dof_update": bpd,
                                         "working_set_bytes": int(batch * N * (32 + 4 + 4 * 4 * (2 * Dx)))}}
    return out


def evaluate_leg(sg, stream, npts):
    """Point evaluation (reconstruct_DG) of a 3D sparse k=3, n=7 expansion
    (seeded Fourier coefficients) at npts uniform points, FP64 on the GPU:
    device-resident (CUDA events around sgdg_evaluate_device) and end to end
    through sgdg_evaluate with host buffers; FP64 operations counted per point
    from the level blocks (k^(D-1) (2k + 2 + D - 1) per block) and the 1D
    tables (2 k^2 per dimension and level)."""
    import ctypes
    import torch
    Dv, kv, nv = 3, 3, 7
    rng = np.random.default_rng(21)
    modes = [(tuple(int(v) for v in rng.integers(1, 4, Dv)), float(rng.uniform(-1, 1)),
              "sin" if rng.random() < 0.5 else "cos", 0.0) for _ in range(6)]
    c = sg.fourier_coeffs(Dv, kv, nv, modes)
    pts = rng.random((npts, Dv))
    dc = torch.from_numpy(c).to("cuda")
    dx = torch.from_numpy(pts).to("cuda")
    dv = torch.empty(npts, dtype=torch.float64, device="cuda")
    L = sg._lib.lib()

    def run():
        sg.check(L.sgdg_evaluate_device(Dv, kv, nv, 0, ctypes.c_void_p(dc.data_ptr()), npts,
                                        ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dv.data_ptr()),
                                        ctypes.c_void_p(stream.cuda_stream)))
    for _ in range(3):
        run()
    torch.cuda.synchronize()
    reps = 10
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nlev = len({tuple(r) for r in sg.index_map(Dv, kv, nv)[0]})
    # FP64 operations per point (an FMA counts 2): per level block, with two
    # dimensions contracted first (D >= 3), k^(D-2) (2k^2 + 2k + D), else
    # k^(D-1) (2k + D + 1); plus the 1D basis tables
    per_block = kv ** (Dv - 2) * (2 * kv * kv + 2 * kv + Dv) if Dv >= 3 else kv ** (Dv - 1) * (2 * kv + Dv + 1)
    flops = npts * (nlev * per_block + Dv * (nv + 1) * 2 * kv * kv)
    t0 = time.perf_counter()
    vals = sg.reconstruct_DG(Dv, kv, nv, c, pts)
    e2e = time.perf_counter() - t0
    return {"workload": "reconstruct_DG, 3D sparse k=3 n=7 expansion at %d uniform points, FP64" % npts,
            "points": npts, "value": npts / (ms / 1e3), "unit": "points/s", "ms": ms,
            "fp64_gflops": flops / (ms / 1e3) / 1e9, "fp64_nominal_gflops": 1250.0,
            "e2e": {"value": npts / e2e, "unit": "points/s", "h2d_bytes": int(c.nbytes + pts.nbytes),
                    "d2h_bytes": int(vals.nbytes)},
            "max_abs_diff_device_vs_host_api": float(np.max(np.abs(dv.cpu().numpy() - vals)))}


def assembly_leg(sg, D=4, k=3, n=7):
    """Time to the plain form's wave right-hand side [[0, I], [L, 0]] with
    L = sum_d D_d D_d for a 4D sparse k=3, n=7 grid (327,888 DOF): assembled
    on the GPU (the operator the plain evolvers use) and on the host (CSR
    products, the exported operator); both hold the same entries."""
    L = sg._lib.lib()
    import ctypes
    op = sg.SparseGridOperator(D, k, n)
    z = ctypes.c_int64()
    t0 = time.perf_counter()
    sg.check(L.sgdg_op_device_nnz(op._h, -1, ctypes.byref(z)))
    gpu_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    nnz_host = op.nnz(-1)
    host_s = time.perf_counter() - t0
    op.close()
    return {"workload": "wave RHS of the plain form, %dD sparse k=%d n=%d (%d DOF)" % (D, k, n, sg.get_size(D, k, n)),
            "nnz": int(z.value), "gpu_s": gpu_s, "host_s": host_s, "same_nnz": int(z.value) == int(nnz_host)}


def plain_fifo(sg, reqs, y0s, ops):
    """The plain per-request FP64 path run on the GPU as a single first-in-
    first-out server in real time: each request, once it has arrived and the
    previous one is done, assembles -sum_d a_d D_d on the GPU and runs its RK4
    steps (advect_evolve, method plain, host state in and out).  Returns the
    latencies, the results and the wall time from the first arrival to the
    last completion."""
    t0 = time.perf_counter() + 0.05
    lat, results, last = [], [], t0
    for r, y0 in zip(reqs, y0s):
        arrive = t0 + r.t_arrival
        wait = arrive - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        op = ops[(r.D, r.k, r.n)]
        _, st = sg.advect_evolve(r.D, r.k, r.n, r.a, y0, 0.0, r.nsteps * r.dt, nsteps=r.nsteps, method="plain", op=op)
        last = time.perf_counter()
        lat.append(last - arrive)
        results.append(st[-1])
    return np.array(lat), results, last - (t0 + reqs[0].t_arrival)


def serving_leg(sg, args):
    """Poisson stream of advection requests of uneven (D, k, n) through the
    request loop (continuous batching), and the same stream through the plain
    per-request FP64 path, run for real on the GPU as a FIFO server (the
    index and 1D tables of each (D, k, n) built beforehand, as a serving
    process would keep them); every served result is compared with its plain
    FP64 result."""
    import importlib
    sv = importlib.import_module(sg.__name__ + ".serving")
    reqs = sv.poisson_stream(sg, args.serve_requests, args.serve_rate, seed=5)
    y0s = [sv.initial_state(sg, r) for r in reqs]
    srv = sg.Server(max_chunk_steps=args.serve_chunk)
    # warm-up: one short request per (k, n) so every 1D table exists before the stream
    for k, n in sorted({(r.k, r.n) for r in reqs}):
        N = sg.get_size(2, k, n)
        srv.submit("advect", 2, k, n, np.zeros(N), 1e-3, 1, a=[1.0, 0.0])
    while srv.counts()[0] + srv.counts()[1] > 0:
        srv.tick()
    srv.close()
    srv = sg.Server(max_chunk_steps=args.serve_chunk)
    times, results, dof, makespan = sv.run_stream(sg, srv, reqs, y0s)
    lat = np.array([t[2] - t[0] for t in times])
    wait = np.array([t[1] - t[0] for t in times])
    ok = sum(1 for t in times if t[3] == srv.DONE)
    srv.close()

    # plain per-request FP64 path, warmed with one step of every (D, k, n)
    ops = {}
    for r, y0 in zip(reqs, y0s):
        key = (r.D, r.k, r.n)
        if key not in ops:
            ops[key] = sg.SparseGridOperator(r.D, r.k, r.n)
            sg.advect_evolve(r.D, r.k, r.n, r.a, y0, 0.0, r.dt, nsteps=1, method="plain", op=ops[key])
    plain_lat, plain_res, plain_makespan = plain_fifo(sg, reqs, y0s, ops)
    for op in ops.values():
        op.close()
    total_dof = float(sum(4.0 * y.size * r.nsteps for r, y in zip(reqs, y0s)))
    errs = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(results, plain_res)]
    big = int(np.argmax([y.size for y in y0s]))

    return {
        "workload": "Poisson stream of advection solves, D 2-5, k 2-3, n 4-8, 100-1000 RK4 steps",
        "requests": len(reqs), "completed": ok, "arrival_rate_per_s": args.serve_rate,
        "max_chunk_steps": args.serve_chunk, "state_dofs": int(sum(y.size for y in y0s)),
        "matfree": {"p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                    "p50_queue_wait_s": float(np.percentile(wait, 50)),
                    "dof_updates_per_s": dof / makespan, "makespan_s": makespan},
        "plain_fp64_per_request": {"p50_latency_s": float(np.percentile(plain_lat, 50)),
                                   "p99_latency_s": float(np.percentile(plain_lat, 99)),
                                   "dof_updates_per_s": total_dof / plain_makespan, "makespan_s": plain_makespan,
                                   "run": "FIFO on the GPU in real time, assembly of -sum_d a_d D_d per request"},
        "rel_l2_vs_plain_fp64": {"max": max(errs), "median": float(np.median(errs)), "requests": len(errs),
                                 "largest_request": {"D": reqs[big].D, "k": reqs[big].k, "n": reqs[big].n,
                                                     "dofs": int(y0s[big].size), "steps": reqs[big].nsteps,
                                                     "rel_l2": errs[big]}},
    }


REF_SAMPLE_SOLVES = 16  # solves the reference arm advances per timed step


def run_reference(args):
    """The reference's CPU path on the host cores: Julia is not installed, so
    the oracle's C restatement (FP64 CSR SpMV + RK4, OpenMP on every host
    thread) advances a bounded sample of the batch's solves per step.  Only
    the oracle is loaded (initial states from its own Fourier projection)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    nth = O.max_threads()
    sample = max(1, min(args.solves, REF_SAMPLE_SOLVES))
    ys = initial_states(O.fourier_coeffs, sample, 1000)
    A = O.CSR(O.wave_rhs_raw(D, K, NLEV))
    for _ in range(args.warmup):
        ys = [A.rk4(y, DT, 1, nthreads=nth) for y in ys]
    t = time.perf_counter()
    for _ in range(args.steps):
        ys = [A.rk4(y, DT, 1, nthreads=nth) for y in ys]
    el = time.perf_counter() - t
    value = sample * ys[0].size * 4.0 * args.steps / el
    desc = ("%d of the %d solves per step (every solve has the same operator and cost), one RK4 step each, "
            "FP64 CSR oracle" % (sample, args.solves))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps * args.solves / sample,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Fourier ICs)", "config": workload_config(args.solves, ys[0].size),
            "form": "FP64 CSR SpMV + FP64 RK4 (the oracle's C restatement of the reference, OpenMP)",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference is Julia (not installed here or on the GPU host); its C restatement in oracle/ is timed"}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    torch.cuda.set_device(local)
    import __graft_entry__ as g
    sg = g.load_package()
    dev = torch.device("cuda", local)
    # a dedicated (non-default) stream: the library launches on it and the
    # CUDA events below are recorded on it
    stream = torch.cuda.Stream(device=dev)

    clk = Clocks(local)
    clk.start()
    states = initial_states(sg.fourier_coeffs, args.solves, 1000 + 100000 * rank)
    b = sg.Batch()
    ids = [b.add("wave", D, K, NLEV, y0, DT) for y0 in states]
    b.set_stream(stream.cuda_stream)
    sg.clear_tile_shapes()
    b.autotune()  # tile shape of (D, k) tuned on this batch (no state change)
    tile = sg.tile_shape(D, K)
    launches_per_step, dofs_per_step = b.step_info()

    for _ in range(args.warmup):
        b.step(1)
    torch.cuda.synchronize()

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    tw0 = time.time()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    tw1 = time.time()
    if dist:
        dist.barrier()
    clocks = clk.stop(tw0, tw1)
    ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    gpu_state0 = b.state(ids[0]) if rank == 0 else None
    value = job_rate(dofs_per_step, args.steps, world, ms / 1e3)

    # end to end through the C ABI with host buffers
    total = b.total_size()
    host = torch.empty(total, dtype=torch.float64, pin_memory=True)
    b.download(host.data_ptr())
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    # one call per step: host states in, one RK4 step, host states out, with
    # the copies of each pipeline chunk overlapping the other chunks' steps;
    # three repeats of e2e_steps calls, the median reported
    b.step_host(host.data_ptr(), host.data_ptr(), 1, args.e2e_chunks)  # builds the chunk graphs
    reps = []
    for _ in range(3):
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            b.step_host(host.data_ptr(), host.data_ptr(), 1, args.e2e_chunks)
        reps.append(max_over_ranks(time.perf_counter() - t0, dist, dev))
    e2e_s = statistics.median(reps)
    e2e_value = job_rate(dofs_per_step, args.e2e_steps, world, e2e_s)
    # the same without the pipeline: upload, step, download in turn
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        b.upload(host.data_ptr())
        b.step(1)
        b.download(host.data_ptr())
    e2e_serial = job_rate(dofs_per_step, args.e2e_steps, world, max_over_ranks(time.perf_counter() - t0, dist, dev))
    b.close()
    del host

    # the plain FP64 drop-in form on the same batch: every solve's
    # *(RHS, x) (src/pdes.jl:63) as an FP64 CSR SpMV fused with the RK4 stage
    # update, all solves of a stage in one launch, states resident in HBM
    op = sg.SparseGridOperator(D, K, NLEV)
    plain_nnz = op.nnz(-1)
    ydev = torch.tensor(np.concatenate(states), dtype=torch.float64, device=dev)
    plain_warm, plain_steps = 3, max(3, min(args.steps, 20))
    op.plain_steps_device(ydev.data_ptr(), args.solves, DT, plain_warm, stream=stream.cuda_stream)  # device operator
    timings = []
    for ns in (1, 1 + plain_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op.plain_steps_device(ydev.data_ptr(), args.solves, DT, ns, stream=stream.cuda_stream)
        timings.append(time.perf_counter() - t0)
    plain_s = max_over_ranks(max(timings[1] - timings[0], 1e-9), dist, dev)  # the fixed cost of a call cancels
    plain_value = job_rate(dofs_per_step, plain_steps, world, plain_s)
    plain_done = plain_warm + 2 + plain_steps
    plain_state0 = ydev[:states[0].size].cpu().numpy() if rank == 0 else None
    del ydev
    op.close()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    cpu = None
    from oracle import oracle as O
    if not args.no_cpu:
        cpu = cpu_oracle_leg(states[0], gpu_state0, args.warmup + args.steps, O.max_threads())
    # the plain batch's solve 0 against the oracle after the same steps
    ref0 = O.CSR(O.wave_rhs_raw(D, K, NLEV)).rk4(states[0], DT, plain_done, nthreads=O.max_threads())
    plain_err = float(np.linalg.norm(plain_state0 - ref0) / np.linalg.norm(ref0))

    peak, peak_kind = measured_peak_hbm()
    step_s = ms / 1e3 / args.steps
    achieved = BYTES_PER_DOF_UPDATE * dofs_per_step / step_s / 1e9
    prof = profiled_traffic()
    traffic = None
    if prof:
        # per-launch DRAM bytes scaled to this batch from the profiled case
        traffic = prof.get("dram_bytes_per_launch_per_solve", 0) * args.solves
    working_set = total * (8 + 8 + 4 * 4) + args.solves * (total // args.solves // 2) * 4
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 apply / f64 RK state", "data": "synthetic (seeded Fourier ICs)",
        "config": workload_config(args.solves, total // args.solves),
        "form": "matrix-free FP32 pencil apply, FP64 RK4, CUDA graph per step",
        "working_set_bytes_per_gpu": int(working_set), "tile_shape_wlog_coop": list(tile[:2]),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(total * 8),
                "d2h_bytes_per_step": int(total * 8), "steps": args.e2e_steps, "pipeline_chunks": args.e2e_chunks,
                "serial_upload_step_download": e2e_serial},
        "gpu_launches": int(launches_per_step * args.steps),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "bytes_per_dof_update": BYTES_PER_DOF_UPDATE},
        "plain_fp64_batch": {"form": "FP64 CSR SpMV + FP64 RK4 stage update per solve, all solves of a stage in "
                                     "one launch, CUDA graph per step (sgdg_op_plain_steps_device)",
                             "value": plain_value, "unit": UNIT, "solves": args.solves, "nnz": int(plain_nnz),
                             "steps": plain_steps, "ms_per_step": 1e3 * plain_s / plain_steps,
                             "chosen_over_plain": value / plain_value,
                             "rel_l2_vs_oracle": {"value": plain_err, "solve": 0, "steps": plain_done}},
        "clocks": clocks,
    }
    line["uneven_batch"] = uneven_batch_leg(sg, stream)
    if args.vlasov_steps > 0:
        line["vlasov"] = vlasov_leg(sg, stream, args.vlasov_steps)
    if args.serve_requests > 0:
        line["serving"] = serving_leg(sg, args)
    if args.assembly:
        line["assembly"] = assembly_leg(sg)
    if args.eval_points > 0:
        line["evaluate"] = evaluate_leg(sg, stream, args.eval_points)
    if cpu:
        line["cpu_baseline"] = {"value": cpu[0], "unit": UNIT, "cores": cpu[2], "kind": "port",
                                "sample": "1 solve, %d RK4 steps (%.1f s), FP64 CSR oracle" % (
                                    args.warmup + args.steps, cpu[1])}
        line["err_vs_oracle"] = {"rel_l2": cpu[3][0], "rel_linf": cpu[3][1], "solve": 0,
                                 "steps": args.warmup + args.steps}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
