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
plain_fp64: the drop-in form (assembled FP64 CSR SpMV + FP64 RK4) on one solve.
cpu_baseline: the FP64 CPU oracle (OpenMP, all host threads) on a bounded
        sample; it also checks the error of solve 0 against the GPU result.

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
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def initial_states(sg, nsolves, seed0):
    """Seeded 6-mode Fourier f0 and v0 per solve, wave vectors in [1,3]^3,
    amplitudes U(-1,1) (the shape of the reference's traveling-wave inputs)."""
    out = []
    for s in range(nsolves):
        rng = np.random.default_rng(seed0 + s)
        fields = []
        for _ in range(2):
            modes = []
            for _ in range(6):
                a = tuple(int(v) for v in rng.integers(1, 4, size=D))
                modes.append((a, float(rng.uniform(-1, 1)), "sin" if rng.random() < 0.5 else "cos", 0.0))
            fields.append(sg.fourier_coeffs(D, K, NLEV, modes))
        out.append(np.concatenate(fields))
    return out


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
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
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


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
    seconds, threads, rel L2 error of the GPU state)."""
    from oracle import oracle as O
    A = O.CSR(O.wave_rhs_raw(D, K, NLEV))
    A.rk4(y0, DT, 1, nthreads=nthreads)  # warm
    t = time.perf_counter()
    ref = A.rk4(y0, DT, steps, nthreads=nthreads)
    el = time.perf_counter() - t
    err = None
    if gpu_state is not None:
        err = float(np.linalg.norm(gpu_state - ref) / np.linalg.norm(ref))
    return y0.size * 4.0 * steps / el, el, nthreads, err


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    import __graft_entry__ as g
    sg = g.load_package()
    y0 = initial_states(sg, 1, 1000)[0]
    nth = O.max_threads()
    A = O.CSR(O.wave_rhs_raw(D, K, NLEV))
    y = y0.copy()
    for _ in range(args.warmup):
        y = A.rk4(y, DT, 1, nthreads=nth)
    t = time.perf_counter()
    for _ in range(args.steps):
        y = A.rk4(y, DT, 1, nthreads=nth)
    el = time.perf_counter() - t
    value = y0.size * 4.0 * args.steps / el
    sample = "1 of the %d solves per step (solves are identical in cost), RK4 steps on the host" % args.solves
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Fourier ICs)",
            "config": {"workload": "wave3d_sparse_k3_n7", "D": D, "k": K, "n": NLEV, "dt": DT,
                       "state_dofs_per_solve": int(y0.size), "form": "FP64 CSR SpMV + FP64 RK4 (oracle port)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference is Julia (not installed); its C restatement in oracle/ is timed"}
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

    states = initial_states(sg, args.solves, 1000 + 100000 * rank)
    b = sg.Batch()
    ids = [b.add("wave", D, K, NLEV, y0, DT) for y0 in states]
    b.set_stream(stream.cuda_stream)
    launches_per_step, dofs_per_step = b.step_info()

    for _ in range(args.warmup):
        b.step(1)
    torch.cuda.synchronize()

    clk = Clocks(local)
    clk.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    gpu_state0 = b.state(ids[0]) if rank == 0 else None
    value = dofs_per_step * args.steps * world / (ms / 1e3)

    # end to end through the C ABI with host buffers
    total = b.total_size()
    host = torch.empty(total, dtype=torch.float64, pin_memory=True)
    b.download(host.data_ptr())
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        b.upload(host.data_ptr())
        b.step(1)
        b.download(host.data_ptr())
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = dofs_per_step * args.e2e_steps * world / e2e_s

    # plain FP64 drop-in form on one solve (same problem)
    op = sg.SparseGridOperator(D, K, NLEV)
    f0, v0 = states[0][:op.N], states[0][op.N:]
    sg.wave_evolve(D, K, NLEV, f0, v0, 0.0, DT, nsteps=1, method="plain", op=op)  # assemble + upload once
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sg.wave_evolve(D, K, NLEV, f0, v0, 0.0, args.steps * DT, nsteps=args.steps, method="plain", op=op)
    plain_s = time.perf_counter() - t0
    plain_value = 2 * op.N * 4.0 * args.steps / plain_s
    plain_nnz = op.nnz(-1)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        cpu = cpu_oracle_leg(states[0], gpu_state0, args.warmup + args.steps, O.max_threads())

    peak, peak_kind = measured_peak_hbm()
    step_s = ms / 1e3 / args.steps
    achieved = BYTES_PER_DOF_UPDATE * dofs_per_step / step_s / 1e9
    prof = profiled_traffic()
    traffic = None
    if prof:
        # per-launch DRAM bytes scaled to this batch from the profiled case
        traffic = prof.get("dram_bytes_per_launch_per_solve", 0) * args.solves
    working_set = total * (8 + 8 + 4 + 4) + args.solves * (total // args.solves // 2) * 4
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 apply / f64 RK state", "data": "synthetic (seeded Fourier ICs)",
        "config": {"workload": "wave3d_sparse_k3_n7_batch", "D": D, "k": K, "n": NLEV, "dt": DT,
                   "solves_per_gpu": args.solves, "state_dofs_per_solve": int(total // args.solves),
                   "working_set_bytes_per_gpu": int(working_set), "l2": "working set > 126 MB L2, no flush",
                   "form": "matrix-free FP32 pencil apply, FP64 RK4, CUDA graph per step"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(total * 8),
                "d2h_bytes_per_step": int(total * 8), "steps": args.e2e_steps},
        "gpu_launches": int(launches_per_step * args.steps),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "bytes_per_dof_update": BYTES_PER_DOF_UPDATE},
        "plain_fp64": {"value": plain_value, "unit": UNIT, "solves": 1, "nnz": int(plain_nnz),
                       "ms_per_step": 1e3 * plain_s / args.steps},
        "clocks": clocks,
    }
    if cpu:
        line["cpu_baseline"] = {"value": cpu[0], "unit": UNIT, "cores": cpu[2], "kind": "port",
                                "sample": "1 solve, %d RK4 steps (%.1f s), FP64 CSR oracle" % (
                                    args.warmup + args.steps, cpu[1])}
        line["err_vs_oracle"] = {"rel_l2": cpu[3], "solve": 0, "steps": args.warmup + args.steps}
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
