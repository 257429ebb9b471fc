"""Benchmark of the spectral collision step (batched Q-hat evaluations/s).

Workload (one GPU): the uniform batch of 4096 independent solves at N = 24,
L = 7, Maxwell molecules (gamma = 0, filter off, ALIASED index mode), all
sharing one kernel table; BKW initial data at seeded t0 ~ U[5.5, 8] plus a
Gaussian bump, mass renormalised to 1; RK4 with dt = 0.01, with the FP64
inverse transform, entropy and EntropyFix rule after every step.  One step =
one RK4 step of every solve = 4 x 4096 Q-hat evaluations, each N^6 = 1.91e8
terms.

value: Q-hat evaluations/s with the state resident in HBM (device-timed,
CUDA events on the launching stream).  e2e: the same metric through the C ABI
with host buffers — per step, edb_batch_load (pinned host real-space f in,
forward FFT), one RK4 step, edb_batch_read (inverse FFT, real-space f out).
Also reported: the FP64 drop-in single-solve path at N = 24 and N = 32
(evals/s and B-stream bandwidth), the BKW L-infinity error after every step
of the batched FP32 path (50 RK4 steps) and of the FP64 testBKW3D case
(N = 16, L = 6, 100 RK4 steps; odd companions N = 17, 21, 25), the roofline
of the dominant kernel, the CPU baseline (the oracle's restatement of
QCalculator::calQ on host threads), the serving engine on the serving-stream
mix (N in {16, 24, 32} with probabilities 0.5/0.3/0.2, gamma in {0, 1},
horizons log-uniform in [20, 500] RK4 steps, 5% BKW requests, 80 GB budget):
its capacity (requests in flight) and p50/p99 time-to-solution under Poisson
arrivals at 70% of that capacity for 60 s, and the uneven batch (512 solves
each at N = 16, 24, 32, gamma in {0, 0.5, 1}, SSP3 dt = 0.005, U{20..200}
steps).

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
        python bench.py --probe calq32|calq64 [--probe-N N] [--probe-S S] ...
For N > 1 (torchrun) every rank runs an independent replica of the workload
(the solves are independent: replicas only, no collective on the data path).
--probe runs one hot kernel on a small fixed case (the command the ncu
captures in profiles/ run) and prints its per-launch time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched Q̂ evals/s vs plain FP64 on GB300 at BKW L∞≤1e-6; serve p50/p99"
UNIT = "Q̂ evals/s"
S_BATCH, N_MODES, L_BOX, DT = 4096, 24, 7.0, 0.01
WORKLOAD = "uniform batch: 4096 solves, N=24, L=7, Maxwell (gamma=0), RK4 dt=0.01, shared B table"
TRAFFIC_BYTES = 7.516e9 + 0.457e9  # DRAM read + write of one batched-kernel launch (ncu)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, device: str) -> float:
    """The largest of every rank's x (the job's time is its slowest replica);
    x itself when no process group is running."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            try:
                pw.append(float(p[2]))
            except ValueError:
                pass
            for nm, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w": float(np.median(pw)) if pw else None}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def data_module():
    """The seeded initial-data helpers (numpy only), loaded by path so that
    the reference arm never imports the package (which loads libedb.so)."""
    import importlib.util

    if "edb_bench_data" in sys.modules:
        return sys.modules["edb_bench_data"]
    path = os.path.join(ROOT, "entropydecreaseboltzmann_gb300", "data.py")
    spec = importlib.util.spec_from_file_location("edb_bench_data", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sys.modules["edb_bench_data"] = mod
    return mod


def make_batch_inputs(S, seed=1002):
    F0, t0, amp = data_module().bkw_bump_batch(S, N_MODES, L_BOX, seed)
    return F0, t0, amp


def cpu_baseline(seconds=12.0, threads=None):
    """The oracle's restatement of QCalculator::calQ (same loop structure as
    the reference, ALIASED index mode) on host threads, independent solves."""
    from oracle.oracle import INDEX_ALIASED, Oracle, build_oracle

    build_oracle()
    o = Oracle()
    threads = threads or os.cpu_count() or 1
    N = N_MODES
    B = o.genB(N, 0.0, L_BOX, False, INDEX_ALIASED)
    F0, _, _ = make_batch_inputs(threads, seed=99)
    fh = np.fft.fftn(F0.reshape(threads, N, N, N), axes=(1, 2, 3)).reshape(threads, -1)
    evals = 0
    t0 = time.perf_counter()
    while True:
        o.calQ_batch(N, B, fh, INDEX_ALIASED, nthreads=threads)
        evals += threads
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return {"value": evals / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{evals} calQ evaluations at N=24 (one independent solve per thread, "
                      f"{threads} threads, {el:.1f} s), oracle restatement of "
                      "QCalculator::calQ, ALIASED mode"}


def run_reference_arm(args):
    """The reference's CPU path on this host's cores: the oracle's
    restatement of QCalculator::calQ (the reference's loops; ALIASED index
    mode) inside BKW3D::RK4's step (BKW.h:480-510: four calQ, the stage
    updates, then ifft, calEntropy and the fix rule), one independent solve
    per host thread.  Imports nothing from the package."""
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    from oracle.oracle import INDEX_ALIASED, EntropyFixOracle, Oracle, build_oracle

    build_oracle()
    o = Oracle()
    threads = os.cpu_count() or 1
    N = N_MODES
    NQ = N ** 3
    B = o.genB(N, 0.0, L_BOX, False, INDEX_ALIASED)
    F0, _, _ = make_batch_inputs(threads, seed=1002)
    fh = np.fft.fftn(F0.reshape(threads, N, N, N), axes=(1, 2, 3)).reshape(threads, -1)
    dt = DT
    efix = [EntropyFixOracle(o, NQ) for _ in range(threads)]
    H_prev = [1.0] * threads
    step_no = [0]

    def rk4_step(fh):
        # BKW.h:481-494 on `threads` independent solves, each calQ on its own thread
        q0 = o.calQ_batch(N, B, fh, INDEX_ALIASED, nthreads=threads)
        q1 = o.calQ_batch(N, B, fh + 0.5 * dt * q0, INDEX_ALIASED, nthreads=threads)
        q2 = o.calQ_batch(N, B, fh + 0.5 * dt * q1, INDEX_ALIASED, nthreads=threads)
        q3 = o.calQ_batch(N, B, fh + dt * q2, INDEX_ALIASED, nthreads=threads)
        fh = fh + dt / 6.0 * (q0 + 2.0 * q1 + 2.0 * q2 + q3)
        # BKW.h:497-510: ifft, calEntropy, the fix rule on Re F
        for s in range(threads):
            F = o.fft3d(N, fh[s], inverse=True)
            H = o.calentropy(N, L_BOX, F)
            if step_no[0] and H - H_prev[s] > 1.0e-10:
                f = np.ascontiguousarray(F.real)
                efix[s].FixSol(f, H_prev[s] / (2.0 * L_BOX) ** 3)
                H = o.calentropy(N, L_BOX, f.astype(np.complex128))
            H_prev[s] = H
        step_no[0] += 1
        return fh

    for _ in range(args.warmup):
        fh = rk4_step(fh)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fh = rk4_step(fh)
    el = time.perf_counter() - t0
    evals = 4 * threads * args.steps
    value = evals / el
    sample = (f"{threads} solves x {args.steps} RK4 steps (4 calQ each, then ifft, entropy and "
              "the fix rule) of the 4096-solve N=24 workload, one solve per host thread; the "
              "reference's C++ is not on the GPU host (its sources are not there, and its "
              "x86 build does not run on Arm), so the oracle's restatement of the same loops "
              "is timed")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD + ", fix on" +
                   f" (CPU sample: {threads} of the 4096 solves per step; the metric is a "
                   "per-evaluation rate)", "cpu_threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch", type=int, default=S_BATCH)
    ap.add_argument("--serve-requests", type=int, default=600,
                    help="request pool of the capacity run (0: skip serving)")
    ap.add_argument("--serve-capacity-seconds", type=float, default=20.0,
                    help="window of the steady-state capacity run")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="arrival window of the Poisson run")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven batch")
    ap.add_argument("--uneven-per-n", type=int, default=512)
    ap.add_argument("--probe", choices=["calq32", "calq64"], default=None,
                    help="run one hot kernel on a small fixed case (see probe())")
    ap.add_argument("--probe-N", type=int, default=24)
    ap.add_argument("--probe-S", type=int, default=256)
    ap.add_argument("--probe-L", type=float, default=7.0)
    ap.add_argument("--probe-mode", type=int, default=1, help="calq64: index mode")
    ap.add_argument("--probe-kernel", type=int, default=0,
                    help="calq64: FP64 kernel (0 double-float streamed, 1 native, 2 on the fly)")
    ap.add_argument("--probe-compact", action="store_true",
                    help="calq64: build only the compact tables (genB_compact)")
    ap.add_argument("--probe-reps", type=int, default=2)
    ap.add_argument("--probe-variant", type=int, default=-1,
                    help="calq32: this kernel variant instead of the autotuned one; "
                         "calq64: this launch shape of the double-float kernel")
    ap.add_argument("--probe-sweep", action="store_true",
                    help="calq32: time every kernel variant (no chunks and 8 chunks); "
                         "calq64: every launch shape of the double-float kernel")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.probe:
        return probe(args)

    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    import entropydecreaseboltzmann_gb300 as edb
    from entropydecreaseboltzmann_gb300 import data

    S = args.batch
    N = N_MODES
    NQ = N ** 3
    # a dedicated (non-default) stream: every launch of the timed region and the
    # CUDA events bracketing it go to this stream
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    q = edb.QCalculator(N, 0, L=L_BOX, filter=False, index_mode=edb.INDEX_ALIASED)
    q.genB()
    F0, t0s, _ = make_batch_inputs(S, seed=1002 + rank)
    # every step: four batched Q-hat stages, the FP64 stage updates, then the
    # FP64 inverse transform, entropy and the EntropyFix rule (BKW.h:480-510)
    bs = edb.BatchSolver(q, S, L_BOX, edb.SCHEME_RK4, DT, fix_entropy=True)
    d_F0 = torch.from_numpy(F0).cuda()
    bs.load_device(d_F0, stream)
    torch.cuda.synchronize()

    # ---- device-resident throughput
    for _ in range(args.warmup):
        bs.step(1, stream)
    barrier()
    launches0 = edb.kernel_launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    bs.step(args.steps, stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    launches = edb.kernel_launch_count() - launches0
    ms_max = max_over_ranks(ms, "cuda")
    evals_per_step = 4 * S
    value = evals_per_step * args.steps * ws / (ms_max * 1e-3)

    # ---- dominant kernel alone: the batched Q-hat kernel, CUDA events
    fin32 = torch.from_numpy(
        np.fft.fftn(F0.reshape(S, N, N, N), axes=(1, 2, 3)).reshape(S, -1).astype(np.complex64)).cuda()
    qout = torch.empty_like(fin32)
    q.calQ_batch_f32(S, fin32, qout, stream)
    kreps = 3
    k0 = torch.cuda.Event(enable_timing=True)
    k1 = torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    for _ in range(kreps):
        q.calQ_batch_f32(S, fin32, qout, stream)
    k1.record(stream)
    torch.cuda.synchronize()
    k_ms = k0.elapsed_time(k1) / kreps
    terms = float(NQ) * NQ * S
    # l1 planes visited per k1: [0, k1/2] and [k1+1, (k1+N)/2]
    executed_terms = float(S) * N ** 4 * sum(
        k1 // 2 + 1 + max(0, (k1 + N) // 2 - k1) for k1 in range(N))
    algo_bytes = 4.0 * NQ * NQ + S * NQ * (8 + 8)  # B32 once, FP32 f-hat in, FP32 Q-hat out
    peak_tf = C_double_peak(edb)
    achieved_tf = 10.0 * terms / (k_ms * 1e-3) / 1e12

    # ---- e2e through the C ABI with pinned host buffers
    h_in = torch.from_numpy(F0).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    bs.load(h_in.numpy())
    bs.step(1)
    _ = bs.read(real=True)
    torch.cuda.synchronize()
    e2e_steps = args.steps
    # one batch, synchronous calls: each step's copies and transforms in series
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        bs.load(h_in.numpy())
        bs.step(1)
        bs.read(real=True, out=h_out.numpy())
    e2e_sync_value = evals_per_step * e2e_steps / (time.perf_counter() - t0)
    # two batches in flight through the asynchronous calls: every step still
    # copies its inputs in and its result out, and one batch's copies overlap
    # the other's step
    bs2 = edb.BatchSolver(q, S, L_BOX, edb.SCHEME_RK4, DT, fix_entropy=True)
    pair = (bs, bs2)
    h_outs = (h_out, torch.empty_like(h_in).pin_memory())
    bs2.load(h_in.numpy())
    bs2.step(1)
    bs2.read(real=True, out=h_outs[1].numpy())
    e2e_clocks = ClockSampler(local)
    e2e_clocks.start()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        b = pair[i % 2]
        b.load_async(h_in.numpy())
        b.step_async(1)
        b.read_async(h_outs[i % 2].numpy())
    for b in pair:
        b.sync()
    e2e_s = time.perf_counter() - t0
    e2e_clk = e2e_clocks.stop()
    del bs2
    e2e_value = evals_per_step * e2e_steps / e2e_s
    h2d = S * NQ * 8
    d2h = S * NQ * 8

    # ---- FP64 drop-in single solve (reference calQ semantics, B streamed)
    fp64 = {}
    for Nf, Lf in ((24, L_BOX), (32, 8.0)):
        q64 = edb.QCalculator(Nf, 0, L=Lf, filter=False, index_mode=edb.INDEX_ALIASED)
        q64.genB()
        f = data.bkw_grid(Nf, Lf, 5.5)
        fh = torch.from_numpy(np.fft.fftn(f.reshape(Nf, Nf, Nf)).reshape(-1)).cuda()
        out = torch.empty_like(fh)
        res = {}
        for kind, name in ((0, "emulated"), (1, "native"), (2, "onthefly")):
            q64.set_fp64_kernel(kind)
            for _ in range(2):
                q64.calQ_device(fh, out, stream)
            reps = 3 if kind == 1 else 5
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            for _ in range(reps):
                q64.calQ_device(fh, out, stream)
            a1.record(stream)
            torch.cuda.synchronize()
            t = a0.elapsed_time(a1) / reps * 1e-3
            nb = float(Nf) ** 6 * 8
            # the double-float kernel reads the ALIASED pair table on the l1
            # planes it visits (l1 <= (k1 - l1) mod N); the native kernel all
            # of B; the on-the-fly kernel no table of N^6 size (its gathers
            # from the compact F-table hit L2)
            visited = sum(k1 // 2 + 1 + max(0, (k1 + Nf) // 2 - k1) for k1 in range(Nf)) / Nf ** 2
            frac = {0: visited, 1: 1.0, 2: 0.0}[kind]
            n2 = 3 * (2 * (Nf - 1 - (Nf - 1) // 2)) ** 2  # largest squared norm (genB's amax)
            table = {0: nb, 1: nb, 2: (n2 + 1) * (n2 // 4 + 1) * 8 + Nf ** 3 * 16}[kind]
            # the kernel each kind runs on this ALIASED table (the double-float
            # one in the launch shape genB timed fastest)
            kern = {0: "calq64p_kernel" if Nf % 4 == 0 else "calq64x_kernel",
                    1: "calq64_kernel", 2: "calq64f_kernel"}[kind]
            res[name] = {"evals_per_s": 1.0 / t, "ms_per_eval": t * 1e3,
                         "B_stream_GBs": nb / t / 1e9,
                         "B_read_GBs": nb * frac / t / 1e9,
                         "table_bytes": table, "kernel": kern}
            if kind == 0:
                res[name]["launch_shape"] = q64.fp64_shape()
        fp64[f"N{Nf}"] = res
        del q64
    peaks, peak_src = measured_peaks()
    for k, v in fp64.items():
        for kind in v.values():
            kind["hbm_frac"] = kind["B_stream_GBs"] / peaks["hbm_gbs"]
            kind["hbm_frac_read"] = kind["B_read_GBs"] / peaks["hbm_gbs"]

    # ---- BKW accuracy of the batched FP32 path (50 RK4 steps, pure BKW
    # solves, fix on as in the timed region): L-inf after every step
    Sb = 32
    t0b = np.linspace(5.5, 8.0, Sb)
    fb = np.stack([data.bkw_grid(N, L_BOX, t) for t in t0b])
    bb = edb.BatchSolver(q, Sb, L_BOX, edb.SCHEME_RK4, DT, fix_entropy=True)
    bb.load(fb)
    bkw_by_step = []
    for st in range(1, 51):
        bb.step(1)
        f = bb.read(real=True)
        exact = np.stack([data.bkw_grid(N, L_BOX, t + st * DT) for t in t0b])
        bkw_by_step.append(float(np.max(np.abs(f - exact))))
    bkw_linf = max(bkw_by_step)

    del bb, bs
    torch.cuda.synchronize()
    cfg1 = run_config1(edb, data)
    serve = run_serving(edb, args, rank) if args.serve_requests > 0 else None
    uneven = None if args.no_uneven else run_uneven(edb, args, rank)
    grouped = None if args.no_uneven else run_grouped(edb, args)

    line = None
    if rank == 0:
        cpu = None if args.no_cpu_baseline else cpu_baseline()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32c (complex FP32, compensated sums; FP64 state)",
            "data": "synthetic (seeded BKW + Gaussian bump, mass 1)",
            "config": {"workload": WORKLOAD + ", FP64 ifft + entropy + EntropyFix rule every step",
                       "solves": S, "N": N, "L": L_BOX, "scheme": "RK4", "fix_entropy": True,
                       "dt": DT, "evals_per_step": evals_per_step,
                       "l2": "inputs larger than L2 (FP32 pair table 414 MB, FP64 state 906 MB); no flush",
                       "parallelism": f"replicas x{ws}"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "path": "two batches in flight: edb_batch_load_async (pinned host) + "
                            "edb_batch_step_async + edb_batch_read_async (pinned host), "
                            "edb_batch_sync at the end",
                    "sync_value": e2e_sync_value,
                    "sync_path": "one batch: edb_batch_load + edb_batch_step + edb_batch_read",
                    "clocks": e2e_clk},
            "gpu_launches": int(launches),
            "clocks": clk,
            "roofline": {"bound": "fp32", "achieved": achieved_tf, "peak": peak_tf,
                         "unit": "TFLOP/s", "frac": achieved_tf / peak_tf,
                         # dram__bytes_read.sum + dram__bytes_write.sum per launch, one ncu
                         # capture of this launch (N=24, S=4096, the autotuned variant)
                         "traffic": TRAFFIC_BYTES if S == S_BATCH else None,
                         "traffic_note": "bytes per launch from ncu; algorithmic bytes are "
                                         f"{algo_bytes / 1e9:.2f} GB (table once + f-hat in, "
                                         "Q-hat out): the table streams once per block of "
                                         "solve groups, and the kernel is FP32-bound",
                         "kernel": "calq32_multi_kernel (the persistent form of "
                                   "calq32_kernel's CTA work)", "ms_per_launch": k_ms,
                         "flop_per_launch": 10.0 * terms,
                         # the kernel sums each symmetric pair of terms (l, k - l) once:
                         # the pair terms it executes, and their rate on the FP32 pipe
                         "executed_terms_per_launch": executed_terms,
                         "executed_tflops": 10.0 * executed_terms / (k_ms * 1e-3) / 1e12,
                         "executed_frac": 10.0 * executed_terms / (k_ms * 1e-3) / 1e12 / peak_tf,
                         "frac_note": "achieved counts the algorithmic 10 S N^6 flop; the kernel "
                                      "sums each symmetric pair of terms (l, k - l) once "
                                      "(about half the terms), so achieved can exceed the FMA "
                                      "rate: executed_frac is the pipe's measure",
                         "peak_source": "FP32 FMA probe measured in this run (edb_measure_fp32_peak)"},
            "fp64_dropin": fp64, "hbm_peak_GBs": peaks["hbm_gbs"], "hbm_peak_source": peak_src,
            # the plain FP64 single-solve path (native FP64 arithmetic) and the
            # FP64-accurate double-float drop-in (the default FP64 kernel)
            "batched_over_plain_fp64_N24": value / fp64["N24"]["native"]["evals_per_s"],
            "batched_over_fp64_dropin_N24": value / fp64["N24"]["emulated"]["evals_per_s"],
            "bkw_linf_fp32_50_steps": bkw_linf,
            "bkw_linf_fp32_by_step": bkw_by_step,
            "bkw_fp64_config1": cfg1,
            "serve": serve,
            "cpu_baseline": cpu,
        }
        if uneven is not None:
            line["uneven_batch"] = uneven
            line["grouped_launch"] = grouped
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.barrier()
        pg.destroy_process_group()
    return 0


def probe(args):
    """One hot kernel on a small fixed case, the command the ncu captures in
    profiles/ run:
      --probe calq32: batched FP32 Q-hat of --probe-S BKW solves (ALIASED
        table, L = --probe-L), the autotuned variant or --probe-variant;
        --probe-sweep times every variant with 1 and 8 chunks first;
      --probe calq64: FP64 drop-in Q-hat of one BKW solve (index mode
        --probe-mode); the double-float kernel in its tuned launch shape or
        --probe-variant, --probe-sweep times every shape first.
    Prints the per-launch time from CUDA events (not meaningful under ncu)."""
    import ctypes as C

    import torch

    import entropydecreaseboltzmann_gb300 as edb
    from entropydecreaseboltzmann_gb300 import data

    N, S, L = args.probe_N, args.probe_S, args.probe_L
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    if args.probe == "calq32":
        q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=edb.INDEX_ALIASED)
        q.genB()
        F0, _, _ = data.bkw_bump_batch(S, N, L, seed=5)
        fh = np.fft.fftn(F0.reshape(S, N, N, N), axes=(1, 2, 3)).reshape(S, -1)
        fin = torch.from_numpy(fh.astype(np.complex64)).cuda()
        out = torch.empty_like(fin)
        if args.probe_sweep:
            part = torch.empty(8 * S * N ** 3 * 4, dtype=torch.float32, device="cuda")
            for Cn in (1, 8):
                first = None
                for var in range(edb.lib.edb_qcalc_batch_variants()):
                    try:
                        q.calQ_batch_f32_ex(S, var, Cn, part, fin, out, stream)
                    except edb.EdbError as e:
                        if e.status == 1 and var > 0:
                            continue
                        raise
                    torch.cuda.synchronize()
                    if first is None:
                        first = out.clone()
                    same = bool(torch.equal(out.view(torch.float32), first.view(torch.float32)))
                    a0 = torch.cuda.Event(enable_timing=True)
                    a1 = torch.cuda.Event(enable_timing=True)
                    a0.record(stream)
                    for _ in range(args.probe_reps):
                        q.calQ_batch_f32_ex(S, var, Cn, part, fin, out, stream)
                    a1.record(stream)
                    torch.cuda.synchronize()
                    t = a0.elapsed_time(a1) / args.probe_reps
                    print(f"variant {var} chunks {Cn}: {t:.3f} ms, "
                          f"{10 * float(N) ** 6 * S / (t * 1e-3) / 1e12:.2f} TFLOP/s, "
                          f"bits {'same' if same else 'DIFFER'}")
                del first
            del part
        if args.probe_variant >= 0:
            def run():
                q.calQ_batch_f32_ex(S, args.probe_variant, 1, None, fin, out, stream)
        else:
            print(f"autotuned variant {q.autotune_batch(S, fin, out, stream)}")

            def run():
                q.calQ_batch_f32(S, fin, out, stream)
        terms = float(N) ** 6 * S
    else:
        q = edb.QCalculator(N, 0, L=L, filter=False, index_mode=args.probe_mode)
        if args.probe_compact:
            q.genB_compact()
        else:
            q.genB()
            q.set_fp64_kernel(args.probe_kernel)
        f = data.bkw_grid(N, L, 5.5)
        fin = torch.from_numpy(np.fft.fftn(f.reshape(N, N, N)).reshape(-1)).cuda()
        out = torch.empty_like(fin)

        def run():
            q.calQ_device(fin, out, stream)
        terms = float(q.info()["terms"])
        if not args.probe_compact and args.probe_kernel == 0:
            tuned = q.fp64_shape()
            if args.probe_sweep:  # every launch shape of the double-float kernel
                first = None
                for shp in range(edb.lib.edb_qcalc_fp64_shapes()):
                    q.fp64_shape(shp)
                    run()
                    torch.cuda.synchronize()
                    first = out.clone() if first is None else first
                    a0 = torch.cuda.Event(enable_timing=True)
                    a1 = torch.cuda.Event(enable_timing=True)
                    a0.record(stream)
                    for _ in range(args.probe_reps):
                        run()
                    a1.record(stream)
                    torch.cuda.synchronize()
                    print(f"shape {shp}: {a0.elapsed_time(a1) / args.probe_reps:.3f} ms, bits "
                          f"{'same' if torch.equal(out, first) else 'DIFFER'}")
            q.fp64_shape(tuned if args.probe_variant < 0 else args.probe_variant)
            print(f"double-float kernel shape {q.fp64_shape()} (tuned at genB: {tuned})")
    run()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.probe_reps):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.probe_reps
    st = edb.device_status(clear=True)
    print(f"device status {st}, finite {bool(torch.isfinite(torch.view_as_real(out)).all())}")
    p1, p2 = C.c_double(), C.c_double()
    edb.lib.edb_measure_fp32_peak(C.byref(p1))
    edb.lib.edb_measure_fp32x2_peak(C.byref(p2))
    print(f"FP32 FMA peak probe: scalar {p1.value:.1f} TFLOP/s, packed f32x2 {p2.value:.1f} TFLOP/s")
    print(f"{args.probe} N={N} S={S}: {ms:.3f} ms/launch, "
          f"{10 * terms / (ms * 1e-3) / 1e12:.2f} TFLOP/s (10 flop/term)")
    return 0


SERVE_KEYS = ("completed", "tts_p50_s", "tts_p99_s", "tts_mean_s", "tts_max_s", "wait_p50_s",
              "wait_p99_s", "throughput_rps", "qhat_evals_per_s", "qhat_evals",
              "qhat_evals_padded", "steps_launched", "kernel_launches", "groups")


def run_serving(edb, args, rank):
    """Serving-stream mix through edb.Server: steady-state capacity with a
    fixed number of requests in flight, then Poisson arrivals at 70% of it
    (all requests run to completion; times are on the server clock, host
    data in and out)."""
    from entropydecreaseboltzmann_gb300 import serving

    budget = 80e9
    srv = edb.Server(hbm_budget_bytes=budget, scheme=edb.SCHEME_RK4, dt=DT)
    pool = serving.stream_requests(rate=1e6, duration=args.serve_requests * 1e-6 * 4,
                                   seed=3000 + rank)
    capacity, cap_evals, cap_pad, ncap = serving.measure_capacity(
        srv, pool, concurrency=96, seconds=args.serve_capacity_seconds)
    srv.close()
    rate = 0.7 * capacity
    srv = edb.Server(hbm_budget_bytes=budget, scheme=edb.SCHEME_RK4, dt=DT)
    reqs = serving.stream_requests(rate=rate, duration=args.serve_seconds, seed=4000 + rank)
    st, _ = serving.run(srv, reqs, DT)
    srv.close()
    gpu_s_per_req = 1.0 / capacity
    out = {
        "workload": "serving stream: N 16/24/32 (p .5/.3/.2, L 6/7/8), gamma {0,1}, mixture of "
                    "1-3 Maxwellians, 5% BKW, horizon log-U[20,500] RK4 steps dt=0.01, 80 GB "
                    "HBM budget; tables built before the clock starts",
        "capacity_rps": capacity,
        "capacity_run": {"in_flight": 96, "window_s": args.serve_capacity_seconds,
                         "completions_counted": ncap, "qhat_evals_per_s": cap_evals,
                         "padding_overhead": cap_pad},
        "offered_rps": rate,
        "arrival_window_s": args.serve_seconds,
        "requests": st["submitted"],
        "hbm_peak_GB": st["hbm_bytes_peak"] / 1e9,
        "bkw_linf_by_N": st["bkw_linf_by_N"],
        "bkw_requests": st["bkw_requests"],
        "padding_overhead": st["qhat_evals_padded"] / max(st["qhat_evals"], 1.0),
        "note": (f"one GPU sustains {capacity:.1f} req/s of this mix ({gpu_s_per_req * 1e3:.0f} "
                 f"GPU-ms per request), so 2000 req/s would need {2000 * gpu_s_per_req:.0f} GPUs; "
                 f"p50/p99 are reported at a sustained 70% of the measured capacity"),
    }
    out.update({k: st[k] for k in SERVE_KEYS})
    return out


def run_config1(edb, data):
    """The testBKW3D case on RK4 through the FP64 device-resident integrator:
    N = 16 on [-6, 6]^3, BKW initial data at t0 = 5.5, dt = 0.01, 100 steps,
    ALIASED index mode with L = 6 in the kernel scale and the filter off; L-inf
    of Re F against the exact BKW solution after every step.  The odd
    companions N = 17, 21, 25 show how the discretisation floor falls with N
    (L-inf after every step, reported as the maximum and the final value)."""
    dt, steps, L = 0.01, 100, 6.0
    out = {"workload": "N=16, L=6, BKW t0=5.5, RK4 dt=0.01 x 100 steps, FP64, aliased, filter off"}
    for N in (16, 17, 21, 25):
        b = edb.BKW3D(N, L, L=L, filter=False, index_mode=edb.INDEX_ALIASED, record_F=True)
        b.setInitial(data.bkw_grid(N, L, 5.5))
        t0 = time.perf_counter()
        b.RK4(0.0, (steps - 0.5) * dt, dt)
        wall = time.perf_counter() - t0
        linf = [float(np.max(np.abs(b.F_history[s] - data.bkw_grid(N, L, 5.5 + (s + 1) * dt))))
                for s in range(b.nsteps)]
        rec = {"steps": b.nsteps, "linf_max": max(linf), "linf_final": linf[-1],
               "wall_s_with_genB": wall}
        if N == 16:
            rec["linf_by_step"] = linf
        out[f"N{N}"] = rec
        del b
    return out


def run_uneven(edb, args, rank):
    """Uneven batch: every request at t = 0, 9 kernel tables, SSP3 with the
    moment-preserving entropy fix (conservative mode)."""
    from entropydecreaseboltzmann_gb300 import serving

    srv = edb.Server(hbm_budget_bytes=80e9, scheme=edb.SCHEME_SSP3, dt=0.005, fix_entropy=True,
                     conserve=True)
    reqs = serving.uneven_requests(args.uneven_per_n, seed=5000 + rank)
    st, _ = serving.run(srv, reqs, 0.005)
    srv.close()
    out = {"workload": f"uneven batch: {args.uneven_per_n} solves each at N=16/24/32 (L 6/7/8), "
                       "gamma U{0,0.5,1}, SSP3 dt=0.005, U{20..200} steps, fix on, conservative",
           "makespan_s": st["last_done_s"], "hbm_peak_GB": st["hbm_bytes_peak"] / 1e9}
    out.update({k: st[k] for k in SERVE_KEYS})
    return out


def run_grouped(edb, args):
    """The uneven mix's nine kernel tables (N = 16/24/32 x gamma = 0/0.5/1,
    L 6/7/8), each with per_N / 3 solves, one Q-hat evaluation each: one
    grouped launch (a descriptor per table, indexed by CTA; its autotuned
    variant, and variant 4) against the per-table launches on nine streams
    and on one stream (variant 4, and each table's autotuned variant).  Tables
    larger than L2 (2.1 GB at N = 32); CUDA events on the launching stream."""
    import torch
    from entropydecreaseboltzmann_gb300 import serving

    S = max(1, args.uneven_per_n // 3)
    tabs = []
    for N in (16, 24, 32):
        for gamma in (0.0, 0.5, 1.0):
            q = edb.QCalculator(N, int(gamma), gamma=gamma, L=serving.L_OF_N[N], filter=False,
                                index_mode=edb.INDEX_ALIASED)
            q.genB()
            g = torch.Generator(device="cuda").manual_seed(N * 10 + int(2 * gamma))
            fin = torch.randn(S, N ** 3, dtype=torch.complex64, device="cuda", generator=g)
            tabs.append([q, S, fin, torch.empty_like(fin)])
    for t in tabs:
        t.append(t[0].autotune_batch(S, t[2], t[3]))
    main = torch.cuda.current_stream()
    streams = [torch.cuda.Stream() for _ in tabs]

    group = [t[:4] for t in tabs]
    gvar = edb.QCalculator.autotune_batch_multi(group, stream=main)

    def grouped(var=None):
        edb.QCalculator.calQ_batch_multi(group, variant=gvar if var is None else var, stream=main)

    def per_stream(var):
        ev = torch.cuda.Event()
        ev.record(main)
        done = []
        for t, st in zip(tabs, streams):
            st.wait_event(ev)
            t[0].calQ_batch_f32_ex(S, t[4] if var is None else var, 1, None, t[2], t[3], stream=st)
            e = torch.cuda.Event()
            e.record(st)
            done.append(e)
        for e in done:
            main.wait_event(e)

    def one_stream(var):
        for t in tabs:
            t[0].calQ_batch_f32_ex(S, t[4] if var is None else var, 1, None, t[2], t[3],
                                   stream=main)

    def timed(fn, reps=5):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(main)
        for _ in range(reps):
            fn()
        b.record(main)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    out = {"workload": f"9 tables (N 16/24/32 x gamma 0/0.5/1), {S} solves each, one Q-hat "
                       "evaluation per solve", "solves": 9 * S,
           "grouped_ms": timed(grouped), "grouped_variant": gvar,
           "grouped_variant4_ms": timed(lambda: grouped(4)),
           "streams_variant4_ms": timed(lambda: per_stream(4)),
           "streams_autotuned_ms": timed(lambda: per_stream(None)),
           "one_stream_variant4_ms": timed(lambda: one_stream(4)),
           "one_stream_autotuned_ms": timed(lambda: one_stream(None)),
           "autotuned_variants": [t[4] for t in tabs]}
    # the grouped launch's bits equal the per-table launches' (any variant, one chunk)
    ref = [t[3].clone() for t in tabs]
    grouped()
    torch.cuda.synchronize()
    out["bit_identical_to_per_table"] = all(torch.equal(r, t[3]) for r, t in zip(ref, tabs))
    del tabs
    torch.cuda.synchronize()
    return out


def C_double_peak(edb):
    import ctypes as C

    v = C.c_double()
    edb.lib.edb_measure_fp32_peak(C.byref(v))
    return v.value


if __name__ == "__main__":
    sys.exit(main())
