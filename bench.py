"""Benchmark of the spectral collision step (batched Q-hat evaluations/s).

Workload (one GPU): the uniform batch of 4096 independent solves at N = 24,
L = 7, Maxwell molecules (gamma = 0, filter off, ALIASED index mode), all
sharing one kernel table; BKW initial data at seeded t0 ~ U[5.5, 8] plus a
Gaussian bump, mass renormalised to 1; RK4 with dt = 0.01.  One step = one
RK4 step of every solve = 4 x 4096 Q-hat evaluations, each N^6 = 1.91e8 terms.

value: Q-hat evaluations/s with the state resident in HBM (device-timed,
CUDA events on the launching stream).  e2e: the same metric through the C ABI
with host buffers — per step, edb_batch_load (pinned host real-space f in,
forward FFT), one RK4 step, edb_batch_read (inverse FFT, real-space f out).
Also reported: the FP64 drop-in single-solve path at N = 24 and N = 32
(evals/s and B-stream bandwidth), the BKW L-infinity error of the batched
FP32 path after 50 RK4 steps, the roofline of the dominant kernel, the
CPU baseline (the oracle's restatement of QCalculator::calQ on host threads)
and the serving engine on the serving-stream mix (N in {16, 24, 32} with
probabilities 0.5/0.3/0.2, gamma in {0, 1}, horizons log-uniform in [20, 500]
RK4 steps, 5% BKW requests, 80 GB budget): its capacity (all requests at
once) and p50/p99 time-to-solution under Poisson arrivals at 70% of that
capacity.  --uneven adds the uneven batch (512 solves each at N = 16, 24,
32, gamma in {0, 0.5, 1}, SSP3 dt = 0.005, U{20..200} steps).

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
For N > 1 (torchrun) every rank runs an independent replica of the workload
(the solves are independent: replicas only, no collective on the data path).
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
TRAFFIC_BYTES = 7.53e9 + 0.46e9  # DRAM read + write of one batched-kernel launch (ncu)


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
        sm, smax, reasons = [], [], set()
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
            for nm, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def make_batch_inputs(S, seed=1002):
    from entropydecreaseboltzmann_gb300 import data

    F0, t0, amp = data.bkw_bump_batch(S, N_MODES, L_BOX, seed)
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
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    from oracle.oracle import INDEX_ALIASED, Oracle, build_oracle

    build_oracle()
    o = Oracle()
    threads = os.cpu_count() or 1
    N = N_MODES
    B = o.genB(N, 0.0, L_BOX, False, INDEX_ALIASED)
    F0, _, _ = make_batch_inputs(threads, seed=1002)
    fh = np.fft.fftn(F0.reshape(threads, N, N, N), axes=(1, 2, 3)).reshape(threads, -1)
    dt = DT

    def rk4_step(fh):
        # BKW.h:481-494 on `threads` independent solves, each calQ on its own thread
        q0 = o.calQ_batch(N, B, fh, INDEX_ALIASED, nthreads=threads)
        q1 = o.calQ_batch(N, B, fh + 0.5 * dt * q0, INDEX_ALIASED, nthreads=threads)
        q2 = o.calQ_batch(N, B, fh + 0.5 * dt * q1, INDEX_ALIASED, nthreads=threads)
        q3 = o.calQ_batch(N, B, fh + dt * q2, INDEX_ALIASED, nthreads=threads)
        return fh + dt / 6.0 * (q0 + 2.0 * q1 + 2.0 * q2 + q3)

    for _ in range(args.warmup):
        fh = rk4_step(fh)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fh = rk4_step(fh)
    el = time.perf_counter() - t0
    evals = 4 * threads * args.steps
    value = evals / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD + f" (CPU sample: {threads} of the 4096 solves per step)",
                                        "cpu_threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{threads} solves x {args.steps} RK4 steps (4 calQ each) of "
                                   "the 4096-solve N=24 workload, one solve per host thread; the "
                                   "reference's C++ cannot be built on the GPU host (its sources "
                                   "are not there), so the oracle's restatement of "
                                   "QCalculator::calQ (same loops) is timed"},
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
    ap.add_argument("--serve-seconds", type=float, default=20.0,
                    help="arrival window of the Poisson run")
    ap.add_argument("--uneven", action="store_true", help="also run the uneven batch")
    ap.add_argument("--uneven-per-n", type=int, default=512)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)

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
    bs = edb.BatchSolver(q, S, L_BOX, edb.SCHEME_RK4, DT)
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
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        bs.load(h_in.numpy())
        bs.step(1)
        bs.read(real=True, out=h_out.numpy())
    e2e_s = time.perf_counter() - t0
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
        for kind, name in ((0, "emulated"), (1, "native")):
            q64.set_fp64_kernel(kind)
            for _ in range(2):
                q64.calQ_device(fh, out, stream)
            reps = 5 if kind == 0 else 3
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
            # planes it visits (l1 <= (k1 - l1) mod N); the native kernel all of B
            frac = (sum(k1 // 2 + 1 + max(0, (k1 + Nf) // 2 - k1) for k1 in range(Nf)) / Nf ** 2
                    if kind == 0 else 1.0)
            res[name] = {"evals_per_s": 1.0 / t, "ms_per_eval": t * 1e3,
                         "B_stream_GBs": nb / t / 1e9,
                         "B_read_GBs": nb * frac / t / 1e9}
        fp64[f"N{Nf}"] = res
        del q64
    peaks, peak_src = measured_peaks()
    for k, v in fp64.items():
        for kind in v.values():
            kind["hbm_frac"] = kind["B_stream_GBs"] / peaks["hbm_gbs"]
            kind["hbm_frac_read"] = kind["B_read_GBs"] / peaks["hbm_gbs"]

    # ---- BKW accuracy of the batched FP32 path (50 RK4 steps, pure BKW solves)
    Sb = 32
    t0b = np.linspace(5.5, 8.0, Sb)
    fb = np.stack([data.bkw_grid(N, L_BOX, t) for t in t0b])
    bb = edb.BatchSolver(q, Sb, L_BOX, edb.SCHEME_RK4, DT)
    bb.load(fb)
    bb.step(50)
    fend = bb.read(real=True)
    exact = np.stack([data.bkw_grid(N, L_BOX, t + 50 * DT) for t in t0b])
    bkw_linf = float(np.max(np.abs(fend - exact)))

    del bb, bs
    torch.cuda.synchronize()
    serve = run_serving(edb, args, rank) if args.serve_requests > 0 else None
    uneven = run_uneven(edb, args, rank) if args.uneven else None

    line = None
    if rank == 0:
        cpu = None if args.no_cpu_baseline else cpu_baseline()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32c (complex FP32, compensated sums; FP64 state)",
            "data": "synthetic (seeded BKW + Gaussian bump, mass 1)",
            "config": {"workload": WORKLOAD, "solves": S, "N": N, "L": L_BOX, "scheme": "RK4",
                       "dt": DT, "evals_per_step": evals_per_step,
                       "l2": "inputs larger than L2 (FP32 pair table 414 MB, FP64 state 906 MB); no flush",
                       "parallelism": f"replicas x{ws}"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "path": "edb_batch_load (pinned host) + edb_batch_step + edb_batch_read"},
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
                         "kernel": "calq32_kernel", "ms_per_launch": k_ms,
                         "flop_per_launch": 10.0 * terms,
                         # the kernel sums each symmetric pair of terms (l, k - l) once:
                         # the pair terms it executes, and their rate on the FP32 pipe
                         "executed_terms_per_launch": executed_terms,
                         "executed_tflops": 10.0 * executed_terms / (k_ms * 1e-3) / 1e12,
                         "executed_frac": 10.0 * executed_terms / (k_ms * 1e-3) / 1e12 / peak_tf,
                         "peak_source": "FP32 FMA probe measured in this run (edb_measure_fp32_peak)"},
            "fp64_dropin": fp64, "hbm_peak_GBs": peaks["hbm_gbs"], "hbm_peak_source": peak_src,
            # the plain FP64 single-solve path (native FP64 arithmetic) and the
            # FP64-accurate double-float drop-in (the default FP64 kernel)
            "batched_over_plain_fp64_N24": value / fp64["N24"]["native"]["evals_per_s"],
            "batched_over_fp64_dropin_N24": value / fp64["N24"]["emulated"]["evals_per_s"],
            "bkw_linf_fp32_50_steps": bkw_linf,
            "serve": serve,
            "cpu_baseline": cpu,
        }
        if uneven is not None:
            line["uneven_batch"] = uneven
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.barrier()
        pg.destroy_process_group()
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


def C_double_peak(edb):
    import ctypes as C

    v = C.c_double()
    edb.lib.edb_measure_fp32_peak(C.byref(v))
    return v.value


if __name__ == "__main__":
    sys.exit(main())
