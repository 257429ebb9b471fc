"""Request streams for the serving engine and their measurement.

Two workloads of independent solves, with seeded synthetic initial data:

* serving stream: Poisson arrivals at a given rate; N in {16, 24, 32} with
  probabilities 0.5 / 0.3 / 0.2 (box L = 6, 7, 8), gamma in {0, 1}; initial
  data a mixture of 1-3 isotropic Maxwellians (Dirichlet(1) weights, drifts
  U[-2, 2]^3, temperatures U[0.5, 1.5]); horizon log-uniform in [20, 500]
  RK4 steps of dt = 0.01.  A fraction (5%) of requests are BKW-initialised
  Maxwell-molecule solves (gamma = 0, t0 ~ U[5.5, 8]) whose result is checked
  against the exact BKW solution.
* uneven batch: 512 solves each at (N, L) = (16, 6), (24, 7), (32, 8), gamma
  drawn from {0, 0.5, 1} per solve (9 kernel tables), mixture initial data,
  SSP3 with dt = 0.005 for U{20..200} steps; everything arrives at once.

Both run through ``Server`` (the C ABI's request loop).
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import data

L_OF_N = {16: 6.0, 24: 7.0, 32: 8.0}


def stream_requests(rate: float, duration: float, seed: int, n_probs=(0.5, 0.3, 0.2),
                    gammas=(0.0, 1.0), horizon=(20, 500), bkw_frac=0.05):
    """Poisson arrivals on [0, duration): list of request dicts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Ns = (16, 24, 32)
    out = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        N = int(rng.choice(Ns, p=n_probs))
        steps = int(round(math.exp(rng.uniform(math.log(horizon[0]), math.log(horizon[1])))))
        bkw = bool(rng.uniform() < bkw_frac)
        g = 0.0 if bkw else float(rng.choice(gammas))
        out.append({"N": N, "gamma": g, "L": L_OF_N[N], "steps": steps, "arrival": t,
                    "bkw_t0": float(rng.uniform(5.5, 8.0)) if bkw else None,
                    "seed": int(rng.integers(1 << 31))})
    return out


def uneven_requests(per_N: int, seed: int, gammas=(0.0, 0.5, 1.0), steps=(20, 200)):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for N in (16, 24, 32):
        for _ in range(per_N):
            out.append({"N": N, "gamma": float(rng.choice(gammas)), "L": L_OF_N[N],
                        "steps": int(rng.integers(steps[0], steps[1] + 1)), "arrival": 0.0,
                        "bkw_t0": None, "seed": int(rng.integers(1 << 31))})
    return out


def initial_data(req) -> np.ndarray:
    N, L = req["N"], req["L"]
    if req["bkw_t0"] is not None:
        return data.bkw_grid(N, L, req["bkw_t0"])
    return data.maxwellian_mixture_batch(1, N, L, seed=req["seed"])[0]


def run(server, reqs, dt: float, max_wall_s: float = 0.0):
    """Submits every request (initial data built beforehand, so generation is
    not inside the served time), runs the loop, returns (stats, per-request
    results summary)."""
    inits = [initial_data(r) for r in reqs]
    for r in reqs:
        server.prepare(r["N"], r["gamma"], r["L"])
    ids = []
    for r, f in zip(reqs, inits):
        ids.append(server.submit(r["N"], r["gamma"], r["L"], r["steps"], f, arrival_s=r["arrival"],
                                 want_result=r["bkw_t0"] is not None))
    t0 = time.perf_counter()
    server.run(max_wall_s)
    wall = time.perf_counter() - t0
    st = server.stats()
    bkw = {}
    for r, rid in zip(reqs, ids):
        if r["bkw_t0"] is None or server.info(rid)["state"] != 2:
            continue
        F, _ = server.result(rid)
        exact = data.bkw_grid(r["N"], r["L"], r["bkw_t0"] + r["steps"] * dt)
        bkw.setdefault(r["N"], []).append(float(np.max(np.abs(F - exact))))
    st["wall_s"] = wall
    st["bkw_linf_by_N"] = {str(k): max(v) for k, v in sorted(bkw.items())}
    st["bkw_requests"] = int(sum(len(v) for v in bkw.values()))
    return st, ids


def measure_capacity(server, reqs, concurrency: int, seconds: float, poll_s: float = 0.02):
    """Steady-state throughput: keeps `concurrency` requests in flight (a new
    request arrives as soon as one finishes) for `seconds` of server time and
    measures the last two thirds of the window.  Requests are taken from
    `reqs` in order (initial data built beforehand).  Returns (requests/s,
    useful Q-hat evals/s, padded / useful evals, completions counted)."""
    inits = [initial_data(r) for r in reqs]
    for r in reqs:
        server.prepare(r["N"], r["gamma"], r["L"])
    ids, nxt = [], 0
    snap = None  # (clock, completed, evals, padded) at the window start
    t_lo = seconds / 3.0
    while True:
        st = server.stats()
        inflight = len(ids) - st["completed"]
        while inflight < concurrency and nxt < len(reqs):
            r = reqs[nxt]
            ids.append(server.submit(r["N"], r["gamma"], r["L"], r["steps"], inits[nxt]))
            nxt += 1
            inflight += 1
        server.run(poll_s)
        now = server.clock()
        if snap is None and now >= t_lo:
            st = server.stats()
            snap = (now, st["completed"], st["qhat_evals"], st["qhat_evals_padded"])
        if now >= seconds or (nxt >= len(reqs) and inflight == 0):
            break
    st = server.stats()
    if snap is None:
        snap = (0.0, 0, 0.0, 0.0)
    span = max(now - snap[0], 1e-9)
    done = st["completed"] - snap[1]
    evals = st["qhat_evals"] - snap[2]
    padded = st["qhat_evals_padded"] - snap[3]
    return done / span, evals / span, padded / max(evals, 1.0), done
