"""Runs one hot kernel on a small, fixed case: the command profiled with ncu.

  python -m entropydecreaseboltzmann_gb300.kernel_probe --kernel calq32 --N 24 --S 256
  python -m entropydecreaseboltzmann_gb300.kernel_probe --kernel calq64 --N 24

calq32: batched FP32 Q-hat of S BKW solves (ALIASED table, L = 7).
calq64: FP64 drop-in Q-hat of one solve (REFERENCE or ALIASED table).
Prints the per-launch time from CUDA events (not meaningful under ncu).
"""
from __future__ import annotations

import argparse

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", choices=["calq32", "calq64"], default="calq32")
    ap.add_argument("--N", type=int, default=24)
    ap.add_argument("--S", type=int, default=256)
    ap.add_argument("--L", type=float, default=7.0)
    ap.add_argument("--mode", type=int, default=1)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--sweep", action="store_true",
                    help="calq32: time every kernel variant (no chunks and 8 chunks)")
    ap.add_argument("--variant", type=int, default=-1,
                    help="calq32: run this kernel variant instead of the autotuned one")
    args = ap.parse_args()

    import torch

    import entropydecreaseboltzmann_gb300 as edb
    from entropydecreaseboltzmann_gb300 import data

    N, S = args.N, args.S
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    if args.kernel == "calq32":
        q = edb.QCalculator(N, 0, L=args.L, filter=False, index_mode=edb.INDEX_ALIASED)
        q.genB()
        F0, _, _ = data.bkw_bump_batch(S, N, args.L, seed=5)
        fh = np.fft.fftn(F0.reshape(S, N, N, N), axes=(1, 2, 3)).reshape(S, -1)
        fin = torch.from_numpy(fh.astype(np.complex64)).cuda()
        out = torch.empty_like(fin)
        if args.sweep:
            part = torch.empty(8 * S * N ** 3 * 4, dtype=torch.float32, device="cuda")
            nv = edb.lib.edb_qcalc_calQ_batch_f32_ex  # noqa: F841 (presence check)
            nvar = edb.lib.edb_qcalc_batch_variants()
            for C in (1, 8):
                first = None
                for var in range(nvar):
                    try:
                        q.calQ_batch_f32_ex(S, var, C, part, fin, out, stream)
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
                    for _ in range(args.reps):
                        q.calQ_batch_f32_ex(S, var, C, part, fin, out, stream)
                    a1.record(stream)
                    torch.cuda.synchronize()
                    t = a0.elapsed_time(a1) / args.reps
                    print(f"variant {var} chunks {C}: {t:.3f} ms, "
                          f"{10 * float(N) ** 6 * S / (t * 1e-3) / 1e12:.2f} TFLOP/s, "
                          f"bits {'same' if same else 'DIFFER'}")
                del first
            del part
        if args.variant >= 0:
            run = lambda: q.calQ_batch_f32_ex(S, args.variant, 1, None, fin, out, stream)  # noqa
        else:
            v = q.autotune_batch(S, fin, out, stream)  # 3 launches per variant
            print(f"autotuned variant {v}")
            run = lambda: q.calQ_batch_f32(S, fin, out, stream)  # noqa: E731
        terms = float(N) ** 6 * S
    else:
        q = edb.QCalculator(N, 0, L=args.L, filter=False, index_mode=args.mode)
        q.genB()
        f = data.bkw_grid(N, args.L, 5.5)
        fin = torch.from_numpy(np.fft.fftn(f.reshape(N, N, N)).reshape(-1)).cuda()
        out = torch.empty_like(fin)
        run = lambda: q.calQ_device(fin, out, stream)  # noqa: E731
        terms = float(q.info()["terms"])
    run()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.reps):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.reps
    if args.kernel == "calq32":
        ref = out.clone()
        torch.cuda.synchronize()
        st = edb.device_status(clear=True)
        print(f"device status {st}, finite {bool(torch.isfinite(torch.view_as_real(ref)).all())}")
    import ctypes as C

    p1, p2 = C.c_double(), C.c_double()
    edb.lib.edb_measure_fp32_peak(C.byref(p1))
    edb.lib.edb_measure_fp32x2_peak(C.byref(p2))
    print(f"FP32 FMA peak probe: scalar {p1.value:.1f} TFLOP/s, packed f32x2 {p2.value:.1f} TFLOP/s")
    print(f"{args.kernel} N={N} S={S}: {ms:.3f} ms/launch, "
          f"{10 * terms / (ms * 1e-3) / 1e12:.2f} TFLOP/s (10 flop/term)")


if __name__ == "__main__":
    main()
