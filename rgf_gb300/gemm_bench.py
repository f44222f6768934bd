"""Time one shape of the device GEMM entry point (``rgf_dgemm_device``).

    python -m rgf_gb300.gemm_bench --m 2000 --n 2000 --k 2000 --precision split --syrk

runs C := -A op(A|B) + C on device buffers ``--reps`` times after ``--warmup``
calls and prints one JSON line: microseconds per call (CUDA events on the
stream the library launches on) and the FP64-equivalent rate.  ``--syrk``
makes the product A A^T (the Schur-update shape of the factorization).  This
is the command the GEMM kernel profiles are taken with; every call also
creates and frees the split engine, as the entry point does.
"""
from __future__ import annotations

import argparse
import json


def main() -> None:
    import numpy as np
    import torch

    import rgf_gb300

    p = argparse.ArgumentParser()
    p.add_argument("--m", type=int, default=2000)
    p.add_argument("--n", type=int, default=2000)
    p.add_argument("--k", type=int, default=2000)
    p.add_argument("--precision", choices=["fp64", "split"], default="split")
    p.add_argument("--slices", type=int, default=0)
    p.add_argument("--syrk", action="store_true", help="B = A (product A A^T)")
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--reps", type=int, default=10)
    args = p.parse_args()
    m, n, k = args.m, (args.m if args.syrk else args.n), args.k
    dev = torch.device("cuda", 0)
    g = torch.Generator(device="cpu").manual_seed(1)
    A = torch.randn(k, m, dtype=torch.float64, generator=g).to(dev)      # column-major m x k
    B = A if args.syrk else torch.randn(n, k, dtype=torch.float64, generator=g).to(dev)
    C = torch.randn(n, m, dtype=torch.float64, generator=g).to(dev)
    stream = torch.cuda.current_stream(dev)

    def call():
        rgf_gb300.dgemm_device(args.precision, "N", "T", m, n, k, -1.0, A.data_ptr(), m,
                               B.data_ptr(), n, 1.0, C.data_ptr(), m,
                               stream=stream.cuda_stream, slices=args.slices)

    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.reps):
        call()
    e1.record(stream)
    e1.synchronize()
    us = e0.elapsed_time(e1) * 1e3 / args.reps
    flops = 2.0 * m * n * k
    print(json.dumps({"m": m, "n": n, "k": k, "precision": args.precision,
                      "slices": args.slices or None, "syrk": args.syrk,
                      "us_per_call": us, "fp64_equiv_tflops": flops / (us * 1e-6) / 1e12,
                      "finite": bool(np.isfinite(C.cpu().numpy()).all())}))


if __name__ == "__main__":
    main()
