"""Algorithmic (LAPACK-convention) flop counts of the RGF stages.

With b = ns and d = nd, per block column i (i < nt):
  factorize: b^3/3 (POTRF) + (b [i<nt-1] + d) b^2 (TRSM)
             + [i<nt-1] (b^2 (b+1) + 2 d b^2) (SYRK + arrowhead GEMM)
             + d^2 (b+1) (corner update), plus d^3/3 once (corner POTRF);
  selected inversion: b^3/3 (TRTRI) + 2 b^3 (two TRMM) + [i<nt-1] 4 b^3
             (two GEMM) + 2 d^2 b + 2 d b^2 + [i<nt-1] 4 d b^2, plus 4 d^3/3 once.
These are the counts behind "FP64-equivalent TFLOP/s", independent of the
precision the work actually runs in.
"""


def algorithmic_flops(ns: int, nt: int, nd: int) -> dict:
    b, d = float(ns), float(nd)
    fac = sel = 0.0
    for i in range(nt):
        last = i == nt - 1
        fac += b ** 3 / 3 + ((0 if last else b) + d) * b * b
        if not last:
            fac += b * b * (b + 1) + 2 * d * b * b
        fac += d * d * (b + 1)
        sel += b ** 3 / 3 + 2 * b ** 3 + 2 * d * d * b + 2 * d * b * b
        if not last:
            sel += 4 * b ** 3 + 4 * d * b * b
    fac += d ** 3 / 3
    sel += 4 * d ** 3 / 3
    return {"factor": fac, "selinv": sel, "total": fac + sel}
