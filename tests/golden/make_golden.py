"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the CPU replay of the reference (oracle/_ref/rgf_replay: the reference's
unmodified RGF.H compiled with oracle/replay/) on
  * the three matrices the reference ships in data/ (A_9_9_ns3_nt3,
    A_11_11_ns3_nt3_nd2, A_126_126_ns42_nt3), and
  * seeded matrices from rgf_gb300.gen (ns=3, nt=3, nd=2 seed 1 is the
    configuration the reference's small case is quoted on),
with seeded right-hand sides, and stores inputs and outputs per case in
golden_<name>.npz: ia, ja, a, b, ns, nt, nd, mf (factor after factorize),
x (solve), diag (the reference's RGFdiag), logdet, res, resn, plus a dense
LAPACK diag(inv(A)) and logdet for the exact values.  Also stores the
stdout of the reference's own main.C driver on A_11 (ref_main_A11.txt).

Needs the reference tree (located by oracle/replay/build_replay.py) and g++; run
it on a development machine: python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.replay import build_replay  # noqa: E402
from rgf_gb300 import gen  # noqa: E402

REF = build_replay.REF

CASES = [
    # name, ns, nt, nd, source, nrhs
    ("A9", 3, 3, 0, "data/A_9_9_ns3_nt3.dat", 1),
    ("A11", 3, 3, 2, "data/A_11_11_ns3_nt3_nd2.dat", 2),
    ("A126", 42, 3, 0, "data/A_126_126_ns42_nt3.dat", 3),
    ("gen_ns3_nt3_nd2_s1", 3, 3, 2, 1, 1),
    ("gen_ns5_nt4_nd1_s2", 5, 4, 1, 2, 2),
    ("gen_ns16_nt5_nd0_s3", 16, 5, 0, 3, 1),
    ("gen_ns7_nt1_nd0_s4", 7, 1, 0, 4, 1),
    ("gen_ns12_nt3_nd3_s5", 12, 3, 3, 5, 2),
    ("gen_ns30_nt4_nd2_s6", 30, 4, 2, 6, 1),
    ("gen_ns70_nt3_nd6_s7", 70, 3, 6, 7, 4),
]


def dense_exact(ia, ja, a):
    n = len(ia) - 1
    A = np.zeros((n, n))
    c = np.repeat(np.arange(n), np.diff(ia.astype(np.int64)))
    A[ja.astype(np.int64), c] = a
    A = np.tril(A) + np.tril(A, -1).T
    sign, ld = np.linalg.slogdet(A)
    return ld, np.diag(np.linalg.inv(A)).copy()


def main():
    exe = build_replay.build()
    with tempfile.TemporaryDirectory() as tmp:
        for name, ns, nt, nd, src, nrhs in CASES:
            if isinstance(src, str):
                mat = os.path.join(REF, src)
                n, ia, ja, a = gen.read_dat(mat)
                seed = 100 + len(name)
            else:
                ia, ja, a = gen.generate_bta(ns, nt, nd, src)
                n = ns * nt + nd
                mat = os.path.join(tmp, name + ".dat")
                gen.write_dat(mat, ia, ja, a)
                seed = src
            b = gen.random_rhs(n, nrhs, seed)
            rhs = os.path.join(tmp, name + ".rhs")
            gen.write_rhs(rhs, b)
            prefix = os.path.join(tmp, name)
            subprocess.run([exe["rgf_replay"], str(ns), str(nt), str(nd), mat, rhs, str(nrhs),
                            prefix], check=True)
            logdet, res, resn = (float(v) for v in open(prefix + ".txt").read().split())
            ld_dense, diag_dense = dense_exact(ia, ja, a)
            np.savez_compressed(
                os.path.join(HERE, f"golden_{name}.npz"), ia=ia, ja=ja, a=a, b=b, ns=ns, nt=nt,
                nd=nd, mf=np.fromfile(prefix + ".mf"), x=np.fromfile(prefix + ".x").reshape(
                    (n, nrhs), order="F"), diag=np.fromfile(prefix + ".diag"), logdet=logdet,
                res=res, resn=resn, logdet_dense=ld_dense, diag_dense=diag_dense)
            print(f"{name}: logdet={logdet:.17g} res={resn:.3g}")
        # the reference's own driver (main.C) on A11 with a one-column RHS
        mat = os.path.join(REF, "data/A_11_11_ns3_nt3_nd2.dat")
        rhs = os.path.join(tmp, "main.rhs")
        gen.write_rhs(rhs, gen.random_rhs(11, 1, 0))
        out = subprocess.run([exe["rgf_ref_main"], "3", "3", "2", mat, rhs], check=True,
                             capture_output=True, text=True).stdout
        lines = [ln for ln in out.splitlines() if not ln.startswith("The current date/time")
                 and "time:" not in ln]
        with open(os.path.join(HERE, "ref_main_A11.txt"), "w") as f:
            f.write("\n".join(lines).strip() + "\n")
        np.save(os.path.join(HERE, "ref_main_A11_rhs.npy"), gen.random_rhs(11, 1, 0))


if __name__ == "__main__":
    main()
