"""Build the CPU replay of the reference (oracle/_ref/) from its own sources.

Compiles the reference's unmodified RGF.H (through replay_driver.C) and its
unmodified main.C + Utilities.C against the host stand-ins in this folder
(MAGMA v2 subset, Fortran BLAS subset, CWC_utility entry points).  Needs the
reference tree and g++; outputs go only to oracle/_ref/.  This recipe is the
one place that locates the reference tree: $RGF_REFERENCE when set, else the
development machine's mount point (reference_root()).  Test infrastructure:
used to generate the golden vectors in tests/golden/.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
CUDA_INC = "/usr/local/cuda/include"


def reference_root() -> str:
    """The reference tree: $RGF_REFERENCE, else the development machine's mount."""
    return os.environ.get("RGF_REFERENCE", "/root/reference")


REF = reference_root()


def build() -> dict:
    if not os.path.isdir(REF):
        raise RuntimeError(f"reference sources not found at {REF}")
    cxx = shutil.which("g++")
    if cxx is None:
        raise RuntimeError("g++ not found")
    os.makedirs(OUT, exist_ok=True)
    flags = ["-O2", "-std=c++14", "-DAdd_", "-w", "-I", os.path.join(HERE, "shim"), "-I", REF,
             "-I", CUDA_INC]
    shim = os.path.join(HERE, "replay_shim.cpp")
    targets = {
        "rgf_replay": [os.path.join(HERE, "replay_driver.C"), os.path.join(REF, "Utilities.C"), shim],
        "rgf_ref_main": [os.path.join(REF, "main.C"), os.path.join(REF, "Utilities.C"), shim],
    }
    out = {}
    for name, srcs in targets.items():
        exe = os.path.join(OUT, name)
        cmd = [cxx, *flags, *srcs, "-o", exe, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"replay build failed ({name}):\n{r.stderr}")
        out[name] = exe
    return out


if __name__ == "__main__":
    print(build())
    sys.exit(0)
