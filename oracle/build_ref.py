"""Build recipe for oracle/_ref: the reference's own element kernels, compiled
unchanged from its sources into cubins for the GB300 (sm_103a).

TEST INFRASTRUCTURE ONLY (the parity tests run these kernels through
oracle/refpin.cpp to pin the CPU oracle); nothing here is product code.

  oracle/_ref/kernels.cubin        <reference>/src/kernels.cu
  oracle/_ref/sparse_matrix.cubin  <reference>/src/sparse_matrix.cu

Only device code goes into a cubin: the reference's host layer (Boost,
cuSPARSE / cuSOLVER calls) is not needed.  The reference's FP32 build is
the one that compiles (its FP64 switch does not), and kernels.cu /
sparse_matrix.cu need unistd.h ahead of include/jsf_compliance.h:352.  The
outputs are git-ignored; the GPU machines use the copies built here.

Usage:  python oracle/build_ref.py [path/to/reference]
(default: the reference checkout of this build container, /root/reference).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
DEFAULT_REF = "/root/reference"
UNITS = ("kernels", "sparse_matrix")


def build(ref=DEFAULT_REF, force=False):
    """Compile the cubins when the reference sources are present; returns the
    list of cubins that exist afterwards."""
    srcs = [os.path.join(ref, "src", u + ".cu") for u in UNITS]
    outs = [os.path.join(OUT, u + ".cubin") for u in UNITS]
    if not all(os.path.exists(s) for s in srcs):
        return [o for o in outs if os.path.exists(o)]
    os.makedirs(OUT, exist_ok=True)
    for s, o in zip(srcs, outs):
        if not force and os.path.exists(o) and os.path.getmtime(o) >= os.path.getmtime(s):
            continue
        cmd = [NVCC, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
               "-I", os.path.join(ref, "include"), "-include", "unistd.h", "-w", s, "-o", o]
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError("reference kernel build failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return outs


if __name__ == "__main__":
    for path in build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF, force=True):
        print(path)
