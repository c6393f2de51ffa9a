"""Build recipe for the native libraries (no cmake; parallel nvcc / g++ calls).

Outputs (in-tree, git-ignored):
  state_estimation_with_cuda_gb300/lib/libsle_gb300.so  C ABI + engine + sm_103a kernels
  state_estimation_with_cuda_gb300/lib/libsegen.so      synthetic grid generator
  oracle/_build/liboracle.so                            CPU FP64 oracle (test infrastructure)
  oracle/_build/librefpin.so                            harness that runs the reference's own kernels
                                                        (test infrastructure)
  oracle/_ref/*.cubin                                   the reference's kernels, built only where its
                                                        sources are present (oracle/build_ref.py)

Every translation unit is rebuilt only when a source or header it may include
is newer than its object.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(LIB, "obj")
ORACLE = os.path.join(REPO, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CUDA_INC = "/usr/local/cuda/include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wno-unused-function"]

CORE_CU = ["kernels/network.cu", "kernels/factor.cu", "engine/engine.cu"]
CORE_CPP = ["model/model.cpp", "symbolic/symbolic.cpp", "symbolic/amd.cpp", "serve/server.cpp", "api/sle_api.cpp"]


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _headers():
    hs = glob.glob(os.path.join(CSRC, "**", "*.h"), recursive=True)
    hs += glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
    hs += glob.glob(os.path.join(CSRC, "**", "*.inc"), recursive=True)
    hs += glob.glob(os.path.join(REPO, "include", "*.h"))
    return hs


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(out, deps):
    return not os.path.exists(out) or os.path.getmtime(out) < _newest(deps)


def build_core(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    hdr = _headers()
    jobs, objs = [], []
    for rel in CORE_CU:
        src = os.path.join(CSRC, rel)
        obj = os.path.join(OBJ, rel.replace("/", "_") + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdr):
            jobs.append([NVCC] + NVCC_FLAGS + ["-I", os.path.join(REPO, "include"), "-c", src, "-o", obj])
    for rel in CORE_CPP:
        src = os.path.join(CSRC, rel)
        obj = os.path.join(OBJ, rel.replace("/", "_") + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdr):
            jobs.append(["g++"] + CXX_FLAGS + ["-I", CUDA_INC, "-I", os.path.join(REPO, "include"), "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    so = os.path.join(LIB, "libsle_gb300.so")
    if _stale(so, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", so] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"])
    return so


def build_segen():
    os.makedirs(LIB, exist_ok=True)
    src = os.path.join(CSRC, "gen", "segen.cpp")
    so = os.path.join(LIB, "libsegen.so")
    if _stale(so, [src, os.path.join(CSRC, "gen", "segen.h")]):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", src, "-o", so])
    return so


def build_oracle():
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    srcs = [os.path.join(ORACLE, "oracle.cpp")]
    hdrs = [os.path.join(ORACLE, "oracle.h")]
    so = os.path.join(ORACLE_BUILD, "liboracle.so")
    if srcs and _stale(so, srcs + hdrs):
        _run(["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-fopenmp"] + srcs + ["-o", so])
    return so


def build_refpin():
    """The reference-kernel harness (driver API; libcuda resolved at run time)."""
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    src = os.path.join(ORACLE, "refpin.cpp")
    so = os.path.join(ORACLE_BUILD, "librefpin.so")
    if _stale(so, [src]):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", CUDA_INC, src, "-o", so,
              "-L", "/usr/local/cuda/lib64/stubs", "-lcuda"])
    return so


def build_ref_kernels():
    """oracle/_ref cubins from the reference's sources, where they are present."""
    sys.path.insert(0, ORACLE)
    try:
        import build_ref
    finally:
        sys.path.pop(0)
    return build_ref.build()


def build_all(verbose=False):
    with ThreadPoolExecutor(max_workers=5) as ex:
        futs = [ex.submit(build_core, verbose), ex.submit(build_segen), ex.submit(build_oracle),
                ex.submit(build_refpin), ex.submit(build_ref_kernels)]
        return [f.result() for f in futs]


if __name__ == "__main__":
    for p in build_all(verbose="-v" in sys.argv):
        print(p)
